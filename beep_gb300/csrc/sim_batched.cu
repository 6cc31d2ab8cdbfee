// Fast form, step-synchronous layout: every particle of the batch advances one
// step at a time, so that the area-mixing contraction of the force of
// infection (src/state.cc:164-219, 223-290) is one dense product over the
// whole batch per step, on the tensor cores:
//
//   Y[(p,st,a)][t] = sum_c I[(p,st,a)][c] * M[c][t]       [P*NS*G x A] . [A x A]
//
// Per step three kernels run on the model's stream:
//   bx_foi   the product, one CTA per (128-row tile of (particle, strain,
//            age) rows, target chunk): tcgen05.mma kind::f16 with M = 128
//            rows, N = the chunk's targets of the model's matrix image
//            (foi_tc.cuh: three BF16 pieces Mh + Mm + Ml of M[c][t],
//            K-major), K = sources in chunks of 32; thread 0 keeps two
//            stages full with bulk copies of the A block and the matrix chunk.
//            The counts are split into two BF16 pieces Ih + Il (exact below
//            65536) when the previous step's observation kernel packs them,
//            and the five products Ih.Mh, Ih.Mm, Ih.Ml, Il.Mh, Il.Mm
//            accumulate in FP32 in tensor memory (the dropped Il.Ml is below
//            2^-24 of each term).
//   bx_step  CTAs take (particle, column chunk) items from the step's counter:
//            NMI, transition means, keyed FP32 draws and the population
//            update per column (c, dp), with the same arithmetic and the same
//            variate streams as the fast kernel of sim_fast.cuh, and the
//            next step's infectious counts.
//   bx_obs   one CTA per particle: the step's observation terms (completed
//            observations -> compensated log-density sums), the next
//            product's A operand and the next step's strain shift.
// The particles' populations, infectious counts, contraction, observation
// slots and compensated log-likelihood partials stay in global memory (L2)
// between steps; bx_init sets them up and bx_final reduces L in FP64.
#include <algorithm>

#include "sim_fast.cuh"

namespace beep {
namespace {

constexpr int kBxRows = 128;          // MMA M: rows (particle, strain, age) per product CTA
constexpr int kBxThreads = 256;       // threads of a product CTA
constexpr int kBxK = tc::kChunkK;     // sources per chunk (the matrix image's chunking)
constexpr int kBxStages = 2;
constexpr int kBxUnits = kBxRows * kBxK / 8 / kBxThreads;   // 16-byte units of a chunk's A pieces per thread
static_assert(kBxUnits * kBxThreads * 8 == kBxRows * kBxK && kBxThreads == 2 * kBxRows, "A-operand staging split");
constexpr int kBxStepThreads = 256;   // threads of a step CTA
constexpr int kBxObsThreads = 128;    // threads of an observation CTA (one particle)
constexpr int kMaxC = 8;              // compartments of a model in this layout, at most

__device__ __forceinline__ uint32_t idesc_m128(int n)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kBxRows >> 4) << 24);
}

// One product CTA computes one 128-row tile against one target chunk (tw columns of
// the matrix): the grid is tiles x target chunks.
struct BxGeom {
	int nct, tw, nkc;
	uint32_t a_piece, b_bytes, stage;   // bytes: one A piece (128 x 32 BF16), one target chunk's B pieces, a stage
};

__host__ __device__ inline BxGeom bx_geometry(int A, int NS)
{
	const tc::Geom g = tc::geometry(A, NS);
	BxGeom x;
	x.nct = g.nct;
	x.tw = g.tw;
	x.nkc = g.nkc;
	x.a_piece = (uint32_t)kBxRows * kBxK * 2;
	x.b_bytes = g.chunk_bytes();
	x.stage = (2 * x.a_piece + x.b_bytes + 127) & ~127u;
	return x;
}

// ---------------------------------------------------------------------------
// the product Y = I . M for one tile of 128 rows

__global__ void __launch_bounds__(kBxThreads, 1) bx_foi(const ModelDev m, const BatchDev b)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ uint64_t full[kBxStages], empty[kBxStages], done;
	__shared__ uint32_t tslot;
	__shared__ int abort_flag;
	const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
	const int A = m.A, G = m.G;
	const int rows = b.P * m.NS * G;
	const BxGeom x = bx_geometry(A, m.NS);
	const int ct = blockIdx.x % x.nct;            // the target chunk
	const int r0 = (blockIdx.x / x.nct) * kBxRows;
	const tc::Geom g = tc::geometry(A, m.NS);
	unsigned char *stage0 = smem_raw;
	uint32_t tcols = 32;
	while (tcols < (uint32_t)x.tw) tcols <<= 1;
	if (warp == 0) tc::tmem_alloc(&tslot, tcols);
	if (tid == 0) {
		abort_flag = 0;
		for (int s = 0; s < kBxStages; s++) {
			tc::mbar_init(&full[s], 1);
			tc::mbar_init(&empty[s], 1);
		}
		tc::mbar_init(&done, 1);
		tc::fence_mbar_init();
	}
	tc::tc_before_sync();
	__syncthreads();
	tc::tc_after_sync();
	const uint32_t taddr = tslot;
	uint32_t pending = 0, pend_par = 0;           // thread 0: stages with a bulk load in flight, and its phase parity
	const int tile = blockIdx.x / x.nct;
	// thread 0: the A block (tile, source chunk kc) and the matrix chunk (ct, kc) into stage s
	auto load = [&](int kc, int s) {
		unsigned char *dst = stage0 + (size_t)s * x.stage;
		tc::mbar_expect_tx(&full[s], 2 * x.a_piece + x.b_bytes);
		tc::bulk_load(dst, b.bx_a + ((size_t)tile * x.nkc + kc) * 2 * x.a_piece, 2 * x.a_piece, &full[s]);
		const unsigned char *src = m.tc_image + (size_t)(ct * x.nkc + kc) * g.chunk_bytes();
		for (int pc = 0; pc < tc::kPieces; pc++)
			tc::bulk_load(dst + 2 * x.a_piece + pc * g.piece_bytes(), src + pc * g.piece_bytes(), g.piece_bytes(),
			              &full[s]);
		pending |= 1u << s;
		pend_par = (pend_par & ~(1u << s)) | ((uint32_t)((kc / kBxStages) & 1) << s);
	};
	const uint32_t id = idesc_m128(x.tw);
	const uint32_t albo = (uint32_t)kBxRows * 16, blbo = (uint32_t)x.tw * 16;
	if (tid == 0) {
		// every stage filled up front; a stage is refilled once its products are done
		bool ok = true;
		for (int kc = 0; kc < x.nkc && kc < kBxStages; kc++) load(kc, kc);
		for (int kc = 0; kc < x.nkc && ok; kc++) {
			const int s = kc % kBxStages;
			const uint32_t use = (uint32_t)(kc / kBxStages);
			ok = tc::mbar_wait(&full[s], use & 1u);
			if (!ok) break;
			pending &= ~(1u << s);
			tc::tc_after_sync();
			const uint32_t sa = tc::smem_u32(stage0 + (size_t)s * x.stage);
#pragma unroll
			for (int ks = 0; ks < kBxK / 16; ks++) {
				const uint64_t ah = tc::sdesc(sa + (uint32_t)(ks * 2) * albo, albo, 128);
				const uint64_t al = tc::sdesc(sa + x.a_piece + (uint32_t)(ks * 2) * albo, albo, 128);
				const uint32_t bb = sa + 2 * x.a_piece + (uint32_t)(ks * 2) * blbo;
				const uint64_t bh = tc::sdesc(bb, blbo, 128);
				const uint64_t bm = tc::sdesc(bb + g.piece_bytes(), blbo, 128);
				const uint64_t bl = tc::sdesc(bb + 2 * g.piece_bytes(), blbo, 128);
				tc::mma_bf16(taddr, ah, bh, id, !(kc == 0 && ks == 0));
				tc::mma_bf16(taddr, ah, bm, id, true);
				tc::mma_bf16(taddr, ah, bl, id, true);
				tc::mma_bf16(taddr, al, bh, id, true);
				tc::mma_bf16(taddr, al, bm, id, true);
			}
			tc::mma_commit(&empty[s]);
			if (kc + kBxStages < x.nkc) {
				ok = tc::mbar_wait(&empty[s], use & 1u);
				if (ok) load(kc + kBxStages, s);
			}
		}
		if (ok) tc::mma_commit(&done);
		else abort_flag = 1;
		// loads still in flight (only after a timeout) land before the CTA exits
		for (int s = 0; s < kBxStages; s++)
			if (pending & (1u << s)) tc::mbar_wait(&full[s], (pend_par >> s) & 1u);
	}
	__syncthreads();
	const bool ok = !*(volatile int *)&abort_flag && tc::mbar_wait(&done, 0);
	tc::tc_after_sync();
	if (ok) {
		// rows of warp quarter q: lanes 32q..32q+31; the two warps of a quarter split the column groups
		const int q = warp & 3, half = warp >> 2;
		const int r = r0 + q * 32 + lane;
		const int gi = r / G, a = r - gi * G;
		float *Y = b.bx_y + (size_t)gi * A * G + a;
		const int ngrp = x.tw / 16;
		for (int gp = half; gp < ngrp; gp += kBxThreads / 128) {
			float v[16];
			tc::tmem_ld16(taddr + ((uint32_t)(q * 32) << 16) + (uint32_t)(gp * 16), v);
			if (r < rows) {
#pragma unroll
				for (int i = 0; i < 16; i++) {
					const int t = ct * x.tw + gp * 16 + i;
					if (t < A) Y[(size_t)t * G] = v[i];
				}
			}
		}
	} else if (tid == 0) {
		for (int r = r0; r < r0 + kBxRows && r < rows; r += G) atomicCAS(b.status + r / (G * m.NS), 0, BEEP_TIMEOUT);
	}
	tc::tc_before_sync();
	__syncthreads();
	if (warp == 0) {
		tc::tc_after_sync();
		tc::tmem_dealloc(taddr, tcols);
	}
}

// ---------------------------------------------------------------------------
// per-particle kernels

__device__ __forceinline__ Tabs bx_tabs(const BatchDev &b, int p)
{
	const GroupDir dir = b.dirs[b.group_of ? b.group_of[p] : 0];
	const float *fp = b.fpool32;
	Tabs tb;
	tb.rate = fp + dir.transrate; tb.sus = fp + dir.susceptibility; tb.inf = fp + dir.infectivity;
	tb.beta_rows = fp + dir.beta_rows; tb.areafactor = fp + dir.areafactor; tb.Ntime = fp + dir.Ntime;
	tb.geo = fp + dir.geo_spline; tb.efoi_spline = fp + dir.efoi_spline; tb.efoi_age = fp + dir.efoi_agedist;
	tb.obs_spline = fp + dir.obs_spline;
	tb.beta_row_of = b.ipool + dir.beta_row_of; tb.efoi_ref = b.ipool + dir.efoi_ref;
	tb.efoi_mult = dir.efoi_mult >= 0 ? fp + dir.efoi_mult : nullptr;
	tb.tm_mult = dir.tm_mult >= 0 ? fp + dir.tm_mult : nullptr;
	return tb;
}

// populations of particle p (buffer k of the pair, or the single buffer), layout [comp][col]
__device__ __forceinline__ int32_t *bx_pop(const ModelDev &m, const BatchDev &b, int p, int k)
{
	const size_t popsz = (size_t)m.C * m.A * m.DP;
	return b.bx_pop + ((size_t)(b.pop_single ? 0 : k) * b.P + p) * popsz;
}

// The product's A operand for particle p: its rows (p, strain, age) of the infectious
// counts Ic [NS][A][G], split into BF16 hi and lo = bf16(v - hi), written as the
// 16-byte rows (8 consecutive sources) of the K-major core matrices of each
// (128-row tile, 32-source chunk) block [hi piece][lo piece], so that the product
// kernel bulk-loads a block per stage.  Slots of rows or sources beyond the batch
// stay zero (the buffer is cleared before a run).
__device__ void bx_pack_a(const ModelDev &m, const BatchDev &b, int p, const float *Ic, int tid, int nt)
{
	const int A = m.A, G = m.G, NS = m.NS;
	const BxGeom x = bx_geometry(A, NS);
	const int units = (A + 7) / 8, nrl = NS * G;
	// adjacent threads take adjacent rows of one source unit: their loads are the
	// contiguous ages of a source, their stores consecutive rows of a core matrix
	for (int idx = tid; idx < nrl * units; idx += nt) {
		const int u = idx / nrl, rl = idx - u * nrl;       // source unit, row (strain, age) of the particle
		const int st = rl / G, a = rl - st * G;
		const int row = p * NS * G + rl;
		const int tile = row / kBxRows, rr = row - tile * kBxRows;
		const int c0 = u * 8, kc = c0 / kBxK, kl = c0 - kc * kBxK;
		const float *src = Ic + ((size_t)st * A) * G + a;
		float v[8];
#pragma unroll
		for (int i = 0; i < 8; i++) v[i] = c0 + i < A ? src[(size_t)(c0 + i) * G] : 0.f;
		uint32_t hw[4], lw[4];
#pragma unroll
		for (int i = 0; i < 4; i++) {
			const __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * i]), h1 = __float2bfloat16_rn(v[2 * i + 1]);
			const __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * i] - __bfloat162float(h0));
			const __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * i + 1] - __bfloat162float(h1));
			hw[i] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
			lw[i] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
		}
		unsigned char *blk = b.bx_a + ((size_t)tile * x.nkc + kc) * 2 * x.a_piece;
		const uint32_t o = tc::kmajor_offset(rr, kl, kBxRows);
		*(uint4 *)(blk + o) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
		*(uint4 *)(blk + x.a_piece + o) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
	}
}

// strain shift of the susceptible population before a step (src/state.cc:392-401): the
// susceptibles of strains 1.. join strain 0's, whose pool every strain's infection draws on
__device__ __forceinline__ void strain_shift(const ModelDev &m, int32_t *pop, int tid, int nt)
{
	const int A = m.A, DP = m.DP, DPS = m.DPS, NS = m.NS, ncol = A * DP;
	const int inf_from = m.trans_from[m.infection_trans];
	for (int idx = tid; idx < A * DPS; idx += nt) {
		const int dp = idx % DPS, c = idx / DPS;
		int32_t *sp = pop + inf_from * ncol + c * DP;
		int32_t sum = 0;
		for (int st = 1; st < NS; st++) { sum += sp[DPS * st + dp]; sp[DPS * st + dp] = 0; }
		sp[dp] += sum;
	}
}

// start populations (and the first step's strain shift), infectious counts of the first
// step, cleared slots and partial sums, the steps' work counters
__global__ void __launch_bounds__(256) bx_init(const ModelDev m, const BatchDev b)
{
	const int p = blockIdx.x, tid = threadIdx.x;
	const int A = m.A, G = m.G, DP = m.DP, DPS = m.DPS, C = m.C, NS = m.NS, ncol = A * DP, popsz = C * ncol;
	int32_t *pop = bx_pop(m, b, p, 0);
	for (int k = tid; k < popsz; k += blockDim.x) {
		const int dp = k % DP, co = (k / DP) % C, c = k / (DP * C);
		pop[co * ncol + c * DP + dp] = b.ti == 0 ? m.pop_init[k] : b.pop_in[(size_t)p * popsz + k];
	}
	__syncthreads();
	if (NS > 1) {
		strain_shift(m, pop, tid, blockDim.x);
		__syncthreads();
	}
	const Tabs tb = bx_tabs(b, p);
	float *Ic = b.bx_ic + (size_t)p * NS * A * G;          // buffer 0 holds the counts of step ti
	for (int idx = tid; idx < NS * A * G; idx += blockDim.x) {
		const int a = idx % G, c = (idx / G) % A, st = idx / (G * A);
		float v = 0.f;
		for (int co = 0; co < C; co++) {
			const float inf = tb.inf[co];
			if (inf != 0.f)
				for (int dp = 0; dp < DPS; dp++)
					if (m.dp_age[dp] == a) v += inf * (float)pop[co * ncol + c * DP + st * DPS + dp];
		}
		Ic[idx] = v;
		if (!m.dp_age_unique) Ic[(size_t)b.P * NS * A * G + idx] = 0.f;   // the first step's accumulation target
	}
	__syncthreads();
	bx_pack_a(m, b, p, Ic, tid, blockDim.x);                 // the first product's operand
	for (int k = tid; k < b.nslots; k += blockDim.x) b.bx_slot[(size_t)p * b.nslots + k] = 0.f;
	for (int k = tid; k < kBxObsThreads; k += blockDim.x) b.bx_kahan[(size_t)p * kBxObsThreads + k] = make_float2(0.f, 0.f);
	if (p == 0)
		for (int k = tid; k < b.tf - b.ti; k += blockDim.x) b.bx_work[k] = 0;
}

// One step of every particle: CTAs take work items (particle p, column chunk k) from
// the step's counter.  Per column (c, dp): NMI, the transition means, the keyed draws
// and the population update, then the column's infectious count for the next step;
// the counts of observed transitions go to the step's count buffer.
template <int MG, int MB>
__global__ void __launch_bounds__(kBxStepThreads, MB) bx_step(const ModelDev m, const BatchDev b, int sett, int chunk)
{
	constexpr int NT = kBxStepThreads;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ int next_item, cur_group, reload;
	const int tid = threadIdx.x;
	const int A = m.A, G = m.G, DP = m.DP, NS = m.NS, DPS = m.DPS, C = m.C, T = m.T;
	const int ncol = A * DP, popsz = C * ncol, tnsz = T * ncol;
	const int tnrows = b.tn_full ? T : m.tn_rows;
	const int nsteps = b.tf - b.ti, s_rel = sett - b.ti;
	const int cur = s_rel & 1;
	const int rows_ic = b.P * NS * A * G;
	const int nchunk = (ncol + chunk - 1) / chunk, nitem = b.P * nchunk;
	// shared memory: the step's table slices of the current parameter set, its rates and
	// the model's small tables
	size_t off = 0;
	auto take = [&](size_t bytes) { unsigned char *q = smem_raw + off; off += (bytes + 15) & ~(size_t)15; return q; };
	float *be = (float *)take(4 * (size_t)NS * A);
	float *et = (float *)take(4 * (size_t)NS * A);
	float *Nm = (float *)take(4 * (size_t)G * G);
	float *rate = (float *)take(4 * (size_t)T * DP);
	float *sus = (float *)take(4 * (size_t)DP);
	float *inf = (float *)take(4 * (size_t)C);
	float *rcp = (float *)take(4 * 64);
	float *lnfact = (float *)take(4 * 32);
	int32_t *from = (int32_t *)take(4 * (size_t)T);
	int32_t *to = (int32_t *)take(4 * (size_t)T);
	int32_t *trow = (int32_t *)take(4 * (size_t)T);
	int32_t *age = (int32_t *)take(4 * (size_t)DPS);
	float *dgeo = (float *)take(16);
	// each thread's column: populations and transition means, [row][thread] (the 32
	// threads of a warp touch 32 consecutive words), indexed by compartment and transition
	int32_t *cpv = (int32_t *)take(4 * (size_t)kMaxC * NT) + tid;
	float *cmv = (float *)take(4 * (size_t)kMaxT * NT) + tid;
	for (int k = tid; k < T; k += NT) {
		from[k] = m.trans_from[k];
		to[k] = m.trans_to[k];
		trow[k] = b.tn_full ? k : m.tn_row[k];
	}
	for (int k = tid; k < DPS; k += NT) age[k] = m.dp_age[k];
	for (int k = tid; k < 64; k += NT) rcp[k] = k == 0 ? 0.f : 1.f / (float)k;
	for (int k = tid; k < 32; k += NT) lnfact[k] = c_lnfact[k];
	if (tid == 0) cur_group = -1;
	const int itr = m.infection_trans;
	const int inf_from = m.trans_from[itr];
	const float dt = (float)m.dt;
	const uint32_t lim = b.sampler_limit ? b.sampler_limit : 65536u;
	const float *Ic_all = b.bx_ic + (size_t)cur * rows_ic;
	float *Icn_all = b.bx_ic + (size_t)(cur ^ 1) * rows_ic;
	for (;;) {
		__syncthreads();                            // the previous item is finished with shared memory
		if (tid == 0) {
			// the next item, and whether its parameter set's tables must be loaded: decided
			// by one thread before the barrier, so that every thread takes the same branch
			// (the tables' barrier below is reached by all threads or by none)
			const int it = atomicAdd(b.bx_work + s_rel, 1);
			next_item = it;
			if (it < nitem) {
				const int g = b.group_of ? b.group_of[it / nchunk] : 0;
				reload = g != cur_group;
				cur_group = g;
			}
		}
		__syncthreads();
		const int item = next_item;
		if (item >= nitem) break;
		const int p = item / nchunk, k = item - p * nchunk;
		const Tabs tb = bx_tabs(b, p);
		if (reload) {                               // the parameter set's rates and slices (kept while it repeats)
			for (int j = tid; j < T * DP; j += NT) rate[j] = tb.rate[j];
			for (int j = tid; j < DP; j += NT) sus[j] = tb.sus[j];
			for (int j = tid; j < C; j += NT) inf[j] = tb.inf[j];
			for (int i = tid; i < NS * A; i += NT) {
				const int c = i % A;
				be[i] = __ldg(tb.beta_rows + (size_t)__ldg(tb.beta_row_of + i) * m.S + sett) *
				        __ldg(tb.areafactor + (size_t)(sett / m.div_per_time) * A + c);
				float e = __ldg(tb.efoi_spline + (size_t)__ldg(tb.efoi_ref + i) * m.S + sett) * m.inv_popsize_f;
				if (tb.efoi_mult) e *= __ldg(tb.efoi_mult + ((size_t)sett * A + c) * NS + i / A);
				et[i] = e;
			}
			for (int j = tid; j < G * G; j += NT) Nm[j] = __ldg(tb.Ntime + (size_t)sett * G * G + j);
			if (tid == 0) dgeo[0] = __ldg(tb.geo + sett);
			__syncthreads();
		}
		const uint32_t stream = b.stream_of ? b.stream_of[p] : (uint32_t)p;
		const uint32_t k0 = b.key_of ? b.key_of[p].x : b.k0, k1 = b.key_of ? b.key_of[p].y : b.k1;
		int32_t *status = b.status + p;
		const int32_t *pc = bx_pop(m, b, p, cur);
		int32_t *pn = bx_pop(m, b, p, cur ^ 1);
		const float *Ic = Ic_all + (size_t)p * NS * A * G;
		const float *Y = b.bx_y + (size_t)p * NS * A * G;
		float *Icp = Icn_all + (size_t)p * NS * A * G;
		int32_t *tn = b.bx_tn + (size_t)p * tnrows * ncol;
		const float d = dgeo[0], omd = 1.f - d;
		const int col1 = min(ncol, (k + 1) * chunk);
		// ---- per column (c, dp): NMI, means, draws, population update, next infectious count
		for (int col = k * chunk + tid; col < col1; col += NT) {
			const int c = col / DP, dp = col - c * DP;
			const int st = dp / DPS, dpl = dp - st * DPS, a = age[dpl];
			for (int co = 0; co < C; co++) cpv[co * NT] = pc[co * ncol + col];
			if (b.pop_traj)
				for (int co = 0; co < C; co++)
					b.pop_traj[((size_t)p * nsteps + s_rel) * popsz + ((size_t)c * C + co) * DP + dp] = cpv[co * NT];
			U4 inv{0, 0, 0, 0};
			uint32_t inv_call = 0xffffffffu;
			float minf = 0.f;
			{
				// the infection transition's source of strain st is read at its strain-0 column
				const float popu = st == 0 ? (float)cpv[inf_from * NT] : (float)pc[inf_from * ncol + c * DP + dpl];
				if (popu > 0.f) {
					const float fac = m.M_factor_f[c], dg = m.M_diag_f[c];
					const float *Icc = Ic + (st * A + c) * G, *Yc = Y + (st * A + c) * G;
					const float *N = Nm + a * G;
					float nmi = 0.f;
#pragma unroll
					for (int aa = 0; aa < MG; aa++) {
						if (aa < G) {
							const float id = __ldg(Icc + aa) * dg;
							nmi = fmaf(N[aa], (id + __ldg(Yc + aa)) * d + fac * id * omd, nmi);
						}
					}
					nmi = fmaxf(nmi, 0.f);
					const int sc = st * A + c;
					const float eage = __ldg(tb.efoi_age + (size_t)__ldg(tb.efoi_ref + sc) * G + a);
					minf = dt * popu * sus[dp] * (be[sc] * nmi + et[sc] * eage);
				}
			}
			// every mean from the step's populations before any count is applied
			for (int tr = 0; tr < T; tr++) {
				float mv;
				if (tr == itr) mv = minf;
				else {
					const float popu = (float)cpv[from[tr] * NT];
					mv = popu <= 0.f ? 0.f : dt * popu * rate[tr * DP + dp];
				}
				if (tb.tm_mult) mv *= __ldg(tb.tm_mult + ((size_t)sett * A + c) * T * DP + tr * DP + dp);
				cmv[tr * NT] = mv;
			}
			for (int tr = 0; tr < T; tr++) {
				const float mean = cmv[tr * NT];
				int32_t n = 0;
				if (mean > 0.f) {
					if (mean > 1.0e9f) atomicCAS(status, 0, BEEP_COUNT_OVERFLOW);
					else {
						n = poisson_fp32(mean, k0, k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett, stream, inv, inv_call,
						                 rcp, lnfact, lim);
						if (n < 0) { atomicCAS(status, 0, BEEP_TIMEOUT); n = 0; }
					}
				} else if (mean != mean) atomicCAS(status, 0, BEEP_NAN_RATE);
				const int row = trow[tr];
				if (row >= 0) tn[row * ncol + col] = n;
				if (b.tn_traj) b.tn_traj[((size_t)p * nsteps + s_rel) * tnsz + ((size_t)c * T + tr) * DP + dp] = n;
				if (n != 0) {
					cpv[from[tr] * NT] -= n;
					cpv[to[tr] * NT] += n;
				}
			}
			float iv = 0.f;
			for (int co = 0; co < C; co++) {
				const int32_t v = cpv[co * NT];
				pn[co * ncol + col] = v;
				if (inf[co] != 0.f) iv = fmaf(inf[co], (float)v, iv);
			}
			if (m.dp_age_unique) Icp[(st * A + c) * G + a] = iv;
			else atomicAdd(Icp + (st * A + c) * G + a, iv);   // cleared by the step's observation kernel
		}
	}
}

// The step's observation terms of particle p (completed observations -> log-density,
// compensated per thread), then the next step's strain shift; with several dp per age
// the next infectious counts are accumulated by atomics, so the buffer the step after
// next accumulates into is cleared here.
__global__ void __launch_bounds__(kBxObsThreads) bx_obs(const ModelDev m, const BatchDev b, int sett)
{
	const int p = blockIdx.x, tid = threadIdx.x;
	const int A = m.A, G = m.G, NS = m.NS, ncol = A * m.DP;
	const int tnrows = b.tn_full ? m.T : m.tn_rows;
	const int s_rel = sett - b.ti, cur = s_rel & 1;
	const Tabs tb = bx_tabs(b, p);
	const int32_t *pc = bx_pop(m, b, p, cur);
	const int32_t *tn = b.bx_tn + (size_t)p * tnrows * ncol;
	float *slot = b.bx_slot + (size_t)p * b.nslots;
	float2 kah = b.bx_kahan[(size_t)p * kBxObsThreads + tid];
	float Lsum = kah.x, Lcmp = kah.y;
	const int a0 = b.step_ptr[s_rel], a1 = b.step_ptr[s_rel + 1];
	// one task ahead: the next task's record, slot and first cell are loaded before the
	// current one is summed (the observations active at a step have distinct slots); each
	// task's sum and the thread's log-density sum keep their order
	auto first_of = [&](const int4 &q0) {
		const int cell = q0.z;
		return (q0.w & 0x7fffffff) > 0 ? (cell >= 0 ? (float)tn[cell] : (float)pc[-1 - cell]) : 0.f;
	};
	int k = a0 + tid;
	int4 n0 = make_int4(0, 0, 0, 0), n1 = make_int4(0, 0, 0, 0);
	float nv = 0.f, nf = 0.f;
	if (k < a1) {
		n0 = __ldg(b.tasks + 2 * k);
		n1 = __ldg(b.tasks + 2 * k + 1);
		nv = slot[n0.x];
		nf = first_of(n0);
	}
	for (; k < a1; k += kBxObsThreads) {
		const int4 q0 = n0, q1 = n1;
		float x = nv;
		const float f = nf;
		const int kn = k + kBxObsThreads;
		if (kn < a1) {
			n0 = __ldg(b.tasks + 2 * kn);
			n1 = __ldg(b.tasks + 2 * kn + 1);
			nv = slot[n0.x];
			nf = first_of(n0);
		}
		const float fac = __int_as_float(q1.x);
		const int spl = q1.y;
		const float w = spl < 0 ? fac : fac * tb.obs_spline[(size_t)spl * m.S + sett];
		const int nc = q0.w & 0x7fffffff;
		if (nc > 0) x = fmaf(w, f, x);
		if (q1.w != 0) {                  // consecutive counts or populations: no cell list
			const int32_t *src = q1.w == 1 ? tn + q0.z : pc + (-1 - q0.z);
#pragma unroll 4
			for (int i = 1; i < nc; i++) x = fmaf(w, (float)src[i], x);
		} else {
			for (int i = 1; i < nc; i++) {
				const int cell = __ldg((b.tn_full ? m.obs_cells_full : m.obs_cells_f) + q1.z + i);
				x = fmaf(w, cell >= 0 ? (float)tn[cell] : (float)pc[-1 - cell], x);
			}
		}
		if (q0.w < 0) {                  // the observation's last step: log-density
			const float lp = obs_lp_fast(x, q0.y, m);
			x = 0.f;
			const float y = lp - Lcmp;      // Kahan
			const float tt = Lsum + y;
			Lcmp = (tt - Lsum) - y;
			Lsum = tt;
		}
		slot[q0.x] = x;
	}
	if (Lsum != kah.x || Lcmp != kah.y) b.bx_kahan[(size_t)p * kBxObsThreads + tid] = make_float2(Lsum, Lcmp);
	if (sett + 1 < b.tf) {
		// the next product's operand from the counts the step kernel left for the next step
		bx_pack_a(m, b, p, b.bx_ic + (size_t)(cur ^ 1) * b.P * NS * A * G + (size_t)p * NS * A * G, tid,
		          kBxObsThreads);
		if (NS > 1) strain_shift(m, bx_pop(m, b, p, cur ^ 1), tid, kBxObsThreads);
		if (!m.dp_age_unique) {
			float *Ic = b.bx_ic + (size_t)cur * b.P * NS * A * G + (size_t)p * NS * A * G;
			for (int k = tid; k < NS * A * G; k += kBxObsThreads) Ic[k] = 0.f;
		}
	}
}

// L per particle (FP64 reduction of the threads' compensated partial sums) and final populations
__global__ void __launch_bounds__(256) bx_final(const ModelDev m, const BatchDev b)
{
	__shared__ double red[8];
	const int p = blockIdx.x, tid = threadIdx.x;
	const int A = m.A, DP = m.DP, C = m.C, ncol = A * DP, popsz = C * ncol;
	if (b.L) {
		double S = 0.0;
		for (int k = tid; k < kBxObsThreads; k += blockDim.x) {
			const float2 v = b.bx_kahan[(size_t)p * kBxObsThreads + k];
			S += (double)v.x - (double)v.y;
		}
		for (int o = 16; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
		if ((tid & 31) == 0) red[tid >> 5] = S;
		__syncthreads();
		if (tid == 0) {
			double t = 0.0;
			for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
			if (t != t) atomicCAS(b.status + p, 0, BEEP_NAN_RATE);
			b.L[p] = t;
		}
	}
	if (b.pop_out) {
		const int32_t *pf = bx_pop(m, b, p, (b.tf - b.ti) & 1);
		for (int k = tid; k < popsz; k += blockDim.x) {
			const int dp = k % DP, co = (k / DP) % C, c = k / (DP * C);
			b.pop_out[(size_t)p * popsz + k] = pf[co * ncol + c * DP + dp];
		}
	}
}

template <int MG, int MB>
int launch_steps(const ModelDev &m, const BatchDev &b, size_t smem_step, int sms, cudaStream_t st, cudaEvent_t *ev)
{
	auto kstep = bx_step<MG, MB>;
	cudaError_t e = allow_dynamic_smem(kstep, smem_step);
	if (e != cudaSuccess) return (int)e;
	const BxGeom x = bx_geometry(m.A, m.NS);
	const size_t smem_foi = (size_t)kBxStages * x.stage;
	e = allow_dynamic_smem(bx_foi, smem_foi);
	if (e != cudaSuccess) return (int)e;
	const int rows = b.P * m.NS * m.G;
	const int ntile = (rows + kBxRows - 1) / kBxRows * x.nct;   // (row tile, target chunk) pairs
	// columns per work item: a multiple of the CTA's threads (a particle's columns then take
	// the same passes whatever the multiple), as large as leaves six items per CTA of the
	// grid -- each item costs two barriers, a counter and (parameter set per particle) the
	// reload of the step's table slices
	const int ncol = m.A * m.DP, grid0 = sms * MB;
	int chunk = kBxStepThreads;
	for (int c2 = 2 * kBxStepThreads; c2 < ncol + kBxStepThreads; c2 += kBxStepThreads) {
		if ((long long)b.P * ((ncol + c2 - 1) / c2) < 6LL * grid0) break;
		chunk = c2;
	}
	const int nitem = b.P * ((ncol + chunk - 1) / chunk);
	const int grid = std::min(nitem, grid0);
	e = cudaMemsetAsync(b.bx_a, 0, batched_a_bytes(m, b.P), st);   // padding rows and sources stay zero
	if (e != cudaSuccess) return (int)e;
	bx_init<<<b.P, 256, 0, st>>>(m, b);
	for (int s = b.ti; s < b.tf; s++) {
		cudaEvent_t *e4 = ev ? ev + 4 * (s - b.ti) : nullptr;   // before and after each of the step's kernels
		if (e4) cudaEventRecord(e4[0], st);
		bx_foi<<<ntile, kBxThreads, smem_foi, st>>>(m, b);
		if (e4) cudaEventRecord(e4[1], st);
		kstep<<<grid, kBxStepThreads, smem_step, st>>>(m, b, s, chunk);
		if (e4) cudaEventRecord(e4[2], st);
		bx_obs<<<b.P, kBxObsThreads, 0, st>>>(m, b, s);
		if (e4) cudaEventRecord(e4[3], st);
	}
	bx_final<<<b.P, 256, 0, st>>>(m, b);
	return (int)cudaGetLastError();
}

}  // namespace

bool batched_supported(const ModelDev &m)
{
	return m.tc_image != nullptr && tc::supported(m.A, m.NS) && m.C <= kMaxC && m.T <= kMaxT && m.G <= 16 &&
	       (size_t)kBxStages * bx_geometry(m.A, m.NS).stage <= 227 * 1024;
}

size_t batched_step_smem(const ModelDev &m, int)
{
	auto r = [](size_t x) { return (x + 15) & ~(size_t)15; };
	const size_t A = m.A, G = m.G, DP = m.DP, NS = m.NS, C = m.C, T = m.T, DPS = m.DPS;
	return 2 * r(4 * NS * A) + r(4 * G * G) + r(4 * T * DP) + r(4 * DP) + r(4 * C) + r(4 * 64) + r(4 * 32) +
	       3 * r(4 * T) + r(4 * DPS) + 16 + 4 * (size_t)(kMaxC + kMaxT) * kBxStepThreads;
}

int batched_obs_threads() { return kBxObsThreads; }

int batched_prepare() { return prepare_constants(); }

int batched_launches(int nsteps) { return 3 * nsteps + 2; }

size_t batched_a_bytes(const ModelDev &m, int P)
{
	const BxGeom x = bx_geometry(m.A, m.NS);
	const size_t tiles = ((size_t)P * m.NS * m.G + kBxRows - 1) / kBxRows;
	return tiles * (size_t)x.nkc * 2 * x.a_piece;
}

int launch_sim_batched(const ModelDev &m, const BatchDev &b, int sms, void *stream, void *events)
{
	if (b.P == 0) return 0;
	if (!batched_supported(m) || !b.bx_pop || b.mode != 0) return (int)cudaErrorInvalidValue;
	const int e0 = prepare_constants();
	if (e0 != 0) return e0;
	const size_t smem = batched_step_smem(m, 0);
	cudaStream_t st = (cudaStream_t)stream;
	cudaEvent_t *ev = (cudaEvent_t *)events;
	return m.G <= 4 ? launch_steps<4, 6>(m, b, smem, sms, st, ev) : m.G <= 8 ? launch_steps<8, 6>(m, b, smem, sms, st, ev)
	     : m.G <= 12 ? launch_steps<12, 6>(m, b, smem, sms, st, ev) : launch_steps<16, 5>(m, b, smem, sms, st, ev);
}

}  // namespace beep
