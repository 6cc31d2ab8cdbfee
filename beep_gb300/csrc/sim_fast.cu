// Fast (mixed-precision) form of the tau-leap + observation log-likelihood.
//
// One CTA keeps one particle resident in shared memory for the whole step
// range: populations, the step's transition counts, the infectious counts and
// the force-of-infection map never leave the SM.  HBM is touched only for the
// parameter tables (shared by many particles, served from L2), the
// observation index and the final outputs.
//
// Arithmetic: rates, means and the Poisson sampler in FP32; the area-mixing
// contraction Imap = M^T I (src/state.cc:223-290) in FP32 from the current
// infectious counts (the reference updates Imap incrementally in FP64; both
// are the same sum, here formed directly each step); observation sums of
// integer counts in FP64 (exact); per-observation log-densities in FP32,
// summed per thread with compensation (Kahan) and reduced across the CTA in
// FP64.  The variates come from the same keyed Philox streams as the plain
// form (same counters, same words), so a particle follows the FP64
// trajectory except where an FP32 comparison lands on the other side of a
// near tie.
//
// Per step (barriers between phases):
//   1 infectious counts Icnt[st][c][a] from pop           (set_I_from_pop)
//   2 Imap[st][t][a] = sum_c M[c][t] Icnt[st][c][a]      (genQ.M contraction)
//   3 per column (c, dp): NMI, means, draws -> tn          (get_NMI, set_transmean, draws)
//   4 observation gathers of the step                     (get_obs_value_section)
//   5 population update; completed observations -> log-density
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "beep_internal.h"
#include "rng_fp64.cuh"

namespace beep {
namespace {

constexpr int kFastThreads = 640;

__constant__ float c_rcp[256];   // 1/k for the inversion recurrence

__device__ __forceinline__ float u01_f(uint32_t w)
{
	return __uint2float_rn(w) * 2.3283064365386963e-10f + 1.1641532182693481e-10f;
}

// FP32 Poisson draw on the keyed stream of poisson_fp64 (same counters/words).
__device__ __forceinline__ int32_t poisson_fp32(float mean, uint32_t k0, uint32_t k1, uint32_t col, uint32_t tr,
                                                uint32_t sett, uint32_t stream, U4 &inv, uint32_t &inv_call)
{
	if (!(mean > 0.f)) return 0;
	if (mean < 10.f) {
		const uint32_t call = tr >> 2;
		if (inv_call != call) {
			inv = philox10(U4{col, sett, stream, (PURPOSE_INV << 24) | call}, k0, k1);
			inv_call = call;
		}
		const float u = u01_f(word_of(inv, tr & 3u));
		float p = expf(-mean);
		float F = p;
		int32_t k = 0;
		while (u > F && k < 255) {
			k++;
			p = p * mean * c_rcp[k];
			const float Fn = F + p;
			if (Fn == F) break;          // FP32 tail exhausted
			F = Fn;
		}
		return k;
	}
	const float slam = sqrtf(mean);
	const float loglam = logf(mean);
	const float b = 0.931f + 2.53f * slam;
	const float a = -0.059f + 0.02483f * b;
	const float invalpha = 1.1239f + 1.1328f / (b - 3.4f);
	const float vr = 0.9277f - 3.6224f / (b - 2.0f);
	const float log_invalpha = logf(invalpha);
	for (uint32_t it = 0; it < 65536u; it++) {
		const U4 r = philox10(U4{col, sett, stream, (PURPOSE_PTRS << 24) | (tr << 16) | it}, k0, k1);
		const float U = u01_f(r.x) - 0.5f;
		const float V = u01_f(r.y);
		const float us = 0.5f - fabsf(U);
		const float k = floorf((2.0f * a / us + b) * U + mean + 0.43f);
		if (us >= 0.07f && V <= vr) return (int32_t)k;
		if (k < 0.0f || (us < 0.013f && V > us)) continue;
		const float lhs = logf(V) + log_invalpha - logf(a / (us * us) + b);
		const float rhs = -mean + k * loglam - lgammaf(k + 1.0f);
		if (lhs <= rhs) return (int32_t)k;
	}
	return -1;
}

__device__ float obs_lp_fast(float vf, int o, const ModelDev &m)
{
	const int kind = m.obs_kind[o], model = m.obs_model[o];
	double value = vf < 0.f ? 0.0 : (double)vf;
	if (kind == BEEP_OBSVAL_UNKNOWN) return 0.f;
	if (kind == BEEP_OBSVAL_VALUE && (model == BEEP_OBS_NORMAL || model == BEEP_OBS_NORMAL_PERCENT)) {
		const float2 np = m.obs_np[o];                       // (-0.5 log(2 pi var), 1/(2 var))
		const float d = m.obs_value_f[o] - (vf < 0.f ? 0.f : vf);
		return np.x - d * d * np.y;
	}
	if (kind == BEEP_OBSVAL_VALUE && model == BEEP_OBS_POISSON) {
		const float lam = value < 1 ? 1.f : (float)value;
		const int i = (int)(m.obs_value[o] + 0.5);
		return (float)i * logf(lam) - lam - lgammaf((float)i + 1.f);
	}
	if (kind == BEEP_OBSVAL_VALUE && model == BEEP_OBS_NEGBIN) {
		const float mm = value < 1 ? 1.f : (float)value, sh = (float)m.obs_shape[o];
		const float v = (float)(int)(m.obs_value[o] + 0.5);
		return lgammaf(sh + v) - lgammaf(v + 1.f) - lgammaf(sh) + sh * logf(sh / (sh + mm)) + v * logf(mm / (sh + mm));
	}
	// thresholded values: rare; evaluated in FP64 as the reference does (src/obsmodel.cc:251-280)
	const double thresh = m.obs_thresh[o], sd = m.obs_sd[o];
	if (model == BEEP_OBS_NORMAL || model == BEEP_OBS_NORMAL_PERCENT) {
		const double var = sd * sd;
		const double x = value < thresh ? thresh : value;
		return (float)(-0.5 * log(2 * 3.14159265358979323846 * var) - (thresh - x) * (thresh - x) / (2 * var));
	}
	const double lam = value < 1 ? 1 : value, sh = m.obs_shape[o];
	double sum = 0.0;
	for (double v = 0; v <= thresh; v++) {
		if (model == BEEP_OBS_POISSON) sum += exp(v * log(lam) - lam - lgamma(v + 1));
		else sum += exp(lgamma(sh + v) - lgamma(v + 1) - lgamma(sh) + sh * log(sh / (sh + lam)) + v * log(lam / (sh + lam)));
	}
	return (float)log(sum);
}

// Row stride of the area-mixing matrix in shared memory: congruent to 8 mod 32
// so that the FOI loop's 4 source rows x 8 targets per warp hit 32 banks.
__host__ __device__ inline int ms_lda(int A) { return A + ((40 - A % 32) % 32); }

struct FastSmem {
	float *Ms;         // [A][lda] source-major, diagonal zero (or null: M read from global)
	int32_t *pop[2];   // [A][C][DP] current / next
	int32_t *tn;       // [A][T][DP]
	float *Icnt[2];    // [NS][A][G] current / next
	float *Imap;       // [NS][A][G]
	float *slot;       // [nslots]
	float *red;        // [2*NT]
};

// Imap[st][t][a] = sum_c M[c][t] Icnt[st][c][a] (off-diagonal M).  Lane layout:
// 4 consecutive lanes share a target t and split the sources c = cg (mod 4);
// the quad's partial sums are combined with two butterfly shuffles.
template <int NT, int kMaxG>
__device__ __forceinline__ void foi(const ModelDev &m, const float *Ms, int lda, const float *Icnt, float *Imap, int tid)
{
	const int A = m.A, G = m.G;
	const int cg = tid & 3;
	for (int st = 0; st < m.NS; st++) {
		const float *I = Icnt + st * A * G;
		for (int t0 = 0; t0 < A; t0 += NT / 4) {
			const int t = t0 + (tid >> 2);
			float acc[kMaxG];
#pragma unroll
			for (int a = 0; a < kMaxG; a++) acc[a] = 0.f;
			if (t < A) {
				if (Ms) {
#pragma unroll 2
					for (int c = cg; c < A; c += 4) {
						const float mv = Ms[c * lda + t];
						const float *Ic = I + c * G;
#pragma unroll
						for (int a = 0; a < kMaxG; a++)
							if (a < G) acc[a] = fmaf(mv, Ic[a], acc[a]);
					}
				} else {
					for (int c = cg; c < A; c += 4) {
						const float mv = __ldg(m.Mdense + (size_t)c * A + t);
						const float *Ic = I + c * G;
#pragma unroll
						for (int a = 0; a < kMaxG; a++)
							if (a < G) acc[a] = fmaf(mv, Ic[a], acc[a]);
					}
				}
			}
#pragma unroll
			for (int a = 0; a < kMaxG; a++) {
				if (a < G) {
					acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 1);
					acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 2);
				}
			}
			if (t < A && cg == 0)
#pragma unroll
				for (int a = 0; a < kMaxG; a++)
					if (a < G) Imap[(st * A + t) * G + a] = acc[a];
		}
	}
}

template <int NT, int kMaxG>
__global__ void __launch_bounds__(NT, 1) sim_fast_kernel(const ModelDev m, const BatchDev b)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const int p = blockIdx.x;
	if (p >= b.P) return;
	const int tid = threadIdx.x;
	const int A = m.A, G = m.G, DP = m.DP, NS = m.NS, DPS = m.DPS, C = m.C, T = m.T;
	const int popsz = A * C * DP, tnsz = A * T * DP, agsz = NS * A * G, ncol = A * DP;
	const int nsteps = b.tf - b.ti;
	const int lda = ms_lda(A);
	const GroupDir dir = b.dirs[b.group_of ? b.group_of[p] : 0];
	const uint32_t stream = b.stream_of ? b.stream_of[p] : (uint32_t)p;
	const float *fp = b.fpool32;
	const int32_t *ip = b.ipool;
	const float *transrate = fp + dir.transrate, *sus = fp + dir.susceptibility, *infectivity = fp + dir.infectivity;
	const float *beta_rows = fp + dir.beta_rows, *areafactor = fp + dir.areafactor, *Ntime = fp + dir.Ntime;
	const float *geo = fp + dir.geo_spline, *efoi_spline = fp + dir.efoi_spline, *efoi_age = fp + dir.efoi_agedist;
	const double *obs_spline = b.fpool + dir.obs_spline;
	const int32_t *beta_row_of = ip + dir.beta_row_of, *efoi_ref = ip + dir.efoi_ref;
	int32_t *status = b.status + p;

	FastSmem s;
	{
		size_t off = 0;
		auto take = [&](size_t bytes) { unsigned char *q = smem_raw + off; off += (bytes + 15) & ~(size_t)15; return q; };
		s.Ms = b.m_in_smem ? (float *)take(sizeof(float) * A * lda) : nullptr;
		s.pop[0] = (int32_t *)take(sizeof(int32_t) * popsz);
		s.pop[1] = (int32_t *)take(sizeof(int32_t) * popsz);
		s.tn = (int32_t *)take(sizeof(int32_t) * tnsz);
		s.Icnt[0] = (float *)take(sizeof(float) * agsz);
		s.Icnt[1] = (float *)take(sizeof(float) * agsz);
		s.Imap = (float *)take(sizeof(float) * agsz);
		s.slot = (float *)take(sizeof(float) * b.nslots);
		s.red = (float *)take(sizeof(float) * 2 * NT);
	}
	if (s.Ms)
		for (int k = tid; k < A * A; k += NT) s.Ms[(k / A) * lda + k % A] = m.Mdense[k];
	for (int k = tid; k < popsz; k += NT) s.pop[0][k] = b.ti == 0 ? m.pop_init[k] : b.pop_in[(size_t)p * popsz + k];
	for (int k = tid; k < b.nslots; k += NT) s.slot[k] = 0.f;
	for (int k = tid; k < agsz; k += NT) s.Icnt[1][k] = 0.f;
	__syncthreads();
	// infectious counts of the start populations (set_I_from_pop, src/state.cc:223-290)
	for (int idx = tid; idx < agsz; idx += NT) {
		const int a = idx % G, c = (idx / G) % A, st = idx / (G * A);
		float v = 0.f;
		for (int co = 0; co < C; co++) {
			const float inf = infectivity[co];
			if (inf != 0.f)
				for (int dp = 0; dp < DPS; dp++)
					if (m.dp_age[dp] == a) v += inf * (float)s.pop[0][(c * C + co) * DP + st * DPS + dp];
		}
		s.Icnt[0][idx] = v;
	}
	__syncthreads();
	foi<NT, kMaxG>(m, s.Ms, lda, s.Icnt[0], s.Imap, tid);
	float Lsum = 0.f, Lcmp = 0.f;           // compensated per-thread log-likelihood
	__syncthreads();

	const int itr = m.infection_trans;
	const int inf_from = m.trans_from[itr];
	const float dt = (float)m.dt;
	const float inv_popsize = (float)(1.0 / m.popsize);
	int cur = 0;
	for (int sett = b.ti; sett < b.tf; sett++) {
		int32_t *pc = cur ? s.pop[1] : s.pop[0], *pn = cur ? s.pop[0] : s.pop[1];
		const float *Ic_cur = cur ? s.Icnt[1] : s.Icnt[0];
		float *Ic_nxt = cur ? s.Icnt[0] : s.Icnt[1];
		if (NS > 1) {
			// strain shift of the susceptible population (src/state.cc:392-401)
			for (int idx = tid; idx < A * DPS; idx += NT) {
				const int dp = idx % DPS, c = idx / DPS;
				int32_t *sp = pc + (c * C + inf_from) * DP;
				int32_t sum = 0;
				for (int st = 1; st < NS; st++) { sum += sp[DPS * st + dp]; sp[DPS * st + dp] = 0; }
				sp[dp] += sum;
			}
			__syncthreads();
		}

		// ---- A: per column (c, dp): NMI, means, draws, next population, next infectious count
		const float d = geo[sett], omd = 1.f - d;
		for (int col = tid; col < ncol; col += NT) {
			const int c = col / DP, dp = col % DP;
			const int st = dp / DPS, dpl = dp % DPS, a = m.dp_age[dpl];
			U4 inv{0, 0, 0, 0};
			uint32_t inv_call = 0xffffffffu;
			int32_t *pcol = pc + c * C * DP + dp, *ncol_p = pn + c * C * DP + dp;
			for (int co = 0; co < C; co++) ncol_p[co * DP] = pcol[co * DP];
			for (int tr = 0; tr < T; tr++) {
				float mean;
				if (tr == itr) {
					const float popu = (float)pc[(c * C + inf_from) * DP + dpl];
					if (popu <= 0.f) mean = 0.f;
					else {
						const float fac = m.M_factor_f[c], dg = m.M_diag_f[c];
						const float *Ic = Ic_cur + (st * A + c) * G, *Im = s.Imap + (st * A + c) * G;
						const float *N = Ntime + ((size_t)sett * G + a) * G;
						float nmi = 0.f;
						for (int aa = 0; aa < G; aa++) {
							const float id = Ic[aa] * dg;
							nmi = fmaf(N[aa], (id + Im[aa]) * d + fac * id * omd, nmi);
						}
						nmi = fmaxf(nmi, 0.f);
						const float be = beta_rows[(size_t)beta_row_of[st * A + c] * m.S + sett] *
						                 areafactor[(size_t)(sett / m.div_per_time) * A + c];
						const int ei = efoi_ref[st * A + c];
						const float eta = efoi_spline[(size_t)ei * m.S + sett] * inv_popsize * efoi_age[(size_t)ei * G + a];
						mean = dt * popu * sus[dp] * (be * nmi + eta);
					}
				} else {
					const float popu = (float)pcol[m.trans_from[tr] * DP];
					mean = popu <= 0.f ? 0.f : dt * popu * transrate[tr * DP + dp];
				}
				int32_t n = 0;
				if (mean != mean) atomicCAS(status, 0, BEEP_NAN_RATE);
				else if (mean > 0.f) {
					if (mean > 1.0e9f) atomicCAS(status, 0, BEEP_COUNT_OVERFLOW);
					else {
						n = poisson_fp32(mean, b.k0, b.k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett, stream, inv, inv_call);
						if (n < 0) { atomicCAS(status, 0, BEEP_TIMEOUT); n = 0; }
					}
				}
				s.tn[(c * T + tr) * DP + dp] = n;
				if (n != 0) {
					ncol_p[m.trans_from[tr] * DP] -= n;
					ncol_p[m.trans_to[tr] * DP] += n;
				}
			}
			float iv = 0.f;
			for (int co = 0; co < C; co++) {
				const float inf = infectivity[co];
				if (inf != 0.f) iv = fmaf(inf, (float)ncol_p[co * DP], iv);
			}
			if (m.dp_age_unique) Ic_nxt[(st * A + c) * G + a] = iv;
			else atomicAdd(Ic_nxt + (st * A + c) * G + a, iv);
		}
		__syncthreads();

		// ---- B: observation sums of the step (completed ones -> log-density); FOI for the next step
		if (b.pop_traj)
			for (int k = tid; k < popsz; k += NT) b.pop_traj[((size_t)p * nsteps + (sett - b.ti)) * popsz + k] = pc[k];
		if (b.tn_traj)
			for (int k = tid; k < tnsz; k += NT) b.tn_traj[((size_t)p * nsteps + (sett - b.ti)) * tnsz + k] = s.tn[k];
		const int a0 = b.step_ptr[sett - b.ti], a1 = b.step_ptr[sett - b.ti + 1];
		for (int k = a0 + tid; k < a1; k += NT) {
			const int pos = b.step_obs[k];
			const int o = b.scored[pos];
			const float fac = (float)m.obs_factor[o];
			const int spl = m.obs_spline[o];
			const int sl = b.slot_of[pos];
			float v = s.slot[sl];
			for (int q = m.obs_cell_ptr[o]; q < m.obs_cell_ptr[o + 1]; q++) {
				const int cell = m.obs_cells[q];
				const float num = cell >= 0 ? (float)s.tn[cell] : (float)pc[-1 - cell];
				v += spl < 0 ? fac * num : fac * num * (float)obs_spline[(size_t)spl * m.S + sett];
			}
			if (sett == m.obs_sett_f[o] - 1) {
				const float lp = obs_lp_fast(v, o, m);
				v = 0.f;
				const float y = lp - Lcmp;      // Kahan
				const float tt = Lsum + y;
				Lcmp = (tt - Lsum) - y;
				Lsum = tt;
			}
			s.slot[sl] = v;
		}
		if (!m.dp_age_unique)
			for (int k = tid; k < agsz; k += NT) (cur ? s.Icnt[1] : s.Icnt[0])[k] = 0.f;   // next step's accumulation target
		foi<NT, kMaxG>(m, s.Ms, lda, Ic_nxt, s.Imap, tid);
		__syncthreads();
		cur ^= 1;
	}

	if (b.pop_out)
		for (int k = tid; k < popsz; k += NT) b.pop_out[(size_t)p * popsz + k] = (cur ? s.pop[1] : s.pop[0])[k];
	if (b.L) {
		s.red[tid] = Lsum;
		s.red[NT + tid] = Lcmp;
		__syncthreads();
		if (tid < 32) {
			double S = 0.0;
			for (int k = tid; k < NT; k += 32) S += (double)s.red[k] - (double)s.red[NT + k];
			for (int o = 16; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
			if (tid == 0) {
				if (S != S) atomicCAS(status, 0, BEEP_NAN_RATE);
				b.L[p] = S;
			}
		}
	}
}

}  // namespace

size_t fast_smem_bytes(const ModelDev &m, int nslots, bool m_in_smem)
{
	auto r = [](size_t x) { return (x + 15) & ~(size_t)15; };
	const size_t agsz = (size_t)m.NS * m.A * m.G;
	return (m_in_smem ? r(4 * (size_t)m.A * ms_lda(m.A)) : 0) + 2 * r(4 * (size_t)m.A * m.C * m.DP) +
	       r(4 * (size_t)m.A * m.T * m.DP) + 3 * r(4 * agsz) + r(4 * (size_t)nslots) + r(4 * 2 * (size_t)kFastThreads);
}

int fast_threads() { return kFastThreads; }

int launch_sim_fast(const ModelDev &m, const BatchDev &b, void *stream)
{
	static bool init = false;
	if (!init) {
		float rcp[256];
		rcp[0] = 0.f;
		for (int k = 1; k < 256; k++) rcp[k] = 1.0f / (float)k;
		cudaMemcpyToSymbol(c_rcp, rcp, sizeof rcp);
		init = true;
	}
	if (b.P == 0) return 0;
	if (m.G > 16) return (int)cudaErrorInvalidValue;
	const size_t smem = fast_smem_bytes(m, b.nslots, b.m_in_smem != 0);
	auto kern = m.G <= 4 ? sim_fast_kernel<kFastThreads, 4> : sim_fast_kernel<kFastThreads, 16>;
	cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
	if (e != cudaSuccess) return (int)e;
	kern<<<b.P, kFastThreads, smem, (cudaStream_t)stream>>>(m, b);
	return (int)cudaGetLastError();
}

}  // namespace beep
