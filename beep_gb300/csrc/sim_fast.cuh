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
// This header holds the device code; it is compiled by sim_fast.cu (the
// simulation kernels) and mbp_fast.cu (the MBP-chain variants), each with
// its own copy of the constant tables (prepare_constants).
//
// Per step (barriers between phases):
//   1 infectious counts Icnt[st][c][a] from pop           (set_I_from_pop)
//   2 Imap[st][t][a] = sum_c M[c][t] Icnt[st][c][a]      (genQ.M contraction)
//   3 per column (c, dp): NMI, means, draws -> tn          (get_NMI, set_transmean, draws)
//   4 observation gathers of the step                     (get_obs_value_section)
//   5 population update; completed observations -> log-density
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "beep_internal.h"
#include "rng_fp64.cuh"
#include "foi_tc.cuh"

namespace beep {
namespace {

constexpr int kFastThreads = 640;   // largest CTA; smaller models use 128 or 256 threads
constexpr int kMaxT = 8;            // transitions per model in the fast form's usual instantiations
constexpr int kWideT = 16;          // transitions in the wide instantiation (one 640-thread CTA per SM)
constexpr int kWideG = 20;          // age groups in the wide instantiation

__constant__ float c_lnfact[32];   // log k!, k < 32

__device__ __forceinline__ float u01_f(uint32_t w)
{
	return __uint2float_rn(w) * 2.3283064365386963e-10f + 1.1641532182693481e-10f;
}

// Shared-memory image of one particle and of the tables it reads.  State is
// stored column-major (index [comp or trans][col], col = c*DP + dp) so that the
// 32 columns of a warp touch 32 consecutive words.
struct FastSmem {
	float *Ms;            // [A][lda] source-major area mixing, diagonal zero (or null)
	int32_t *pop0, *pop1; // [C][ncol] current / next (swapped every step)
	int32_t *tn;          // [T][ncol]
	float *Ic0, *Ic1;     // [NS][A][G] infectious counts, current / next
	float *Imap;          // [NS][A][G]
	float *slot;          // [nslots]
	// per-particle constants
	int32_t *from, *to;   // [T]
	int32_t *trow;        // [T] row of the transition in tn, or -1 (not observed)
	int32_t *age;         // [DPS]
	float *inf;           // [C]
	float *rate;          // [T][DP]
	float *sus;           // [DP]
	float *rcp;           // [64] 1/k
	float *lnfact;        // [32] log k!
	int32_t *brow, *eref; // [NS][A] beta row and efoi spline of each (strain, area)
	float *eage;          // [nefoi][G] efoi age distributions (when they fit)
	// per-step slices, double-buffered: [0] the step simulated, [1] the next one
	float *be0, *be1;     // [NS][A] beta * areafactor
	float *et0, *et1;     // [NS][A] external force of infection per capita (before the age factor)
	float *N0, *N1;       // [G][G] age mixing
	float *dgeo;          // [2] geographic spline value
	float *red;           // [2*NT]
	float *mv;            // [T][NT] each thread's transition means (320-thread CTAs, whose registers are tight)
	float *pm;            // [T][ncol] the step's transition means (draws per (transition, column)), or null
};

__host__ __device__ inline int ms_lda(int A) { return A + ((40 - A % 32) % 32); }

// log k! - (-mean + k log mean), written without cancellation: for k >= 32
// Stirling's series of log Gamma(k+1) with x = (mean - n)/n, n = k+1, gives
// rhs = k (log1p(x) - x) - x - log(n)/2 - log(2 pi)/2 - 1/(12n) + 1/(360n^3).
__device__ __forceinline__ float ptrs_rhs(float k, float mean, float loglam, const float *lnfact)
{
	if (k < 32.f) return fmaf(k, loglam, -mean) - lnfact[(int)k];
	const float n = k + 1.f;
	const float in = __fdividef(1.f, n);
	const float x = (mean - n) * in;
	const float corr = in * (0.083333333f - in * in * 0.0027777778f);
	return k * (log1pf(x) - x) - x - 0.5f * __logf(n) - 0.91893853f - corr;
}

// FP32 Poisson draw on the keyed stream of the FP64 form (same counters/words).
// The Philox blocks are computed by the warp's calling lanes together: when a
// lane of the warp needs the inversion words of its column or the first PTRS
// pair, every calling lane computes its own (same counters, so the same
// values), instead of the warp issuing the block once for the inversion lanes
// and again for the PTRS lanes.
__device__ __forceinline__ int32_t poisson_fp32(float mean, uint32_t k0, uint32_t k1, uint32_t col, uint32_t tr,
                                                uint32_t sett, uint32_t stream, U4 &inv, uint32_t &inv_call,
                                                const float *rcp, const float *lnfact, uint32_t limit)
{
	const unsigned act = __activemask();
	const bool big = mean >= 10.f;
	const uint32_t call = tr >> 2;
	if (__any_sync(act, !big && inv_call != call)) {
		inv = philox10(U4{col, sett, stream, (PURPOSE_INV << 24) | call}, k0, k1);
		inv_call = call;
	}
	U4 r0{0, 0, 0, 0};
	if (__any_sync(act, big)) r0 = philox10(U4{col, sett, stream, (PURPOSE_PTRS << 24) | (tr << 16)}, k0, k1);
	if (!big) {
		// sequential search of the FP32 CDF: the smallest k with u <= F(k), or the k at
		// which adding p(k) no longer changes F (the FP32 tail is exhausted), at most 63.
		// kInvTerms terms per pass: the same products and sums in the same order as one
		// term per pass, so the same k, with fewer of the loop's passes and branches
		constexpr int kInvTerms = 2;
		const float u = u01_f(word_of(inv, tr & 3u));
		float p = expf(-mean);
		float F = p;
		int32_t k = 0;
		if (!(u > F)) return 0;
		while (k <= 63 - kInvTerms) {
			float pt[kInvTerms], Ft[kInvTerms];
#pragma unroll
			for (int j = 0; j < kInvTerms; j++) {
				pt[j] = (j == 0 ? p : pt[j - 1]) * mean * rcp[k + 1 + j];
				Ft[j] = (j == 0 ? F : Ft[j - 1]) + pt[j];
			}
#pragma unroll
			for (int j = 0; j < kInvTerms; j++)       // exhausted at k + 1 + j, or u <= F(k + 1 + j)
				if (Ft[j] == (j == 0 ? F : Ft[j - 1]) || !(u > Ft[j])) return k + 1 + j;
			k += kInvTerms;
			p = pt[kInvTerms - 1];
			F = Ft[kInvTerms - 1];
		}
		while (u > F && k < 63) {                      // the last terms, one at a time
			k++;
			p = p * mean * rcp[k];
			const float Fn = F + p;
			if (Fn == F) break;
			F = Fn;
		}
		return k;
	}
	const float slam = sqrtf(mean);
	const float loglam = __logf(mean);
	const float b = 0.931f + 2.53f * slam;
	const float a = -0.059f + 0.02483f * b;
	const float invalpha = 1.1239f + __fdividef(1.1328f, b - 3.4f);
	const float vr = 0.9277f - __fdividef(3.6224f, b - 2.0f);
	const float log_invalpha = __logf(invalpha);
	const float two_a = 2.0f * a;
	for (uint32_t it = 0; it < limit; it++) {
		const U4 r = it == 0 ? r0 : philox10(U4{col, sett, stream, (PURPOSE_PTRS << 24) | (tr << 16) | it}, k0, k1);
		const float U = u01_f(r.x) - 0.5f;
		const float V = u01_f(r.y);
		const float us = 0.5f - fabsf(U);
		const float k = floorf((__fdividef(two_a, us) + b) * U + mean + 0.43f);
		if (us >= 0.07f && V <= vr) return (int32_t)k;
		if (k < 0.0f || (us < 0.013f && V > us)) continue;
		const float lhs = __logf(V) + log_invalpha - __logf(__fdividef(a, us * us) + b);
		if (lhs <= ptrs_rhs(k, mean, loglam, lnfact)) return (int32_t)k;
	}
	return -1;
}

// log-density of one completed observation (src/obsmodel.cc:245-305) in FP32;
// thresholded values (rare) in FP64 as the reference evaluates them.
__device__ float obs_lp_fast(float vf, int o, const ModelDev &m)
{
	const int kind = m.obs_kind[o], model = m.obs_model[o];
	const float v = vf < 0.f ? 0.f : vf;
	if (kind == BEEP_OBSVAL_UNKNOWN) return 0.f;
	if (kind == BEEP_OBSVAL_VALUE) {
		if (model == BEEP_OBS_NORMAL || model == BEEP_OBS_NORMAL_PERCENT) {
			const float2 np = m.obs_np[o];                     // (-0.5 log(2 pi var), 1/(2 var))
			const float d = m.obs_value_f[o] - v;
			return np.x - d * d * np.y;
		}
		const float lam = v < 1.f ? 1.f : v;
		const float y = floorf(m.obs_value_f[o] + 0.5f);
		if (model == BEEP_OBS_POISSON) return y * logf(lam) - lam - lgammaf(y + 1.f);
		const float sh = m.obs_shape_f[o];
		return lgammaf(sh + y) - lgammaf(y + 1.f) - lgammaf(sh) + sh * logf(sh / (sh + lam)) + y * logf(lam / (sh + lam));
	}
	const double value = v, thresh = m.obs_thresh[o], sd = m.obs_sd[o];
	if (model == BEEP_OBS_NORMAL || model == BEEP_OBS_NORMAL_PERCENT) {
		const double var = sd * sd;
		const double x = value < thresh ? thresh : value;
		return (float)(-0.5 * log(2 * 3.14159265358979323846 * var) - (thresh - x) * (thresh - x) / (2 * var));
	}
	const double lam = value < 1 ? 1 : value, sh = m.obs_shape[o];
	double sum = 0.0;
	for (double k = 0; k <= thresh; k++) {
		if (model == BEEP_OBS_POISSON) sum += exp(k * log(lam) - lam - lgamma(k + 1));
		else sum += exp(lgamma(sh + k) - lgamma(k + 1) - lgamma(sh) + sh * log(sh / (sh + lam)) + k * log(lam / (sh + lam)));
	}
	return (float)log(sum);
}

// Imap[st][t][a] = sum_c M[c][t] Icnt[st][c][a] (off-diagonal M).  The
// infectious counts are stored with the age stride MG (the age count rounded
// up to a multiple of 4) so that a source's ages load as float4.
//  * M in shared memory: four consecutive lanes share a target t and split the
//    sources c = cg (mod 4); the row stride is congruent to 8 mod 32 so that a
//    warp's 4 rows x 8 targets hit 32 banks.
//  * M in global memory (L2): four lanes share a target pair (t, t+1), each pair
//    of matrix entries loads as one float2, eight sources in flight per lane
//    (four in the 320-thread layouts).
// The quad's partial sums are combined with two butterfly shuffles.
template <int NT, int MG>
__device__ __forceinline__ void foi(const ModelDev &m, const float *Ms, int lda, const float *Icnt, float *Imap, int tid)
{
	const int A = m.A;
	const int cg = tid & 3;
	for (int st = 0; st < m.NS; st++) {
		const float *I = Icnt + st * A * MG;
		float *Y = Imap + st * A * MG;
		if (Ms) {
			for (int t0 = 0; t0 < A; t0 += NT / 4) {
				const int t = t0 + (tid >> 2);
				float acc[MG];
#pragma unroll
				for (int a = 0; a < MG; a++) acc[a] = 0.f;
				if (t < A) {
#pragma unroll 2
					for (int c = cg; c < A; c += 4) {
						const float mv = Ms[c * lda + t];
						const float4 *Ic = reinterpret_cast<const float4 *>(I + c * MG);
#pragma unroll
						for (int q = 0; q < MG / 4; q++) {
							const float4 v = Ic[q];
							acc[4 * q] = fmaf(mv, v.x, acc[4 * q]);
							acc[4 * q + 1] = fmaf(mv, v.y, acc[4 * q + 1]);
							acc[4 * q + 2] = fmaf(mv, v.z, acc[4 * q + 2]);
							acc[4 * q + 3] = fmaf(mv, v.w, acc[4 * q + 3]);
						}
					}
				}
#pragma unroll
				for (int a = 0; a < MG; a++) {
					acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 1);
					acc[a] += __shfl_xor_sync(0xffffffffu, acc[a], 2);
				}
				if (t < A && cg == 0) {
					float4 *Yt = reinterpret_cast<float4 *>(Y + t * MG);
#pragma unroll
					for (int q = 0; q < MG / 4; q++) Yt[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
				}
			}
		} else {
			const int npair = (A + 1) / 2;
			const bool even = (A & 1) == 0;
			for (int p0 = 0; p0 < npair; p0 += NT / 4) {
				const int tp = p0 + (tid >> 2);
				const int t = 2 * tp;
				float a0[MG], a1[MG];
#pragma unroll
				for (int a = 0; a < MG; a++) { a0[a] = 0.f; a1[a] = 0.f; }
				if (tp < npair) {
					const bool has1 = t + 1 < A;
					// sources in flight per lane: 8, or 4 in the 320-thread layouts (their tighter
					// register budget; measured 1.3% faster on the ABC-SMC workload)
					constexpr int kU = NT == kDualThreads ? 4 : 8;
					for (int cb = cg; cb < A; cb += 4 * kU) {
						float2 mv[kU];
#pragma unroll
						for (int u = 0; u < kU; u++) {
							const int c = cb + 4 * u;
							mv[u] = make_float2(0.f, 0.f);
							if (c < A) {
								const float *row = m.Mdense + (size_t)c * A + t;
								if (even) mv[u] = __ldg(reinterpret_cast<const float2 *>(row));
								else mv[u] = make_float2(__ldg(row), has1 ? __ldg(row + 1) : 0.f);
							}
						}
#pragma unroll
						for (int u = 0; u < kU; u++) {
							const int c = cb + 4 * u;
							if (c < A) {
								const float4 *Ic = reinterpret_cast<const float4 *>(I + c * MG);
#pragma unroll
								for (int q = 0; q < MG / 4; q++) {
									const float4 v = Ic[q];
									a0[4 * q] = fmaf(mv[u].x, v.x, a0[4 * q]);
									a0[4 * q + 1] = fmaf(mv[u].x, v.y, a0[4 * q + 1]);
									a0[4 * q + 2] = fmaf(mv[u].x, v.z, a0[4 * q + 2]);
									a0[4 * q + 3] = fmaf(mv[u].x, v.w, a0[4 * q + 3]);
									a1[4 * q] = fmaf(mv[u].y, v.x, a1[4 * q]);
									a1[4 * q + 1] = fmaf(mv[u].y, v.y, a1[4 * q + 1]);
									a1[4 * q + 2] = fmaf(mv[u].y, v.z, a1[4 * q + 2]);
									a1[4 * q + 3] = fmaf(mv[u].y, v.w, a1[4 * q + 3]);
								}
							}
						}
					}
				}
#pragma unroll
				for (int a = 0; a < MG; a++) {
					a0[a] += __shfl_xor_sync(0xffffffffu, a0[a], 1);
					a0[a] += __shfl_xor_sync(0xffffffffu, a0[a], 2);
					a1[a] += __shfl_xor_sync(0xffffffffu, a1[a], 1);
					a1[a] += __shfl_xor_sync(0xffffffffu, a1[a], 2);
				}
				if (tp < npair && cg == 0) {
					float4 *Y0 = reinterpret_cast<float4 *>(Y + t * MG);
#pragma unroll
					for (int q = 0; q < MG / 4; q++) Y0[q] = make_float4(a0[4 * q], a0[4 * q + 1], a0[4 * q + 2], a0[4 * q + 3]);
					if (t + 1 < A) {
						float4 *Y1 = reinterpret_cast<float4 *>(Y + (t + 1) * MG);
#pragma unroll
						for (int q = 0; q < MG / 4; q++) Y1[q] = make_float4(a1[4 * q], a1[4 * q + 1], a1[4 * q + 2], a1[4 * q + 3]);
					}
				}
			}
		}
	}
}

// Force of infection on the tensor cores (foi_tc.cuh) for one step, in two
// halves so that the CTA's other warps work while the tensor cores run:
//   foi_tensor_issue   every thread: counts Icnt [NS][A][MG] -> stacked BF16
//                      pieces; then thread 0 streams the matrix chunks and
//                      issues the MMAs (warp 0 is busy until it returns);
//   foi_tensor_collect every thread: waits for the MMAs, thread 0 issues the
//                      next step's first loads (with `more`), and the
//                      accumulators are read back into Imap [NS][A][MG] (hi
//                      rows written, a barrier, lo rows added).
// Both return false (for every thread, after collect) if a wait gave up.
template <int NT, int MG>
__device__ void foi_tensor_issue(tc::Foi &f, uint32_t taddr, uint32_t step_no, const float *Icnt, int tid,
                                 int *abort_flag)
{
	const tc::Geom &g = f.g;
	const int A = g.A, NS = g.NS, kp = g.kpad(), R = g.arows();
	for (int idx = tid; idx < NS * kp * 16; idx += NT) {
		const int a = idx & 15, c = (idx >> 4) % kp, st = idx / (16 * kp);
		const float v = (c < A && a < MG) ? Icnt[(st * A + c) * MG + a] : 0.f;
		const __nv_bfloat16 h = __float2bfloat16_rn(v);
		const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
		*(__nv_bfloat16 *)(f.a + tc::kmajor_offset(st * 32 + a, c, R)) = h;
		*(__nv_bfloat16 *)(f.a + tc::kmajor_offset(st * 32 + 16 + a, c, R)) = l;
	}
	tc::fence_async_smem();
	__syncthreads();
	if (tid == 0) {
		if (!tc::issue_step(f, taddr, step_no)) {
			atomicExch(abort_flag, 1);
			tc::drain(f);
		}
	}
}

template <int NT, int MG>
__device__ bool foi_tensor_collect(tc::Foi &f, uint32_t taddr, uint32_t step_no, bool more, float *Imap, int tid,
                                   int *abort_flag)
{
	const tc::Geom &g = f.g;
	const int A = g.A, NS = g.NS;
	__syncwarp();
	if (!tc::mbar_wait(f.done, step_no & 1u)) atomicExch(abort_flag, 1);
	tc::tc_after_sync();
	__syncwarp();
	if (tid == 0 && more && !*(volatile int *)abort_flag) tc::prefetch(f, step_no + 1);
	// rows of warp quarter qd: r = qd*16 + lane (lane < 16) = strain qd/2, piece qd%2, age lane
	const int warp = tid >> 5, lane = tid & 31, qd = warp & 3, st = qd >> 1;
	const int ngroups = (g.nct * g.tw + 15) >> 4;
	for (int pass = 0; pass < 2; pass++) {
		if ((qd & 1) == pass && st < NS) {
			for (int gi = warp >> 2; gi < ngroups; gi += NT / 128) {
				float v[16];
				tc::tmem_ld16(taddr + ((uint32_t)(qd * 32) << 16) + (uint32_t)(gi * 16), v);
				if (lane < MG) {
					float *y = Imap + (st * A + gi * 16) * MG + lane;
#pragma unroll
					for (int i = 0; i < 16; i++)
						if (gi * 16 + i < A) y[i * MG] = pass ? y[i * MG] + v[i] : v[i];
				}
			}
		}
		__syncthreads();
	}
	tc::tc_before_sync();
	return !*(volatile int *)abort_flag;
}

struct Tabs {
	const float *rate, *sus, *inf, *beta_rows, *areafactor, *Ntime, *geo, *efoi_spline, *efoi_age, *obs_spline;
	const int32_t *beta_row_of, *efoi_ref;
	const float *efoi_mult, *tm_mult;       // prediction modifications, or null
};

// Per-step table slices: beta*areafactor and the external force of infection
// per (strain, area), the age-mixing matrix and the geographic spline
// (src/state.cc:403-423, 547-553).  The loads for step sett are issued by
// slice_load early in the previous step's draw phase (their latency hides
// behind the draws) and stored by slice_store after it.
struct SliceRegs {
	float be, et, N, d;
};

// item i (strain, area) of a step's slices: beta * areafactor, external force of infection per capita
__device__ __forceinline__ float2 slice_item(const ModelDev &m, const Tabs &tb, const FastSmem &s, int sett, int i)
{
	const int A = m.A, c = i % A;
	const float be = __ldg(tb.beta_rows + (size_t)s.brow[i] * m.S + sett) *
	                 __ldg(tb.areafactor + (size_t)(sett / m.div_per_time) * A + c);
	float et = __ldg(tb.efoi_spline + (size_t)s.eref[i] * m.S + sett) * m.inv_popsize_f;
	if (tb.efoi_mult) et *= __ldg(tb.efoi_mult + ((size_t)sett * A + c) * m.NS + i / A);
	return make_float2(be, et);
}

// the first NT items of each kind go through registers; items beyond (models
// with more (strain, area) pairs or age pairs than threads) are loaded when stored
template <int NT>
__device__ __forceinline__ SliceRegs slice_load(const ModelDev &m, const Tabs &tb, const FastSmem &s, int sett, int tid)
{
	SliceRegs r{0.f, 0.f, 0.f, 0.f};
	if (tid < m.NS * m.A) {
		const float2 v = slice_item(m, tb, s, sett, tid);
		r.be = v.x;
		r.et = v.y;
	}
	if (tid < m.G * m.G) r.N = __ldg(tb.Ntime + (size_t)sett * m.G * m.G + tid);
	if (tid == 0) r.d = __ldg(tb.geo + sett);
	return r;
}

template <int NT>
__device__ __forceinline__ void slice_store(const ModelDev &m, const Tabs &tb, FastSmem &s, const SliceRegs &r, int buf,
                                            int sett, int tid)
{
	float *be = buf ? s.be1 : s.be0, *et = buf ? s.et1 : s.et0, *N = buf ? s.N1 : s.N0;
	const int NSA = m.NS * m.A, GG = m.G * m.G;
	if (tid < NSA) { be[tid] = r.be; et[tid] = r.et; }
	if (tid < GG) N[tid] = r.N;
	if (tid == 0) s.dgeo[buf] = r.d;
	for (int i = tid + NT; i < NSA; i += NT) {
		const float2 v = slice_item(m, tb, s, sett, i);
		be[i] = v.x;
		et[i] = v.y;
	}
	for (int i = tid + NT; i < GG; i += NT) N[i] = __ldg(tb.Ntime + (size_t)sett * GG + i);
}

// Stirling remainder of log Gamma(z): log Gamma(z) - ((z - 1/2) log z - z + log(2 pi)/2)
__device__ __forceinline__ float stirling_rem(float z)
{
	const float iz = __fdividef(1.f, z), iz2 = iz * iz;
	return iz * (0.083333333f - iz2 * (0.0027777778f - iz2 * 0.00079365079f));
}

// Binomial(n, p) thinning in FP32 on the keyed stream of the FP64 form (same
// counters and words): inversion below n q = 10, BTRS (Hoermann 1993) above.
// The BTRS acceptance test log f(k)/f(m) is formed without cancellation as
//   -(m+1/2) log1p(d/(m+1)) - (n-m+1/2) log1p(-d/(n-m+1))
//   + d log((n-k+1) q / ((k+1) (1-q))) + Stirling remainders,  d = k - m,
// instead of differences of large log-factorials.
__device__ __forceinline__ int32_t binomial_fp32(float p, int32_t n, uint32_t k0, uint32_t k1, uint32_t col, uint32_t tr,
                                                 uint32_t sett, uint32_t stream, uint32_t limit)
{
	if (n <= 0 || !(p > 0.f)) return 0;
	if (p >= 1.f) return n;
	const bool flip = p > 0.5f;
	const float q = flip ? 1.f - p : p, qc = 1.f - q;
	const float nd = (float)n;
	int32_t k = 0;
	if (nd * q < 10.f) {
		const U4 r = philox10(U4{col, sett, stream, (PURPOSE_THIN << 24) | (tr >> 2)}, k0, k1);
		const float u = u01_f(word_of(r, tr & 3u));
		const float ratio = q / qc;
		float f = expf(nd * log1pf(-q));
		float F = f;
		while (u > F && k < n) {
			f = f * ratio * (float)(n - k) / (float)(k + 1);
			k++;
			const float Fn = F + f;
			if (Fn == F) break;                       // FP32 tail exhausted
			F = Fn;
		}
	} else {
		const float spq = sqrtf(nd * q * qc);
		const float b = 1.15f + 2.53f * spq;
		const float a = -0.0873f + 0.0248f * b + 0.01f * q;
		const float c = nd * q + 0.5f;
		const float alpha = (2.83f + __fdividef(5.1f, b)) * spq;
		const float vr = 0.92f - __fdividef(4.2f, b);
		const float m = floorf((nd + 1.f) * q);
		const float em = stirling_rem(m + 1.f) + stirling_rem(nd - m + 1.f);
		k = -1;
		for (uint32_t it = 0; it < limit; it++) {
			const U4 r = philox10(U4{col, sett, stream, (PURPOSE_BTRS << 24) | (tr << 16) | it}, k0, k1);
			const float U = u01_f(r.x) - 0.5f;
			const float V = u01_f(r.y);
			const float us = 0.5f - fabsf(U);
			const float kd = floorf((__fdividef(2.f * a, us) + b) * U + c);
			if (kd < 0.f || kd > nd) continue;
			if (us >= 0.07f && V <= vr) { k = (int32_t)kd; break; }
			const float lhs = __logf(V * alpha / (__fdividef(a, us * us) + b));
			const float d = kd - m;
			const float rhs = -(m + 0.5f) * log1pf(d / (m + 1.f)) - (nd - m + 0.5f) * log1pf(-d / (nd - m + 1.f)) +
			                  d * __logf((nd - kd + 1.f) * q / ((kd + 1.f) * qc)) + em - stirling_rem(kd + 1.f) -
			                  stirling_rem(nd - kd + 1.f);
			if (lhs <= rhs) { k = (int32_t)kd; break; }
		}
		if (k < 0) return -1;
	}
	return flip ? n - k : k;
}

// CTAs resident per SM (MB): one of 640 threads; two to four of 320
// (kDualThreads) when that many particles' state fits the SM's shared memory
// -- the register budget per thread shrinks to 96 / 64 / 48 and the warps per
// SM grow to 20 / 30 / 40, which hides the latency of the sampler and Philox
// chains; two of 256 or four of 128 threads for small models.
constexpr int min_ctas(int nt) { return nt >= 640 ? 1 : nt >= 256 ? 2 : 4; }

// One particle (or MBP chain) p of a batch over its whole step range, run by
// the NT threads of a CTA.  MT: the most transitions the per-column mean
// registers hold (kMaxT, or kWideT for models with more transitions).
template <int NT, int MG, bool TC, bool CH, int MT, bool PD = false>
__device__ __forceinline__ void sim_fast_body(const ModelDev &m, const BatchDev &b, const int p)
{
	extern __shared__ __align__(16) unsigned char smem_raw[];
	if (p >= b.P) return;
	const int tid = threadIdx.x;
	const int A = m.A, G = m.G, DP = m.DP, NS = m.NS, DPS = m.DPS, C = m.C, T = m.T;
	const int ncol = A * DP, popsz = C * ncol, tnsz = T * ncol, agsz = NS * A * MG;   // ages padded to MG
	const int tnrows = b.tn_full ? T : m.tn_rows;        // stored transition rows
	const int nsteps = b.tf - b.ti;
	const int lda = ms_lda(A);
	const GroupDir dir = b.dirs[b.group_of ? b.group_of[p] : 0];
	const uint32_t stream = b.stream_of ? b.stream_of[p] : (uint32_t)p;
	const uint32_t k0 = b.key_of ? b.key_of[p].x : b.k0, k1 = b.key_of ? b.key_of[p].y : b.k1;   // the particle's key
	Tabs tb;
	{
		const float *fp = b.fpool32;
		tb.rate = fp + dir.transrate; tb.sus = fp + dir.susceptibility; tb.inf = fp + dir.infectivity;
		tb.beta_rows = fp + dir.beta_rows; tb.areafactor = fp + dir.areafactor; tb.Ntime = fp + dir.Ntime;
		tb.geo = fp + dir.geo_spline; tb.efoi_spline = fp + dir.efoi_spline; tb.efoi_age = fp + dir.efoi_agedist;
		tb.obs_spline = fp + dir.obs_spline;
		tb.beta_row_of = b.ipool + dir.beta_row_of; tb.efoi_ref = b.ipool + dir.efoi_ref;
		tb.efoi_mult = dir.efoi_mult >= 0 ? fp + dir.efoi_mult : nullptr;
		tb.tm_mult = dir.tm_mult >= 0 ? fp + dir.tm_mult : nullptr;
	}
	int32_t *status = b.status + p;
	// MBP chains (CH): slot of the current state and of the state written; chain
	// arrays [slot][chain][step][transition][column]
	const int cmode = CH ? b.mode : 0;
	const int cs_i = CH ? b.cur[p] : 0, cs_p = 1 - cs_i;
	float Lst = 0.f, Lstc = 0.f;            // mode 2: compensated state log-likelihood of this thread

	FastSmem s;
	{
		size_t off = 0;
		auto take = [&](size_t bytes) { unsigned char *q = smem_raw + off; off += (bytes + 15) & ~(size_t)15; return q; };
		s.Ms = b.m_in_smem ? (float *)take(sizeof(float) * A * lda) : nullptr;
		if (b.gstate) {
			// models too large for shared memory keep the particle's state in a global
			// (L2-resident) region of the same layout
			unsigned char *g = (unsigned char *)b.gstate + (size_t)p * b.gstate_stride;
			size_t go = 0;
			auto gtake = [&](size_t bytes) { unsigned char *q = g + go; go += (bytes + 255) & ~(size_t)255; return q; };
			s.pop0 = (int32_t *)gtake(4 * (size_t)popsz);
			s.pop1 = b.pop_single ? s.pop0 : (int32_t *)gtake(4 * (size_t)popsz);
			s.tn = b.tn_smem ? (int32_t *)take(4 * (size_t)tnrows * ncol) : (int32_t *)gtake(4 * (size_t)tnrows * ncol);
		} else {
			s.pop0 = (int32_t *)take(4 * (size_t)popsz);
			s.pop1 = b.pop_single ? s.pop0 : (int32_t *)take(4 * (size_t)popsz);
			s.tn = (int32_t *)take(4 * (size_t)tnrows * ncol);
		}
		// the infectious counts and the force of infection stay on chip in both cases
		// (the FOI reads each of them A times per step)
		s.Ic0 = (float *)take(4 * (size_t)agsz);
		s.Ic1 = (float *)take(4 * (size_t)agsz);
		s.Imap = (float *)take(4 * (size_t)agsz);
		s.slot = (float *)take(4 * (size_t)b.nslots);
		s.from = (int32_t *)take(4 * (size_t)T);
		s.trow = (int32_t *)take(4 * (size_t)T);
		s.to = (int32_t *)take(4 * (size_t)T);
		s.age = (int32_t *)take(4 * (size_t)DPS);
		s.inf = (float *)take(4 * (size_t)C);
		s.rate = (float *)take(4 * (size_t)T * DP);
		s.sus = (float *)take(4 * (size_t)DP);
		s.rcp = (float *)take(4 * 64);
		s.lnfact = (float *)take(4 * 32);
		s.brow = (int32_t *)take(4 * (size_t)NS * A);
		s.eref = (int32_t *)take(4 * (size_t)NS * A);
		s.eage = (float *)take(4 * (size_t)b.nefoi_stage * G);
		s.be0 = (float *)take(4 * (size_t)NS * A);
		s.et0 = (float *)take(4 * (size_t)NS * A);
		s.N0 = (float *)take(4 * (size_t)G * G);
		s.be1 = (float *)take(4 * (size_t)NS * A);
		s.et1 = (float *)take(4 * (size_t)NS * A);
		s.N1 = (float *)take(4 * (size_t)G * G);
		s.dgeo = (float *)take(4 * 2);
		s.red = (float *)take(4 * 2 * (size_t)NT);
		s.mv = NT == kDualThreads ? (float *)take(4 * (size_t)T * NT) : nullptr;
		s.pm = PD ? (float *)take(4 * (size_t)T * ncol) : nullptr;
	}
	// tensor-core FOI (large models, 640 threads): chunk ring, stacked counts, barriers, tensor memory
	__shared__ uint64_t tc_bars[2 * tc::kStages + 1];
	__shared__ uint32_t tc_slot;
	__shared__ int tc_abort;
	tc::Foi tf;
	constexpr bool use_tc = TC;   // tensor-core FOI (instantiated for 640 threads only)
	uint32_t taddr = 0, tcols = 0;
	if (use_tc) {
		size_t off = b.tc_smem_off;
		tf.g = tc::geometry(A, NS);
		tf.stage0 = smem_raw + off;
		tf.stage_stride = (tf.g.chunk_bytes() + 127) & ~(uint32_t)127;
		tf.a = smem_raw + off + (size_t)tc::kStages * tf.stage_stride;
		tf.full = tc_bars; tf.empty = tc_bars + tc::kStages; tf.done = tc_bars + 2 * tc::kStages;
		tf.image = m.tc_image;
		tf.pending = 0; tf.pend_par = 0;
		tcols = tf.g.tmem_cols();
		if ((tid >> 5) == 0) tc::tmem_alloc(&tc_slot, tcols);
		if (tid == 0) {
			tc_abort = 0;
			for (int k = 0; k < tc::kStages; k++) { tc::mbar_init(&tf.full[k], 1); tc::mbar_init(&tf.empty[k], 1); }
			tc::mbar_init(tf.done, 1);
			tc::fence_mbar_init();
		}
		for (uint32_t k = tid; k < tf.g.a_bytes() / 4; k += NT) ((uint32_t *)tf.a)[k] = 0u;
		tc::tc_before_sync();
		__syncthreads();
		tc::tc_after_sync();
		taddr = tc_slot;
		if (tid == 0) tc::prefetch(tf, 0);
	}
	uint32_t tc_step = 0;
	if (s.Ms)
		for (int k = tid; k < A * A; k += NT) s.Ms[(k / A) * lda + k % A] = m.Mdense[k];
	for (int k = tid; k < popsz; k += NT) {
		// global layout [c][co][dp] -> shared [co][c*DP+dp]
		const int dp = k % DP, co = (k / DP) % C, c = k / (DP * C);
		s.pop0[co * ncol + c * DP + dp] = b.ti == 0 ? m.pop_init[k] : b.pop_in[(size_t)p * popsz + k];
	}
	for (int k = tid; k < b.nslots; k += NT) s.slot[k] = 0.f;
	for (int k = tid; k < agsz; k += NT) s.Ic1[k] = 0.f;
	for (int k = tid; k < T; k += NT) {
		s.from[k] = m.trans_from[k];
		s.to[k] = m.trans_to[k];
		s.trow[k] = b.tn_full ? k : m.tn_row[k];
	}
	for (int k = tid; k < DPS; k += NT) s.age[k] = m.dp_age[k];
	for (int k = tid; k < C; k += NT) s.inf[k] = tb.inf[k];
	for (int k = tid; k < T * DP; k += NT) s.rate[k] = tb.rate[k];
	for (int k = tid; k < DP; k += NT) s.sus[k] = tb.sus[k];
	for (int k = tid; k < 64; k += NT) s.rcp[k] = k == 0 ? 0.f : 1.f / (float)k;
	for (int k = tid; k < 32; k += NT) s.lnfact[k] = c_lnfact[k];
	for (int k = tid; k < NS * A; k += NT) { s.brow[k] = tb.beta_row_of[k]; s.eref[k] = tb.efoi_ref[k]; }
	for (int k = tid; k < b.nefoi_stage * G; k += NT) s.eage[k] = tb.efoi_age[k];
	__syncthreads();
	// infectious counts of the start populations (set_I_from_pop, src/state.cc:223-290)
	for (int idx = tid; idx < agsz; idx += NT) {
		const int a = idx % MG, c = (idx / MG) % A, st = idx / (MG * A);
		float v = 0.f;
		for (int co = 0; co < C && a < G; co++) {
			const float inf = s.inf[co];
			if (inf != 0.f)
				for (int dp = 0; dp < DPS; dp++)
					if (s.age[dp] == a) v += inf * (float)s.pop0[co * ncol + c * DP + st * DPS + dp];
		}
		s.Ic0[idx] = v;
	}
	slice_store<NT>(m, tb, s, slice_load<NT>(m, tb, s, b.ti, tid), 0, b.ti, tid);
	__syncthreads();
	bool tc_ok = true;
	if (use_tc) {
		foi_tensor_issue<NT, MG>(tf, taddr, tc_step, s.Ic0, tid, &tc_abort);
		tc_ok = foi_tensor_collect<NT, MG>(tf, taddr, tc_step, nsteps > 1, s.Imap, tid, &tc_abort);
		tc_step++;
	} else {
		foi<NT, MG>(m, s.Ms, lda, s.Ic0, s.Imap, tid);
	}
	float Lsum = 0.f, Lcmp = 0.f;           // compensated per-thread log-likelihood
	__syncthreads();

	const int itr = m.infection_trans;
	const int inf_from = m.trans_from[itr];
	const uint32_t lim = b.sampler_limit ? b.sampler_limit : 65536u;
	const float dt = (float)m.dt;
	bool cur = false;
	int sb = 0;                                          // slice buffer of the step simulated
	for (int sett = b.ti; sett < b.tf && tc_ok; sett++) {
		int32_t *pc = cur ? s.pop1 : s.pop0, *pn = cur ? s.pop0 : s.pop1;
		const SliceRegs nxt = sett + 1 < b.tf ? slice_load<NT>(m, tb, s, sett + 1, tid) : SliceRegs{0.f, 0.f, 0.f, 0.f};
		const float *be = sb ? s.be1 : s.be0, *et = sb ? s.et1 : s.et0, *Nm = sb ? s.N1 : s.N0;
		const float *Ic_cur = cur ? s.Ic1 : s.Ic0;
		float *Ic_nxt = cur ? s.Ic0 : s.Ic1;
		if (NS > 1) {
			// strain shift of the susceptible population (src/state.cc:392-401)
			for (int idx = tid; idx < A * DPS; idx += NT) {
				const int dp = idx % DPS, c = idx / DPS;
				int32_t *sp = pc + inf_from * ncol + c * DP;
				int32_t sum = 0;
				for (int st = 1; st < NS; st++) { sum += sp[DPS * st + dp]; sp[DPS * st + dp] = 0; }
				sp[dp] += sum;
			}
			__syncthreads();
		}

		// ---- A: per column (c, dp): NMI, means, draws, next population and infectious count
		const float d = s.dgeo[sb], omd = 1.f - d;
		if constexpr (PD) {
		// ---- A, small models: the means of every column, then one draw per (transition,
		//      column) -- the draws of a column run on T threads at once instead of one after
		//      another on one -- then every column's next infectious count
		for (int col = tid; col < ncol; col += NT) {
			const int c = col / DP, dp = col - c * DP;
			const int st = dp / DPS, dpl = dp - st * DPS, a = s.age[dpl];
			float minf = 0.f;
			{
				const float popu = (float)pc[inf_from * ncol + c * DP + dpl];
				if (popu > 0.f) {
					const float fac = m.M_factor_f[c], dg = m.M_diag_f[c];
					const float *Ic = Ic_cur + (st * A + c) * MG, *Im = s.Imap + (st * A + c) * MG;
					const float *N = Nm + a * G;
					float nmi = 0.f;
#pragma unroll
					for (int aa = 0; aa < MG; aa++) {
						if (aa < G) {
							const float id = Ic[aa] * dg;
							nmi = fmaf(N[aa], (id + Im[aa]) * d + fac * id * omd, nmi);
						}
					}
					nmi = fmaxf(nmi, 0.f);
					const int sc = st * A + c;
					const float eage = b.nefoi_stage ? s.eage[s.eref[sc] * G + a] : __ldg(tb.efoi_age + (size_t)s.eref[sc] * G + a);
					minf = dt * popu * s.sus[dp] * (be[sc] * nmi + et[sc] * eage);
				}
			}
			for (int tr = 0; tr < T; tr++) {
				float v;
				if (tr == itr) v = minf;
				else {
					const float popu = (float)pc[s.from[tr] * ncol + col];
					v = popu <= 0.f ? 0.f : dt * popu * s.rate[tr * DP + dp];
				}
				if (tb.tm_mult) v *= __ldg(tb.tm_mult + ((size_t)sett * A + c) * T * DP + tr * DP + dp);
				s.pm[tr * ncol + col] = v;
			}
			if (pn != pc)
				for (int co = 0; co < C; co++) pn[co * ncol + col] = pc[co * ncol + col];
		}
		__syncthreads();
		for (int idx = tid; idx < T * ncol; idx += NT) {
			const int tr = idx / ncol, col = idx - tr * ncol;
			const float mean = s.pm[idx];
			U4 inv{0, 0, 0, 0};
			uint32_t inv_call = 0xffffffffu;
			int32_t n = 0;
			if (mean > 0.f) {
				if (mean > 1.0e9f) atomicCAS(status, 0, BEEP_COUNT_OVERFLOW);
				else {
					n = poisson_fp32(mean, k0, k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett, stream, inv, inv_call,
					                 s.rcp, s.lnfact, lim);
					if (n < 0) { atomicCAS(status, 0, BEEP_TIMEOUT); n = 0; }
				}
			} else if (mean != mean) atomicCAS(status, 0, BEEP_NAN_RATE);
			const int row = s.trow[tr];
			if (row >= 0) s.tn[row * ncol + col] = n;
			if (n != 0) {                                // integer updates: their order does not matter
				atomicSub(pn + s.from[tr] * ncol + col, n);
				atomicAdd(pn + s.to[tr] * ncol + col, n);
			}
		}
		__syncthreads();
		for (int col = tid; col < ncol; col += NT) {
			const int c = col / DP, dp = col - c * DP;
			const int st = dp / DPS, dpl = dp - st * DPS, a = s.age[dpl];
			float iv = 0.f;
			for (int co = 0; co < C; co++) {
				const float inf = s.inf[co];
				if (inf != 0.f) iv = fmaf(inf, (float)pn[co * ncol + col], iv);
			}
			if (m.dp_age_unique) Ic_nxt[(st * A + c) * MG + a] = iv;
			else atomicAdd(Ic_nxt + (st * A + c) * MG + a, iv);
		}
		} else {
		for (int col = tid; col < ncol; col += NT) {
			const int c = col / DP, dp = col - c * DP;
			const int st = dp / DPS, dpl = dp - st * DPS, a = s.age[dpl];
			U4 inv{0, 0, 0, 0};
			uint32_t inv_call = 0xffffffffu;
			// means of all transitions from the step's populations (src/state.cc:380-456)
			float minf = 0.f;
			{
				const float popu = (float)pc[inf_from * ncol + c * DP + dpl];
				if (popu > 0.f) {
					const float fac = m.M_factor_f[c], dg = m.M_diag_f[c];
					const float *Ic = Ic_cur + (st * A + c) * MG, *Im = s.Imap + (st * A + c) * MG;
					const float *N = Nm + a * G;
					float nmi = 0.f;
#pragma unroll
					for (int aa = 0; aa < MG; aa++) {
						if (aa < G) {
							const float id = Ic[aa] * dg;
							nmi = fmaf(N[aa], (id + Im[aa]) * d + fac * id * omd, nmi);
						}
					}
					nmi = fmaxf(nmi, 0.f);
					const int sc = st * A + c;
					const float eage = b.nefoi_stage ? s.eage[s.eref[sc] * G + a] : __ldg(tb.efoi_age + (size_t)s.eref[sc] * G + a);
					minf = dt * popu * s.sus[dp] * (be[sc] * nmi + et[sc] * eage);
				}
			}
			// the means: in registers, or (320-thread CTAs) in the thread's shared-memory column
			constexpr bool kMvSmem = NT == kDualThreads;
			float mv[kMvSmem ? 1 : MT];
			float *mvs = s.mv + tid;
			auto mean_of = [&](int tr) {
				float v;
				if (tr == itr) v = minf;
				else {
					const float popu = (float)pc[s.from[tr] * ncol + col];
					v = popu <= 0.f ? 0.f : dt * popu * s.rate[tr * DP + dp];
				}
				if (tb.tm_mult) v *= __ldg(tb.tm_mult + ((size_t)sett * A + c) * T * DP + tr * DP + dp);
				return v;
			};
			if constexpr (kMvSmem) {
				for (int tr = 0; tr < T; tr++) mvs[tr * NT] = mean_of(tr);
			} else {
#pragma unroll
				for (int tr = 0; tr < MT; tr++) mv[tr] = tr < T ? mean_of(tr) : 0.f;
			}
			if (pn != pc)
				for (int co = 0; co < C; co++) pn[co * ncol + col] = pc[co * ncol + col];
			// draws; the populations are updated after every mean was formed
			for (int tr = 0; tr < T; tr++) {
				float mean;
				if constexpr (kMvSmem) {
					mean = mvs[tr * NT];
				} else {
					mean = mv[0];
#pragma unroll
					for (int k = 1; k < MT; k++) mean = tr == k ? mv[k] : mean;
				}
				int32_t n = 0;
				if constexpr (CH) {
					const size_t tcell = (size_t)tr * ncol + col, step_cells = (size_t)T * ncol;
					const size_t ci = (((size_t)cs_i * b.P + p) * m.S + sett) * step_cells + tcell;
					const size_t cp = (((size_t)cs_p * b.P + p) * m.S + sett) * step_cells + tcell;
					if (mean != mean) atomicCAS(status, 0, BEEP_NAN_RATE);
					if (cmode == 2) {                      // State::likelihood term of the fixed count
						n = b.ch_tn[ci];
						float lp;
						if (mean == 0.f) lp = n == 0 ? 0.f : -1.0e9f;
						else lp = (float)n * __logf(mean) - mean - lgammaf((float)n + 1.f);
						const float y = lp - Lstc;
						const float t2 = Lst + y;
						Lstc = (t2 - Lst) - y;
						Lst = t2;
					} else if (cmode == 3) {               // the given counts stay
						n = b.ch_tn[cp];
						b.ch_mean_f[cp] = mean;
					} else {
						if (mean > 0.f) {
							if (mean > 1.0e9f) atomicCAS(status, 0, BEEP_COUNT_OVERFLOW);
							else if (b.simu_all || (b.simu && b.simu[((size_t)p * m.S + sett) * A + c])) {
								n = poisson_fp32(mean, k0, k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett, stream, inv,
								                 inv_call, s.rcp, s.lnfact, lim);
							} else {                       // coupled to the current state (src/mbp.cc:293-305)
								const int32_t ni = b.ch_tn[ci];
								const float ri = b.ch_mean_f[ci];
								if (mean > ri) {
									n = poisson_fp32(mean - ri, k0, k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett,
									                 stream, inv, inv_call, s.rcp, s.lnfact, lim);
									if (n >= 0) n += ni;
								} else if (mean == ri) n = ni;
								else n = binomial_fp32(mean / ri, ni, k0, k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett,
								                       stream, lim);
							}
							if (n < 0) { atomicCAS(status, 0, BEEP_TIMEOUT); n = 0; }
						}
						b.ch_tn[cp] = n;
						b.ch_mean_f[cp] = mean;
					}
				} else {
				if (mean > 0.f) {
					if (mean > 1.0e9f) atomicCAS(status, 0, BEEP_COUNT_OVERFLOW);
					else {
						n = poisson_fp32(mean, k0, k1, (uint32_t)col, (uint32_t)tr, (uint32_t)sett, stream, inv, inv_call,
						                 s.rcp, s.lnfact, lim);
						if (n < 0) { atomicCAS(status, 0, BEEP_TIMEOUT); n = 0; }
					}
				} else if (mean != mean) atomicCAS(status, 0, BEEP_NAN_RATE);
				}
				const int row = s.trow[tr];
				if (row >= 0) s.tn[row * ncol + col] = n;
				if (n != 0) {
					pn[s.from[tr] * ncol + col] -= n;
					pn[s.to[tr] * ncol + col] += n;
				}
			}
			float iv = 0.f;
			for (int co = 0; co < C; co++) {
				const float inf = s.inf[co];
				if (inf != 0.f) iv = fmaf(inf, (float)pn[co * ncol + col], iv);
			}
			if (m.dp_age_unique) Ic_nxt[(st * A + c) * MG + a] = iv;
			else atomicAdd(Ic_nxt + (st * A + c) * MG + a, iv);
		}
		}
		if (sett + 1 < b.tf) slice_store<NT>(m, tb, s, nxt, sb ^ 1, sett + 1, tid);
		__syncthreads();

		// ---- B: observation sums of the step (completed ones -> log-density),
		//         next step's table slices and force of infection
		if (b.pop_traj)
			for (int k = tid; k < popsz; k += NT) {
				const int dp = k % DP, co = (k / DP) % C, c = k / (DP * C);
				b.pop_traj[((size_t)p * nsteps + (sett - b.ti)) * popsz + k] = pc[co * ncol + c * DP + dp];
			}
		if (b.tn_traj)
			for (int k = tid; k < tnsz; k += NT) {
				const int dp = k % DP, tr = (k / DP) % T, c = k / (DP * T);
				b.tn_traj[((size_t)p * nsteps + (sett - b.ti)) * tnsz + k] = s.tn[tr * ncol + c * DP + dp];
			}
		const bool tc_now = use_tc && sett + 1 < b.tf;
		if (tc_now) foi_tensor_issue<NT, MG>(tf, taddr, tc_step, Ic_nxt, tid, &tc_abort);
		// with the tensor cores busy for warp 0, warps 1.. take the observations
		const int ow = tc_now ? 32 : 0;
		const int a0 = b.step_ptr[sett - b.ti], a1 = b.step_ptr[sett - b.ti + 1];
		for (int k = a0 + tid - ow; tid >= ow && k < a1; k += NT - ow) {
			const int4 t0 = __ldg(b.tasks + 2 * k), t1 = __ldg(b.tasks + 2 * k + 1);
			const float fac = __int_as_float(t1.x);
			const int spl = t1.y;
			const float w = spl < 0 ? fac : fac * tb.obs_spline[(size_t)spl * m.S + sett];
			const int nc = t0.w & 0x7fffffff;
			float v = s.slot[t0.x];
			if (t1.w != 0) {                  // consecutive counts or populations: no cell list
				const int32_t *src = t1.w == 1 ? s.tn + t0.z : pc + (-1 - t0.z);
#pragma unroll 4
				for (int i = 0; i < nc; i++) v = fmaf(w, (float)src[i], v);
			} else {
				if (nc > 0) {
					const int cell = t0.z;
					v = fmaf(w, cell >= 0 ? (float)s.tn[cell] : (float)pc[-1 - cell], v);
				}
				for (int i = 1; i < nc; i++) {
					const int cell = __ldg((b.tn_full ? m.obs_cells_full : m.obs_cells_f) + t1.z + i);
					v = fmaf(w, cell >= 0 ? (float)s.tn[cell] : (float)pc[-1 - cell], v);
				}
			}
			if (t0.w < 0) {                  // the observation's last step: log-density
				const float lp = obs_lp_fast(v, t0.y, m);
				v = 0.f;
				const float y = lp - Lcmp;      // Kahan
				const float tt = Lsum + y;
				Lcmp = (tt - Lsum) - y;
				Lsum = tt;
			}
			s.slot[t0.x] = v;
		}
		if (!m.dp_age_unique)
			for (int k = tid; k < agsz; k += NT) (cur ? s.Ic1 : s.Ic0)[k] = 0.f;   // next step's accumulation target
		if (use_tc) {
			if (tc_now) {
				tc_ok = foi_tensor_collect<NT, MG>(tf, taddr, tc_step, sett + 2 < b.tf, s.Imap, tid, &tc_abort);
				tc_step++;
			}
		} else {
			foi<NT, MG>(m, s.Ms, lda, Ic_nxt, s.Imap, tid);
		}
		__syncthreads();
		cur = !cur;
		sb ^= 1;
	}

	if (use_tc) {
		if (tid == 0) {
			tc::drain(tf);                             // loads still in flight (only after a timeout)
			if (!tc_ok) atomicCAS(status, 0, BEEP_TIMEOUT);
		}
		tc::tc_before_sync();
		__syncthreads();
		if ((tid >> 5) == 0) {
			tc::tc_after_sync();
			tc::tmem_dealloc(taddr, tcols);
		}
	}
	if (b.pop_out) {
		const int32_t *pf = cur ? s.pop1 : s.pop0;
		for (int k = tid; k < popsz; k += NT) {
			const int dp = k % DP, co = (k / DP) % C, c = k / (DP * C);
			b.pop_out[(size_t)p * popsz + k] = pf[co * ncol + c * DP + dp];
		}
	}
	if (CH && cmode == 2) {
		__syncthreads();
		s.red[tid] = Lst;
		s.red[NT + tid] = Lstc;
		__syncthreads();
		if (tid < 32) {
			double S = 0.0;
			for (int k = tid; k < NT; k += 32) S += (double)s.red[k] - (double)s.red[NT + k];
			for (int o = 16; o > 0; o >>= 1) S += __shfl_xor_sync(0xffffffffu, S, o);
			if (tid == 0) b.Li[p] = S;
		}
	}
	if (b.L) {
		__syncthreads();
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

// One CTA per particle (or MBP chain): CTA p runs particle p.  PD: the draws of a step
// one per (transition, column) thread (small models, fast_parallel_draws).
template <int NT, int MG, bool TC, bool CH = false, int MB = min_ctas(NT), int MT = kMaxT, bool PD = false>
__global__ void __launch_bounds__(NT, MB) sim_fast_kernel(const ModelDev m, const BatchDev b)
{
	sim_fast_body<NT, MG, TC, CH, MT, PD>(m, b, blockIdx.x);
}

// log k! for k < 32 in this translation unit's constant memory, once (before
// any graph capture)
inline int prepare_constants()
{
	static std::mutex mu;
	static bool done = false;
	std::lock_guard<std::mutex> lock(mu);
	if (done) return 0;
	float lf[32];
	for (int k = 0; k < 32; k++) lf[k] = (float)std::lgamma((double)k + 1.0);
	cudaError_t e = cudaMemcpyToSymbol(c_lnfact, lf, sizeof lf);
	// a copy from pageable memory may return before its bytes land, and the kernels run on
	// non-blocking streams that do not wait for the legacy stream: wait for it here
	if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
	if (e != cudaSuccess) return (int)e;
	done = true;
	return 0;
}

}  // namespace
}  // namespace beep
