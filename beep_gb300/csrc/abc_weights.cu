// beep_abcsmc_weights: ABC-SMC importance weights of a generation
// (ABCSMC::calculate_particle_weight, src/abcsmc.cc:260-271, with
// MVN::probability, src/mvn.cc:185-196, and normalise_particle_weights,
// src/abcsmc.cc:275-283):
//   w_i = exp(logprior_i) / sum_j w_j^last exp(-0.5 (d/size)^T M^-1 (d/size)),
//   d = theta_i - theta_j over the inferred parameters; then w /= mean(w).
// The N_new x N_last kernel terms are formed in FP32 from parameters centred
// on the last generation's FP64 mean (the differences are unchanged, and no
// cancellation against a large common offset is left to FP32).  Each new
// particle's sum  sum_j w_j exp(-q_j / 2)  is accumulated as a running
// log-sum-exp -- the largest exponent so far, m, and the compensated sum of
// exp(x_j - m) -- so that it cannot underflow even when every term would
// (far-away particles); the per-particle log sums, the prior factor and the
// normalisation are FP64.  Where the reference's FP64 sum underflows to zero
// (its weight is then infinite) this one stays finite.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "capi_internal.h"

namespace beep {
namespace {

constexpr int kAbcThreads = 256;
constexpr int kAbcTile = 256;        // last-generation particles staged per pass
constexpr int kMaxVar = 16;

__global__ void __launch_bounds__(kAbcThreads) abc_kernel_logsums(int nvar, int nnew, const float *th_new, int nlast,
                                                                  const float *th_last, const float *logw_last,
                                                                  const float *A, double *logsum_out)
{
	__shared__ float s_th[kAbcTile * kMaxVar];
	__shared__ float s_lw[kAbcTile];
	__shared__ float s_A[kMaxVar * kMaxVar];
	const int i = blockIdx.x * kAbcThreads + threadIdx.x;
	for (int k = threadIdx.x; k < nvar * nvar; k += kAbcThreads) s_A[k] = A[k];
	float x[kMaxVar];
#pragma unroll
	for (int v = 0; v < kMaxVar; v++) x[v] = (i < nnew && v < nvar) ? th_new[(size_t)i * nvar + v] : 0.f;
	float mx = -INFINITY, s = 0.f, cmp = 0.f;      // running max exponent; compensated sum of exp(x_j - mx)
	for (int j0 = 0; j0 < nlast; j0 += kAbcTile) {
		const int nj = min(kAbcTile, nlast - j0);
		__syncthreads();
		for (int k = threadIdx.x; k < nj * nvar; k += kAbcThreads) s_th[k] = th_last[(size_t)j0 * nvar + k];
		for (int k = threadIdx.x; k < nj; k += kAbcThreads) s_lw[k] = logw_last[j0 + k];
		__syncthreads();
		if (i < nnew) {
			for (int j = 0; j < nj; j++) {
				float d[kMaxVar];
#pragma unroll
				for (int v = 0; v < kMaxVar; v++) d[v] = v < nvar ? x[v] - s_th[j * nvar + v] : 0.f;
				float q = 0.f;
#pragma unroll
				for (int v1 = 0; v1 < kMaxVar; v1++) {
					if (v1 < nvar) {
						float r = 0.f;
#pragma unroll
						for (int v2 = 0; v2 < kMaxVar; v2++)
							if (v2 < nvar) r = fmaf(s_A[v1 * nvar + v2], d[v2], r);
						q = fmaf(d[v1], r, q);
					}
				}
				const float xe = s_lw[j] - 0.5f * q;
				if (xe == -INFINITY) continue;       // a previous particle of weight zero
				if (xe > mx) {                       // new largest exponent: rescale the sum
					const float f = expf(mx - xe);
					s *= f;
					cmp *= f;
					mx = xe;
				}
				const float y = expf(xe - mx) - cmp;   // Kahan
				const float t = s + y;
				cmp = (t - s) - y;
				s = t;
			}
		}
	}
	if (i < nnew) logsum_out[i] = (double)mx + log((double)s - (double)cmp);
}

}  // namespace
}  // namespace beep

using namespace beep;

extern "C" BEEP_API beep_status beep_abcsmc_weights(int32_t nvar, int32_t nnew, const double *theta_new,
                                                    const double *logprior_new, int32_t nlast,
                                                    const double *theta_last, const double *w_last,
                                                    const double *inv_cov, double size, int32_t normalise,
                                                    double *w_out)
{
	if (nvar <= 0 || nvar > kMaxVar || nnew <= 0 || nlast <= 0 || !theta_new || !logprior_new || !theta_last ||
	    !w_last || !inv_cov || !w_out || !(size > 0))
		return fail(BEEP_BAD_INPUT, "abcsmc weights: bad arguments (nvar must be 1..16, size > 0)");
	int dev = 0;
	CUDA_TRY(cudaGetDevice(&dev));
	// (d/size)^T M^-1 (d/size) = d^T (M^-1 / size^2) d
	std::vector<float> A((size_t)nvar * nvar), tn((size_t)nnew * nvar), tl((size_t)nlast * nvar), lwl(nlast);
	for (int k = 0; k < nvar * nvar; k++) A[k] = (float)(inv_cov[k] / (size * size));
	// both generations centred on the last one's mean (FP64) before rounding to FP32
	std::vector<double> mean(nvar, 0.0);
	for (int j = 0; j < nlast; j++)
		for (int v = 0; v < nvar; v++) mean[v] += theta_last[(size_t)j * nvar + v];
	for (int v = 0; v < nvar; v++) mean[v] /= nlast;
	for (int i = 0; i < nnew; i++)
		for (int v = 0; v < nvar; v++) tn[(size_t)i * nvar + v] = (float)(theta_new[(size_t)i * nvar + v] - mean[v]);
	for (int j = 0; j < nlast; j++)
		for (int v = 0; v < nvar; v++) tl[(size_t)j * nvar + v] = (float)(theta_last[(size_t)j * nvar + v] - mean[v]);
	bool any_weight = false;
	for (int k = 0; k < nlast; k++) {
		if (!(w_last[k] >= 0.0)) return fail(BEEP_BAD_INPUT, "abcsmc weights: negative or NaN previous weight");
		lwl[k] = w_last[k] > 0.0 ? (float)std::log(w_last[k]) : -INFINITY;
		any_weight |= w_last[k] > 0.0;
	}
	if (!any_weight) return fail(BEEP_BAD_INPUT, "abcsmc weights: every previous weight is zero");
	Layout L;
	const size_t o_A = L.add(4 * A.size()), o_tn = L.add(4 * tn.size()), o_tl = L.add(4 * tl.size()),
	             o_wl = L.add(4 * lwl.size()), o_s = L.add(8 * (size_t)nnew);
	DevBuf buf;
	CUDA_TRY(buf.reserve(L.size));
	char *d = (char *)buf.ptr;
	std::vector<double> logsums(nnew);
	cudaError_t e = cudaMemcpy(d + o_A, A.data(), 4 * A.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_tn, tn.data(), 4 * tn.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_tl, tl.data(), 4 * tl.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_wl, lwl.data(), 4 * lwl.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) {
		abc_kernel_logsums<<<(nnew + kAbcThreads - 1) / kAbcThreads, kAbcThreads>>>(
		    nvar, nnew, (const float *)(d + o_tn), nlast, (const float *)(d + o_tl), (const float *)(d + o_wl),
		    (const float *)(d + o_A), (double *)(d + o_s));
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpy(logsums.data(), d + o_s, 8 * (size_t)nnew, cudaMemcpyDeviceToHost);
	buf.release();
	if (e != cudaSuccess) return fail(BEEP_DEVICE_ERROR, std::string("abcsmc weights: ") + cudaGetErrorString(e));
	std::vector<double> logw(nnew);
	double lmax = -INFINITY;
	for (int i = 0; i < nnew; i++) {
		if (logsums[i] != logsums[i]) return fail(BEEP_NAN_RATE, "abcsmc weights: NaN kernel sum (non-finite parameters?)");
		logw[i] = logprior_new[i] - logsums[i];
		lmax = std::max(lmax, logw[i]);
	}
	if (!normalise) {
		for (int i = 0; i < nnew; i++) w_out[i] = std::exp(logw[i]);
	} else {
		// ABCSMC::normalise_particle_weights, w /= mean(w), formed relative to the
		// largest weight so that no weight overflows on the way
		if (!(lmax > -INFINITY)) return fail(BEEP_BAD_INPUT, "abcsmc weights: every new particle has prior weight zero");
		double wsum = 0.0;
		for (int i = 0; i < nnew; i++) {
			w_out[i] = std::exp(logw[i] - lmax);
			wsum += w_out[i];
		}
		wsum /= nnew;
		for (int i = 0; i < nnew; i++) w_out[i] /= wsum;
	}
	return BEEP_OK;
}
