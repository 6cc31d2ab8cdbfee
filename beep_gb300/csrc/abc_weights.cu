// beep_abcsmc_weights: ABC-SMC importance weights of a generation
// (ABCSMC::calculate_particle_weight, src/abcsmc.cc:260-271, with
// MVN::probability, src/mvn.cc:185-196, and normalise_particle_weights,
// src/abcsmc.cc:275-283):
//   w_i = exp(logprior_i) / sum_j w_j^last exp(-0.5 (d/size)^T M^-1 (d/size)),
//   d = theta_i - theta_j over the inferred parameters; then w /= mean(w).
// The N_new x N_last kernel terms are formed in FP32 (each is a quadratic form
// of parameter differences of order one) and summed per particle with
// compensation; the per-particle sums, the prior factor and the normalisation
// are FP64.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "capi_internal.h"

namespace beep {
namespace {

constexpr int kAbcThreads = 256;
constexpr int kAbcTile = 256;        // last-generation particles staged per pass
constexpr int kMaxVar = 16;

__global__ void __launch_bounds__(kAbcThreads) abc_kernel_sums(int nvar, int nnew, const float *th_new, int nlast,
                                                               const float *th_last, const float *w_last,
                                                               const float *A, double *sum_out)
{
	__shared__ float s_th[kAbcTile * kMaxVar];
	__shared__ float s_w[kAbcTile];
	__shared__ float s_A[kMaxVar * kMaxVar];
	const int i = blockIdx.x * kAbcThreads + threadIdx.x;
	for (int k = threadIdx.x; k < nvar * nvar; k += kAbcThreads) s_A[k] = A[k];
	float x[kMaxVar];
#pragma unroll
	for (int v = 0; v < kMaxVar; v++) x[v] = (i < nnew && v < nvar) ? th_new[(size_t)i * nvar + v] : 0.f;
	float s = 0.f, cmp = 0.f;
	for (int j0 = 0; j0 < nlast; j0 += kAbcTile) {
		const int nj = min(kAbcTile, nlast - j0);
		__syncthreads();
		for (int k = threadIdx.x; k < nj * nvar; k += kAbcThreads) s_th[k] = th_last[(size_t)j0 * nvar + k];
		for (int k = threadIdx.x; k < nj; k += kAbcThreads) s_w[k] = w_last[j0 + k];
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
				const float term = s_w[j] * expf(-0.5f * q);
				const float y = term - cmp;          // Kahan
				const float t = s + y;
				cmp = (t - s) - y;
				s = t;
			}
		}
	}
	if (i < nnew) sum_out[i] = (double)s - (double)cmp;
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
	std::vector<float> A((size_t)nvar * nvar), tn((size_t)nnew * nvar), tl((size_t)nlast * nvar), wl(nlast);
	for (int k = 0; k < nvar * nvar; k++) A[k] = (float)(inv_cov[k] / (size * size));
	for (size_t k = 0; k < tn.size(); k++) tn[k] = (float)theta_new[k];
	for (size_t k = 0; k < tl.size(); k++) tl[k] = (float)theta_last[k];
	for (int k = 0; k < nlast; k++) wl[k] = (float)w_last[k];
	Layout L;
	const size_t o_A = L.add(4 * A.size()), o_tn = L.add(4 * tn.size()), o_tl = L.add(4 * tl.size()),
	             o_wl = L.add(4 * wl.size()), o_s = L.add(8 * (size_t)nnew);
	DevBuf buf;
	CUDA_TRY(buf.reserve(L.size));
	char *d = (char *)buf.ptr;
	std::vector<double> sums(nnew);
	cudaError_t e = cudaMemcpy(d + o_A, A.data(), 4 * A.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_tn, tn.data(), 4 * tn.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_tl, tl.data(), 4 * tl.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_wl, wl.data(), 4 * wl.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) {
		abc_kernel_sums<<<(nnew + kAbcThreads - 1) / kAbcThreads, kAbcThreads>>>(
		    nvar, nnew, (const float *)(d + o_tn), nlast, (const float *)(d + o_tl), (const float *)(d + o_wl),
		    (const float *)(d + o_A), (double *)(d + o_s));
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpy(sums.data(), d + o_s, 8 * (size_t)nnew, cudaMemcpyDeviceToHost);
	buf.release();
	if (e != cudaSuccess) return fail(BEEP_DEVICE_ERROR, std::string("abcsmc weights: ") + cudaGetErrorString(e));
	for (int i = 0; i < nnew; i++) w_out[i] = std::exp(logprior_new[i]) / sums[i];
	if (normalise) {                                  // ABCSMC::normalise_particle_weights
		double wsum = 0.0;
		for (int i = 0; i < nnew; i++) wsum += w_out[i];
		wsum /= nnew;
		for (int i = 0; i < nnew; i++) w_out[i] /= wsum;
	}
	return BEEP_OK;
}
