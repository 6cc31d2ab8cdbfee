// beep_abcsmc_weights: ABC-SMC importance weights of a generation
// (ABCSMC::calculate_particle_weight, src/abcsmc.cc:260-271, with
// MVN::probability, src/mvn.cc:185-196, and normalise_particle_weights,
// src/abcsmc.cc:275-283):
//   w_i = exp(logprior_i) / sum_j w_j^last exp(-0.5 (d/size)^T M^-1 (d/size)),
//   d = theta_i - theta_j over the inferred parameters; then w /= mean(w).
//
// The quadratic form is evaluated as a sum of squares: with the Cholesky
// factor L of M^-1 / size^2 (= L L^T, FP64 on the host) every particle is
// mapped to z = L^T (theta - mean of the last generation), and
// q_ij = |z_i - z_j|^2 -- no cancellation between positive and negative
// terms of the form, whatever the correlations (centring removes any large
// common offset).  A matrix that is not positive definite (the reference
// inverts whatever sample covariance it has, singular or not) is used as
// given: q_ij = d^T A d on the centred parameters, as the reference does.
// Each new particle's sum  sum_j w_j exp(-q_ij / 2)  is accumulated as a
// running log-sum-exp -- the largest exponent so far and the compensated sum
// of exp(x_j - max) -- so it cannot underflow.
//   pass 1  FP32 differences and sums, one thread per new particle;
//   pass 2  FP64, for the new particles whose nearest previous particles are
//           far (largest term below exp(-10) of the heaviest previous
//           weight): there the FP32 rounding of q (a few 1e-8 of q) would
//           reach the 1e-6 level in exp(-q/2).
// The log sums, the prior factor and the normalisation (relative to the
// largest weight, so nothing overflows) are FP64.  Where the reference's FP64
// sum underflows to zero (its weight is then infinite) this one stays finite.
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
constexpr double kFarExponent = 10.0;

// q of a difference d: |d|^2 (whitened coordinates) or d^T A d (A row-major nvar x nvar)
template <bool WHITE, typename R>
__device__ __forceinline__ R quad_form(const R *d, const R *A, int nvar)
{
	R q = 0;
	if (WHITE) {
#pragma unroll
		for (int v = 0; v < kMaxVar; v++)
			if (v < nvar) q = fma(d[v], d[v], q);
	} else {
#pragma unroll
		for (int v1 = 0; v1 < kMaxVar; v1++) {
			if (v1 < nvar) {
				R r = 0;
#pragma unroll
				for (int v2 = 0; v2 < kMaxVar; v2++)
					if (v2 < nvar) r = fma(A[v1 * nvar + v2], d[v2], r);
				q = fma(d[v1], r, q);
			}
		}
	}
	return q;
}

template <bool WHITE>
__global__ void __launch_bounds__(kAbcThreads) abc_logsums_f32(int nvar, int nnew, const float *z_new, int nlast,
                                                               const float *z_last, const float *logw_last,
                                                               const float *A, double *logsum_out, float *max_out)
{
	__shared__ float s_z[kAbcTile * kMaxVar];
	__shared__ float s_lw[kAbcTile];
	__shared__ float s_A[kMaxVar * kMaxVar];
	const int i = blockIdx.x * kAbcThreads + threadIdx.x;
	if (!WHITE)
		for (int k = threadIdx.x; k < nvar * nvar; k += kAbcThreads) s_A[k] = A[k];
	float x[kMaxVar];
#pragma unroll
	for (int v = 0; v < kMaxVar; v++) x[v] = (i < nnew && v < nvar) ? z_new[(size_t)i * nvar + v] : 0.f;
	float mx = -INFINITY, s = 0.f, cmp = 0.f;      // running max exponent; compensated sum of exp(x_j - mx)
	for (int j0 = 0; j0 < nlast; j0 += kAbcTile) {
		const int nj = min(kAbcTile, nlast - j0);
		__syncthreads();
		for (int k = threadIdx.x; k < nj * nvar; k += kAbcThreads) s_z[k] = z_last[(size_t)j0 * nvar + k];
		for (int k = threadIdx.x; k < nj; k += kAbcThreads) s_lw[k] = logw_last[j0 + k];
		__syncthreads();
		if (i < nnew) {
			for (int j = 0; j < nj; j++) {
				float d[kMaxVar];
#pragma unroll
				for (int v = 0; v < kMaxVar; v++) d[v] = v < nvar ? x[v] - s_z[j * nvar + v] : 0.f;
				const float q = quad_form<WHITE>(d, s_A, nvar);
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
	if (i < nnew) {
		logsum_out[i] = (double)mx + log((double)s - (double)cmp);
		max_out[i] = mx;
	}
}

// FP64 log sums of the listed new particles (one thread each)
template <bool WHITE>
__global__ void __launch_bounds__(kAbcThreads) abc_logsums_f64(int nvar, int nfar, const int *far_idx,
                                                               const double *z_new, int nlast, const double *z_last,
                                                               const double *logw_last, const double *A,
                                                               double *logsum_out)
{
	const int k = blockIdx.x * kAbcThreads + threadIdx.x;
	if (k >= nfar) return;
	const int i = far_idx[k];
	double x[kMaxVar];
#pragma unroll
	for (int v = 0; v < kMaxVar; v++) x[v] = v < nvar ? z_new[(size_t)i * nvar + v] : 0.0;
	double mx = -INFINITY, s = 0.0;
	for (int j = 0; j < nlast; j++) {
		const double lw = logw_last[j];
		if (lw == -INFINITY) continue;
		double d[kMaxVar];
#pragma unroll
		for (int v = 0; v < kMaxVar; v++) d[v] = v < nvar ? x[v] - z_last[(size_t)j * nvar + v] : 0.0;
		const double xe = lw - 0.5 * quad_form<WHITE>(d, A, nvar);
		if (xe > mx) {
			s *= exp(mx - xe);
			mx = xe;
		}
		s += exp(xe - mx);
	}
	logsum_out[i] = mx + log(s);
}

// L with A = L L^T (A symmetric positive definite, row-major n x n); false otherwise
bool cholesky(int n, const std::vector<double> &A, std::vector<double> &L)
{
	L.assign((size_t)n * n, 0.0);
	for (int i = 0; i < n; i++)
		for (int j = 0; j <= i; j++) {
			double s = A[(size_t)i * n + j];
			for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
			if (i == j) {
				if (!(s > 0.0)) return false;
				L[(size_t)i * n + i] = std::sqrt(s);
			} else {
				L[(size_t)i * n + j] = s / L[(size_t)j * n + j];
			}
		}
	return true;
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
	// (d/size)^T M^-1 (d/size) = |L^T d|^2 with L L^T = M^-1 / size^2
	std::vector<double> Am((size_t)nvar * nvar), Lc;
	for (int i = 0; i < nvar; i++)
		for (int j = 0; j < nvar; j++)   // the symmetric part (the form only sees it)
			Am[(size_t)i * nvar + j] = 0.5 * (inv_cov[i * nvar + j] + inv_cov[j * nvar + i]) / (size * size);
	const bool white = cholesky(nvar, Am, Lc);
	if (!white) {                                  // the form as given, on centred parameters
		Lc.assign((size_t)nvar * nvar, 0.0);
		for (int v = 0; v < nvar; v++) Lc[(size_t)v * nvar + v] = 1.0;
	}
	std::vector<float> Af(Am.begin(), Am.end());
	std::vector<double> mean(nvar, 0.0);
	for (int j = 0; j < nlast; j++)
		for (int v = 0; v < nvar; v++) mean[v] += theta_last[(size_t)j * nvar + v];
	for (int v = 0; v < nvar; v++) mean[v] /= nlast;
	auto whiten = [&](const double *th, int n, std::vector<double> &z64, std::vector<float> &z32) {
		z64.assign((size_t)n * nvar, 0.0);
		z32.resize((size_t)n * nvar);
		for (int i = 0; i < n; i++)
			for (int k = 0; k < nvar; k++) {
				double s = 0.0;
				for (int v = k; v < nvar; v++) s += Lc[(size_t)v * nvar + k] * (th[(size_t)i * nvar + v] - mean[v]);
				z64[(size_t)i * nvar + k] = s;
				z32[(size_t)i * nvar + k] = (float)s;
			}
	};
	std::vector<double> zn64, zl64;
	std::vector<float> zn32, zl32;
	whiten(theta_new, nnew, zn64, zn32);
	whiten(theta_last, nlast, zl64, zl32);
	std::vector<double> lw64(nlast);
	std::vector<float> lw32(nlast);
	double lwmax = -INFINITY;
	for (int k = 0; k < nlast; k++) {
		if (!(w_last[k] >= 0.0)) return fail(BEEP_BAD_INPUT, "abcsmc weights: negative or NaN previous weight");
		lw64[k] = w_last[k] > 0.0 ? std::log(w_last[k]) : -INFINITY;
		lw32[k] = (float)lw64[k];
		lwmax = std::max(lwmax, lw64[k]);
	}
	if (!(lwmax > -INFINITY)) return fail(BEEP_BAD_INPUT, "abcsmc weights: every previous weight is zero");
	Layout L;
	const size_t o_zn = L.add(4 * zn32.size()), o_zl = L.add(4 * zl32.size()), o_wl = L.add(4 * (size_t)nlast),
	             o_s = L.add(8 * (size_t)nnew), o_mx = L.add(4 * (size_t)nnew), o_zn64 = L.add(8 * zn64.size()),
	             o_zl64 = L.add(8 * zl64.size()), o_wl64 = L.add(8 * (size_t)nlast), o_far = L.add(4 * (size_t)nnew),
	             o_A = L.add(4 * Af.size()), o_A64 = L.add(8 * Am.size());
	DevBuf buf;
	CUDA_TRY(buf.reserve(L.size));
	char *d = (char *)buf.ptr;
	std::vector<double> logsums(nnew);
	std::vector<float> mx(nnew);
	std::vector<int> far;
	cudaError_t e = cudaMemcpy(d + o_zn, zn32.data(), 4 * zn32.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_zl, zl32.data(), 4 * zl32.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_wl, lw32.data(), 4 * (size_t)nlast, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_A, Af.data(), 4 * Af.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d + o_A64, Am.data(), 8 * Am.size(), cudaMemcpyHostToDevice);
	if (e == cudaSuccess) {
		auto k32 = white ? abc_logsums_f32<true> : abc_logsums_f32<false>;
		k32<<<(nnew + kAbcThreads - 1) / kAbcThreads, kAbcThreads>>>(
		    nvar, nnew, (const float *)(d + o_zn), nlast, (const float *)(d + o_zl), (const float *)(d + o_wl),
		    (const float *)(d + o_A), (double *)(d + o_s), (float *)(d + o_mx));
		e = cudaGetLastError();
	}
	if (e == cudaSuccess) e = cudaMemcpy(mx.data(), d + o_mx, 4 * (size_t)nnew, cudaMemcpyDeviceToHost);
	if (e == cudaSuccess) {
		for (int i = 0; i < nnew; i++)
			if (!((double)mx[i] >= lwmax - kFarExponent)) far.push_back(i);   // also NaN: recomputed, then checked
		if (!far.empty()) {
			e = cudaMemcpy(d + o_zn64, zn64.data(), 8 * zn64.size(), cudaMemcpyHostToDevice);
			if (e == cudaSuccess) e = cudaMemcpy(d + o_zl64, zl64.data(), 8 * zl64.size(), cudaMemcpyHostToDevice);
			if (e == cudaSuccess) e = cudaMemcpy(d + o_wl64, lw64.data(), 8 * (size_t)nlast, cudaMemcpyHostToDevice);
			if (e == cudaSuccess) e = cudaMemcpy(d + o_far, far.data(), 4 * far.size(), cudaMemcpyHostToDevice);
			if (e == cudaSuccess) {
				auto k64 = white ? abc_logsums_f64<true> : abc_logsums_f64<false>;
				k64<<<((int)far.size() + kAbcThreads - 1) / kAbcThreads, kAbcThreads>>>(
				    nvar, (int)far.size(), (const int *)(d + o_far), (const double *)(d + o_zn64), nlast,
				    (const double *)(d + o_zl64), (const double *)(d + o_wl64), (const double *)(d + o_A64),
				    (double *)(d + o_s));
				e = cudaGetLastError();
			}
		}
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
