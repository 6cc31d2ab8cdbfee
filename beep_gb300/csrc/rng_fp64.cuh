// Keyed variate streams for the FP64 plain form.
//
// uniforms: Philox4x32-10 (Salmon et al., SC'11); key = 64-bit seed; a word
//           w gives u = (w + 1/2) 2^-32, strictly inside (0,1).
// Poisson:  draw of transition tr in column col = c*ndemocatpos + dp at step
//           sett of stream s:
//           mean < 10  sequential inversion, u from word tr%4 of
//                      Philox({col, sett, s, (0<<24) | tr/4});
//           mean >= 10 PTRS (Hoermann 1993), iteration it takes (U, V) from
//                      words 0,1 of Philox({col, sett, s, (1<<24)|(tr<<16)|it}).
// Binomial: thinning of a count n with probability p, q = min(p, 1-p):
//           n q < 10   sequential inversion, u from word tr%4 of
//                      Philox({col, sett, s, (2<<24) | tr/4});
//           n q >= 10  BTRS (Hoermann 1993), iteration it takes (U, V) from
//                      words 0,1 of Philox({col, sett, s, (4<<24)|(tr<<16)|it});
//           for q = 1-p the draw is n minus the draw for q.
// exp/log:  Cody-Waite reduction by ln 2 with a degree-14 Taylor series for
//           e^r; log(m) = 2 atanh((m-1)/(m+1)) series; log k! exact below 23,
//           Stirling series above.  Only IEEE +,-,*,/,sqrt are used, and this
//           header is compiled without FMA contraction (--fmad=false), so the
//           draws are a pure function of (seed, counter, mean) -- identical to
//           any other IEEE-754 implementation of the same recipe.
#pragma once

#include <cstdint>

namespace beep {

constexpr uint32_t PURPOSE_INV = 0u;
constexpr uint32_t PURPOSE_PTRS = 1u;
constexpr uint32_t PURPOSE_THIN = 2u;
constexpr uint32_t PURPOSE_RESAMPLE = 3u;
constexpr uint32_t PURPOSE_BTRS = 4u;

struct U4 { uint32_t x, y, z, w; };

__device__ __forceinline__ U4 philox10(U4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
	for (int r = 0; r < 10; r++) {
		const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
		const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
		c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
	return c;
}

__device__ __forceinline__ double u01_d(uint32_t w)
{
	return (double)w * 2.3283064365386963e-10 + 1.1641532182693481e-10;
}

__device__ __forceinline__ uint32_t word_of(const U4 &r, uint32_t i)
{
	return i == 0 ? r.x : i == 1 ? r.y : i == 2 ? r.z : r.w;
}

__device__ __forceinline__ double scale2(double x, int k)
{
	while (k > 1000) { x *= 1.0715086071862673e+301; k -= 1000; }
	while (k < -1000) { x *= 9.332636185032189e-302; k += 1000; }
	return x * __longlong_as_double((long long)((uint64_t)(k + 1023) << 52));
}

__device__ __forceinline__ double exp_p(double x)
{
	if (x != x) return x;
	if (x > 709.0) return __longlong_as_double(0x7ff0000000000000ll);
	if (x < -745.0) return 0.0;
	const double kd = floor(x * 1.4426950408889634 + 0.5);
	const int k = (int)kd;
	const double r = (x - kd * 0.6931471803691238) - kd * 1.9082149292705877e-10;
	double p = 1.1470745597729725e-11;
	p = p * r + 1.6059043836821613e-10;
	p = p * r + 2.08767569878681e-09;
	p = p * r + 2.505210838544172e-08;
	p = p * r + 2.755731922398589e-07;
	p = p * r + 2.7557319223985893e-06;
	p = p * r + 2.48015873015873e-05;
	p = p * r + 0.0001984126984126984;
	p = p * r + 0.001388888888888889;
	p = p * r + 0.008333333333333333;
	p = p * r + 0.041666666666666664;
	p = p * r + 0.16666666666666666;
	p = p * r + 0.5;
	p = p * r + 1.0;
	p = p * r + 1.0;
	return scale2(p, k);
}

__device__ __forceinline__ double log_p(double x)
{
	if (!(x > 0.0)) return x == 0.0 ? -__longlong_as_double(0x7ff0000000000000ll) : __longlong_as_double(0x7ff8000000000000ll);
	if (x == __longlong_as_double(0x7ff0000000000000ll)) return x;
	int e = 0;
	if (x < 9.332636185032189e-302) { x *= 1.2676506002282294e+30; e = -100; }
	uint64_t b = (uint64_t)__double_as_longlong(x);
	e += (int)((b >> 52) & 0x7ff) - 1023;
	b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
	double m = __longlong_as_double((long long)b);
	if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
	const double s = (m - 1.0) / (m + 1.0);
	const double z = s * s;
	double q = 1.0 / 21.0;
	q = q * z + 1.0 / 19.0;
	q = q * z + 1.0 / 17.0;
	q = q * z + 1.0 / 15.0;
	q = q * z + 1.0 / 13.0;
	q = q * z + 1.0 / 11.0;
	q = q * z + 1.0 / 9.0;
	q = q * z + 1.0 / 7.0;
	q = q * z + 1.0 / 5.0;
	q = q * z + 1.0 / 3.0;
	q = q * z + 1.0;
	const double lm = 2.0 * s * q;
	const double ed = (double)e;
	return ed * 0.6931471803691238 + (ed * 1.9082149292705877e-10 + lm);
}

__device__ __forceinline__ double log_factorial_p(double k)
{
	if (k <= 22.0) {
		double f = 1.0;
		for (double j = 2.0; j <= k; j += 1.0) f *= j;
		return log_p(f);
	}
	const double n = k + 1.0;
	const double in = 1.0 / n, in2 = in * in;
	const double corr = in * (1.0 / 12.0 - in2 * (1.0 / 360.0 - in2 * (1.0 / 1260.0 - in2 * (1.0 / 1680.0))));
	return (n - 0.5) * log_p(n) - n + 0.9189385332046728 + corr;
}

// Poisson(mean) of transition tr in column col at step sett; -1 after `limit`
// rejections (65536 unless a test lowers it; reported as an error by the caller).
static __device__ __noinline__ int32_t poisson_fp64(double mean, uint32_t k0, uint32_t k1, uint32_t col, uint32_t tr,
                                              uint32_t sett, uint32_t stream, uint32_t limit = 65536u)
{
	if (!(mean > 0.0)) return 0;
	if (mean < 10.0) {
		const U4 r = philox10(U4{col, sett, stream, (PURPOSE_INV << 24) | (tr >> 2)}, k0, k1);
		const double u = u01_d(word_of(r, tr & 3u));
		double p = exp_p(-mean);
		double F = p;
		int32_t k = 0;
		while (u > F && k < 1000) {
			k++;
			p = p * mean / (double)k;
			F = F + p;
		}
		return k;
	}
	const double slam = sqrt(mean);
	const double loglam = log_p(mean);
	const double b = 0.931 + 2.53 * slam;
	const double a = -0.059 + 0.02483 * b;
	const double invalpha = 1.1239 + 1.1328 / (b - 3.4);
	const double vr = 0.9277 - 3.6224 / (b - 2.0);
	const double log_invalpha = log_p(invalpha);
	for (uint32_t it = 0; it < limit; it++) {
		const U4 r = philox10(U4{col, sett, stream, (PURPOSE_PTRS << 24) | (tr << 16) | it}, k0, k1);
		const double U = u01_d(r.x) - 0.5;
		const double V = u01_d(r.y);
		const double us = 0.5 - fabs(U);
		const double k = floor((2.0 * a / us + b) * U + mean + 0.43);
		if (us >= 0.07 && V <= vr) return (int32_t)k;
		if (k < 0.0 || (us < 0.013 && V > us)) continue;
		const double lhs = log_p(V) + log_invalpha - log_p(a / (us * us) + b);
		const double rhs = -mean + k * loglam - log_factorial_p(k);
		if (lhs <= rhs) return (int32_t)k;
	}
	return -1;
}

// Binomial(n, p) thinning of transition tr in column col at step sett (the
// coupled proposal's count when the proposed mean is below the current one);
// -1 after `limit` rejections.
static __device__ __noinline__ int32_t binomial_fp64(double p, int32_t n, uint32_t k0, uint32_t k1, uint32_t col,
                                               uint32_t tr, uint32_t sett, uint32_t stream, uint32_t limit = 65536u)
{
	if (n <= 0 || !(p > 0.0)) return 0;
	if (p >= 1.0) return n;
	const bool flip = p > 0.5;
	const double q = flip ? 1.0 - p : p;
	const double nd = (double)n;
	int32_t k;
	if (nd * q < 10.0) {
		const U4 r = philox10(U4{col, sett, stream, (PURPOSE_THIN << 24) | (tr >> 2)}, k0, k1);
		const double u = u01_d(word_of(r, tr & 3u));
		const double ratio = q / (1.0 - q);
		double f = exp_p(nd * log_p(1.0 - q));
		double F = f;
		k = 0;
		while (u > F && k < n) {
			f = f * ratio * (double)(n - k) / (double)(k + 1);
			k++;
			F = F + f;
		}
	} else {
		const double spq = sqrt(nd * q * (1.0 - q));
		const double b = 1.15 + 2.53 * spq;
		const double a = -0.0873 + 0.0248 * b + 0.01 * q;
		const double c = nd * q + 0.5;
		const double alpha = (2.83 + 5.1 / b) * spq;
		const double vr = 0.92 - 4.2 / b;
		const double m = floor((nd + 1.0) * q);
		const double lpq = log_p(q / (1.0 - q));
		const double h = log_factorial_p(m) + log_factorial_p(nd - m);
		k = -1;
		for (uint32_t it = 0; it < limit; it++) {
			const U4 r = philox10(U4{col, sett, stream, (PURPOSE_BTRS << 24) | (tr << 16) | it}, k0, k1);
			const double U = u01_d(r.x) - 0.5;
			const double V = u01_d(r.y);
			const double us = 0.5 - fabs(U);
			const double kd = floor((2.0 * a / us + b) * U + c);
			if (kd < 0.0 || kd > nd) continue;
			if (us >= 0.07 && V <= vr) { k = (int32_t)kd; break; }
			const double lhs = log_p(V * alpha / (a / (us * us) + b));
			const double rhs = h - log_factorial_p(kd) - log_factorial_p(nd - kd) + (kd - m) * lpq;
			if (lhs <= rhs) { k = (int32_t)kd; break; }
		}
		if (k < 0) return -1;
	}
	return flip ? n - k : k;
}

}  // namespace beep
