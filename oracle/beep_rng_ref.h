/* beep_rng_ref.h -- CPU statement of the project's counter-based variate
 * streams.  TEST INFRASTRUCTURE (oracle): used by the oracle restatement and
 * by the replay hook that drives the compiled reference; never shipped.
 *
 * The reference draws every transition count with
 *     poisson_sample(mean)  ->  std::poisson_distribution<int>  (src/utils.cc:148-153)
 * on one global engine, so its draws depend on call order.  For parity the
 * oracle, the replayed reference and the CUDA kernels all draw from the same
 * keyed stream instead:
 *
 *   uniforms : Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random
 *              numbers: as easy as 1, 2, 3", SC'11).  key = 64-bit seed.
 *              A 32-bit word w gives u = (w + 1/2) 2^-32, strictly in (0, 1).
 *   Poisson  : the draw of transition tr in column (area c, dp) at step sett
 *              of stream s, column index col = c*ndemocatpos + dp:
 *              mean < 10  -> sequential inversion with the word tr%4 of
 *                            Philox({col, sett, s, (0<<24) | tr/4}), so one
 *                            Philox call serves four transitions;
 *              mean >= 10 -> PTRS, transformed rejection with squeeze
 *                            (W. Hoermann, "The transformed rejection method
 *                            for generating Poisson random variables",
 *                            Insurance: Math. & Econ. 12, 1993); iteration it
 *                            takes (U, V) from words 0, 1 of
 *                            Philox({col, sett, s, (1<<24) | (tr<<16) | it}).
 *   Binomial : thinning of a count n with probability p (coupled proposals,
 *              src/mbp.cc:300-303); with q = min(p, 1-p):
 *              n q < 10   -> sequential inversion with the word tr%4 of
 *                            Philox({col, sett, s, (2<<24) | tr/4});
 *              n q >= 10  -> BTRS, transformed rejection with squeeze
 *                            (W. Hoermann, "The generation of binomial random
 *                            variates", J. Statist. Comput. Simul. 46, 1993);
 *                            iteration it takes (U, V) from words 0, 1 of
 *                            Philox({col, sett, s, (4<<24) | (tr<<16) | it});
 *              a draw for q = 1-p is n minus the draw for q.
 *   exp/log  : written here from the mathematics (Cody-Waite reduction by
 *              ln 2 + Taylor series of e^r; log by the atanh series), using
 *              only IEEE-754 +,-,*,/ and sqrt so that the host and the GPU
 *              produce identical bits.  Compile with -ffp-contract=off.
 */
#ifndef BEEP_RNG_REF_H
#define BEEP_RNG_REF_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#define BEEP_PURPOSE_INV 0u      /* inversion words of transition draws       */
#define BEEP_PURPOSE_PTRS 1u     /* rejection pairs of transition draws       */
#define BEEP_PURPOSE_THIN 2u     /* binomial thinning of coupled proposals    */
#define BEEP_PURPOSE_RESAMPLE 3u /* particle-filter resampling uniforms       */
#define BEEP_PURPOSE_BTRS 4u     /* rejection pairs of binomial thinning      */

typedef struct { uint32_t v[4]; } beep_u32x4;

static inline void beep_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo)
{
	uint64_t p = (uint64_t)a * (uint64_t)b;
	*hi = (uint32_t)(p >> 32);
	*lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds (multipliers and Weyl increments of the SC'11 paper). */
static inline beep_u32x4 beep_philox4x32_10(beep_u32x4 ctr, uint32_t k0, uint32_t k1)
{
	for (int r = 0; r < 10; r++) {
		uint32_t hi0, lo0, hi1, lo1;
		beep_mulhilo32(0xD2511F53u, ctr.v[0], &hi0, &lo0);
		beep_mulhilo32(0xCD9E8D57u, ctr.v[2], &hi1, &lo1);
		beep_u32x4 n;
		n.v[0] = hi1 ^ ctr.v[1] ^ k0;
		n.v[1] = lo1;
		n.v[2] = hi0 ^ ctr.v[3] ^ k1;
		n.v[3] = lo0;
		ctr = n;
		k0 += 0x9E3779B9u;
		k1 += 0xBB67AE85u;
	}
	return ctr;
}

static inline double beep_u01(uint32_t w)
{
	return (double)w * 2.3283064365386963e-10 + 1.1641532182693481e-10;   /* (w + 1/2) 2^-32, exact */
}

/* ---- exp / log / log-factorial written from the mathematics ------------- */

static inline double beep_scale2(double x, int k)
{
	/* x * 2^k for |k| <= 1100 using exact power-of-two factors */
	while (k > 1000) { x *= 1.0715086071862673e+301; k -= 1000; }
	while (k < -1000) { x *= 9.332636185032189e-302; k += 1000; }
	uint64_t b = (uint64_t)(k + 1023) << 52;
	double s;
	memcpy(&s, &b, sizeof s);
	return x * s;
}

static inline double beep_exp(double x)
{
	if (x != x) return x;
	if (x > 709.0) return INFINITY;
	if (x < -745.0) return 0.0;
	double kd = floor(x * 1.4426950408889634 + 0.5);
	int k = (int)kd;
	/* ln2 split: LN2_HI keeps 32 significant bits so kd*LN2_HI is exact */
	double r = (x - kd * 0.6931471803691238) - kd * 1.9082149292705877e-10;
	/* Taylor series of e^r, |r| <= 0.347, degree 14 (Horner) */
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
	return beep_scale2(p, k);
}

static inline double beep_log(double x)
{
	if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
	if (x == INFINITY) return x;
	int e = 0;
	if (x < 9.332636185032189e-302) { x *= 1.2676506002282294e+30; e = -100; }
	uint64_t b;
	memcpy(&b, &x, sizeof b);
	e += (int)((b >> 52) & 0x7ff) - 1023;
	b = (b & 0x000fffffffffffffull) | 0x3ff0000000000000ull;
	double m;
	memcpy(&m, &b, sizeof m);                    /* m in [1, 2) */
	if (m > 1.4142135623730951) { m *= 0.5; e += 1; }
	double s = (m - 1.0) / (m + 1.0);            /* |s| <= 0.1716 */
	double z = s * s;
	/* log(m) = 2 atanh(s) = 2 s (1 + z/3 + z^2/5 + ... + z^10/21) */
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
	double lm = 2.0 * s * q;
	double ed = (double)e;
	return ed * 0.6931471803691238 + (ed * 1.9082149292705877e-10 + lm);
}

/* log(k!) for integer k >= 0: exact factorial up to 22!, else Stirling's
 * series for log Gamma(n), n = k+1, through the n^-7 term. */
static inline double beep_log_factorial(double k)
{
	if (k <= 22.0) {
		double f = 1.0;
		for (double j = 2.0; j <= k; j += 1.0) f *= j;
		return beep_log(f);
	}
	double n = k + 1.0;
	double in = 1.0 / n, in2 = in * in;
	double corr = in * (1.0 / 12.0 - in2 * (1.0 / 360.0 - in2 * (1.0 / 1260.0 - in2 * (1.0 / 1680.0))));
	return (n - 0.5) * beep_log(n) - n + 0.9189385332046728 + corr;
}

/* ---- Poisson(mean) from the keyed stream --------------------------------- */

#define BEEP_INV_KMAX 1000

/* Draw of transition tr of column col (= c*ndemocatpos + dp) at step sett. */
static inline int32_t beep_poisson_ref(double mean, uint32_t k0, uint32_t k1, uint32_t col,
                                       uint32_t tr, uint32_t sett, uint32_t stream)
{
	if (!(mean > 0.0)) return 0;
	if (mean < 10.0) {
		beep_u32x4 c = {{col, sett, stream, (BEEP_PURPOSE_INV << 24) | (tr >> 2)}};
		beep_u32x4 r = beep_philox4x32_10(c, k0, k1);
		double u = beep_u01(r.v[tr & 3u]);
		double p = beep_exp(-mean);
		double F = p;
		int32_t k = 0;
		while (u > F && k < BEEP_INV_KMAX) {
			k++;
			p = p * mean / (double)k;
			F = F + p;
		}
		return k;
	}
	double slam = sqrt(mean);
	double loglam = beep_log(mean);
	double b = 0.931 + 2.53 * slam;
	double a = -0.059 + 0.02483 * b;
	double invalpha = 1.1239 + 1.1328 / (b - 3.4);
	double vr = 0.9277 - 3.6224 / (b - 2.0);
	double log_invalpha = beep_log(invalpha);
	for (uint32_t it = 0; it < 65536u; it++) {
		beep_u32x4 c = {{col, sett, stream, (BEEP_PURPOSE_PTRS << 24) | (tr << 16) | it}};
		beep_u32x4 r = beep_philox4x32_10(c, k0, k1);
		double U = beep_u01(r.v[0]) - 0.5;
		double V = beep_u01(r.v[1]);
		double us = 0.5 - fabs(U);
		double k = floor((2.0 * a / us + b) * U + mean + 0.43);
		if (us >= 0.07 && V <= vr) return (int32_t)k;
		if (k < 0.0 || (us < 0.013 && V > us)) continue;
		double lhs = beep_log(V) + log_invalpha - beep_log(a / (us * us) + b);
		double rhs = -mean + k * loglam - beep_log_factorial(k);
		if (lhs <= rhs) return (int32_t)k;
	}
	return -1;   /* 65536 rejections: reported as an error by the callers */
}

/* ---- Binomial(n, p) from the keyed stream -------------------------------- */

/* Thinning of count n of transition tr of column col at step sett; -1 after
 * 65536 rejections. */
static inline int32_t beep_binomial_ref(double p, int32_t n, uint32_t k0, uint32_t k1, uint32_t col,
                                        uint32_t tr, uint32_t sett, uint32_t stream)
{
	if (n <= 0 || !(p > 0.0)) return 0;
	if (p >= 1.0) return n;
	const int flip = p > 0.5;
	const double q = flip ? 1.0 - p : p;
	const double nd = (double)n;
	int32_t k;
	if (nd * q < 10.0) {
		beep_u32x4 c = {{col, sett, stream, (BEEP_PURPOSE_THIN << 24) | (tr >> 2)}};
		beep_u32x4 r = beep_philox4x32_10(c, k0, k1);
		const double u = beep_u01(r.v[tr & 3u]);
		const double ratio = q / (1.0 - q);
		double f = beep_exp(nd * beep_log(1.0 - q));
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
		const double lpq = beep_log(q / (1.0 - q));
		const double h = beep_log_factorial(m) + beep_log_factorial(nd - m);
		k = -1;
		for (uint32_t it = 0; it < 65536u; it++) {
			beep_u32x4 cc = {{col, sett, stream, (BEEP_PURPOSE_BTRS << 24) | (tr << 16) | it}};
			beep_u32x4 r = beep_philox4x32_10(cc, k0, k1);
			const double U = beep_u01(r.v[0]) - 0.5;
			const double V = beep_u01(r.v[1]);
			const double us = 0.5 - fabs(U);
			const double kd = floor((2.0 * a / us + b) * U + c);
			if (kd < 0.0 || kd > nd) continue;
			if (us >= 0.07 && V <= vr) { k = (int32_t)kd; break; }
			const double lhs = beep_log(V * alpha / (a / (us * us) + b));
			const double rhs = h - beep_log_factorial(kd) - beep_log_factorial(nd - kd) + (kd - m) * lpq;
			if (lhs <= rhs) { k = (int32_t)kd; break; }
		}
		if (k < 0) return -1;
	}
	return flip ? n - k : k;
}

#endif
