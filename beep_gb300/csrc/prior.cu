// beep_log_prior: the log-prior and bounds of parameter sets on the host --
// Model::prior with Model::spline_prior (src/model.cc:1590-1706) and
// Model::inbounds (src/model.cc:2625-2669), each term as the reference forms
// it, so the values equal the reference's to rounding.  Host code only: the
// caller's MCMC / ABC step evaluates it once per proposal beside the device
// simulation.
#include <cmath>
#include <vector>

#include "capi_internal.h"

namespace {

constexpr double kUnset = 999999999.0;   // the reference's UNSET

double val_of(double v, int32_t par, const double *theta)
{
	return v == kUnset && par >= 0 ? theta[par] : v;
}

// normal_probability / gamma_probability (src/utils.cc:107-120)
double normal_lp(double x, double mean, double var)
{
	return -0.5 * std::log(2 * 3.14159265358979323846 * var) - (x - mean) * (x - mean) / (2 * var);
}

bool inbounds(const beep_prior_spec &s, const double *th)
{
	for (int32_t k = 0; k < s.nparam; k++) {
		const double v = th[k];
		switch (s.type[k]) {
		case BEEP_PRIOR_FIXED: if (v != s.val1[k]) return false; break;
		case BEEP_PRIOR_UNIFORM: if (v < s.val1[k] || v > s.val2[k]) return false; break;
		case BEEP_PRIOR_NORMAL: break;
		default: if (v < 0) return false; break;   // exponential and Dirichlet kinds
		}
		for (int32_t j = s.gt_ptr[k]; j < s.gt_ptr[k + 1]; j++)
			if (v < th[s.gt_param[j]]) return false;
		for (int32_t j = s.lt_ptr[k]; j < s.lt_ptr[k + 1]; j++)
			if (v > th[s.lt_param[j]]) return false;
	}
	return true;
}

// log-prior; false if a term is undefined (a gamma density at a non-positive value)
bool log_prior(const beep_prior_spec &s, const double *th, std::vector<double> &dir, double &Pr)
{
	Pr = 0.0;
	for (int32_t k = 0; k < s.nparam; k++) {
		const double v = th[k];
		switch (s.type[k]) {
		case BEEP_PRIOR_FIXED: break;
		case BEEP_PRIOR_UNIFORM: {
			const double mn = val_of(s.val1[k], s.val1_param[k], th), mx = val_of(s.val2[k], s.val2_param[k], th);
			Pr += std::log(1.0 / (mx - mn));
		} break;
		case BEEP_PRIOR_EXP: {
			const double rate = val_of(s.val1[k], s.val1_param[k], th);
			Pr += std::log(rate) - rate * v;
		} break;
		case BEEP_PRIOR_NORMAL: {
			const double mu = val_of(s.val1[k], s.val1_param[k], th), sd = val_of(s.val2[k], s.val2_param[k], th);
			Pr += normal_lp(v, mu, sd * sd);
		} break;
		case BEEP_PRIOR_DIRICHLET: case BEEP_PRIOR_DIRICHLET_ALPHA: case BEEP_PRIOR_MDIRICHLET: {
			const double a = val_of(s.val1[k], s.val1_param[k], th), b = val_of(s.val2[k], s.val2_param[k], th);
			if (s.ml_mode) {
				if (a != 1) Pr += (a - 1) * std::log(v);
			} else {
				if (!(v > 0) || !(a > 0) || !(b > 0)) return false;
				Pr += (a - 1) * std::log(v) - b * v + a * std::log(b) - std::lgamma(a);
			}
		} break;
		case BEEP_PRIOR_DIRICHLET_FLAT:
			if (!s.ml_mode) Pr += -v;
			break;
		}
	}
	if (s.nsmooth > 0) {
		// Model::dirichlet_correct, then the smoothing terms of spline_prior
		dir.assign(th, th + s.nparam);
		for (int32_t g = 0; g < s.ndirichlet; g++) {
			double sum = 0.0;
			for (int32_t j = s.dir_ptr[g]; j < s.dir_ptr[g + 1]; j++) sum += th[s.dir_param[j]];
			for (int32_t j = s.dir_ptr[g]; j < s.dir_ptr[g + 1]; j++) dir[s.dir_param[j]] = th[s.dir_param[j]] / (s.dir_frac[j] * sum);
		}
		for (int32_t i = 0; i < s.nsmooth; i++) {
			const double value = s.smooth_value[i];
			if (s.smooth_kind[i] == 1) {
				const double mu = std::log(dir[s.smooth_par1[i]] * s.smooth_mult1[i]);
				const double logx = std::log(dir[s.smooth_par2[i]] * s.smooth_mult2[i]);
				Pr += -(logx - mu) * (logx - mu) / (2 * value * value) - logx;
			} else {
				const double d = dir[s.smooth_par1[i]] - dir[s.smooth_par2[i]];
				Pr += -d * d / (2 * value * value);
			}
		}
	}
	return true;
}

}  // namespace

extern "C" BEEP_API beep_status beep_log_prior(const beep_prior_spec *spec, int32_t nset, const double *paramval,
                                               double *logprior_out, int32_t *inbounds_out)
{
	if (!spec || nset < 0 || (nset > 0 && (!paramval || !logprior_out))) return beep::fail(BEEP_BAD_INPUT, "null argument");
	const beep_prior_spec &s = *spec;
	if (s.nparam <= 0 || !s.type || !s.val1 || !s.val2 || !s.val1_param || !s.val2_param || !s.gt_ptr || !s.lt_ptr)
		return beep::fail(BEEP_BAD_INPUT, "prior specification: missing array");
	if (s.ndirichlet < 0 || s.nsmooth < 0 || (s.ndirichlet > 0 && (!s.dir_ptr || !s.dir_param || !s.dir_frac)) ||
	    (s.nsmooth > 0 && (!s.smooth_kind || !s.smooth_par1 || !s.smooth_par2 || !s.smooth_mult1 || !s.smooth_mult2 ||
	                       !s.smooth_value)))
		return beep::fail(BEEP_BAD_INPUT, "prior specification: missing Dirichlet or smoothing array");
	auto par_ok = [&](int32_t p) { return p >= 0 && p < s.nparam; };
	for (int32_t k = 0; k < s.nparam; k++) {
		if (s.type[k] < BEEP_PRIOR_FIXED || s.type[k] > BEEP_PRIOR_MDIRICHLET) return beep::fail(BEEP_BAD_INPUT, "unknown prior type");
		if ((s.val1[k] == kUnset && !par_ok(s.val1_param[k])) || (s.val2[k] == kUnset && s.type[k] != BEEP_PRIOR_EXP &&
		    s.type[k] != BEEP_PRIOR_FIXED && s.type[k] != BEEP_PRIOR_DIRICHLET_FLAT && !par_ok(s.val2_param[k])))
			return beep::fail(BEEP_BAD_INPUT, "prior hyperparameter taken from an unknown parameter");
		for (int32_t j = s.gt_ptr[k]; j < s.gt_ptr[k + 1]; j++) if (!par_ok(s.gt_param[j])) return beep::fail(BEEP_BAD_INPUT, "greater-than parameter out of range");
		for (int32_t j = s.lt_ptr[k]; j < s.lt_ptr[k + 1]; j++) if (!par_ok(s.lt_param[j])) return beep::fail(BEEP_BAD_INPUT, "less-than parameter out of range");
		if (s.ml_mode && (s.type[k] == BEEP_PRIOR_DIRICHLET || s.type[k] == BEEP_PRIOR_DIRICHLET_ALPHA ||
		                  s.type[k] == BEEP_PRIOR_MDIRICHLET) && s.val2[k] != 1.0)
			return beep::fail(BEEP_BAD_INPUT, "in the maximum-likelihood mode a Dirichlet prior needs beta 1 (src/model.cc:1631)");
	}
	for (int32_t g = 0; g < s.ndirichlet; g++)
		for (int32_t j = s.dir_ptr[g]; j < s.dir_ptr[g + 1]; j++) if (!par_ok(s.dir_param[j])) return beep::fail(BEEP_BAD_INPUT, "Dirichlet parameter out of range");
	for (int32_t i = 0; i < s.nsmooth; i++)
		if (!par_ok(s.smooth_par1[i]) || !par_ok(s.smooth_par2[i]) || (s.smooth_kind[i] != 1 && s.smooth_kind[i] != 2))
			return beep::fail(BEEP_BAD_INPUT, "bad smoothing term");
	std::vector<double> dir;
	for (int32_t n = 0; n < nset; n++) {
		const double *th = paramval + (size_t)n * s.nparam;
		const bool ok = inbounds(s, th);
		if (inbounds_out) inbounds_out[n] = ok ? 1 : 0;
		double Pr = 0.0;
		logprior_out[n] = ok && log_prior(s, th, dir, Pr) ? Pr : -INFINITY;
	}
	return BEEP_OK;
}
