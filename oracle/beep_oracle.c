/* beep_oracle.c -- CPU restatement of the reference's tau-leap + observation
 * log-likelihood.  TEST INFRASTRUCTURE ONLY (parity checker and the timed CPU
 * baseline); see beep_oracle.h for the reference functions it follows.
 * Build with -ffp-contract=off so every FP64 operation is rounded as written. */
#include "beep_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "beep_rng_ref.h"

double beep_oracle_exp(double x) { return beep_exp(x); }
double beep_oracle_log(double x) { return beep_log(x); }
double beep_oracle_log_factorial(double k) { return beep_log_factorial(k); }

int32_t beep_oracle_poisson(double mean, uint64_t seed, uint32_t col, uint32_t tr, uint32_t step,
                            uint32_t stream)
{
	return beep_poisson_ref(mean, (uint32_t)seed, (uint32_t)(seed >> 32), col, tr, step, stream);
}

int32_t beep_oracle_binomial(double p, int32_t n, uint64_t seed, uint32_t col, uint32_t tr, uint32_t step,
                             uint32_t stream)
{
	return beep_binomial_ref(p, n, (uint32_t)seed, (uint32_t)(seed >> 32), col, tr, step, stream);
}

/* ---- log-densities: src/utils.cc:107-170 ------------------------------- */

static double normal_probability(double x, double mean, double var)
{
	return -0.5 * log(2 * M_PI * var) - (x - mean) * (x - mean) / (2 * var);
}

static double poisson_probability(int i, double lam)
{
	if (lam == 0) return i == 0 ? 0 : -1000000000.0;
	if (i < 0) return -1000000000.0;
	return i * log(lam) - lam - lgamma(i + 1);
}

static double negative_binomial_probability(unsigned int val, double m, double shape)
{
	return lgamma(shape + val) - lgamma(val + 1) - lgamma(shape) + shape * log(shape / (shape + m))
	       + val * log(m / (shape + m));
}

/* ObservationModel::obs_prob, src/obsmodel.cc:245-305 */
double beep_oracle_obs_prob(double value, int32_t value_kind, double val, int32_t model,
                            double sd, double shape, double thresh)
{
	if (value < 0) value = 0;
	if (value_kind == BEEP_OBSVAL_UNKNOWN) return 0;
	if (value_kind == BEEP_OBSVAL_THRESH) {
		switch (model) {
		case BEEP_OBS_NORMAL:
		case BEEP_OBS_NORMAL_PERCENT:
			if (value < thresh) return normal_probability(thresh, thresh, sd * sd);
			return normal_probability(thresh, value, sd * sd);
		case BEEP_OBS_POISSON: {
			double lam = value; if (lam < 1) lam = 1;
			double sum = 0.0;
			for (double v = 0; v <= thresh; v++) sum += exp(poisson_probability((int)v, lam));
			return log(sum);
		}
		case BEEP_OBS_NEGBIN: {
			double mm = value; if (mm < 1) mm = 1;
			double sum = 0.0;
			for (double v = 0; v <= thresh; v++) sum += exp(negative_binomial_probability((unsigned)v, mm, shape));
			return log(sum);
		}
		}
		return NAN;
	}
	switch (model) {
	case BEEP_OBS_NORMAL:
	case BEEP_OBS_NORMAL_PERCENT:
		return normal_probability(val, value, sd * sd);
	case BEEP_OBS_POISSON: {
		double lam = value; if (lam < 1) lam = 1;
		return poisson_probability((int)(val + 0.5), lam);
	}
	case BEEP_OBS_NEGBIN: {
		double mm = value; if (mm < 1) mm = 1;
		return negative_binomial_probability((unsigned)(int)(val + 0.5), mm, shape);
	}
	}
	return NAN;
}

/* ---- per-batch observation index (src/obsmodel.cc:174-217) -------------- */

typedef struct {
	int32_t ti, tf;
	int32_t ncell_t, ncell_p;
	int32_t *t_ptr, *t_obs;   /* [(tf-ti)*ncell_t + 1], obs lists of transition cells */
	int32_t *p_ptr, *p_obs;   /* same for population cells */
	int32_t *scored;          /* observation indices scored, ascending */
	int32_t nscored;
} obs_index;

static void obs_index_free(obs_index *ix)
{
	free(ix->t_ptr); free(ix->t_obs); free(ix->p_ptr); free(ix->p_obs); free(ix->scored);
}

static int obs_index_build(const beep_model_desc *m, int32_t ti, int32_t tf, obs_index *ix)
{
	memset(ix, 0, sizeof *ix);
	ix->ti = ti; ix->tf = tf;
	int32_t ns = tf - ti;
	ix->ncell_t = m->narea * m->ntrans * m->ndemocatpos;
	ix->ncell_p = m->narea * m->ncomp * m->ndemocatpos;
	size_t nt = (size_t)ns * ix->ncell_t, np = (size_t)ns * ix->ncell_p;
	ix->t_ptr = calloc(nt + 1, sizeof(int32_t));
	ix->p_ptr = calloc(np + 1, sizeof(int32_t));
	ix->scored = malloc(sizeof(int32_t) * (size_t)(m->nobs > 0 ? m->nobs : 1));
	if (!ix->t_ptr || !ix->p_ptr || !ix->scored) return BEEP_OOM;
	for (int32_t i = 0; i < m->nobs; i++) {
		if (m->obs_sett_i[i] >= ti && m->obs_sett_f[i] <= tf) ix->scored[ix->nscored++] = i;
	}
	for (int pass = 0; pass < 2; pass++) {
		for (int32_t k = 0; k < ix->nscored; k++) {
			int32_t i = ix->scored[k];
			for (int32_t s = m->obs_sett_i[i]; s < m->obs_sett_f[i]; s++) {
				for (int32_t q = m->obs_cell_ptr[i]; q < m->obs_cell_ptr[i + 1]; q++) {
					int32_t cell = m->obs_cells[q];
					if (cell >= 0) {
						size_t slot = (size_t)(s - ti) * ix->ncell_t + cell;
						if (pass == 0) ix->t_ptr[slot + 1]++;
						else ix->t_obs[ix->t_ptr[slot]++] = i;
					} else {
						size_t slot = (size_t)(s - ti) * ix->ncell_p + (size_t)(-1 - cell);
						if (pass == 0) ix->p_ptr[slot + 1]++;
						else ix->p_obs[ix->p_ptr[slot]++] = i;
					}
				}
			}
		}
		if (pass == 0) {
			for (size_t k = 0; k < nt; k++) ix->t_ptr[k + 1] += ix->t_ptr[k];
			for (size_t k = 0; k < np; k++) ix->p_ptr[k + 1] += ix->p_ptr[k];
			ix->t_obs = malloc(sizeof(int32_t) * (size_t)(ix->t_ptr[nt] + 1));
			ix->p_obs = malloc(sizeof(int32_t) * (size_t)(ix->p_ptr[np] + 1));
			if (!ix->t_obs || !ix->p_obs) return BEEP_OOM;
		} else {
			/* the fill pass advanced each start to the next start: shift back */
			for (size_t k = nt; k > 0; k--) ix->t_ptr[k] = ix->t_ptr[k - 1];
			ix->t_ptr[0] = 0;
			for (size_t k = np; k > 0; k--) ix->p_ptr[k] = ix->p_ptr[k - 1];
			ix->p_ptr[0] = 0;
		}
	}
	return BEEP_OK;
}

/* ---- one particle ------------------------------------------------------- */

typedef struct {
	double *pop, *popnext;      /* [A][C][DP] */
	double *Imap, *Idiag;       /* [nstrain][A*G] */
	double *dinf, *NMI, *I, *eta; /* [G] */
	double *tmean;              /* [T][DP] */
	int32_t *tn_traj;           /* [(tf-ti)][A][T][DP] */
	double *pop_traj;           /* [(tf-ti)][A][C][DP] */
	double *obs_value;          /* [nobs] */
	double *infdif;             /* [T] */
} work;

static void scatter_inf(const beep_model_desc *m, const double *dinf, int32_t c,
                        double *Ima, double *Idia)
{
	int32_t G = m->nage;
	double diag = m->M_diag[c];
	int32_t j0 = m->M_rowptr[c], j1 = m->M_rowptr[c + 1];
	int32_t v = c * G;
	for (int32_t a = 0; a < G; a++) {
		double di = dinf[a];
		if (di != 0) {
			Idia[v + a] += di * diag;
			for (int32_t j = j0; j < j1; j++) Ima[m->M_to[j] * G + a] += di * m->M_val[j];
		}
	}
}

/* set_I_from_pop, src/state.cc:223-290: Imap/Idiag [NS][A*G] from pop */
static void inf_from_pop(const beep_model_desc *m, const beep_param_tables *tb, const double *pop, work *w,
                         double *Imap, double *Idiag)
{
	const int32_t A = m->narea, G = m->nage, C = m->ncomp, DP = m->ndemocatpos, NS = m->nstrain, DPS = DP / NS;
	const size_t AG = (size_t)A * G;
	memset(Imap, 0, sizeof(double) * AG * NS);
	memset(Idiag, 0, sizeof(double) * AG * NS);
	for (int32_t st = 0; st < NS; st++) {
		for (int32_t c = 0; c < A; c++) {
			for (int32_t a = 0; a < G; a++) w->dinf[a] = 0;
			for (int32_t co = 0; co < C; co++) {
				double inf = tb->infectivity[co];
				if (inf != 0) {
					int32_t dpp = st * DPS;
					for (int32_t dp = 0; dp < DPS; dp++) {
						double pv = pop[((size_t)c * C + co) * DP + dpp];
						if (pv != 0) w->dinf[m->democatpos_age[dp]] += inf * pv;
						dpp++;
					}
				}
			}
			scatter_inf(m, w->dinf, c, Imap + st * AG, Idiag + st * AG);
		}
	}
}

/* update_I_from_transnum, src/state.cc:178-219: adds the infectivity change
 * of the counts tn (minus base, when given: the coupled proposal's
 * dtransnum, src/mbp.cc:308-309,320) to Imap/Idiag */
static void inf_update(const beep_model_desc *m, const int32_t *tn, const int32_t *base, work *w, double *Imap,
                       double *Idiag)
{
	const int32_t A = m->narea, G = m->nage, T = m->ntrans, DP = m->ndemocatpos, NS = m->nstrain, DPS = DP / NS;
	const size_t AG = (size_t)A * G;
	for (int32_t st = 0; st < NS; st++) {
		for (int32_t c = 0; c < A; c++) {
			for (int32_t a = 0; a < G; a++) w->dinf[a] = 0;
			for (int32_t tr = 0; tr < T; tr++) {
				double di = w->infdif[tr];
				if (di != 0) {
					int32_t dpp = st * DPS;
					for (int32_t dp = 0; dp < DPS; dp++) {
						const size_t cell = ((size_t)c * T + tr) * DP + dpp;
						double num = base ? (double)(tn[cell] - base[cell]) : (double)tn[cell];
						if (num != 0) w->dinf[m->democatpos_age[dp]] += di * num;
						dpp++;
					}
				}
			}
			scatter_inf(m, w->dinf, c, Imap + st * AG, Idiag + st * AG);
		}
	}
}

/* set_transmean for area c, src/state.cc:380-456 (with get_NMI,
 * src/state.cc:547-578): w->tmean[T][DP] from pop (the susceptible
 * population of other strains is moved to strain 0 in place) */
static int transmean_area(const beep_model_desc *m, const beep_param_tables *tb, double *pop, const double *Imap,
                          const double *Idiag, int32_t sett, int32_t c, work *w)
{
	const int32_t A = m->narea, G = m->nage, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos;
	const int32_t NS = m->nstrain, DPS = DP / NS;
	const size_t AG = (size_t)A * G;
	double *pc = pop + (size_t)c * C * DP;
	int32_t itr = m->infection_trans;
	double *sus_pop = pc + (size_t)m->trans_from[itr] * DP;
	if (NS > 1) {
		for (int32_t dp = 0; dp < DPS; dp++) {
			double sum = 0.0;
			for (int32_t st = 1; st < NS; st++) {
				int32_t dpp = DPS * st + dp;
				sum += sus_pop[dpp]; sus_pop[dpp] = 0;
			}
			sus_pop[dp] += sum;
		}
	}
	for (int32_t st = 0; st < NS; st++) {
		const double *Id = Idiag + st * AG, *Im = Imap + st * AG;
		double d = tb->geo_spline[sett];
		double omd = 1 - d;
		double fac = m->M_factor[c];
		if (G == 1) {
			double val = Id[c] * (d + fac * omd) + Im[c] * d;
			if (val < 0) val = 0;
			w->NMI[0] = val;
		} else {
			int32_t v = c * G;
			for (int32_t a = 0; a < G; a++) w->I[a] = (Id[v + a] + Im[v + a]) * d + fac * Id[v + a] * omd;
			const double *N = tb->Ntime + (size_t)sett * G * G;
			for (int32_t a = 0; a < G; a++) {
				double sum = 0.0;
				for (int32_t aa = 0; aa < G; aa++) sum += N[a * G + aa] * w->I[aa];
				if (sum < 0) sum = 0;
				w->NMI[a] = sum;
			}
		}
		double be = tb->beta_rows[(size_t)tb->beta_row_of[st * A + c] * m->ndivision + sett];
		be *= tb->areafactor[(size_t)(sett / m->division_per_time) * A + c];
		int32_t ei = tb->efoi_ref[st * A + c];
		double et = tb->efoi_spline[(size_t)ei * m->ndivision + sett] / m->popsize;
		if (tb->efoi_mult) et *= tb->efoi_mult[((size_t)sett * A + c) * NS + st];   /* src/state.cc:415 */
		for (int32_t a = 0; a < G; a++) w->eta[a] = et * tb->efoi_agedist[(size_t)ei * G + a];
		int32_t dpp = st * DPS;
		for (int32_t dp = 0; dp < DPS; dp++) {
			double popu = sus_pop[dp];
			if (popu <= 0) w->tmean[itr * DP + dpp] = 0;
			else {
				int32_t a = m->democatpos_age[dp];
				double v = m->dt * popu * tb->susceptibility[dpp] * (be * w->NMI[a] + w->eta[a]);
				if (v != v) return BEEP_NAN_RATE;
				w->tmean[itr * DP + dpp] = v;
			}
			dpp++;
		}
	}
	for (int32_t tr = 0; tr < T; tr++) {
		if (tr == itr) continue;
		int32_t from = m->trans_from[tr];
		for (int32_t dp = 0; dp < DP; dp++) {
			double popu = pc[(size_t)from * DP + dp];
			if (popu <= 0) w->tmean[tr * DP + dp] = 0;
			else w->tmean[tr * DP + dp] = m->dt * popu * tb->transrate[(size_t)tr * DP + dp];
		}
	}
	if (tb->transmean_mult) {                            /* src/state.cc:446-453 */
		const double *mu = tb->transmean_mult + ((size_t)sett * A + c) * T * DP;
		for (int32_t k = 0; k < T * DP; k++) w->tmean[k] *= mu[k];
	}
	return BEEP_OK;
}

/* update_pop, src/state.cc:460-485: popnext = pop + the flows of tn */
static void update_pop(const beep_model_desc *m, const double *pop, const int32_t *tn, double *popnext)
{
	const int32_t A = m->narea, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos;
	memcpy(popnext, pop, sizeof(double) * (size_t)A * C * DP);
	for (int32_t c = 0; c < A; c++) {
		double *pn = popnext + (size_t)c * C * DP;
		for (int32_t tr = 0; tr < T; tr++) {
			int32_t from = m->trans_from[tr], to = m->trans_to[tr];
			for (int32_t dp = 0; dp < DP; dp++) {
				double num = (double)tn[((size_t)c * T + tr) * DP + dp];
				if (num != 0) { pn[(size_t)from * DP + dp] -= num; pn[(size_t)to * DP + dp] += num; }
			}
		}
	}
}

/* State::democat_change_pop_adjust, src/state.cc:339-376: pop[sett] moved
 * between the values of each change's classification so that their shares,
 * summed over the change's areas, groups and compartments, follow the step's
 * fractions */
static void democat_adjust(const beep_model_desc *m, double *pop, int32_t sett)
{
	const int32_t C = m->ncomp, DP = m->ndemocatpos;
	int32_t frac_off = 0;
	for (int32_t k = 0; k < m->ndemocat_change; k++) {
		const int32_t nv = m->dcc_nval[k];
		const int32_t *dpg = m->dcc_dp + m->dcc_dp_ptr[k];
		const int32_t ng = (m->dcc_dp_ptr[k + 1] - m->dcc_dp_ptr[k]) / nv;
		const double *fr = m->dcc_frac + frac_off + (size_t)sett * nv;
		double cat[32], gap[32];
		for (int32_t f = 0; f < nv; f++) cat[f] = 0;
		for (int32_t j = m->dcc_area_ptr[k]; j < m->dcc_area_ptr[k + 1]; j++) {
			const double *pc = pop + (size_t)m->dcc_area[j] * C * DP;
			for (int32_t g = 0; g < ng; g++)
				for (int32_t co = 0; co < C; co++)
					for (int32_t f = 0; f < nv; f++) cat[f] += pc[(size_t)co * DP + dpg[g * nv + f]];
		}
		double tot = 0.0;
		for (int32_t f = 0; f < nv; f++) tot += cat[f];
		for (int32_t f = 0; f < nv; f++) gap[f] = fr[f] - cat[f] / tot;
		for (int32_t j = m->dcc_area_ptr[k]; j < m->dcc_area_ptr[k + 1]; j++) {
			double *pc = pop + (size_t)m->dcc_area[j] * C * DP;
			for (int32_t g = 0; g < ng; g++)
				for (int32_t co = 0; co < C; co++) {
					double sum = 0.0;
					for (int32_t f = 0; f < nv; f++) sum += pc[(size_t)co * DP + dpg[g * nv + f]];
					for (int32_t f = 0; f < nv; f++) pc[(size_t)co * DP + dpg[g * nv + f]] += gap[f] * sum;
				}
		}
		frac_off += m->ndivision * nv;
	}
}

/* get_obs_value_section + calculate, src/obsmodel.cc:22-109, over the
 * trajectory in w (steps ti..tf-1) */
static int loglik_traj(const beep_model_desc *m, const beep_param_tables *tb, const obs_index *ix, int32_t ti,
                       int32_t tf, const int32_t *tn_traj, const double *pop_traj, work *w, double *Lout)
{
	const int32_t A = m->narea, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos;
	const size_t popsz = (size_t)A * C * DP, tnsz = (size_t)A * T * DP;
	for (int32_t k = 0; k < ix->nscored; k++) w->obs_value[ix->scored[k]] = 0;
	for (int32_t sett = ti; sett < tf; sett++) {
		const int32_t *tn = tn_traj + (size_t)(sett - ti) * tnsz;
		const double *pp = pop_traj + (size_t)(sett - ti) * popsz;
		for (int32_t c = 0; c < A; c++) {
			for (int32_t tr = 0; tr < T; tr++) {
				for (int32_t dp = 0; dp < DP; dp++) {
					int32_t cell = (c * T + tr) * DP + dp;
					double num = (double)tn[cell];
					if (num != 0) {
						size_t slot = (size_t)(sett - ti) * ix->ncell_t + cell;
						for (int32_t q = ix->t_ptr[slot]; q < ix->t_ptr[slot + 1]; q++) {
							int32_t ob = ix->t_obs[q];
							int32_t spl = m->obs_factor_spline[ob];
							if (spl < 0) w->obs_value[ob] += m->obs_factor[ob] * num;
							else w->obs_value[ob] += m->obs_factor[ob] * num * tb->obs_spline[(size_t)spl * m->ndivision + sett];
						}
					}
				}
			}
			for (int32_t co = 0; co < C; co++) {
				for (int32_t dp = 0; dp < DP; dp++) {
					int32_t cell = (c * C + co) * DP + dp;
					size_t slot = (size_t)(sett - ti) * ix->ncell_p + cell;
					if (ix->p_ptr[slot + 1] > ix->p_ptr[slot]) {
						double num = pp[cell];
						for (int32_t q = ix->p_ptr[slot]; q < ix->p_ptr[slot + 1]; q++) {
							int32_t ob = ix->p_obs[q];
							w->obs_value[ob] += m->obs_factor[ob] * num;
						}
					}
				}
			}
		}
	}
	double L = 0.0;
	for (int32_t k = 0; k < ix->nscored; k++) {
		int32_t i = ix->scored[k];
		L += beep_oracle_obs_prob(w->obs_value[i], m->obs_value_kind[i], m->obs_value[i], m->obs_model[i],
		                          m->obs_sd[i], m->obs_shape[i], m->obs_threshold[i]);
	}
	if (L != L) return BEEP_NAN_RATE;
	*Lout = L;
	return BEEP_OK;
}

static void set_infdif(const beep_model_desc *m, const beep_param_tables *tb, work *w)
{
	for (int32_t tr = 0; tr < m->ntrans; tr++)
		w->infdif[tr] = tb->infectivity[m->trans_to[tr]] - tb->infectivity[m->trans_from[tr]];
}

static int simulate_particle(const beep_model_desc *m, const beep_sim_batch *b, const obs_index *ix,
                             int32_t p, work *w)
{
	const int32_t A = m->narea, G = m->nage, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos;
	const int32_t NS = m->nstrain;
	const size_t popsz = (size_t)A * C * DP, tnsz = (size_t)A * T * DP, AG = (size_t)A * G;
	const int32_t grp = b->group_of ? b->group_of[p] : 0;
	const beep_param_tables *tb = &b->groups[grp];
	const uint32_t stream = b->stream_of ? b->stream_of[p] : (uint32_t)p;
	const uint32_t k0 = (uint32_t)b->seed, k1 = (uint32_t)(b->seed >> 32);
	(void)AG; (void)NS;

	set_infdif(m, tb, w);
	if (b->ti == 0) memcpy(w->pop, m->pop_init, sizeof(double) * popsz);
	else if (m->ndemocat_change > 0) memcpy(w->pop, b->pop_in_f64 + (size_t)p * popsz, sizeof(double) * popsz);
	else for (size_t k = 0; k < popsz; k++) w->pop[k] = (double)b->pop_in[(size_t)p * popsz + k];

	for (int32_t sett = b->ti; sett < b->tf; sett++) {
		int32_t *tn = w->tn_traj + (size_t)(sett - b->ti) * tnsz;
		if (m->ndemocat_change > 0) democat_adjust(m, w->pop, sett);
		if (sett == b->ti) inf_from_pop(m, tb, w->pop, w, w->Imap, w->Idiag);
		else inf_update(m, tn - tnsz, NULL, w, w->Imap, w->Idiag);

		for (int32_t c = 0; c < A; c++) {
			int s = transmean_area(m, tb, w->pop, w->Imap, w->Idiag, sett, c, w);
			if (s != BEEP_OK) return s;
			for (int32_t tr = 0; tr < T; tr++) {           /* draws, src/state.cc:614-631 */
				for (int32_t dp = 0; dp < DP; dp++) {
					double mean = w->tmean[tr * DP + dp];
					int32_t cell = (c * T + tr) * DP + dp;
					if (mean == 0) tn[cell] = 0;
					else {
						if (mean > 1000000000.0) return BEEP_COUNT_OVERFLOW;
						tn[cell] = beep_poisson_ref(mean, k0, k1, (uint32_t)(c * DP + dp), (uint32_t)tr,
						                            (uint32_t)sett, stream);
						if (tn[cell] < 0) return BEEP_TIMEOUT;
					}
				}
			}
		}
		memcpy(w->pop_traj + (size_t)(sett - b->ti) * popsz, w->pop, sizeof(double) * popsz);

		/* update_pop, src/state.cc:460-485 (pop[sett+1]; also formed after the last step) */
		update_pop(m, w->pop, tn, w->popnext);
		double *sw = w->pop; w->pop = w->popnext; w->popnext = sw;
	}

	/* outputs */
	size_t nsteps = (size_t)(b->tf - b->ti);
	if (b->pop_out_f64) memcpy(b->pop_out_f64 + (size_t)p * popsz, w->pop, sizeof(double) * popsz);
	if (b->pop_traj_out_f64)
		memcpy(b->pop_traj_out_f64 + (size_t)p * nsteps * popsz, w->pop_traj, sizeof(double) * nsteps * popsz);
	if (b->pop_out) {
		int32_t *po = b->pop_out + (size_t)p * popsz;
		for (size_t k = 0; k < popsz; k++) {
			double v = w->pop[k];
			if (v > 2147483647.0 || v < -2147483648.0) return BEEP_COUNT_OVERFLOW;
			po[k] = (int32_t)v;
		}
	}
	if (b->transnum_out) memcpy(b->transnum_out + (size_t)p * nsteps * tnsz, w->tn_traj, sizeof(int32_t) * nsteps * tnsz);
	if (b->pop_traj_out) {
		int32_t *po = b->pop_traj_out + (size_t)p * nsteps * popsz;
		for (size_t k = 0; k < nsteps * popsz; k++) po[k] = (int32_t)w->pop_traj[k];
	}

	if (b->L_out) {
		int s2 = loglik_traj(m, tb, ix, b->ti, b->tf, w->tn_traj, w->pop_traj, w, &b->L_out[p]);
		if (s2 != BEEP_OK) return s2;
	}
	return BEEP_OK;
}

static int work_alloc(const beep_model_desc *m, int32_t nsteps, work *w)
{
	const size_t A = m->narea, G = m->nage, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos, NS = m->nstrain;
	memset(w, 0, sizeof *w);
	w->pop = malloc(sizeof(double) * A * C * DP);
	w->popnext = malloc(sizeof(double) * A * C * DP);
	w->Imap = malloc(sizeof(double) * A * G * NS);
	w->Idiag = malloc(sizeof(double) * A * G * NS);
	w->dinf = malloc(sizeof(double) * G);
	w->NMI = malloc(sizeof(double) * G);
	w->I = malloc(sizeof(double) * G);
	w->eta = malloc(sizeof(double) * G);
	w->tmean = malloc(sizeof(double) * T * DP);
	w->tn_traj = malloc(sizeof(int32_t) * (size_t)nsteps * A * T * DP);
	w->pop_traj = malloc(sizeof(double) * (size_t)nsteps * A * C * DP);
	w->obs_value = malloc(sizeof(double) * (size_t)(m->nobs > 0 ? m->nobs : 1));
	w->infdif = malloc(sizeof(double) * T);
	if (!w->pop || !w->popnext || !w->Imap || !w->Idiag || !w->dinf || !w->NMI || !w->I || !w->eta ||
	    !w->tmean || !w->tn_traj || !w->pop_traj || !w->obs_value || !w->infdif) return BEEP_OOM;
	return BEEP_OK;
}

static void work_free(work *w)
{
	free(w->pop); free(w->popnext); free(w->Imap); free(w->Idiag); free(w->dinf); free(w->NMI);
	free(w->I); free(w->eta); free(w->tmean); free(w->tn_traj); free(w->pop_traj); free(w->obs_value);
	free(w->infdif);
}

int beep_oracle_simulate(const beep_model_desc *m, const beep_sim_batch *b, int nthreads)
{
	if (!m || !b || b->ti < 0 || b->tf <= b->ti || b->tf > m->ndivision || m->nstrain < 1 ||
	    m->ndemocatpos % m->nstrain != 0 || b->nparticle < 0 || !b->groups)
		return BEEP_BAD_INPUT;
	if (b->ti > 0 && !(m->ndemocat_change > 0 ? (const void *)b->pop_in_f64 : (const void *)b->pop_in))
		return BEEP_BAD_INPUT;
	obs_index ix;
	int st = obs_index_build(m, b->ti, b->tf, &ix);
	if (st != BEEP_OK) { obs_index_free(&ix); return st; }
	int status = BEEP_OK;
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#else
	(void)nthreads;
#endif
#pragma omp parallel
	{
		work w;
		int ws = work_alloc(m, b->tf - b->ti, &w);
		if (ws != BEEP_OK) {
#pragma omp critical
			status = ws;
		}
#pragma omp for schedule(dynamic, 1)
		for (int32_t p = 0; p < b->nparticle; p++) {
			if (ws != BEEP_OK || status != BEEP_OK) continue;
			int s = simulate_particle(m, b, &ix, p, &w);
			if (s != BEEP_OK) {
#pragma omp critical
				status = s;
			}
		}
		work_free(&w);
	}
	obs_index_free(&ix);
	return status;
}


/* ---- model-based proposals: src/mbp.cc:252-330, src/state.cc:109-123,812-826 */

typedef struct {
	int32_t *tn;                /* [S][A][T][DP] */
	double *mean;               /* [S][A][T][DP] transmean */
	double *Imap, *Idiag;       /* [S][NS][A*G] */
} chain_state;

static int chain_alloc(const beep_model_desc *m, chain_state *cs)
{
	const size_t S = m->ndivision, tnsz = (size_t)m->narea * m->ntrans * m->ndemocatpos;
	const size_t IG = (size_t)m->nstrain * m->narea * m->nage;
	cs->tn = malloc(sizeof(int32_t) * S * tnsz);
	cs->mean = malloc(sizeof(double) * S * tnsz);
	cs->Imap = malloc(sizeof(double) * S * IG);
	cs->Idiag = malloc(sizeof(double) * S * IG);
	return cs->tn && cs->mean && cs->Imap && cs->Idiag ? BEEP_OK : BEEP_OOM;
}

static void chain_free(chain_state *cs)
{
	free(cs->tn); free(cs->mean); free(cs->Imap); free(cs->Idiag);
}

/* Mbp::mbp (src/mbp.cc:252-330) from the state ini to the state pro under the
 * tables tb.  simu_all: every cell is drawn afresh and Imap follows
 * set_Imap_sett (this is State::simulate(0, S), src/state.cc:596-638, with
 * transmean and Imap kept); otherwise simu [S][A] (or NULL) marks the SIMU
 * cells and the others are coupled to ini. */
static int mbp_chain(const beep_model_desc *m, const beep_param_tables *tb, const obs_index *ix, uint32_t k0,
                     uint32_t k1, uint32_t stream, int32_t infupd, int simu_all, const uint8_t *simu,
                     const chain_state *ini, chain_state *pro, work *w, double *L)
{
	const int32_t A = m->narea, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos, S = m->ndivision;
	const size_t popsz = (size_t)A * C * DP, tnsz = (size_t)A * T * DP;
	const size_t IG = (size_t)m->nstrain * A * m->nage;
	const int dif = !simu_all && infupd == BEEP_INF_DIF_UPDATE;
	set_infdif(m, tb, w);
	memcpy(w->pop, m->pop_init, sizeof(double) * popsz);   /* pop_init, src/state.cc:59-62 */
	memset(w->Imap, 0, sizeof(double) * IG);               /* dImap, dIdiag (src/mbp.cc:405-414) */
	memset(w->Idiag, 0, sizeof(double) * IG);
	for (int32_t sett = 0; sett < S; sett++) {
		double *Im = pro->Imap + sett * IG, *Id = pro->Idiag + sett * IG;
		int32_t *tn = pro->tn + sett * tnsz;
		double *mn = pro->mean + sett * tnsz;
		if (m->ndemocat_change > 0) democat_adjust(m, w->pop, sett);   /* src/mbp.cc:265 */
		if (!dif) {                                        /* set_Imap_sett, src/state.cc:164-174 */
			if (sett == 0) inf_from_pop(m, tb, w->pop, w, Im, Id);
			else {
				memcpy(Im, Im - IG, sizeof(double) * IG);
				memcpy(Id, Id - IG, sizeof(double) * IG);
				inf_update(m, tn - tnsz, NULL, w, Im, Id);
			}
		} else {                                           /* set_Imap_using_dI, src/state.cc:109-123 */
			const double *Ii = ini->Imap + sett * IG, *Idi = ini->Idiag + sett * IG;
			for (size_t v = 0; v < IG; v++) {
				Im[v] = Ii[v] + w->Imap[v];
				Id[v] = Idi[v] + w->Idiag[v];
			}
		}
		for (int32_t c = 0; c < A; c++) {
			int s = transmean_area(m, tb, w->pop, Im, Id, sett, c, w);
			if (s != BEEP_OK) return s;
			const int sim = simu_all || (simu && simu[(size_t)sett * A + c]);
			for (int32_t tr = 0; tr < T; tr++) {
				for (int32_t dp = 0; dp < DP; dp++) {
					const size_t cell = ((size_t)c * T + tr) * DP + dp;
					const uint32_t col = (uint32_t)(c * DP + dp);
					const double rate_p = w->tmean[tr * DP + dp];
					mn[cell] = rate_p;
					const int32_t num_i = sim ? 0 : ini->tn[sett * tnsz + cell];
					int32_t num_p = 0;
					if (rate_p != 0) {
						if (rate_p > 1000000000.0) return BEEP_COUNT_OVERFLOW;
						if (sim) num_p = beep_poisson_ref(rate_p, k0, k1, col, (uint32_t)tr, (uint32_t)sett, stream);
						else {
							const double rate_i = ini->mean[sett * tnsz + cell];
							if (rate_p > rate_i) {
								num_p = beep_poisson_ref(rate_p - rate_i, k0, k1, col, (uint32_t)tr, (uint32_t)sett, stream);
								if (num_p >= 0) num_p += num_i;
							} else if (rate_p == rate_i) num_p = num_i;
							else num_p = beep_binomial_ref(rate_p / rate_i, num_i, k0, k1, col, (uint32_t)tr,
							                               (uint32_t)sett, stream);
						}
						if (num_p < 0) return BEEP_TIMEOUT;
					}
					tn[cell] = num_p;
				}
			}
		}
		memcpy(w->pop_traj + (size_t)sett * popsz, w->pop, sizeof(double) * popsz);
		if (sett < S - 1) {
			update_pop(m, w->pop, tn, w->popnext);
			double *sw = w->pop; w->pop = w->popnext; w->popnext = sw;
			if (dif) inf_update(m, tn, ini->tn + sett * tnsz, w, w->Imap, w->Idiag);
		}
	}
	return L ? loglik_traj(m, tb, ix, 0, S, pro->tn, w->pop_traj, w, L) : BEEP_OK;
}

/* State::likelihood (src/state.cc:812-826) of the state cs; with tb, the
 * transition means are first recomputed under tb on the fixed state
 * (Mbp::parameter_proposal, src/mbp.cc:460-478), else the stored ones are used */
static int state_likelihood(const beep_model_desc *m, const beep_param_tables *tb, const chain_state *cs, work *w,
                            double *Li)
{
	const int32_t A = m->narea, C = m->ncomp, T = m->ntrans, DP = m->ndemocatpos, S = m->ndivision;
	const size_t popsz = (size_t)A * C * DP, tnsz = (size_t)A * T * DP;
	const size_t IG = (size_t)m->nstrain * A * m->nage;
	double L = 0.0;
	memcpy(w->pop, m->pop_init, sizeof(double) * popsz);
	for (int32_t sett = 0; sett < S; sett++) {
		const int32_t *tn = cs->tn + sett * tnsz;
		if (tb && m->ndemocat_change > 0) democat_adjust(m, w->pop, sett);
		for (int32_t c = 0; c < A; c++) {
			if (tb) {
				int s = transmean_area(m, tb, w->pop, cs->Imap + sett * IG, cs->Idiag + sett * IG, sett, c, w);
				if (s != BEEP_OK) return s;
			}
			for (int32_t tr = 0; tr < T; tr++)
				for (int32_t dp = 0; dp < DP; dp++) {
					const size_t cell = ((size_t)c * T + tr) * DP + dp;
					const double mean = tb ? w->tmean[tr * DP + dp] : cs->mean[sett * tnsz + cell];
					L += poisson_probability(tn[cell], mean);
				}
		}
		if (tb) {
			update_pop(m, w->pop, tn, w->popnext);
			double *sw = w->pop; w->pop = w->popnext; w->popnext = sw;
		}
	}
	*Li = L;
	return BEEP_OK;
}

int beep_oracle_mbp(const beep_model_desc *m, int32_t nchain, const beep_param_tables *groups,
                    const int32_t *ginit, const int32_t *gprop, uint64_t seed, const uint32_t *sinit,
                    const uint32_t *sprop, int32_t inf_update, const uint8_t *simu, double *L_init, double *L_prop,
                    double *Li_init, double *Li_fixed, int32_t *tn_init, int32_t *tn_prop, int nthreads)
{
	if (!m || !groups || nchain < 0 || !ginit || !gprop || !sinit || !sprop) return BEEP_BAD_INPUT;
	const int32_t S = m->ndivision;
	const size_t tnsz = (size_t)m->narea * m->ntrans * m->ndemocatpos;
	const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
	obs_index ix;
	int status = obs_index_build(m, 0, S, &ix);
	if (status != BEEP_OK) { obs_index_free(&ix); return status; }
#ifdef _OPENMP
	if (nthreads > 0) omp_set_num_threads(nthreads);
#else
	(void)nthreads;
#endif
#pragma omp parallel
	{
		work w;
		chain_state a, b;
		int ws = work_alloc(m, S, &w);
		if (ws == BEEP_OK) ws = chain_alloc(m, &a);
		if (ws == BEEP_OK) ws = chain_alloc(m, &b);
		if (ws != BEEP_OK) {
#pragma omp critical
			status = ws;
		}
#pragma omp for schedule(dynamic, 1)
		for (int32_t k = 0; k < nchain; k++) {
			if (ws != BEEP_OK || status != BEEP_OK) continue;
			const beep_param_tables *ti = &groups[ginit[k]], *tp = &groups[gprop[k]];
			double Lv;
			int s = mbp_chain(m, ti, &ix, k0, k1, sinit[k], BEEP_INF_UPDATE, 1, NULL, NULL, &a, &w, &Lv);
			if (s == BEEP_OK && L_init) L_init[k] = Lv;
			if (s == BEEP_OK && Li_init) s = state_likelihood(m, NULL, &a, &w, &Li_init[k]);
			if (s == BEEP_OK && Li_fixed) s = state_likelihood(m, tp, &a, &w, &Li_fixed[k]);
			if (s == BEEP_OK)
				s = mbp_chain(m, tp, &ix, k0, k1, sprop[k], inf_update, 0,
				              simu ? simu + (size_t)k * S * m->narea : NULL, &a, &b, &w, &Lv);
			if (s == BEEP_OK && L_prop) L_prop[k] = Lv;
			if (s == BEEP_OK && tn_init) memcpy(tn_init + (size_t)k * S * tnsz, a.tn, sizeof(int32_t) * S * tnsz);
			if (s == BEEP_OK && tn_prop) memcpy(tn_prop + (size_t)k * S * tnsz, b.tn, sizeof(int32_t) * S * tnsz);
			if (s != BEEP_OK) {
#pragma omp critical
				status = s;
			}
		}
		if (ws == BEEP_OK || 1) { work_free(&w); }
		chain_free(&a); chain_free(&b);
	}
	obs_index_free(&ix);
	return status;
}


/* ---- particle filter: src/pmcmc.cc:180-268, src/mpi.cc:215-327 ----------- */

int beep_oracle_pf(const beep_model_desc *m, const beep_param_tables *tab, int32_t N, uint64_t seed,
                   uint32_t resample_stream, double invT, int32_t form, int32_t nsec, const int32_t *sec_ti,
                   const int32_t *sec_tf, double *loglik, double *loglik_sec, double *L_out, int32_t *anc_out,
                   int32_t *lineage_out, int nthreads)
{
	(void)form;
	if (!m || !tab || N <= 0 || nsec <= 0) return BEEP_BAD_INPUT;
	const size_t popsz = (size_t)m->narea * m->ncomp * m->ndemocatpos;
	const size_t tnsz = (size_t)m->narea * m->ntrans * m->ndemocatpos;
	/* every slot's counts of every section, [section start * N + slot * steps][cell] */
	int32_t *tn_all = lineage_out ? malloc(sizeof(int32_t) * tnsz * (size_t)m->ndivision * N) : NULL;
	int32_t *anc_all = lineage_out ? malloc(sizeof(int32_t) * (size_t)nsec * N) : NULL;
	if (lineage_out && (!tn_all || !anc_all)) return BEEP_OOM;
	/* carried populations: int32, or FP64 with demographic changes */
	const size_t pe = m->ndemocat_change > 0 ? sizeof(double) : sizeof(int32_t);
	char *pops = malloc(pe * popsz * N), *pout = malloc(pe * popsz * N);
	double *L = malloc(sizeof(double) * N), *w = malloc(sizeof(double) * N), *wsum = malloc(sizeof(double) * N);
	int32_t *bp = malloc(sizeof(int32_t) * N), *extra = malloc(sizeof(int32_t) * N);
	if (!pops || !pout || !L || !w || !wsum || !bp || !extra) return BEEP_OOM;
	const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
	double obprob = 0.0;
	int st = BEEP_OK;
	for (int32_t s = 0; s < nsec && st == BEEP_OK; s++) {
		beep_sim_batch b;
		memset(&b, 0, sizeof b);
		b.nparticle = N; b.ngroup = 1; b.groups = tab; b.seed = seed;
		b.ti = sec_ti[s]; b.tf = sec_tf[s];
		if (m->ndemocat_change > 0) {
			b.pop_in_f64 = s > 0 ? (const double *)pops : NULL;
			b.pop_out_f64 = (double *)pout;
		} else {
			b.pop_in = s > 0 ? (const int32_t *)pops : NULL;
			b.pop_out = (int32_t *)pout;
		}
		b.L_out = L;
		if (tn_all) b.transnum_out = tn_all + (size_t)N * sec_ti[s] * tnsz;
		st = beep_oracle_simulate(m, &b, nthreads);
		if (st != BEEP_OK) break;
		if (L_out) memcpy(L_out + (size_t)s * N, L, sizeof(double) * N);
		/* PMCMC::bootstrap */
		double Lmax = -1000000000.0;
		for (int32_t p = 0; p < N; p++) if (L[p] > Lmax) Lmax = L[p];
		double sum = 0.0;
		for (int32_t p = 0; p < N; p++) {
			w[p] = exp(invT * (L[p] - Lmax));
			sum += w[p];
			wsum[p] = sum;
		}
		const double ob = invT * Lmax + log(sum / N);
		if (loglik_sec) loglik_sec[s] = ob;
		obprob += ob;
		for (int32_t p = 0; p < N; p++) bp[p] = -1;
		int32_t ne = 0;
		for (int32_t j = 0; j < N; j++) {
			beep_u32x4 c = {{(uint32_t)j, (uint32_t)s, resample_stream, BEEP_PURPOSE_RESAMPLE << 24}};
			beep_u32x4 r = beep_philox4x32_10(c, k0, k1);
			const double z = beep_u01(r.v[0]) * sum;
			int32_t pp = 0;
			while (pp < N && z > wsum[pp]) pp++;
			if (pp == N) { st = BEEP_NAN_RATE; break; }
			if (bp[pp] == -1) bp[pp] = pp;
			else extra[ne++] = pp;
		}
		for (int32_t p = 0; p < N && st == BEEP_OK; p++)
			if (bp[p] == -1) bp[p] = extra[--ne];
		if (anc_out) memcpy(anc_out + (size_t)s * N, bp, sizeof(int32_t) * N);
		if (anc_all) memcpy(anc_all + (size_t)s * N, bp, sizeof(int32_t) * N);
		/* Mpi::end_sec_swap: slot p continues from its ancestor's population */
		for (int32_t p = 0; p < N; p++) memcpy(pops + pe * popsz * p, pout + pe * popsz * bp[p], pe * popsz);
	}
	if (loglik) *loglik = obprob;
	if (lineage_out && st == BEEP_OK) {
		/* Mpi::particle_sample, src/mpi.cc:331-389 */
		int32_t p = anc_all[(size_t)(nsec - 1) * N + 0];
		for (int32_t k = nsec - 1; k >= 0; k--) {
			const int32_t ti = sec_ti[k], nst = sec_tf[k] - ti;
			memcpy(lineage_out + (size_t)ti * tnsz, tn_all + ((size_t)N * ti + (size_t)p * nst) * tnsz,
			       sizeof(int32_t) * (size_t)nst * tnsz);
			if (k > 0) p = anc_all[(size_t)(k - 1) * N + p];
		}
	}
	free(tn_all); free(anc_all);
	free(pops); free(pout); free(L); free(w); free(wsum); free(bp); free(extra);
	return st;
}


/* ---- ABC-SMC importance weights: src/abcsmc.cc:260-283, src/mvn.cc:185-196 */

void beep_oracle_abcsmc_weights(int32_t nvar, int32_t nnew, const double *theta_new, const double *logprior_new,
                                int32_t nlast, const double *theta_last, const double *w_last,
                                const double *inv_cov, double size, int32_t normalise, double *w_out)
{
	/* new particles are independent: spread over the host's threads (each sum in the reference's order) */
#pragma omp parallel for schedule(static)
	for (int32_t i = 0; i < nnew; i++) {
		const double *pend = theta_new + (size_t)i * nvar;
		double sum = 0.0;
		for (int32_t j = 0; j < nlast; j++) {
			const double *pstart = theta_last + (size_t)j * nvar;
			double q = 0;                                   /* MVN::probability */
			for (int32_t v1 = 0; v1 < nvar; v1++)
				for (int32_t v2 = 0; v2 < nvar; v2++) {
					double val1 = pend[v1] - pstart[v1];
					double val2 = pend[v2] - pstart[v2];
					q += (val1 / size) * inv_cov[v1 * nvar + v2] * (val2 / size);
				}
			sum += w_last[j] * exp(-0.5 * q);
		}
		w_out[i] = exp(logprior_new[i]) / sum;
	}
	if (normalise) {
		double wsum = 0.0;
		for (int32_t i = 0; i < nnew; i++) wsum += w_out[i];
		wsum /= nnew;
		for (int32_t i = 0; i < nnew; i++) w_out[i] /= wsum;
	}
}
