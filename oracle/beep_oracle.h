/* beep_oracle.h -- CPU restatement of BEEP's tau-leap simulation and
 * observation log-likelihood.  TEST INFRASTRUCTURE ONLY: the parity checker
 * and the timed CPU baseline.  The product never links it.
 *
 * It consumes the same plain tables as the C ABI in include/beep_gpu.h and
 * follows the reference loop by loop:
 *   State::simulate(ti,tf)            src/state.cc:596-638
 *   State::set_I_from_pop             src/state.cc:223-290
 *   State::set_Imap_sett / update_I_from_transnum  src/state.cc:164-219
 *   State::get_NMI                    src/state.cc:547-578
 *   State::set_transmean              src/state.cc:380-456
 *   State::update_pop                 src/state.cc:460-485
 *   ObservationModel::calculate(_section), get_obs_value_section, obs_prob
 *                                     src/obsmodel.cc:22-109,245-305
 *   normal/poisson/negative_binomial_probability  src/utils.cc:107-170
 * Transition counts are drawn from the keyed stream of beep_rng_ref.h (the
 * same stream the replay hook feeds to the compiled reference).
 */
#ifndef BEEP_ORACLE_H
#define BEEP_ORACLE_H

#include "../include/beep_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runs a batch exactly as beep_simulate specifies, on nthreads host threads
 * (0 = all).  Returns 0 on success, else a beep_status code. */
int beep_oracle_simulate(const beep_model_desc *m, const beep_sim_batch *b, int nthreads);

/* Bootstrap particle filter (PMCMC::obs_prob + bootstrap + Mpi::end_sec_swap,
 * src/pmcmc.cc:180-268, src/mpi.cc:215-327): per section, simulate every
 * particle slot p from its carried population (stream p), weight
 * w = exp(invT (L - Lmax)), add invT Lmax + log(sum w / N) to the estimate, and
 * resample with the "selected particle keeps its own slot" placement; the j-th
 * resampling uniform of section s is word 0 of
 * Philox({j, s, resample_stream, RESAMPLE<<24}).  Outputs: the estimate, the
 * per-section terms, per-section L [nsec][N], ancestors [nsec][N] and the
 * sampled lineage's counts [S][A][T][DP] (Mpi::particle_sample, src/mpi.cc:331-389)
 * (each may be NULL). */
int beep_oracle_pf(const beep_model_desc *m, const beep_param_tables *tab, int32_t N, uint64_t seed,
                   uint32_t resample_stream, double invT, int32_t form, int32_t nsec, const int32_t *sec_ti,
                   const int32_t *sec_tf, double *loglik, double *loglik_sec, double *L_out, int32_t *anc_out,
                   int32_t *lineage_out, int nthreads);

/* Model-based proposals (Mbp::mbp, src/mbp.cc:252-330) for nchain chains.
 * Chain k: the initial state is State::simulate(theta_k) over [0, ndivision)
 * with tables groups[ginit[k]] and variate stream sinit[k]; the proposal is
 * Mbp::mbp(theta'_k, inf_update) with tables groups[gprop[k]] and stream
 * sprop[k], simu [k][ndivision][narea] marking SIMU cells (NULL: none).
 * Outputs (each may be NULL): L_init / L_prop [nchain] log-likelihoods of the
 * two states (EF = -2 L); Li_init [nchain] State::likelihood() of the initial
 * state (src/state.cc:812-826); Li_fixed [nchain] the same with the means
 * recomputed under theta'_k on the fixed initial state (parameter_proposal,
 * src/mbp.cc:460-478); tn_init / tn_prop [nchain][S][A][T][DP]. */
int beep_oracle_mbp(const beep_model_desc *m, int32_t nchain, const beep_param_tables *groups,
                    const int32_t *ginit, const int32_t *gprop, uint64_t seed, const uint32_t *sinit,
                    const uint32_t *sprop, int32_t inf_update, const uint8_t *simu, double *L_init, double *L_prop,
                    double *Li_init, double *Li_fixed, int32_t *tn_init, int32_t *tn_prop, int nthreads);

/* ABC-SMC weights (src/abcsmc.cc:260-283, src/mvn.cc:185-196), FP64 as the
 * reference computes them. */
void beep_oracle_abcsmc_weights(int32_t nvar, int32_t nnew, const double *theta_new, const double *logprior_new,
                                int32_t nlast, const double *theta_last, const double *w_last,
                                const double *inv_cov, double size, int32_t normalise, double *w_out);

/* One Poisson draw from the keyed stream (exposed for sampler tests). */
int32_t beep_oracle_poisson(double mean, uint64_t seed, uint32_t col, uint32_t tr, uint32_t step,
                            uint32_t stream);

/* One Binomial(n, p) thinning draw from the keyed stream (for sampler tests). */
int32_t beep_oracle_binomial(double p, int32_t n, uint64_t seed, uint32_t col, uint32_t tr, uint32_t step,
                             uint32_t stream);

/* Project exp / log / log-factorial used inside the sampler (for tests). */
double beep_oracle_exp(double x);
double beep_oracle_log(double x);
double beep_oracle_log_factorial(double k);

/* obs_prob of one observation value (src/obsmodel.cc:245-305). */
double beep_oracle_obs_prob(double value, int32_t value_kind, double obs_value, int32_t model,
                            double sd, double shape, double threshold);

#ifdef __cplusplus
}
#endif

#endif
