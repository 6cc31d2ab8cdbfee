/* beep_gpu.h -- C ABI of the GB300 implementation of BEEP's tau-leap
 * simulation and observation log-likelihood.
 *
 * The reference has no plugin interface: the hot path is the in-process C++
 * class State (src/state.hh:14-134) with ObservationModel
 * (src/obsmodel.hh:10-41).  A caller that already ran State::set_param for a
 * parameter set (src/state.cc:66-91) holds every table the path reads; this
 * ABI takes those tables as plain arrays and returns what the reference would
 * have stored in State (transnum, pop) and what ObservationModel::calculate /
 * calculate_section would have returned (the log-likelihood L, EF = -2 L).
 *
 * Conventions
 *  - All sizes are int32_t, all real tables are IEEE double, counts int32_t.
 *  - Arrays are row-major in the index order of the reference's nested
 *    vectors, e.g. transnum[sett][c][tr][dp] (src/state.hh:25).
 *  - Every entry point returns beep_status; beep_last_error() gives the text
 *    of the last failure on the calling thread.  The library never exits the
 *    process (the reference calls exit() through emsg, src/utils.cc:296-316).
 *  - Random variates come from a keyed counter-based stream (Philox4x32-10),
 *    key = seed, counter = (cell, step, stream, purpose|iteration), so any
 *    particle's trajectory is reproducible from (seed, stream) alone.
 */
#ifndef BEEP_GPU_H
#define BEEP_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BEEP_GPU_ABI_VERSION 4

#if defined(__GNUC__)
#define BEEP_API __attribute__((visibility("default")))
#else
#define BEEP_API
#endif

typedef enum beep_status {
	BEEP_OK = 0,
	BEEP_BAD_INPUT = 1,      /* inconsistent sizes, indices out of range, NULL where required */
	BEEP_NAN_RATE = 2,       /* a transition mean was NaN (reference: emsgEC("State",4)) */
	BEEP_OOM = 3,            /* device or host allocation failed */
	BEEP_TIMEOUT = 4,        /* a bounded device wait gave up */
	BEEP_DEVICE_ERROR = 5,   /* CUDA runtime error */
	BEEP_NO_DEVICE = 6,      /* no CUDA device, or the kernels were not built for it */
	BEEP_COUNT_OVERFLOW = 7  /* a draw or a population left the int32 range */
} beep_status;

/* Observation model of one observation (src/consts.hh:42, ObsModelFunc). */
enum beep_obs_model {
	BEEP_OBS_NORMAL = 0,
	BEEP_OBS_NORMAL_PERCENT = 1,
	BEEP_OBS_POISSON = 2,
	BEEP_OBS_NEGBIN = 3
};

/* Kind of observed value (src/consts.hh:160-161: THRESH, UNKNOWN sentinels). */
enum beep_obs_value_kind {
	BEEP_OBSVAL_VALUE = 0,
	BEEP_OBSVAL_UNKNOWN = 1,
	BEEP_OBSVAL_THRESH = 2
};

/* Encoding of an observation's contributing cells (the reference's
 * obs_trans / obs_pop index, src/obsmodel.cc:174-217):
 *   cell >= 0 : transition cell, cell = (c*ntrans + tr)*ndemocatpos + dp
 *   cell <  0 : population cell, -1-cell = (c*ncomp + co)*ndemocatpos + dp
 * The cells of one observation are listed in the order the reference visits
 * them (c, then transitions before populations, then tr or co, then dp). */
#define BEEP_POP_CELL(c, co, dp, ncomp, ndp) (-1 - (((c) * (ncomp) + (co)) * (ndp) + (dp)))

/* Parameter-independent model: what State::simulate and ObservationModel read
 * from Details, Data and Model.  Host pointers; copied at beep_model_create. */
typedef struct beep_model_desc {
	int32_t narea, nage, ndemocatpos, nstrain, ncomp, ntrans;
	int32_t ndivision;          /* steps, Details::ndivision */
	int32_t period;             /* Details::period (areafactor rows) */
	int32_t division_per_time;  /* Details::division_per_time */
	double dt;                  /* double(period)/ndivision (src/state.cc:384) */
	double popsize;             /* Data::popsize */

	const int32_t *trans_from;      /* [ntrans] */
	const int32_t *trans_to;        /* [ntrans] */
	int32_t infection_trans;        /* Model::infection_trans */
	const int32_t *democatpos_age;  /* [ndemocatpos/nstrain] Data::democatpos[dp][0] */

	/* geographic mixing Data::genQ.M (src/struct.hh:232-237) and genQ.factor */
	const double *M_diag;       /* [narea] */
	const int32_t *M_rowptr;    /* [narea+1] row c lists genQ.M.to[c] / val[c] */
	const int32_t *M_to;        /* [nnz] */
	const double *M_val;        /* [nnz] */
	const double *M_factor;     /* [narea] */

	const double *pop_init;     /* [narea][ncomp][ndemocatpos] Area::pop_init, integer-valued */

	/* observations Data::obs (src/struct.hh:340-354) */
	int32_t nobs;
	const int32_t *obs_sett_i;      /* [nobs] */
	const int32_t *obs_sett_f;      /* [nobs] */
	const int32_t *obs_value_kind;  /* [nobs] beep_obs_value_kind */
	const double *obs_value;        /* [nobs] */
	const int32_t *obs_model;       /* [nobs] beep_obs_model */
	const double *obs_sd;           /* [nobs] (normal models) */
	const double *obs_shape;        /* [nobs] (negative binomial) */
	const double *obs_threshold;    /* [nobs] datatable threshold (THRESH values) */
	const double *obs_factor;       /* [nobs] */
	const int32_t *obs_factor_spline; /* [nobs] row of beep_param_tables.obs_spline, or -1 */
	const int32_t *obs_cell_ptr;    /* [nobs+1] */
	const int32_t *obs_cells;       /* [obs_cell_ptr[nobs]] encoded cells */

	/* Demographic changes Data::democat_change (src/data.cc:958-1040), applied to
	 * pop[sett] at the start of every step by State::democat_change_pop_adjust
	 * (src/state.cc:339-376): change k moves population between the nval[k]
	 * values of one demographic classification so that, summed over its areas,
	 * groups and compartments, the values' shares follow frac[k][sett][.].
	 * Populations then stop being integers: a model with changes runs the
	 * plain FP64 form only, and its batches pass populations through the
	 * *_f64 fields of beep_sim_batch (since ABI 4).  0 / NULL: none. */
	int32_t ndemocat_change;
	const int32_t *dcc_nval;        /* [n] values of the changed classification (<= 32) */
	const int32_t *dcc_area_ptr;    /* [n+1] areas of change k: dcc_area[dcc_area_ptr[k] .. dcc_area_ptr[k+1]) */
	const int32_t *dcc_area;        /* DemocatChange::area */
	const int32_t *dcc_dp_ptr;      /* [n+1] groups of change k, nval[k] dp each: dcc_dp[dcc_dp_ptr[k] + g*nval[k] + f] */
	const int32_t *dcc_dp;          /* DemocatChange::dp_group[g][f] (dp < ndemocatpos/nstrain) */
	const double *dcc_frac;         /* per change k in turn: [ndivision][nval[k]] DemocatChange::frac */
} beep_model_desc;

/* Tables that State::set_param derives from one parameter set θ
 * (src/state.cc:66-91; src/model.cc:1010-1362).  Host pointers. */
typedef struct beep_param_tables {
	const double *transrate;      /* [ntrans][ndemocatpos] */
	const double *susceptibility; /* [ndemocatpos] */
	const double *infectivity;    /* [ncomp] paramval[comp[co].infectivity_param] */
	int32_t nbeta_row;
	const double *beta_rows;      /* [nbeta_row][ndivision] beta[st][c][.] rows */
	const int32_t *beta_row_of;   /* [nstrain][narea] row of beta_rows */
	const double *areafactor;     /* [period][narea] */
	const double *Ntime;          /* [ndivision][nage][nage] */
	const double *geo_spline;     /* [ndivision] disc_spline[geo_spline_ref] */
	int32_t nefoi;
	const double *efoi_spline;    /* [nefoi][ndivision] disc_spline of each efoi spline */
	const double *efoi_agedist;   /* [nefoi][nage] */
	const int32_t *efoi_ref;      /* [nstrain][narea] Model::efoi_spl_ref */
	int32_t nobs_spline;
	const double *obs_spline;     /* [nobs_spline][ndivision] factor splines of observations */
	/* PREDICTION-mode model modifications (ModelMod, src/model.cc:1446-1585), NULL when
	 * absent: the external force of infection of area c, strain st at step s is
	 * multiplied by efoi_mult[s][c][st] and every transition mean by
	 * transmean_mult[s][c][tr][dp] (State::set_transmean, src/state.cc:415,446-453) */
	const double *efoi_mult;      /* [ndivision][narea][nstrain] or NULL */
	const double *transmean_mult; /* [ndivision][narea][ntrans][ndemocatpos] or NULL */
} beep_param_tables;

/* Arithmetic form of the kernels. */
enum beep_form {
	BEEP_FORM_PLAIN_FP64 = 0, /* FP64 in the reference's summation order: bit-exact transnum/pop */
	BEEP_FORM_FAST = 1        /* particle-resident, FP32 rates and draws on the same keyed streams,
	                             exact integer observation sums, compensated FP32 log-densities
	                             reduced in FP64; models of up to 16 transitions and 20 age
	                             groups (beyond 8 transitions or 16 ages: one 640-thread CTA
	                             per SM with the FOI on FP32 SIMT; MBP chains up to 8 and 16) */
};

/* One batch of particles advanced over steps [ti, tf): State::simulate(ti,tf)
 * (src/state.cc:596-638) followed by the observation log-likelihood over the
 * observations whose window lies inside [ti, tf) -- all observations for
 * (0, ndivision) as in ObservationModel::calculate (src/obsmodel.cc:22-35),
 * a filter section's observations as in calculate_section (:39-58).
 * Host pointers unless the entry point says otherwise. */
typedef struct beep_sim_batch {
	int32_t nparticle;
	int32_t ngroup;                      /* parameter sets */
	const beep_param_tables *groups;     /* [ngroup] */
	const int32_t *group_of;             /* [nparticle] or NULL (all particles use group 0) */
	uint64_t seed;                       /* Philox key */
	const uint32_t *stream_of;           /* [nparticle] or NULL (stream = particle index) */
	int32_t ti, tf;                      /* 0 <= ti < tf <= ndivision */
	const int32_t *pop_in;               /* [nparticle][narea][ncomp][ndemocatpos] pop[ti]; NULL when ti == 0 (Area::pop_init) */
	double *L_out;                       /* [nparticle] log-likelihood, or NULL */
	int32_t *pop_out;                    /* [nparticle][narea][ncomp][ndemocatpos] pop[tf] (pop[tf-1] updated by step tf-1), or NULL */
	int32_t *transnum_out;               /* [nparticle][tf-ti][narea][ntrans][ndemocatpos], or NULL */
	int32_t *pop_traj_out;               /* [nparticle][tf-ti][narea][ncomp][ndemocatpos] pop[ti..tf-1], or NULL */
	int32_t form;                        /* beep_form */
	/* Models with demographic changes (fractional populations; since ABI 4): the
	 * same three populations in FP64, used instead of pop_in, pop_out and
	 * pop_traj_out (which must then be NULL). */
	const double *pop_in_f64;
	double *pop_out_f64;
	double *pop_traj_out_f64;
} beep_sim_batch;

typedef struct beep_model beep_model;    /* device-resident model + work buffers */

/* Library and device. */
BEEP_API int32_t beep_abi_version(void);
BEEP_API const char *beep_last_error(void);
BEEP_API beep_status beep_device_init(int32_t device);

/* Model lifetime (replaces constructing Data/Model/ObservationModel for the
 * hot path: src/main.cc:148-160). */
BEEP_API beep_status beep_model_create(const beep_model_desc *desc, beep_model **out);
BEEP_API beep_status beep_model_destroy(beep_model *model);

/* State::simulate for a batch (src/state.cc:582-638 + src/obsmodel.cc:22-58).
 * Host buffers; host<->device copies happen inside the call.  Equivalent to
 * beep_batch_create + upload + launch + download + destroy. */
BEEP_API beep_status beep_simulate(beep_model *model, const beep_sim_batch *batch);

/* The same call in stages, for callers that keep a batch resident and repeat
 * it (PMCMC proposals, ABC-SMC generations, serving).  The batch keeps the
 * caller's beep_sim_batch host pointers: beep_batch_stage re-reads them into
 * pinned staging memory, beep_batch_upload copies the staging to the device,
 * beep_batch_launch enqueues the kernels on the model's stream (inputs and
 * outputs stay on the device), beep_batch_download copies the outputs into
 * the caller's host arrays and waits.  beep_batch_time runs `iters` launches
 * between two CUDA events on the model's stream and reports the mean device
 * time per launch.  Same reference functions as beep_simulate. */
typedef struct beep_batch beep_batch;
BEEP_API beep_status beep_batch_create(beep_model *model, const beep_sim_batch *batch, beep_batch **out);
BEEP_API beep_status beep_batch_stage(beep_batch *batch);
BEEP_API beep_status beep_batch_upload(beep_batch *batch);
BEEP_API beep_status beep_batch_launch(beep_batch *batch);
BEEP_API beep_status beep_batch_download(beep_batch *batch);
BEEP_API beep_status beep_batch_time(beep_batch *batch, int32_t iters, double *ms_per_launch);
BEEP_API int32_t beep_batch_launches(const beep_batch *batch);   /* kernels per launch */
/* beep_batch_time with the step-synchronous fast form's time split: the mean
 * device time per launch and, of it, the time of the per-step tensor-core
 * products of the force of infection (CUDA events around each product kernel;
 * 0 for the other layouts).  A measurement aid with no counterpart in the
 * reference. */
/* The same split over the three kernels of each step: ms_kernels[0] the products,
 * [1] the step kernels (means, draws, populations), [2] the observation kernels;
 * all 0 for the other layouts. */
BEEP_API beep_status beep_batch_time_kernels(beep_batch *batch, int32_t iters, double *ms_per_launch,
                                             double *ms_kernels);
BEEP_API beep_status beep_batch_time_split(beep_batch *batch, int32_t iters, double *ms_per_launch,
                                           double *ms_product);
/* bytes moved host->device by beep_batch_upload and device->host by beep_batch_download */
BEEP_API beep_status beep_batch_bytes(const beep_batch *batch, int64_t *h2d, int64_t *d2h);
BEEP_API beep_status beep_batch_destroy(beep_batch *batch);
/* stage + upload + launch + download, with the device work (input copy,
 * status reset, kernel, output copy) captured once as a CUDA graph and
 * replayed by later calls (captured again if the staged inputs change size). */
BEEP_API beep_status beep_batch_run_graph(beep_batch *batch);
/* Autotuner of the fast form for a model: times every kernel layout the
 * model supports -- force of infection on FP32 SIMT (one or several particles
 * per SM), on the tensor cores one particle per CTA, or on the tensor cores
 * batched over the particles (step-synchronous layout) -- on a sample of the
 * given batch (up to 64 particles per SM over a window of up to 90 steps in
 * the middle of its range, started from the populations its first steps
 * leave there) and records the
 * fastest on the model; later batches of the model use it while the options
 * fast_foi and fast_ctas_per_sm are automatic (when several particles per SM
 * won, each batch still takes one per SM if it is too small to fill the SMs
 * several deep).  *chosen (may be NULL) receives the force of infection path
 * (1 = FP32 SIMT, 2 = tensor cores per particle, 3 = tensor cores batched). */
BEEP_API beep_status beep_autotune(beep_model *model, const beep_sim_batch *batch, int32_t *chosen);
/* Force-of-infection path the fast form of this batch runs: 1 = FP32 SIMT,
 * 2 = tensor cores one particle per CTA, 3 = tensor cores batched over the
 * particles (every particle advances one step at a time; per step one product
 * [particles x strains x ages, areas] . [areas, areas] and one step kernel);
 * 0 for the plain form. */
BEEP_API int32_t beep_batch_foi_path(const beep_batch *batch);
/* Particles (CTAs) resident per SM that the fast form of this batch is laid
 * out for: 1..4; 0 for the plain form and the step-synchronous layout. */
BEEP_API int32_t beep_batch_ctas_per_sm(const beep_batch *batch);

/* Bootstrap particle filter of PMCMC (PMCMC::obs_prob + bootstrap,
 * src/pmcmc.cc:180-268; ancestor swap Mpi::end_sec_swap, src/mpi.cc:215-327)
 * for one parameter set, run entirely on the device.  Particle slot p draws its
 * transitions from stream p; the j-th resampling uniform of section s is word
 * 0 of Philox({j, s, resample_stream, 3<<24}).  Sections are contiguous and
 * cover [0, ndivision) (ObservationModel::split_observations,
 * src/obsmodel.cc:326-348).  Outputs: the log-likelihood estimate
 * sum_s (invT Lmax_s + log(sum_p w_p / N)), and optionally the per-section
 * terms, per-section L [nsection][nparticle] and ancestors
 * [nsection][nparticle] (backpart[s+1] of the reference).  Host buffers. */
typedef struct beep_pf_request {
	int32_t nparticle;
	const beep_param_tables *tables;
	uint64_t seed;
	uint32_t resample_stream;
	double invT;
	int32_t nsection;
	const int32_t *section_ti, *section_tf;   /* [nsection] */
	int32_t form;                             /* beep_form of the simulation */
	double *loglik_out;                       /* [1] */
	double *loglik_section_out;               /* [nsection] or NULL */
	double *L_out;                            /* [nsection][nparticle] or NULL */
	int32_t *ancestors_out;                   /* [nsection][nparticle] or NULL */
	/* the sampled lineage (Mpi::particle_sample, src/mpi.cc:331-389): the
	 * transition counts [ndivision][narea][ntrans][ndemocatpos] of the particle
	 * the last resampling put in slot 0, each section taken from the slot its
	 * ancestor occupied then; NULL to skip (it keeps every slot's counts on the
	 * device for the whole run) */
	int32_t *lineage_transnum_out;
} beep_pf_request;

/* The section batches and device buffers a call prepares stay with the model
 * and are reused by later calls with the same nparticle, sections, form and
 * lineage request (only the tables and keys are staged again); they are freed
 * by a call of another shape or by beep_model_destroy. */
BEEP_API beep_status beep_pf_loglik(beep_model *model, const beep_pf_request *request);

/* ABC-SMC importance weights of a generation (ABCSMC::calculate_particle_weight
 * + MVN::probability, src/abcsmc.cc:260-271, src/mvn.cc:185-196):
 *   w_i = exp(logprior_i) / sum_j w_last_j exp(-0.5 (d/size)^T inv_cov (d/size)),
 *   d = theta_new_i - theta_last_j over the nvar inferred parameters
 * ([nnew][nvar], [nlast][nvar] row-major, inv_cov [nvar][nvar], nvar <= 16);
 * with normalise != 0 the weights are divided by their mean
 * (normalise_particle_weights, src/abcsmc.cc:275-283).  The pairwise kernel
 * terms are computed in FP32 on the GPU and summed with compensation; the
 * per-particle sums, the prior factor and the normalisation are FP64.
 * The form is evaluated as |L^T d|^2 with L L^T = inv_cov / size^2 when
 * inv_cov is positive definite (as given otherwise); sums are kept as
 * log-sum-exp, so they never underflow, and new particles far from every
 * previous one are summed again in FP64.  Errors: BEEP_BAD_INPUT for
 * negative or NaN previous weights or all of them zero. */
BEEP_API beep_status beep_abcsmc_weights(int32_t nvar, int32_t nnew, const double *theta_new,
                                         const double *logprior_new, int32_t nlast, const double *theta_last,
                                         const double *w_last, const double *inv_cov, double size,
                                         int32_t normalise, double *w_out);

/* Log-prior and bounds of parameter sets: Model::prior with its spline
 * smoothing term (src/model.cc:1590-1706) and Model::inbounds
 * (src/model.cc:2625-2669), on the host.  The prior types are the
 * reference's PriorType in its order; a hyperparameter val1 / val2 equal to
 * 999999999 (the reference's UNSET) is taken from parameter val1_param /
 * val2_param, as Model::get_val1/get_val2 do.  The smoothing terms are the
 * pairs of consecutive spline points that Model::spline_prior visits (points
 * on different parameters and times, not both fixed), evaluated on the
 * Dirichlet-corrected values (Model::dirichlet_correct, src/model.cc:2685-2695);
 * none in simulation modes.  paramval is [nset][nparam]; inbounds_out[k] = 1
 * when set k is inside the bounds, and logprior_out[k] is its log-prior
 * (-inf outside the bounds or where a gamma density's argument is not
 * positive). */
typedef enum beep_prior_type {
	BEEP_PRIOR_FIXED = 0,
	BEEP_PRIOR_UNIFORM = 1,
	BEEP_PRIOR_EXP = 2,
	BEEP_PRIOR_NORMAL = 3,
	BEEP_PRIOR_DIRICHLET = 4,
	BEEP_PRIOR_DIRICHLET_ALPHA = 5,
	BEEP_PRIOR_DIRICHLET_FLAT = 6,
	BEEP_PRIOR_MDIRICHLET = 7
} beep_prior_type;

typedef struct beep_prior_spec {
	int32_t nparam;
	const int32_t *type;                      /* [nparam] beep_prior_type */
	const double *val1, *val2;                /* [nparam] */
	const int32_t *val1_param, *val2_param;   /* [nparam], -1 where unused */
	const int32_t *gt_ptr, *gt_param;         /* [nparam+1] CSR: parameters each must be >= (Param::greaterthan) */
	const int32_t *lt_ptr, *lt_param;         /* [nparam+1] CSR: parameters each must be <= (Param::lessthan) */
	int32_t ndirichlet;
	const int32_t *dir_ptr, *dir_param;       /* [ndirichlet+1] CSR: the members of each Dirichlet group */
	const double *dir_frac;                   /* and their fractions */
	int32_t nsmooth;
	const int32_t *smooth_kind;               /* [nsmooth] 1 log-normal (log_smooth), 2 normal (smooth) */
	const int32_t *smooth_par1, *smooth_par2; /* [nsmooth] the two points' parameters */
	const double *smooth_mult1, *smooth_mult2, *smooth_value;   /* [nsmooth] their factors, the smoothing sd */
	int32_t ml_mode;                          /* 1: the reference's maximum-likelihood mode (mode=map) */
} beep_prior_spec;
BEEP_API beep_status beep_log_prior(const beep_prior_spec *spec, int32_t nset, const double *paramval,
                                    double *logprior_out, int32_t *inbounds_out);

/* Library options (process-wide; no counterpart in the reference):
 *   "fast_foi"  force of infection of the fast form: 0 = automatic (tensor
 *               cores batched over the particles for models of 300 to 512
 *               areas with one or two strains, FP32 SIMT otherwise), 1 = FP32
 *               SIMT, 2 = tensor cores one particle per CTA wherever supported
 *               (64 to 512 areas, one or two strains, more than 256 area x
 *               group columns), 3 = tensor cores batched over the particles
 *               (step-synchronous layout; 64 to 512 areas, one or two strains,
 *               at most 8 compartments and 8 transitions, 16 ages).
 *   "sampler_iteration_limit"  rejection iterations of the PTRS / BTRS
 *               samplers before a draw gives up with BEEP_TIMEOUT: 0 = the
 *               default 65536, or 1..65536 (lowered only to test that status).
 *   "fast_ctas_per_sm"  particles resident per SM in the fast form, for models
 *               of more than 256 area x group columns: 0 = automatic (several
 *               when at least three particles' state fits the SM's shared
 *               memory and the batch is large enough for several per SM to
 *               finish sooner than one, else one), 1 = one (640-thread CTAs),
 *               2..4 = at most that many (320-thread CTAs; at most 3 above 8
 *               ages; the particles' state may then move to global memory).
 *   "fast_parallel_draws"  the fast form's draws of a step one per (transition,
 *               column) thread instead of a column's transitions one after
 *               another on one thread: 0 = automatic (models whose draws fit
 *               two passes of the CTA, in batches of at most four particles
 *               per SM, where a step's latency sets the time), 1 = never,
 *               2 = wherever the draws fit.  The draws are the same.
 * Unknown names or values give BEEP_BAD_INPUT. */
BEEP_API beep_status beep_set_option(const char *name, int64_t value);

/* ---- MBP chains: model-based proposals (Mbp, src/mbp.cc) -----------------
 * A chain set keeps, for each chain, two full trajectory states on the
 * device -- the reference's Mbp::initial and Mbp::propose (transnum,
 * transmean, Imap, Idiag over all ndivision steps, src/state.hh:21-28) -- and
 * which of the two is the chain's current state.  BEEP_FORM_PLAIN_FP64 chains
 * reproduce the reference's counts bit for bit; BEEP_FORM_FAST chains draw
 * from the same keyed streams with FP32 means (counts and means are kept as
 * int32 and FP32; Imap is formed from the counts each step, so inf_update has
 * no effect on them). */
typedef struct beep_mbp_chains beep_mbp_chains;

typedef enum beep_inf_update {
	BEEP_INF_UPDATE = 0,       /* Imap recomputed from the new state's counts (State::set_Imap_sett) */
	BEEP_INF_DIF_UPDATE = 1    /* Imap' = Imap + dImap from the count differences (set_Imap_using_dI) */
} beep_inf_update;

typedef struct beep_mbp_request {
	const beep_param_tables *groups;   /* parameter sets (State::set_param tables) */
	int32_t ngroup;
	const int32_t *group_of;           /* [nchain] parameter set of each chain, or NULL (all set 0) */
	uint64_t seed;
	const uint32_t *stream_of;         /* [nchain] variate stream of each chain's draws, or NULL (chain index) */
	int32_t inf_update;                /* beep_inf_update (beep_mbp_propose) */
	const uint8_t *simu;               /* [nchain][ndivision][narea] 1 = simulate the cell afresh (SIMU,
	                                      Mbp::mbp_slicetime / mbp_fixedtree), or NULL: all coupled */
	double *L_out;                     /* [nchain] log-likelihood of the new state (EF = -2 L), or NULL */
} beep_mbp_request;

BEEP_API beep_status beep_mbp_create(beep_model *model, int32_t nchain, int32_t form, beep_mbp_chains **out);
BEEP_API beep_status beep_mbp_destroy(beep_mbp_chains *chains);
/* State::simulate(theta) (src/state.cc:582-592) of every chain over
 * [0, ndivision); the result becomes the chain's current state. */
BEEP_API beep_status beep_mbp_initialise(beep_mbp_chains *chains, const beep_mbp_request *request);
/* State::initialise_from_particle (src/state.cc:294-322) for every chain: the
 * given transition counts [nchain][ndivision][narea][ntrans][ndemocatpos]
 * become the chain's current state, with Imap, Idiag and the transition means
 * recomputed under the request's tables and L_out (if set) from the
 * observations.  (With several strains the reference applies update_pop
 * before the strain shift of set_transmean here; this call follows
 * State::simulate's order, which is the same for one strain.) */
BEEP_API beep_status beep_mbp_set_state(beep_mbp_chains *chains, const beep_mbp_request *request,
                                        const int32_t *transnum);
/* Mbp::mbp (src/mbp.cc:252-330): every chain's proposed state from its
 * current state, under the request's tables: a coupled cell draws
 * n' = n + Poisson(m'-m) (m' > m), n (m' = m) or Binomial(n, m'/m) (m' < m)
 * from the keyed stream of the chain; a SIMU cell draws Poisson(m'). */
BEEP_API beep_status beep_mbp_propose(beep_mbp_chains *chains, const beep_mbp_request *request);
/* Mbp::mbp (src/mbp.cc:252-330) for the chains of up to 8 chain sets of
 * different models (uneven areas, ages and horizons) at once, in ONE
 * persistent kernel launch: requests[k] is set k's proposal request, as for
 * beep_mbp_propose.  One 640-thread CTA per SM takes chains from a work
 * counter, the sets whose chains cost most first.  Each chain's counts are
 * those beep_mbp_propose gives for its set (the same keyed streams and
 * arithmetic); a set whose own launch runs fewer threads per chain can differ
 * in the last FP32 bits of L (its observation terms are summed over another
 * split of threads).  The sets must be fast-form, initialised, distinct and
 * on one device, with models of at most 8 transitions and 16 age groups.
 * The reference updates its chains one after another (Mbp::mcmc_updates, src/mbp.cc:34-98). */
BEEP_API beep_status beep_mbp_propose_fused(int32_t nset, beep_mbp_chains *const *sets,
                                            const beep_mbp_request *requests);
/* Mbp::swap_initial_propose_state (src/mbp.cc:241-246) for every chain with
 * accept[k] != 0: its last proposal becomes its current state. */
BEEP_API beep_status beep_mbp_accept(beep_mbp_chains *chains, const uint8_t *accept);
/* State::likelihood (src/state.cc:812-826) of every chain's current state,
 * with the transition means recomputed under the request's tables on the
 * fixed state (Mbp::parameter_proposal, src/mbp.cc:460-478); with the chain's
 * own tables this is the likelihood of its stored means.  Li_out [nchain]. */
BEEP_API beep_status beep_mbp_state_likelihood(beep_mbp_chains *chains, const beep_mbp_request *request,
                                               double *Li_out);
/* Mbp::get_al (src/mbp.cc:334-361): with cutoff_mode != 0 (CUTOFF)
 * al = EF_prop < EFcut ? exp(Pr_prop - Pr_init) : 0, else (INVT)
 * al = exp(-invT/2 (EF_prop - EF_init) + Pr_prop - Pr_init); capped at 1. */
BEEP_API double beep_mbp_acceptance(int32_t cutoff_mode, double invT, double EFcut, double EF_prop,
                                    double EF_init, double Pr_prop, double Pr_init);
/* The current state of one chain: transnum [ndivision][narea][ntrans][ndemocatpos]
 * and/or transmean of the same shape (either may be NULL). */
BEEP_API beep_status beep_mbp_read_state(beep_mbp_chains *chains, int32_t chain, int32_t *transnum_out,
                                         double *transmean_out);
/* Chains resident per SM in the fast form's last prepared batch (1..4; 0 for
 * the plain form or before the first call). */
BEEP_API int32_t beep_mbp_ctas_per_sm(const beep_mbp_chains *chains);

/* ---- Serving: continuous batching of requests on one GPU -----------------
 * A server runs simulation and likelihood requests of any model size
 * concurrently.  A request is queued at submit; a worker thread admits
 * queued requests in arrival order as running ones complete and free device
 * memory -- first fit, holding back the room the oldest waiting request needs
 * so that it is never overtaken forever -- up to max_inflight at once.  An
 * admitted request gets its own device model and batch on its own stream, so
 * its kernels overlap with the other running requests' on the device.  The
 * results are those beep_simulate gives for the same model and batch.  The
 * reference runs the same three kinds of work one after another in a
 * single process (src/pmcmc.cc:180-207, src/simulate.cc:42-165). */
typedef enum beep_request_kind {
	BEEP_REQ_LIKELIHOOD = 0,   /* per-particle log-likelihood over [ti, tf) (PMCMC / ABC-SMC evaluations) */
	BEEP_REQ_SCENARIO = 1,     /* trajectories from the initial state (mode=sim, src/simulate.cc:42-65) */
	BEEP_REQ_PREDICTION = 2,   /* continuation of given populations from ti (mode=prediction, src/simulate.cc:77-165) */
	BEEP_REQ_PF_LIKELIHOOD = 3 /* particle-filter likelihood estimate (PMCMC::obs_prob): the particles'
	                              states stay on the device from section to section */
} beep_request_kind;

typedef struct beep_request {
	int32_t kind;                    /* beep_request_kind */
	const beep_model_desc *model;    /* copied at submit; its arrays must stay valid until the request is done */
	const beep_sim_batch *batch;     /* copied at submit (NULL for BEEP_REQ_PF_LIKELIHOOD); arrays as above */
	const beep_pf_request *pf;       /* copied at submit (BEEP_REQ_PF_LIKELIHOOD only); arrays as above */
} beep_request;

typedef struct beep_request_stats {
	double submit_s, admit_s, done_s;   /* host clock, seconds since the server started */
	double gpu_start_s, gpu_end_s;      /* device clock: first copy in, last copy out */
	int64_t device_bytes;               /* device memory the request held */
	int32_t state;                      /* 0 queued, 1 running, 2 done */
	int32_t status;                     /* beep_status once done */
} beep_request_stats;

typedef struct beep_server beep_server;
/* hbm_budget_bytes: device memory the server's requests may hold at once
 * (a request larger than the budget runs alone). */
BEEP_API beep_status beep_server_create(int32_t device, int64_t hbm_budget_bytes, int32_t max_inflight,
                                        beep_server **out);
/* Finishes every submitted request, then releases the server. */
BEEP_API beep_status beep_server_destroy(beep_server *server);
BEEP_API beep_status beep_serve_submit(beep_server *server, const beep_request *request, uint64_t *ticket);
/* *done = 1 once the request finished; the return value is then its status. */
BEEP_API beep_status beep_serve_poll(beep_server *server, uint64_t ticket, int32_t *done);
/* Waits up to timeout_s (< 0: without limit); BEEP_TIMEOUT if still running. */
BEEP_API beep_status beep_serve_wait(beep_server *server, uint64_t ticket, double timeout_s);
BEEP_API beep_status beep_serve_stats(beep_server *server, uint64_t ticket, beep_request_stats *out);
/* Forgets a finished request. */
BEEP_API beep_status beep_serve_release(beep_server *server, uint64_t ticket);

/* Plain FP64 simulation that allocates no memory on the GPU.  No counterpart
 * in the reference: it serves callers that cannot call cudaMalloc -- an
 * application whose allocator or fixed memory budget owns all device memory,
 * where an allocation by a library fails or takes memory the pool counts on.  The
 * caller allocates and passes device pointers: the tables of one parameter
 * set (every pointer in `tables` is a device pointer; the struct itself is in
 * host memory), pop_in (when ti > 0), L_out [nparticle] and pop_out
 * [nparticle][narea][ncomp][ndemocatpos] (either may be NULL).  Particle p
 * uses variate stream p.  Working memory comes from one 64 MiB file-scope
 * device array held by every GPU that loads the library; batches that need
 * more are rejected with BEEP_BAD_INPUT (use fewer particles per call).  The
 * first call on a device looks up the array's device address (make that call
 * before any stream capture).  Calls share the array: the call clears what
 * must start at zero, and calls that overlap on the GPU race.  The call
 * is synchronous: it enqueues on `stream` (a cudaStream_t, NULL = legacy
 * default stream), first reading the index tables back to the host in stream
 * order to check their ranges, and returns after the kernel finished, with
 * its status (also when it fails part-way).  Same results as
 * beep_simulate with BEEP_FORM_PLAIN_FP64 on the same inputs. */
BEEP_API beep_status beep_simulate_plain_noalloc(beep_model *model, const beep_param_tables *tables,
                                                 int32_t nparticle, uint64_t seed, int32_t ti, int32_t tf,
                                                 const int32_t *pop_in, double *L_out, int32_t *pop_out,
                                                 void *stream);

#ifdef __cplusplus
}
#endif

#endif
