// Internal device-side layout of the model, the parameter-set tables and a
// batch.  Shared by the host C++ (capi.cu) and the kernels.
#pragma once

#include <cstdint>

#include <vector_types.h>

#include "../../include/beep_gpu.h"

namespace beep {

// Parameter-independent model in HBM.  Area mixing is stored twice: by source
// (the reference's genQ.M rows) and transposed by target, each target's
// sources in ascending source order, so that a target's incremental sum can
// be formed by one thread in the reference's order (src/state.cc:209-216).
struct ModelDev {
	int32_t A, G, DP, NS, DPS, C, T, S, period, div_per_time, nobs;
	int32_t infection_trans;
	double dt, popsize;
	const int32_t *trans_from, *trans_to, *dp_age;
	const double *M_diag, *M_factor;
	const int32_t *csc_ptr, *csc_src;    // [A+1], [nnz]
	const double *csc_val;               // [nnz]
	const int32_t *pop_init;             // [A][C][DP]
	// observations
	const int32_t *obs_model, *obs_kind, *obs_spline, *obs_cell_ptr, *obs_cells, *obs_sett_i, *obs_sett_f;
	const double *obs_value, *obs_sd, *obs_shape, *obs_thresh, *obs_factor;
	// FP32 copies for the fast form
	const float *Mdense;                 // [A][A] source-major, diagonal zero
	const float *M_diag_f, *M_factor_f;  // [A]
	const float *csc_val_f;              // [nnz]
	const float2 *obs_np;                // [nobs] normal models: (-0.5 log(2 pi sd^2), 1/(2 sd^2))
	const float *obs_value_f;            // [nobs]
	const float *obs_factor_f, *obs_shape_f;  // [nobs]
	const int32_t *obs_cells_f;          // cells in the fast form's column-major shared layout:
	                                     // row*ncol + col (row = tn_row[tr]) or -1-(co*ncol + col) (population)
	const int32_t *obs_cells_full;       // the same with row = tr (all transition rows stored)
	int32_t tn_row[16];                  // row of each observed transition in the fast form's counts, or -1
	int32_t tn_rows;                     // number of observed transitions
	int32_t pop_obs;                     // some observation reads populations
	int32_t dp_age_unique;               // each age has exactly one dp per strain
	float inv_popsize_f;                 // 1 / Data::popsize
	const unsigned char *tc_image;       // area mixing as BF16 pieces for the tensor-core FOI (foi_tc.cuh), or null
	// demographic changes (State::democat_change_pop_adjust); with any, the plain form's
	// populations are FP64 (pop_a/pop_b/pop_in/pop_out/pop_traj hold doubles)
	int32_t ndcc;
	const int32_t *dcc_nval, *dcc_area_ptr, *dcc_area, *dcc_dp_ptr, *dcc_dp;
	const int32_t *dcc_frac_ptr;         // [ndcc] offset of change k's [S][nval] fractions
	const double *dcc_frac;
};
constexpr int kMaxDccValues = 32;        // values of a changed classification, at most

// One parameter set's tables: offsets into the batch's table pool (doubles /
// int32).  Tables shared between parameter sets share offsets.
struct GroupDir {
	int64_t transrate, susceptibility, infectivity, infdif, beta_rows, areafactor, Ntime, geo_spline,
	    efoi_spline, efoi_agedist, obs_spline;          // double pool offsets
	int64_t beta_row_of, efoi_ref;                      // int pool offsets
	int64_t efoi_mult, tm_mult;                         // prediction multipliers (double pool), -1 if absent
};

struct BatchDev {
	int32_t P, ti, tf, ngroup;
	uint32_t k0, k1;
	const GroupDir *dirs;               // [ngroup]
	const double *fpool;
	const float *fpool32;               // FP32 copy of fpool (fast form)
	const int32_t *ipool;
	const int32_t *group_of;            // [P] or null
	const uint32_t *stream_of;          // [P] or null
	const uint2 *key_of;                // [P] Philox key (seed words) of each particle, or null: (k0, k1) for all
	const int32_t *pop_in;              // [P][A][C][DP] or null (ti == 0)
	// scored observations and their per-step activity
	int32_t nscored;
	const int32_t *scored;              // [nscored] ascending obs index
	const int32_t *step_ptr;            // [tf-ti+1]
	const int32_t *step_obs;            // scored-position of obs active at each step
	// fast form: observation accumulator slots and completion lists
	int32_t nslots, m_in_smem, nefoi_stage;
	int32_t tn_full, pop_single;        // fast form: store every transition row / one population buffer
	void *gstate;                       // fast form, large models: per-particle state in global memory (or null)
	int32_t tn_smem;                    // with gstate: the transition counts stay in shared memory
	size_t gstate_stride;               // bytes per particle   // nefoi_stage: efoi age tables staged in shared memory (0 = read from L2)
	const int4 *tasks;                  // [2 * step_ptr[tf-ti]] per (step, active observation):
	                                    // {slot, obs, first cell, ncell | last<<31}, {factor bits, spline, cell offset, 0}
	// per-particle work (device)
	int32_t *pop_a, *pop_b;             // [P][A][C][DP] (doubles when the model has demographic changes,
	                                    // as are pop_in, pop_out and pop_traj)
	int32_t *tn;                        // [P][A][T][DP] current step's counts (when not writing a trajectory)
	double *Imap, *Idiag, *dinf, *NMI;  // [P][NS][A][G]
	double *obs_acc;                    // [P][nscored]
	// outputs (device)
	double *L;                          // [P] or null
	int32_t *pop_out;                   // [P][A][C][DP] or null
	int32_t *tn_traj;                   // [P][tf-ti][A][T][DP] or null
	int32_t *pop_traj;                  // [P][tf-ti][A][C][DP] or null
	int32_t *status;                    // [P] beep_status per particle
	// MBP chains (plain form; mode 0 = plain simulation of the fields above)
	int32_t mode;                       // 1: new chain state (Mbp::mbp; initialisation = every cell SIMU)
	                                    // 2: State::likelihood of the current state under this batch's tables
	                                    // 3: state rebuilt from the counts in the non-current slot
	                                    //    (State::initialise_from_particle)
	int32_t inf_dif;                    // mode 1: Imap' = Imap + dImap (INF_DIF_UPDATE)
	int32_t simu_all;                   // mode 1: every cell drawn afresh (State::simulate)
	const uint8_t *simu;                // [P][S][A] 1 = SIMU cell, or null
	const uint8_t *cur;                 // [P] slot (0/1) holding each chain's current state
	int32_t *ch_tn;                     // [2][P][S][A][T][DP]
	double *ch_mean;                    // [2][P][S][A][T][DP]
	double *ch_Imap, *ch_Idiag;         // [2][P][S][NS][A][G]
	double *Li;                         // [P] mode 2 output
	float *ch_mean_f;                   // fast form chains: means [2][P][S][T][A*DP] (counts in ch_tn, same layout)
	// fast form: force of infection on the tensor cores (foi_tc.cuh); its shared
	// memory starts at tc_smem_off bytes into the dynamic shared memory
	int32_t foi_tc;
	size_t tc_smem_off;
	int32_t nt;                         // fast form: threads per CTA (0: fast_pick_threads)
	uint32_t sampler_limit;             // rejection iterations before a draw reports BEEP_TIMEOUT (0: 65536)
	// fast form, step-synchronous layout (sim_batched.cu): every particle advances one step
	// at a time; the force of infection is one tensor-core product over the batch per step
	int32_t batched;
	int32_t *bx_pop;                    // [1 or 2][P][C][A*DP] populations (column-major per particle)
	float *bx_ic;                       // [2][P][NS][A][G] infectious counts of the step / the next step
	float *bx_y;                        // [P][NS][A][G] area-mixing contraction of the step's counts
	float *bx_slot;                     // [P][nslots] observation accumulators
	float2 *bx_kahan;                   // [P][observation threads] compensated log-likelihood partial sums
	int32_t *bx_tn;                     // [P][observed transitions][A*DP] counts of the step
	int32_t *bx_work;                   // [tf-ti] particle counters of the step kernels
	unsigned char *bx_a;                // the next product's A operand: per (128-row tile, 32-source chunk) the
	                                    // infectious counts as split BF16 (hi, lo) in K-major core matrices
	int32_t ctas;                       // fast form, nt == kDualThreads: CTAs resident per SM (2..4)
	int32_t pd;                         // fast form, small models and batches: the draws of a step one per
	                                    // (transition, column) thread (latency: the GPU is not full)
};

#if defined(__CUDACC__)
// Raises a kernel's dynamic shared-memory limit (a per-kernel attribute) to the most the
// device allows beside the kernel's static shared memory, and checks that `need` fits.
// Every host thread sets the same value, so that concurrent launches of one kernel with
// different sizes (requests served from several threads) do not undercut each other.
template <typename K>
inline cudaError_t allow_dynamic_smem(K kern, size_t need)
{
	cudaFuncAttributes fa;
	cudaError_t e = cudaFuncGetAttributes(&fa, (const void *)kern);
	if (e != cudaSuccess) return e;
	int dev = 0, optin = 0;
	e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
	if (e != cudaSuccess) return e;
	const long long lim = (long long)optin - (long long)fa.sharedSizeBytes;
	if ((long long)need > lim) return cudaErrorInvalidValue;
	return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim);
}
#endif

// launchers
int launch_sim_plain(const ModelDev &m, const BatchDev &b, void *stream);   // sim_plain.cu
int launch_sim_fast(const ModelDev &m, const BatchDev &b, void *stream);    // sim_fast.cu
size_t fast_smem_bytes(const ModelDev &m, int nslots, bool m_in_smem, int nefoi_stage, bool state_global, int tnrows,
                       bool pop_single, bool tn_smem = false, int nt = 0, int mg = 0,    // mg: age stride (0: G to 4s)
                       bool pd = false);                                                 // pd: draws per (transition, column)
bool fast_pd_fits(const ModelDev &m, int nt);    // the draws of a step fit two passes of nt threads
size_t fast_gstate_stride(const ModelDev &m);
size_t fast_tc_smem_bytes(const ModelDev &m);   // shared memory of the tensor-core FOI
int fast_pick_threads(const ModelDev &m);        // threads per CTA of the fast kernel for this model
// library options (beep_set_option)
int option_fast_foi();                           // 0 automatic, 1 FP32 SIMT, 2 tensor cores per particle,
                                                 // 3 tensor cores batched over the particles (step-synchronous)
int option_fast_ctas();                          // 0 automatic, 1, or 2..4: particles (CTAs) per SM, at most
int option_parallel_draws();                     // 0 automatic, 1 never, 2 where the draws fit
uint32_t option_sampler_limit();                 // 0 (65536) or the rejection-iteration limit of the samplers
constexpr int kDualThreads = 320;                // threads per CTA with several particles per SM
constexpr size_t kSmemPerSM = 228 * 1024;        // shared memory per SM (each resident CTA reserves 1 KB)
int fast_threads();
int fast_prepare();                              // one-time constant tables of the fast kernel
int fast_chain_prepare();                        // the same for the MBP-chain variants (mbp_fast.cu)
int launch_sim_fast_chain(const ModelDev &m, const BatchDev &b, void *stream);   // mbp_fast.cu
int fast_ctas_prepare();                         // constant tables of sim_fast_ctas.cu
int fast_ctas_max(int G);                        // most 320-thread CTAs per SM for G ages
int launch_sim_fast_ctas(const ModelDev &m, const BatchDev &b, size_t smem, void *stream);   // sim_fast_ctas.cu
int fast_chain_ctas_prepare();                   // constant tables of mbp_fast_ctas.cu
int launch_sim_fast_chain_ctas(const ModelDev &m, const BatchDev &b, size_t smem, void *stream);   // mbp_fast_ctas.cu
// MBP chains of several models in one persistent launch (mbp_fused.cu): n chain batches (mode 1),
// items in array order; counter: one device int32 the launch zeroes and counts on
constexpr int kMaxFusedSets = 8;
bool fused_supported(const ModelDev &m);
int fused_mg(const ModelDev *m, int n);          // age stride of a fused launch over these models
size_t fused_smem_bytes(const ModelDev &m, const BatchDev &b, int mg);
int launch_sim_fast_chain_fused(const ModelDev *m, const BatchDev *b, int n, int32_t *counter, int sms, void *stream);
// fast form for models with more than 8 transitions or 16 age groups (sim_fast_wide.cu)
bool fast_wide_needed(const ModelDev &m);
bool fast_wide_supported(const ModelDev &m);   // up to 16 transitions and 20 age groups
int fast_wide_prepare();
int launch_sim_fast_wide(const ModelDev &m, const BatchDev &b, size_t smem, void *stream);
// step-synchronous fast form (sim_batched.cu)
bool batched_supported(const ModelDev &m);
size_t batched_step_smem(const ModelDev &m, int tnrows);
int batched_obs_threads();
int batched_prepare();                           // constant tables of sim_batched.cu
int batched_launches(int nsteps);                // kernel launches of one batch run
size_t batched_a_bytes(const ModelDev &m, int P);  // bytes of BatchDev::bx_a
// events: null, or 4 * (tf - ti) cudaEvent_t: per step before the product kernel, between it and
// the step kernel, between that and the observation kernel, and after it
int launch_sim_batched(const ModelDev &m, const BatchDev &b, int sms, void *stream, void *events = nullptr);

}  // namespace beep
