// Plain FP64 form of the tau-leap + observation log-likelihood.
//
// One CTA advances one particle over steps [ti, tf).  Every FP64 value the
// reference computes is computed with the same operations in the same order
// (this file is compiled with --fmad=false), so transition counts and
// populations are bit-identical to the reference driven by the same keyed
// variates.  Per step the CTA runs five phases separated by barriers:
//   A  dinf[st][c][a]     set_I_from_pop / update_I_from_transnum   src/state.cc:178-290
//   B  Imap, Idiag         the same functions' scatter, as a gather  src/state.cc:209-216
//   C  NMI[st][c][a]       get_NMI (+ strain shift of S)             src/state.cc:392-401,547-578
//   D  transition counts   set_transmean + poisson draws             src/state.cc:380-456,608-631
//   E  observation sums    get_obs_value_section                    src/obsmodel.cc:74-109
//      and pop[sett+1]     update_pop                               src/state.cc:460-485
// Models with demographic changes first apply State::democat_change_pop_adjust
// (src/state.cc:339-376) to pop[sett] at the start of each step; their
// populations are FP64 (the kernel's PopT = double instantiation), as in the
// reference, whose populations are doubles throughout.
// The log-likelihood of the scored observations is reduced at the end with
// compensated (Neumaier) sums; the reference sums naively in index order
// (src/obsmodel.cc:28), so the two agree to rounding (1e-12 relative).
//
// The same kernel advances MBP chains (src/mbp.cc:252-330), whose two states
// per chain (Mbp::initial, Mbp::propose) are full trajectories in HBM:
//   mode 1  a new state in the slot that is not current: every cell coupled
//           to the current state (n' = n + Poisson(m'-m), n, or
//           Binomial(n, m'/m)) unless it is a SIMU cell; Imap' either
//           recomputed (INF_UPDATE) or Imap + dImap with dImap built from
//           the count differences (INF_DIF_UPDATE, src/state.cc:109-123).
//           Initialisation (State::simulate) is this mode with every cell SIMU.
//   mode 3  State::initialise_from_particle (src/state.cc:294-322): the counts
//           already in the slot that is not current are kept; Imap
//           (set_Imap), the means (set_transmean) and L are recomputed.
//   mode 2  State::likelihood (src/state.cc:812-826) of the current state
//           with the means recomputed under this batch's tables on the fixed
//           state (Mbp::parameter_proposal, src/mbp.cc:460-478).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "beep_internal.h"
#include "rng_fp64.cuh"

namespace beep {
namespace {

constexpr int kThreads = 256;

__device__ double normal_lp(double x, double mean, double var)
{
	return -0.5 * log(2 * 3.14159265358979323846 * var) - (x - mean) * (x - mean) / (2 * var);
}

__device__ double poisson_lp(int i, double lam)
{
	if (lam == 0) return i == 0 ? 0 : -1000000000.0;
	if (i < 0) return -1000000000.0;
	return i * log(lam) - lam - lgamma((double)(i + 1));
}

__device__ double negbin_lp(unsigned int val, double m, double shape)
{
	return lgamma(shape + val) - lgamma((double)val + 1) - lgamma(shape) + shape * log(shape / (shape + m)) +
	       val * log(m / (shape + m));
}

// ObservationModel::obs_prob, src/obsmodel.cc:245-305
__device__ double obs_prob(double value, int kind, double val, int model, double sd, double shape, double thresh)
{
	if (value < 0) value = 0;
	if (kind == BEEP_OBSVAL_UNKNOWN) return 0;
	if (kind == BEEP_OBSVAL_THRESH) {
		if (model == BEEP_OBS_NORMAL || model == BEEP_OBS_NORMAL_PERCENT) {
			if (value < thresh) return normal_lp(thresh, thresh, sd * sd);
			return normal_lp(thresh, value, sd * sd);
		}
		double lam = value < 1 ? 1 : value;
		double sum = 0.0;
		for (double v = 0; v <= thresh; v++)
			sum += exp(model == BEEP_OBS_POISSON ? poisson_lp((int)v, lam) : negbin_lp((unsigned)v, lam, shape));
		return log(sum);
	}
	if (model == BEEP_OBS_NORMAL || model == BEEP_OBS_NORMAL_PERCENT) return normal_lp(val, value, sd * sd);
	double lam = value < 1 ? 1 : value;
	if (model == BEEP_OBS_POISSON) return poisson_lp((int)(val + 0.5), lam);
	return negbin_lp((unsigned)(int)(val + 0.5), lam, shape);
}

__device__ __forceinline__ void set_status(int32_t *st, int v)
{
	atomicCAS(st, 0, v);
}

// State::democat_change_pop_adjust (src/state.cc:339-376) of one particle's
// pop[sett]: per change, each value's population summed over the change's
// areas, groups and compartments (in that order, one thread per value), the
// shares' gap to the step's fractions, and every (area, group, compartment)
// row shifted by gap x the row's total.  The rows are disjoint (areas and dp
// are unique within a change), so they are updated in parallel.
__device__ void democat_adjust(const ModelDev &m, double *pop, int sett, int tid, int nth)
{
	__shared__ double s_cat[kMaxDccValues], s_gap[kMaxDccValues];
	const int C = m.C, DP = m.DP;
	for (int k = 0; k < m.ndcc; k++) {
		const int nv = m.dcc_nval[k], a0 = m.dcc_area_ptr[k], a1 = m.dcc_area_ptr[k + 1];
		const int *dpg = m.dcc_dp + m.dcc_dp_ptr[k];
		const int ng = (m.dcc_dp_ptr[k + 1] - m.dcc_dp_ptr[k]) / nv;
		if (tid < nv) {
			double s = 0.0;
			for (int j = a0; j < a1; j++) {
				const double *pc = pop + (size_t)m.dcc_area[j] * C * DP;
				for (int g = 0; g < ng; g++) {
					const int dp = dpg[g * nv + tid];
					for (int co = 0; co < C; co++) s += pc[(size_t)co * DP + dp];
				}
			}
			s_cat[tid] = s;
		}
		__syncthreads();
		if (tid == 0) {
			const double *fr = m.dcc_frac + m.dcc_frac_ptr[k] + (size_t)sett * nv;
			double tot = 0.0;
			for (int f = 0; f < nv; f++) tot += s_cat[f];
			for (int f = 0; f < nv; f++) s_gap[f] = fr[f] - s_cat[f] / tot;
		}
		__syncthreads();
		const int nrow = (a1 - a0) * ng * C;
		for (int idx = tid; idx < nrow; idx += nth) {
			const int co = idx % C, g = (idx / C) % ng, c = m.dcc_area[a0 + idx / (C * ng)];
			double *pc = pop + ((size_t)c * C + co) * DP;
			const int *dps = dpg + g * nv;
			double sum = 0.0;
			for (int f = 0; f < nv; f++) sum += pc[dps[f]];
			for (int f = 0; f < nv; f++) pc[dps[f]] += s_gap[f] * sum;
		}
		__syncthreads();
	}
}

// PopT: int32_t, or double for models with demographic changes
template <typename PopT>
__global__ void __launch_bounds__(kThreads) sim_plain_kernel(const ModelDev m, const BatchDev b)
{
	constexpr bool kPop64 = sizeof(PopT) == 8;
	const uint32_t lim = b.sampler_limit ? b.sampler_limit : 65536u;   // sampler rejection iterations
	const int p = blockIdx.x;
	if (p >= b.P) return;
	const int tid = threadIdx.x, nth = blockDim.x;
	const int A = m.A, G = m.G, DP = m.DP, NS = m.NS, DPS = m.DPS, C = m.C, T = m.T;
	const size_t popsz = (size_t)A * C * DP, tnsz = (size_t)A * T * DP, agsz = (size_t)NS * A * G;
	const int nsteps = b.tf - b.ti;
	const GroupDir dir = b.dirs[b.group_of ? b.group_of[p] : 0];
	const uint32_t stream = b.stream_of ? b.stream_of[p] : (uint32_t)p;
	const uint32_t k0 = b.key_of ? b.key_of[p].x : b.k0, k1 = b.key_of ? b.key_of[p].y : b.k1;   // the particle's key
	const double *fp = b.fpool;
	const int32_t *ip = b.ipool;
	const double *transrate = fp + dir.transrate, *sus = fp + dir.susceptibility, *infectivity = fp + dir.infectivity;
	const double *infdif = fp + dir.infdif, *beta_rows = fp + dir.beta_rows, *areafactor = fp + dir.areafactor;
	const double *Ntime = fp + dir.Ntime, *geo = fp + dir.geo_spline, *efoi_spline = fp + dir.efoi_spline;
	const double *efoi_age = fp + dir.efoi_agedist, *obs_spline = fp + dir.obs_spline;
	const int32_t *beta_row_of = ip + dir.beta_row_of, *efoi_ref = ip + dir.efoi_ref;
	const double *efoi_mult = dir.efoi_mult >= 0 ? fp + dir.efoi_mult : nullptr;
	const double *tm_mult = dir.tm_mult >= 0 ? fp + dir.tm_mult : nullptr;

	// MBP chains: slot of the current state and of the state being written
	const int mode = b.mode;
	const int cs_i = mode ? b.cur[p] : 0, cs_p = 1 - cs_i;
	const bool dif = mode == 1 && b.inf_dif && !b.simu_all;
	const bool writes = mode == 1 || mode == 3;          // the non-current slot receives a state
	auto chs = [&](int slot, int s) { return ((size_t)slot * b.P + p) * m.S + s; };
	double Lsum = 0.0, Lcmp = 0.0;   // mode 2: compensated partial sum of this thread

	PopT *pop_cur = (PopT *)b.pop_a + (size_t)p * popsz;
	PopT *pop_nxt = (PopT *)b.pop_b + (size_t)p * popsz;
	double *Imap = b.Imap + (size_t)p * agsz, *Idiag = b.Idiag + (size_t)p * agsz;
	double *dinf = b.dinf + (size_t)p * agsz, *NMI = b.NMI + (size_t)p * agsz;
	double *acc = b.obs_acc + (size_t)p * b.nscored;
	int32_t *status = b.status + p;

	for (size_t k = tid; k < popsz; k += nth)
		pop_cur[k] = b.ti == 0 ? (PopT)m.pop_init[k] : ((const PopT *)b.pop_in)[(size_t)p * popsz + k];
	for (int k = tid; k < b.nscored; k += nth) acc[k] = 0.0;
	__syncthreads();

	const int itr = m.infection_trans;
	const int inf_from = m.trans_from[itr];
	for (int sett = b.ti; sett < b.tf; sett++) {
		int32_t *tn = mode ? b.ch_tn + chs(writes ? cs_p : cs_i, sett) * tnsz
		          : b.tn_traj ? b.tn_traj + ((size_t)p * nsteps + (sett - b.ti)) * tnsz : b.tn + (size_t)p * tnsz;
		const int32_t *tn_prev = b.tn_traj || mode ? tn - tnsz : tn;   // single buffer still holds the previous step
		const int32_t *tn_base = dif && sett > 0 ? b.ch_tn + chs(cs_i, sett - 1) * tnsz : nullptr;
		double *Im_s = mode ? b.ch_Imap + chs(writes ? cs_p : cs_i, sett) * agsz : Imap;
		double *Id_s = mode ? b.ch_Idiag + chs(writes ? cs_p : cs_i, sett) * agsz : Idiag;

		if constexpr (kPop64) {
			if (m.ndcc > 0) democat_adjust(m, pop_cur, sett, tid, nth);   // pop[sett] before its step
		}

		// ---- A: dinf per (strain, source area, age)
		for (int idx = tid; idx < (int)agsz && mode != 2 && !(dif && sett == 0); idx += nth) {
			const int a = idx % G, c = (idx / G) % A, st = idx / (G * A);
			double s = 0.0;
			if (sett == b.ti) {
				for (int co = 0; co < C; co++) {
					const double inf = infectivity[co];
					if (inf != 0) {
						for (int dp = 0; dp < DPS; dp++) {
							if (m.dp_age[dp] != a) continue;
							const double pv = (double)pop_cur[((size_t)c * C + co) * DP + st * DPS + dp];
							if (pv != 0) s += inf * pv;
						}
					}
				}
			} else {
				for (int tr = 0; tr < T; tr++) {
					const double di = infdif[tr];
					if (di != 0) {
						for (int dp = 0; dp < DPS; dp++) {
							if (m.dp_age[dp] != a) continue;
							const size_t cl = ((size_t)c * T + tr) * DP + st * DPS + dp;
							const double num = tn_base ? (double)(tn_prev[cl] - tn_base[cl]) : (double)tn_prev[cl];
							if (num != 0) s += di * num;
						}
					}
				}
			}
			dinf[idx] = s;
		}
		__syncthreads();

		// ---- B: Imap/Idiag per (strain, target area, age), sources in ascending order
		// (INF_DIF_UPDATE: the running sums are dImap/dIdiag and the state's maps
		// are the current state's plus them)
		for (int idx = tid; idx < (int)agsz && mode != 2; idx += nth) {
			const int a = idx % G, t = (idx / G) % A, st = idx / (G * A);
			const double *dst = dinf + (size_t)st * A * G;
			double im = sett == b.ti ? 0.0 : Imap[idx];
			double id = sett == b.ti ? 0.0 : Idiag[idx];
			if (!(dif && sett == 0)) {
				const double dself = dst[t * G + a];
				if (dself != 0) id += dself * m.M_diag[t];
				for (int j = m.csc_ptr[t]; j < m.csc_ptr[t + 1]; j++) {
					const double d = dst[m.csc_src[j] * G + a];
					if (d != 0) im += d * m.csc_val[j];
				}
			}
			Imap[idx] = im;
			Idiag[idx] = id;
			if (writes) {
				if (dif) {
					const size_t io = chs(cs_i, sett) * agsz + idx;
					Im_s[idx] = b.ch_Imap[io] + im;
					Id_s[idx] = b.ch_Idiag[io] + id;
				} else {
					Im_s[idx] = im;
					Id_s[idx] = id;
				}
			}
		}
		__syncthreads();

		// ---- C: NMI per (strain, area, age); strain shift of the susceptible population
		for (int idx = tid; idx < (int)agsz; idx += nth) {
			const int a = idx % G, c = (idx / G) % A, st = idx / (G * A);
			const double *Id = Id_s + (size_t)st * A * G, *Im = Im_s + (size_t)st * A * G;
			const double d = geo[sett];
			const double omd = 1 - d;
			const double fac = m.M_factor[c];
			double val;
			if (G == 1) {
				val = Id[c] * (d + fac * omd) + Im[c] * d;
				if (val < 0) val = 0;
			} else {
				const int v = c * G;
				const double *N = Ntime + ((size_t)sett * G + a) * G;
				double sum = 0.0;
				for (int aa = 0; aa < G; aa++) {
					const double I = (Id[v + aa] + Im[v + aa]) * d + fac * Id[v + aa] * omd;
					sum += N[aa] * I;
				}
				if (sum < 0) sum = 0;
				val = sum;
			}
			NMI[idx] = val;
		}
		if (NS > 1) {
			for (int idx = tid; idx < A * DPS; idx += nth) {
				const int dp = idx % DPS, c = idx / DPS;
				PopT *sp = pop_cur + ((size_t)c * C + inf_from) * DP;
				double sum = 0.0;
				for (int st = 1; st < NS; st++) {
					sum += (double)sp[DPS * st + dp];
					sp[DPS * st + dp] = 0;
				}
				if constexpr (kPop64) sp[dp] += sum;
				else sp[dp] = (int32_t)((double)sp[dp] + sum);
			}
		}
		__syncthreads();

		// ---- D: transition means and counts per (area, transition, dp)
		for (int cell = tid; cell < (int)tnsz; cell += nth) {
			const int dp = cell % DP, tr = (cell / DP) % T, c = cell / (DP * T);
			double mean;
			if (tr == itr) {
				const int st = dp / DPS, dpl = dp % DPS;
				const double popu = (double)pop_cur[((size_t)c * C + inf_from) * DP + dpl];
				if (popu <= 0) mean = 0;
				else {
					const int a = m.dp_age[dpl];
					double be = beta_rows[(size_t)beta_row_of[st * A + c] * m.S + sett];
					be *= areafactor[(size_t)(sett / m.div_per_time) * A + c];
					const int ei = efoi_ref[st * A + c];
					double et = efoi_spline[(size_t)ei * m.S + sett] / m.popsize;
					if (efoi_mult) et *= efoi_mult[((size_t)sett * A + c) * NS + st];
					const double eta = et * efoi_age[(size_t)ei * G + a];
					mean = m.dt * popu * sus[dp] * (be * NMI[((size_t)st * A + c) * G + a] + eta);
				}
			} else {
				const double popu = (double)pop_cur[((size_t)c * C + m.trans_from[tr]) * DP + dp];
				mean = popu <= 0 ? 0 : m.dt * popu * transrate[(size_t)tr * DP + dp];
			}
			if (tm_mult) mean *= tm_mult[(size_t)sett * tnsz + cell];   // prediction modifications
			if (mode == 2) {                    // State::likelihood term of the fixed count
				if (mean != mean) set_status(status, BEEP_NAN_RATE);
				const double lp = poisson_lp(tn[cell], mean);
				const double t = Lsum + lp;
				Lcmp += fabs(Lsum) >= fabs(lp) ? (Lsum - t) + lp : (lp - t) + Lsum;
				Lsum = t;
				continue;
			}
			if (mode == 3) {                    // the given counts stay
				if (mean != mean) set_status(status, BEEP_NAN_RATE);
				b.ch_mean[chs(cs_p, sett) * tnsz + cell] = mean;
				continue;
			}
			int32_t n = 0;
			if (mean != mean) set_status(status, BEEP_NAN_RATE);
			else if (mean != 0) {
				if (mean > 1000000000.0) set_status(status, BEEP_COUNT_OVERFLOW);
				else {
					const uint32_t col = (uint32_t)(c * DP + dp);
					if (mode == 0 || b.simu_all || (b.simu && b.simu[((size_t)p * m.S + sett) * A + c])) {
						n = poisson_fp64(mean, k0, k1, col, (uint32_t)tr, (uint32_t)sett, stream, lim);
					} else {                        // coupled to the current state (src/mbp.cc:293-305)
						const size_t ci = chs(cs_i, sett) * tnsz + cell;
						const int32_t ni = b.ch_tn[ci];
						const double ri = b.ch_mean[ci];
						if (mean > ri) {
							n = poisson_fp64(mean - ri, k0, k1, col, (uint32_t)tr, (uint32_t)sett, stream, lim);
							if (n >= 0) n += ni;
						} else if (mean == ri) n = ni;
						else n = binomial_fp64(mean / ri, ni, k0, k1, col, (uint32_t)tr, (uint32_t)sett, stream, lim);
					}
					if (n < 0) { set_status(status, BEEP_TIMEOUT); n = 0; }
				}
			}
			if (mode == 1) b.ch_mean[chs(cs_p, sett) * tnsz + cell] = mean;
			tn[cell] = n;
		}
		__syncthreads();

		// ---- E: observation sums (one thread per active observation, cells in reference order)
		const int s0 = b.step_ptr[sett - b.ti], s1 = mode == 2 ? s0 : b.step_ptr[sett - b.ti + 1];
		for (int k = s0 + tid; k < s1; k += nth) {
			const int pos = b.step_obs[k];
			const int o = b.scored[pos];
			const double fac = m.obs_factor[o];
			const int spl = m.obs_spline[o];
			double v = acc[pos];
			for (int q = m.obs_cell_ptr[o]; q < m.obs_cell_ptr[o + 1]; q++) {
				const int cell = m.obs_cells[q];
				if (cell >= 0) {
					const double num = (double)tn[cell];
					if (num != 0) {
						if (spl < 0) v += fac * num;
						else v += fac * num * obs_spline[(size_t)spl * m.S + sett];
					}
				} else {
					v += fac * (double)pop_cur[-1 - cell];
				}
			}
			acc[pos] = v;
		}
		// update_pop into the other buffer
		for (size_t k = tid; k < popsz; k += nth) {
			const int dp = (int)(k % DP), co = (int)((k / DP) % C), c = (int)(k / ((size_t)DP * C));
			if constexpr (kPop64) {
				// FP64 populations: the flows in transition order, as update_pop applies them
				double v = pop_cur[k];
				for (int tr = 0; tr < T; tr++) {
					const int32_t n = tn[((size_t)c * T + tr) * DP + dp];
					if (n != 0) {
						if (m.trans_from[tr] == co) v -= (double)n;
						if (m.trans_to[tr] == co) v += (double)n;
					}
				}
				pop_nxt[k] = v;
			} else {
				long long v = pop_cur[k];
				for (int tr = 0; tr < T; tr++) {
					const long long n = tn[((size_t)c * T + tr) * DP + dp];
					if (m.trans_from[tr] == co) v -= n;
					if (m.trans_to[tr] == co) v += n;
				}
				if (v > 2147483647ll || v < -2147483648ll) { set_status(status, BEEP_COUNT_OVERFLOW); v = 0; }
				pop_nxt[k] = (int32_t)v;
			}
			if (b.pop_traj) ((PopT *)b.pop_traj)[((size_t)p * nsteps + (sett - b.ti)) * popsz + k] = pop_cur[k];
		}
		__syncthreads();
		PopT *sw = pop_cur; pop_cur = pop_nxt; pop_nxt = sw;
	}

	if (b.pop_out)
		for (size_t k = tid; k < popsz; k += nth) ((PopT *)b.pop_out)[(size_t)p * popsz + k] = pop_cur[k];

	__shared__ double part_s[kThreads], part_c[kThreads];
	if (mode == 2) {
		// the threads' compensated partial sums, combined in thread order
		part_s[tid] = Lsum;
		part_c[tid] = Lcmp;
		__syncthreads();
		if (tid == 0) {
			double S = 0.0, Cc = 0.0;
			for (int k = 0; k < nth; k++) {
				const double x = part_s[k];
				const double t = S + x;
				Cc += fabs(S) >= fabs(x) ? (S - t) + x : (x - t) + S;
				S = t;
				Cc += part_c[k];
			}
			b.Li[p] = S + Cc;
		}
	} else if (b.L) {
		// each thread sums a contiguous run of scored observations (Neumaier), then the
		// partials are combined in thread order by thread 0
		const int per = (b.nscored + nth - 1) / nth;
		const int k0 = tid * per, k1 = min(b.nscored, k0 + per);
		double s = 0.0, cmp = 0.0;
		for (int k = k0; k < k1; k++) {
			const int o = b.scored[k];
			const double lp = obs_prob(acc[k], m.obs_kind[o], m.obs_value[o], m.obs_model[o], m.obs_sd[o],
			                           m.obs_shape[o], m.obs_thresh[o]);
			const double t = s + lp;
			cmp += fabs(s) >= fabs(lp) ? (s - t) + lp : (lp - t) + s;
			s = t;
		}
		part_s[tid] = s;
		part_c[tid] = cmp;
		__syncthreads();
		if (tid == 0) {
			double S = 0.0, Cc = 0.0;
			for (int k = 0; k < nth; k++) {
				const double x = part_s[k];
				const double t = S + x;
				Cc += fabs(S) >= fabs(x) ? (S - t) + x : (x - t) + S;
				S = t;
				Cc += part_c[k];
			}
			const double L = S + Cc;
			if (L != L) set_status(status, BEEP_NAN_RATE);
			b.L[p] = L;
		}
	}
}

}  // namespace

int launch_sim_plain(const ModelDev &m, const BatchDev &b, void *stream)
{
	if (b.P == 0) return 0;
	if (m.ndcc > 0) sim_plain_kernel<double><<<b.P, kThreads, 0, (cudaStream_t)stream>>>(m, b);
	else sim_plain_kernel<int32_t><<<b.P, kThreads, 0, (cudaStream_t)stream>>>(m, b);
	return (int)cudaGetLastError();
}

}  // namespace beep
