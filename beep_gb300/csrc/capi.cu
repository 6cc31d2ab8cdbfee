// C ABI (include/beep_gpu.h): model creation, batch packing, launches.
//
// Host-side work per beep_simulate call:
//   1. validate the batch and pack every input into one pinned staging
//      buffer: the parameter-set tables (deduplicated by host pointer), the
//      per-particle group/stream indices and start populations, and the
//      per-step lists of active observations;
//   2. one host->device copy, the kernel, one device->host copy of the
//      outputs, all on the model's stream;
//   3. per-particle status words are reduced to the returned beep_status.
// Device memory is a per-model arena that only grows, so steady-state calls
// allocate nothing.
#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <unordered_map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "capi_internal.h"
#include "foi_tc.cuh"

using namespace beep;

namespace beep {

thread_local std::string g_err;
std::atomic<int> g_fast_foi{0};
std::atomic<int> g_fast_ctas{0};
std::atomic<uint32_t> g_sampler_limit{0};
std::atomic<int> g_parallel_draws{0};

beep_status fail(beep_status s, const std::string &msg)
{
	g_err = msg;
	return s;
}

void build_obs_lists(const int32_t *sett_i, const int32_t *sett_f, int nobs, int ti, int tf, ObsLists &out)
{
	const int nsteps = tf - ti;
	out.scored.clear();
	out.step_ptr.assign(nsteps + 1, 0);
	for (int o = 0; o < nobs; o++)
		if (sett_i[o] >= ti && sett_f[o] <= tf) out.scored.push_back(o);
	for (int o : out.scored)
		for (int s = sett_i[o]; s < sett_f[o]; s++) out.step_ptr[s - ti + 1]++;
	for (int s = 0; s < nsteps; s++) out.step_ptr[s + 1] += out.step_ptr[s];
	out.step_obs.resize(out.step_ptr[nsteps]);
	std::vector<int32_t> fill(out.step_ptr.begin(), out.step_ptr.end() - 1);
	for (size_t k = 0; k < out.scored.size(); k++) {
		const int o = out.scored[k];
		for (int s = sett_i[o]; s < sett_f[o]; s++) out.step_obs[fill[s - ti]++] = (int32_t)k;
	}
}

}  // namespace beep

extern "C" {

int32_t beep_abi_version(void) { return BEEP_GPU_ABI_VERSION; }

const char *beep_last_error(void) { return g_err.c_str(); }

beep_status beep_set_option(const char *name, int64_t value)
{
	if (!name) return fail(BEEP_BAD_INPUT, "null option name");
	if (std::string(name) == "fast_foi") {
		if (value < 0 || value > 3) return fail(BEEP_BAD_INPUT, "fast_foi must be 0, 1, 2 or 3");
		g_fast_foi.store((int)value);
		return BEEP_OK;
	}
	if (std::string(name) == "fast_ctas_per_sm") {
		if (value < 0 || value > 4) return fail(BEEP_BAD_INPUT, "fast_ctas_per_sm must be 0 (automatic) or 1..4");
		g_fast_ctas.store((int)value);
		return BEEP_OK;
	}
	if (std::string(name) == "fast_parallel_draws") {
		if (value < 0 || value > 2) return fail(BEEP_BAD_INPUT, "fast_parallel_draws must be 0 (automatic), 1 (never) or 2");
		g_parallel_draws.store((int)value);
		return BEEP_OK;
	}
	if (std::string(name) == "sampler_iteration_limit") {
		if (value < 0 || value > 65536) return fail(BEEP_BAD_INPUT, "sampler_iteration_limit must be 0 (default 65536) or 1..65536");
		g_sampler_limit.store((uint32_t)value);
		return BEEP_OK;
	}
	return fail(BEEP_BAD_INPUT, std::string("unknown option ") + name);
}

beep_status beep_device_init(int32_t device)
{
	int n = 0;
	cudaError_t e = cudaGetDeviceCount(&n);
	if (e != cudaSuccess || n == 0) return fail(BEEP_NO_DEVICE, "no CUDA device available");
	if (device < 0 || device >= n) return fail(BEEP_BAD_INPUT, "device index out of range");
	CUDA_TRY(cudaSetDevice(device));
	cudaDeviceProp prop;
	CUDA_TRY(cudaGetDeviceProperties(&prop, device));
	if (prop.major * 10 + prop.minor != 103)
		return fail(BEEP_NO_DEVICE, "the kernels are built for sm_103a; device is sm_" +
		                                std::to_string(prop.major) + std::to_string(prop.minor));
	return BEEP_OK;
}

beep_status beep_model_create(const beep_model_desc *d, beep_model **out)
{
	if (!d || !out) return fail(BEEP_BAD_INPUT, "null argument");
	*out = nullptr;
	const int32_t A = d->narea, G = d->nage, DP = d->ndemocatpos, NS = d->nstrain, C = d->ncomp, T = d->ntrans;
	const int32_t S = d->ndivision;
	if (A <= 0 || G <= 0 || DP <= 0 || NS <= 0 || C <= 0 || T <= 0 || S <= 0 || d->period <= 0 ||
	    d->division_per_time <= 0 || DP % NS != 0 || d->nobs < 0)
		return fail(BEEP_BAD_INPUT, "model sizes must be positive and ndemocatpos a multiple of nstrain");
	if ((S - 1) / d->division_per_time >= d->period) return fail(BEEP_BAD_INPUT, "ndivision exceeds period*division_per_time");
	if (!d->trans_from || !d->trans_to || !d->democatpos_age || !d->M_diag || !d->M_rowptr || !d->M_factor ||
	    !d->pop_init)
		return fail(BEEP_BAD_INPUT, "missing model array");
	if (d->infection_trans < 0 || d->infection_trans >= T) return fail(BEEP_BAD_INPUT, "infection_trans out of range");
	for (int tr = 0; tr < T; tr++)
		if (d->trans_from[tr] < 0 || d->trans_from[tr] >= C || d->trans_to[tr] < 0 || d->trans_to[tr] >= C)
			return fail(BEEP_BAD_INPUT, "transition compartment out of range");
	const int32_t DPS = DP / NS;
	for (int dp = 0; dp < DPS; dp++)
		if (d->democatpos_age[dp] < 0 || d->democatpos_age[dp] >= G) return fail(BEEP_BAD_INPUT, "democatpos_age out of range");
	if (d->M_rowptr[0] != 0) return fail(BEEP_BAD_INPUT, "M_rowptr[0] must be 0");
	for (int c = 0; c < A; c++)
		if (d->M_rowptr[c + 1] < d->M_rowptr[c]) return fail(BEEP_BAD_INPUT, "M_rowptr not monotone");
	const int32_t nnz = d->M_rowptr[A];
	for (int j = 0; j < nnz; j++)
		if (d->M_to[j] < 0 || d->M_to[j] >= A) return fail(BEEP_BAD_INPUT, "M_to out of range");
	const size_t popsz = (size_t)A * C * DP;
	std::vector<int32_t> pop_init(popsz);
	for (size_t k = 0; k < popsz; k++) {
		double v = d->pop_init[k];
		if (v != std::floor(v) || v < -2147483648.0 || v > 2147483647.0)
			return fail(BEEP_BAD_INPUT, "pop_init must be integer-valued within int32");
		pop_init[k] = (int32_t)v;
	}
	const int32_t nobs = d->nobs;
	int32_t ncells = 0;
	if (nobs > 0) {
		if (!d->obs_sett_i || !d->obs_sett_f || !d->obs_value_kind || !d->obs_value || !d->obs_model || !d->obs_sd ||
		    !d->obs_shape || !d->obs_threshold || !d->obs_factor || !d->obs_factor_spline || !d->obs_cell_ptr ||
		    !d->obs_cells)
			return fail(BEEP_BAD_INPUT, "missing observation array");
		if (d->obs_cell_ptr[0] != 0) return fail(BEEP_BAD_INPUT, "obs_cell_ptr[0] must be 0");
		ncells = d->obs_cell_ptr[nobs];
		for (int o = 0; o < nobs; o++) {
			if (d->obs_sett_i[o] < 0 || d->obs_sett_f[o] <= d->obs_sett_i[o] || d->obs_sett_f[o] > S)
				return fail(BEEP_BAD_INPUT, "observation time window out of range");
			if (d->obs_cell_ptr[o + 1] < d->obs_cell_ptr[o]) return fail(BEEP_BAD_INPUT, "obs_cell_ptr not monotone");
			if (d->obs_model[o] < 0 || d->obs_model[o] > 3 || d->obs_value_kind[o] < 0 || d->obs_value_kind[o] > 2)
				return fail(BEEP_BAD_INPUT, "bad observation model or value kind");
			bool has_pop = false;
			for (int q = d->obs_cell_ptr[o]; q < d->obs_cell_ptr[o + 1]; q++) {
				int32_t cell = d->obs_cells[q];
				if (cell >= 0 ? cell >= A * T * DP : (-1 - cell) >= (int64_t)popsz)
					return fail(BEEP_BAD_INPUT, "observation cell out of range");
				has_pop |= cell < 0;
			}
			if (has_pop && d->obs_factor_spline[o] >= 0)
				return fail(BEEP_BAD_INPUT, "population observations cannot carry a factor spline (src/obsmodel.cc:98)");
		}
	}
	// demographic changes: validated, and the offset of each change's fractions
	const int32_t ndcc = d->ndemocat_change;
	std::vector<int32_t> dcc_frac_ptr;
	int32_t dcc_na = 0, dcc_nd = 0, dcc_nf = 0;
	if (ndcc < 0) return fail(BEEP_BAD_INPUT, "ndemocat_change must be >= 0");
	if (ndcc > 0) {
		if (!d->dcc_nval || !d->dcc_area_ptr || !d->dcc_area || !d->dcc_dp_ptr || !d->dcc_dp || !d->dcc_frac)
			return fail(BEEP_BAD_INPUT, "missing demographic-change array");
		if (d->dcc_area_ptr[0] != 0 || d->dcc_dp_ptr[0] != 0)
			return fail(BEEP_BAD_INPUT, "dcc_area_ptr[0] and dcc_dp_ptr[0] must be 0");
		for (int k = 0; k < ndcc; k++) {
			const int32_t nv = d->dcc_nval[k];
			if (nv < 1 || nv > kMaxDccValues) return fail(BEEP_BAD_INPUT, "dcc_nval must lie in 1..32");
			if (d->dcc_area_ptr[k + 1] < d->dcc_area_ptr[k] || d->dcc_dp_ptr[k + 1] < d->dcc_dp_ptr[k] ||
			    (d->dcc_dp_ptr[k + 1] - d->dcc_dp_ptr[k]) % nv != 0)
				return fail(BEEP_BAD_INPUT, "dcc_area_ptr / dcc_dp_ptr not monotone, or a group without nval dp");
			dcc_frac_ptr.push_back(dcc_nf);
			dcc_nf += S * nv;
		}
		dcc_na = d->dcc_area_ptr[ndcc];
		dcc_nd = d->dcc_dp_ptr[ndcc];
		for (int j = 0; j < dcc_na; j++)
			if (d->dcc_area[j] < 0 || d->dcc_area[j] >= A) return fail(BEEP_BAD_INPUT, "dcc_area out of range");
		for (int j = 0; j < dcc_nd; j++)
			if (d->dcc_dp[j] < 0 || d->dcc_dp[j] >= DPS) return fail(BEEP_BAD_INPUT, "dcc_dp out of range");
		// within a change each area and each dp appears once (the rows it shifts are disjoint)
		for (int k = 0; k < ndcc; k++) {
			std::vector<char> seen_a(A, 0), seen_d(DPS, 0);
			for (int j = d->dcc_area_ptr[k]; j < d->dcc_area_ptr[k + 1]; j++) {
				if (seen_a[d->dcc_area[j]]) return fail(BEEP_BAD_INPUT, "an area repeats within a demographic change");
				seen_a[d->dcc_area[j]] = 1;
			}
			for (int j = d->dcc_dp_ptr[k]; j < d->dcc_dp_ptr[k + 1]; j++) {
				if (seen_d[d->dcc_dp[j]]) return fail(BEEP_BAD_INPUT, "a dp repeats within a demographic change");
				seen_d[d->dcc_dp[j]] = 1;
			}
		}
	}

	// transpose of the area mixing matrix, each target's sources ascending
	std::vector<int32_t> csc_ptr(A + 1, 0), csc_src(nnz);
	std::vector<double> csc_val(nnz);
	for (int j = 0; j < nnz; j++) csc_ptr[d->M_to[j] + 1]++;
	for (int t = 0; t < A; t++) csc_ptr[t + 1] += csc_ptr[t];
	{
		std::vector<int32_t> fill(csc_ptr.begin(), csc_ptr.end() - 1);
		for (int c = 0; c < A; c++)
			for (int j = d->M_rowptr[c]; j < d->M_rowptr[c + 1]; j++) {
				int t = d->M_to[j];
				csc_src[fill[t]] = c;
				csc_val[fill[t]] = d->M_val[j];
				fill[t]++;
			}
	}

	// FP32 copies for the fast form: dense source-major mixing matrix (diagonal
	// kept separately), the transpose's values, and per-observation constants
	// of the normal log-density
	std::vector<float> Mdense((size_t)A * A, 0.f), Mdiag_f(A), Mfac_f(A), csc_val_f(nnz);
	for (int c = 0; c < A; c++) {
		Mdiag_f[c] = (float)d->M_diag[c];
		Mfac_f[c] = (float)d->M_factor[c];
		for (int j = d->M_rowptr[c]; j < d->M_rowptr[c + 1]; j++) Mdense[(size_t)c * A + d->M_to[j]] += (float)d->M_val[j];
	}
	for (int j = 0; j < nnz; j++) csc_val_f[j] = (float)csc_val[j];
	// the tensor-core FOI's image of the off-diagonal matrix: per (target chunk,
	// source chunk) three BF16 pieces hi + mid + lo of M[c][t], K-major (foi_tc.cuh)
	std::vector<unsigned char> tc_img;
	if (A >= 64 && tc::supported(A, NS)) {
		const tc::Geom g = tc::geometry(A, NS);
		tc_img.assign(g.image_bytes(), 0);
		auto bf16 = [](float x) {   // round to nearest even; the inputs are finite
			uint32_t u;
			memcpy(&u, &x, 4);
			return (uint16_t)((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
		};
		auto f32 = [](uint16_t h) {
			uint32_t u = (uint32_t)h << 16;
			float x;
			memcpy(&x, &u, 4);
			return x;
		};
		for (int ct = 0; ct < g.nct; ct++)
			for (int kc = 0; kc < g.nkc; kc++) {
				unsigned char *ch = tc_img.data() + (size_t)(ct * g.nkc + kc) * g.chunk_bytes();
				for (int n = 0; n < g.tw; n++)
					for (int kl = 0; kl < tc::kChunkK; kl++) {
						const int t = ct * g.tw + n, c = kc * tc::kChunkK + kl;
						const float x = (t < A && c < A) ? Mdense[(size_t)c * A + t] : 0.f;
						const uint16_t h = bf16(x);
						const float r1 = x - f32(h);
						const uint16_t mid = bf16(r1);
						const uint16_t lo = bf16(r1 - f32(mid));
						const uint32_t o = tc::kmajor_offset(n, kl, g.tw);
						memcpy(ch + o, &h, 2);
						memcpy(ch + g.piece_bytes() + o, &mid, 2);
						memcpy(ch + 2 * g.piece_bytes() + o, &lo, 2);
					}
			}
	}
	std::vector<float2> obs_np(nobs > 0 ? nobs : 1);
	std::vector<float> obs_value_f(nobs > 0 ? nobs : 1), obs_factor_f(nobs > 0 ? nobs : 1), obs_shape_f(nobs > 0 ? nobs : 1);
	std::vector<int32_t> obs_cells_f(ncells > 0 ? ncells : 1), obs_cells_full(ncells > 0 ? ncells : 1);
	int32_t tn_row[16];
	int32_t tn_rows = 0, pop_obs = 0;
	{
		const int ncol = A * DP;
		std::vector<int> seen(T, 0);
		for (int q = 0; q < ncells; q++) {
			const int32_t cell = d->obs_cells[q];
			if (cell >= 0) seen[(cell / DP) % T] = 1;
			else pop_obs = 1;
		}
		for (int tr = 0; tr < 16; tr++) tn_row[tr] = -1;
		for (int tr = 0; tr < T && tr < 16; tr++)
			if (seen[tr]) tn_row[tr] = tn_rows++;
		for (int q = 0; q < ncells; q++) {
			const int32_t cell = d->obs_cells[q];
			if (cell >= 0) {
				const int c = cell / (T * DP), tr = (cell / DP) % T, dp = cell % DP;
				obs_cells_f[q] = (tr < 16 ? tn_row[tr] : 0) * ncol + c * DP + dp;
				obs_cells_full[q] = tr * ncol + c * DP + dp;
			} else {
				const int k = -1 - cell, c = k / (C * DP), co = (k / DP) % C, dp = k % DP;
				obs_cells_f[q] = obs_cells_full[q] = -1 - (co * ncol + c * DP + dp);
			}
		}
	}
	for (int o = 0; o < nobs; o++) {
		obs_value_f[o] = (float)d->obs_value[o];
		obs_factor_f[o] = (float)d->obs_factor[o];
		obs_shape_f[o] = (float)d->obs_shape[o];
		const double var = d->obs_sd[o] * d->obs_sd[o];
		obs_np[o] = make_float2((float)(-0.5 * std::log(2 * 3.14159265358979323846 * var)), (float)(1.0 / (2 * var)));
	}

	beep_model *m = new beep_model();
	m->A = A; m->G = G; m->DP = DP; m->NS = NS; m->C = C; m->T = T; m->S = S;
	m->period = d->period; m->dpt = d->division_per_time; m->nobs = nobs;
	m->obs_sett_i.assign(d->obs_sett_i, d->obs_sett_i + nobs);
	m->obs_sett_f.assign(d->obs_sett_f, d->obs_sett_f + nobs);
	m->obs_spline.assign(d->obs_factor_spline, d->obs_factor_spline + nobs);
	for (int o = 0; o < nobs; o++) m->max_obs_spline = std::max(m->max_obs_spline, d->obs_factor_spline[o]);
	m->obs_cell_ptr_h.assign(d->obs_cell_ptr, d->obs_cell_ptr + (nobs > 0 ? nobs + 1 : 0));
	m->obs_cells_f_h.assign(obs_cells_f.begin(), obs_cells_f.begin() + ncells);
	m->obs_cells_full_h.assign(obs_cells_full.begin(), obs_cells_full.begin() + ncells);
	m->obs_factor_f_h.assign(obs_factor_f.begin(), obs_factor_f.begin() + nobs);
	m->trans_from_h.assign(d->trans_from, d->trans_from + T);
	m->trans_to_h.assign(d->trans_to, d->trans_to + T);
	m->pop64 = ndcc > 0;
	cudaGetDevice(&m->device);
	cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, m->device);

	Layout L;
	size_t o_tf = L.add(4 * T), o_tt = L.add(4 * T), o_age = L.add(4 * DPS), o_diag = L.add(8 * A),
	       o_fac = L.add(8 * A), o_cp = L.add(4 * (A + 1)), o_cs = L.add(4 * (size_t)nnz), o_cv = L.add(8 * (size_t)nnz),
	       o_pi = L.add(4 * popsz), o_om = L.add(4 * (size_t)nobs), o_ok = L.add(4 * (size_t)nobs),
	       o_os = L.add(4 * (size_t)nobs), o_ocp = L.add(4 * (size_t)(nobs + 1)), o_oc = L.add(4 * (size_t)ncells),
	       o_osi = L.add(4 * (size_t)nobs), o_osf = L.add(4 * (size_t)nobs), o_ov = L.add(8 * (size_t)nobs),
	       o_osd = L.add(8 * (size_t)nobs), o_osh = L.add(8 * (size_t)nobs), o_oth = L.add(8 * (size_t)nobs),
	       o_ofa = L.add(8 * (size_t)nobs), o_md = L.add(4 * (size_t)A * A), o_mdg = L.add(4 * (size_t)A),
	       o_mfc = L.add(4 * (size_t)A), o_cvf = L.add(4 * (size_t)nnz), o_onp = L.add(8 * (size_t)nobs),
	       o_ovf = L.add(4 * (size_t)nobs), o_off = L.add(4 * (size_t)nobs), o_oshf = L.add(4 * (size_t)nobs),
	       o_ocf = L.add(4 * (size_t)ncells), o_ocfull = L.add(4 * (size_t)ncells), o_tc = L.add(tc_img.size()),
	       o_dnv = L.add(4 * (size_t)ndcc), o_dap = L.add(ndcc ? 4 * (size_t)(ndcc + 1) : 0),
	       o_da = L.add(4 * (size_t)dcc_na), o_ddp = L.add(ndcc ? 4 * (size_t)(ndcc + 1) : 0),
	       o_dd = L.add(4 * (size_t)dcc_nd), o_dfp = L.add(4 * (size_t)ndcc), o_df = L.add(8 * (size_t)dcc_nf);
	std::vector<char> host(L.size);
	auto put = [&](size_t off, const void *src, size_t n) { if (n) memcpy(host.data() + off, src, n); };
	put(o_tf, d->trans_from, 4 * T); put(o_tt, d->trans_to, 4 * T); put(o_age, d->democatpos_age, 4 * DPS);
	put(o_diag, d->M_diag, 8 * A); put(o_fac, d->M_factor, 8 * A); put(o_cp, csc_ptr.data(), 4 * (A + 1));
	put(o_cs, csc_src.data(), 4 * (size_t)nnz); put(o_cv, csc_val.data(), 8 * (size_t)nnz);
	put(o_pi, pop_init.data(), 4 * popsz);
	if (nobs > 0) {
		put(o_om, d->obs_model, 4 * (size_t)nobs); put(o_ok, d->obs_value_kind, 4 * (size_t)nobs);
		put(o_os, d->obs_factor_spline, 4 * (size_t)nobs); put(o_ocp, d->obs_cell_ptr, 4 * (size_t)(nobs + 1));
		put(o_oc, d->obs_cells, 4 * (size_t)ncells); put(o_osi, d->obs_sett_i, 4 * (size_t)nobs);
		put(o_osf, d->obs_sett_f, 4 * (size_t)nobs); put(o_ov, d->obs_value, 8 * (size_t)nobs);
		put(o_osd, d->obs_sd, 8 * (size_t)nobs); put(o_osh, d->obs_shape, 8 * (size_t)nobs);
		put(o_oth, d->obs_threshold, 8 * (size_t)nobs); put(o_ofa, d->obs_factor, 8 * (size_t)nobs);
	}
	put(o_md, Mdense.data(), 4 * (size_t)A * A); put(o_mdg, Mdiag_f.data(), 4 * (size_t)A);
	put(o_mfc, Mfac_f.data(), 4 * (size_t)A); put(o_cvf, csc_val_f.data(), 4 * (size_t)nnz);
	if (nobs > 0) put(o_onp, obs_np.data(), 8 * (size_t)nobs);
	if (nobs > 0) put(o_ovf, obs_value_f.data(), 4 * (size_t)nobs);
	if (nobs > 0) put(o_off, obs_factor_f.data(), 4 * (size_t)nobs);
	if (nobs > 0) put(o_oshf, obs_shape_f.data(), 4 * (size_t)nobs);
	if (ncells > 0) put(o_ocf, obs_cells_f.data(), 4 * (size_t)ncells);
	if (ncells > 0) put(o_ocfull, obs_cells_full.data(), 4 * (size_t)ncells);
	put(o_tc, tc_img.data(), tc_img.size());
	if (ndcc > 0) {
		put(o_dnv, d->dcc_nval, 4 * (size_t)ndcc); put(o_dap, d->dcc_area_ptr, 4 * (size_t)(ndcc + 1));
		put(o_da, d->dcc_area, 4 * (size_t)dcc_na); put(o_ddp, d->dcc_dp_ptr, 4 * (size_t)(ndcc + 1));
		put(o_dd, d->dcc_dp, 4 * (size_t)dcc_nd); put(o_dfp, dcc_frac_ptr.data(), 4 * (size_t)ndcc);
		put(o_df, d->dcc_frac, 8 * (size_t)dcc_nf);
	}
	cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = m->model_mem.reserve(L.size);
	// on the model's stream, waited for: a cudaMemcpy from pageable memory may return
	// before its last bytes land, and the model's (non-blocking) stream would not wait for
	// the legacy stream's copy
	if (e == cudaSuccess)
		e = cudaMemcpyAsync(m->model_mem.ptr, host.data(), L.size, cudaMemcpyHostToDevice, m->stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
	if (e != cudaSuccess) {
		beep_model_destroy(m);
		return fail(e == cudaErrorMemoryAllocation ? BEEP_OOM : BEEP_DEVICE_ERROR, std::string("model upload: ") + cudaGetErrorString(e));
	}
	char *base = (char *)m->model_mem.ptr;
	ModelDev &md = m->dev;
	md.A = A; md.G = G; md.DP = DP; md.NS = NS; md.DPS = DPS; md.C = C; md.T = T; md.S = S;
	md.period = d->period; md.div_per_time = d->division_per_time; md.nobs = nobs;
	md.infection_trans = d->infection_trans; md.dt = d->dt; md.popsize = d->popsize;
	md.trans_from = (const int32_t *)(base + o_tf); md.trans_to = (const int32_t *)(base + o_tt);
	md.dp_age = (const int32_t *)(base + o_age); md.M_diag = (const double *)(base + o_diag);
	md.M_factor = (const double *)(base + o_fac); md.csc_ptr = (const int32_t *)(base + o_cp);
	md.csc_src = (const int32_t *)(base + o_cs); md.csc_val = (const double *)(base + o_cv);
	md.pop_init = (const int32_t *)(base + o_pi);
	md.obs_model = (const int32_t *)(base + o_om); md.obs_kind = (const int32_t *)(base + o_ok);
	md.obs_spline = (const int32_t *)(base + o_os); md.obs_cell_ptr = (const int32_t *)(base + o_ocp);
	md.obs_cells = (const int32_t *)(base + o_oc); md.obs_sett_i = (const int32_t *)(base + o_osi);
	md.obs_sett_f = (const int32_t *)(base + o_osf); md.obs_value = (const double *)(base + o_ov);
	md.obs_sd = (const double *)(base + o_osd); md.obs_shape = (const double *)(base + o_osh);
	md.obs_thresh = (const double *)(base + o_oth); md.obs_factor = (const double *)(base + o_ofa);
	md.Mdense = (const float *)(base + o_md); md.M_diag_f = (const float *)(base + o_mdg);
	md.M_factor_f = (const float *)(base + o_mfc); md.csc_val_f = (const float *)(base + o_cvf);
	md.obs_np = (const float2 *)(base + o_onp);
	md.obs_value_f = (const float *)(base + o_ovf);
	md.inv_popsize_f = (float)(1.0 / d->popsize);
	md.obs_factor_f = (const float *)(base + o_off);
	md.obs_shape_f = (const float *)(base + o_oshf);
	md.obs_cells_f = (const int32_t *)(base + o_ocf);
	md.ndcc = ndcc;
	md.dcc_nval = (const int32_t *)(base + o_dnv); md.dcc_area_ptr = (const int32_t *)(base + o_dap);
	md.dcc_area = (const int32_t *)(base + o_da); md.dcc_dp_ptr = (const int32_t *)(base + o_ddp);
	md.dcc_dp = (const int32_t *)(base + o_dd); md.dcc_frac_ptr = (const int32_t *)(base + o_dfp);
	md.dcc_frac = (const double *)(base + o_df);
	md.obs_cells_full = (const int32_t *)(base + o_ocfull);
	md.tc_image = tc_img.empty() ? nullptr : (const unsigned char *)(base + o_tc);
	for (int tr = 0; tr < 16; tr++) md.tn_row[tr] = tn_row[tr];
	md.tn_rows = tn_rows;
	md.pop_obs = pop_obs;
	{
		std::vector<int> cnt(G, 0);
		for (int dp = 0; dp < DPS; dp++) cnt[d->democatpos_age[dp]]++;
		md.dp_age_unique = 1;
		for (int a = 0; a < G; a++) if (cnt[a] != 1) md.dp_age_unique = 0;
	}
	*out = m;
	return BEEP_OK;
}

beep_status beep_model_destroy(beep_model *m)
{
	if (!m) return BEEP_OK;
	if (m->stream) cudaStreamSynchronize(m->stream);
	for (beep_batch *q : m->pf.q) beep_batch_destroy(q);
	m->pf.q.clear();
	m->pf.work.release();
	m->model_mem.release();
	if (m->stream) cudaStreamDestroy(m->stream);
	delete m;
	return BEEP_OK;
}

}  // extern "C"

namespace {

// The parameter tables of a batch in one pool, each distinct array once (by
// address and length).  With copy, the pool is built in `f` (FP64, the plain
// form); without, only the offsets are laid out and `pieces` lists what goes
// where, for the caller to write straight into the staging buffer in FP32
// (the fast form, which reads no FP64 table).
struct TablePacker {
	bool copy = true;
	size_t fsize = 0;                     // pool length in values (a multiple of 4)
	std::vector<double> f;
	struct Piece {
		const double *src;
		size_t n;
		int64_t off;
	};
	std::vector<Piece> pieces;
	std::vector<int32_t> i;
	struct KeyHash {
		size_t operator()(const std::pair<const void *, size_t> &k) const
		{
			return std::hash<const void *>()(k.first) * 31u + std::hash<size_t>()(k.second);
		}
	};
	std::unordered_map<std::pair<const void *, size_t>, int64_t, KeyHash> seen;
	std::unordered_map<const int32_t *, std::pair<int32_t, int32_t>> ranges;
	int64_t reserve(size_t n)             // n values, filled by the caller
	{
		const int64_t off = (int64_t)fsize;
		fsize = align_up(fsize + n, 4);
		if (copy) f.resize(fsize, 0.0);
		return off;
	}
	int64_t addf(const double *p, size_t n)
	{
		auto key = std::make_pair((const void *)p, n);
		auto it = seen.find(key);
		if (it != seen.end()) return it->second;
		const int64_t off = (int64_t)fsize;
		if (copy) {
			f.insert(f.end(), p, p + n);
			f.resize(align_up(f.size(), 4), 0.0);
		} else {
			pieces.push_back(Piece{p, n, off});
		}
		fsize = align_up(fsize + n, 4);
		seen[key] = off;
		return off;
	}
	int64_t addi(const int32_t *p, size_t n)
	{
		auto key = std::make_pair((const void *)p, n + ((size_t)1 << 62));
		auto it = seen.find(key);
		if (it != seen.end()) return it->second;
		int64_t off = (int64_t)i.size();
		i.insert(i.end(), p, p + n);
		i.resize(align_up(i.size(), 8));
		seen[key] = off;
		return off;
	}
};

beep_status pack_tables(const beep_model *m, const beep_sim_batch *b, TablePacker &pk, std::vector<GroupDir> &dirs)
{
	const size_t A = m->A, G = m->G, DP = m->DP, NS = m->NS, C = m->C, T = m->T, S = m->S;
	dirs.resize(b->ngroup);
	for (int g = 0; g < b->ngroup; g++) {
		const beep_param_tables &t = b->groups[g];
		if (!t.transrate || !t.susceptibility || !t.infectivity || !t.beta_rows || !t.beta_row_of || !t.areafactor ||
		    !t.Ntime || !t.geo_spline || !t.efoi_spline || !t.efoi_agedist || !t.efoi_ref)
			return fail(BEEP_BAD_INPUT, "parameter set " + std::to_string(g) + ": missing table");
		if (t.nbeta_row <= 0 || t.nefoi <= 0 || t.nobs_spline < 0)
			return fail(BEEP_BAD_INPUT, "parameter set " + std::to_string(g) + ": bad table counts");
		// index tables shared between parameter sets are scanned once (range of values cached)
		auto range_of = [&](const int32_t *p) {
			auto it = pk.ranges.find(p);
			if (it != pk.ranges.end()) return it->second;
			std::pair<int32_t, int32_t> r{INT32_MAX, INT32_MIN};
			for (size_t k = 0; k < NS * A; k++) { r.first = std::min(r.first, p[k]); r.second = std::max(r.second, p[k]); }
			pk.ranges[p] = r;
			return r;
		};
		const auto rb = range_of(t.beta_row_of), re = range_of(t.efoi_ref);
		if (rb.first < 0 || rb.second >= t.nbeta_row) return fail(BEEP_BAD_INPUT, "beta_row_of out of range");
		if (re.first < 0 || re.second >= t.nefoi) return fail(BEEP_BAD_INPUT, "efoi_ref out of range");
		if (m->max_obs_spline >= t.nobs_spline) return fail(BEEP_BAD_INPUT, "obs_factor_spline beyond nobs_spline");
		GroupDir &dd = dirs[g];
		dd.transrate = pk.addf(t.transrate, T * DP);
		dd.susceptibility = pk.addf(t.susceptibility, DP);
		dd.infectivity = pk.addf(t.infectivity, C);
		dd.infdif = pk.reserve(T);           // filled when the pool is staged
		dd.beta_rows = pk.addf(t.beta_rows, (size_t)t.nbeta_row * S);
		dd.areafactor = pk.addf(t.areafactor, (size_t)m->period * A);
		dd.Ntime = pk.addf(t.Ntime, S * G * G);
		dd.geo_spline = pk.addf(t.geo_spline, S);
		dd.efoi_spline = pk.addf(t.efoi_spline, (size_t)t.nefoi * S);
		dd.efoi_agedist = pk.addf(t.efoi_agedist, (size_t)t.nefoi * G);
		dd.obs_spline = t.nobs_spline > 0 && t.obs_spline ? pk.addf(t.obs_spline, (size_t)t.nobs_spline * S) : 0;
		dd.beta_row_of = pk.addi(t.beta_row_of, NS * A);
		dd.efoi_ref = pk.addi(t.efoi_ref, NS * A);
		dd.efoi_mult = t.efoi_mult ? pk.addf(t.efoi_mult, S * A * NS) : -1;
		dd.tm_mult = t.transmean_mult ? pk.addf(t.transmean_mult, S * A * T * DP) : -1;
	}
	return BEEP_OK;
}

}  // namespace


namespace {

beep_status check_batch(const beep_model *m, const beep_sim_batch *b, bool device_io = false)
{
	const int P = b->nparticle;
	if (P <= 0 || b->ngroup <= 0 || !b->groups) return fail(BEEP_BAD_INPUT, "nparticle/ngroup/groups");
	if (b->ti < 0 || b->tf <= b->ti || b->tf > m->S) return fail(BEEP_BAD_INPUT, "step range must satisfy 0 <= ti < tf <= ndivision");
	if (b->form != BEEP_FORM_PLAIN_FP64 && b->form != BEEP_FORM_FAST) return fail(BEEP_BAD_INPUT, "unknown form");
	if (m->pop64) {
		if (b->form != BEEP_FORM_PLAIN_FP64)
			return fail(BEEP_BAD_INPUT, "a model with demographic changes (fractional populations) runs the plain FP64 form only");
		if (b->pop_in || b->pop_out || b->pop_traj_out)
			return fail(BEEP_BAD_INPUT, "a model with demographic changes takes populations through pop_in_f64, pop_out_f64 and pop_traj_out_f64");
		if (b->ti > 0 && !b->pop_in_f64 && !device_io) return fail(BEEP_BAD_INPUT, "pop_in_f64 is required when ti > 0");
	} else {
		if (b->pop_in_f64 || b->pop_out_f64 || b->pop_traj_out_f64)
			return fail(BEEP_BAD_INPUT, "FP64 populations are for models with demographic changes");
		if (b->ti > 0 && !b->pop_in && !device_io) return fail(BEEP_BAD_INPUT, "pop_in is required when ti > 0");
	}
	if (b->group_of)
		for (int p = 0; p < P; p++)
			if (b->group_of[p] < 0 || b->group_of[p] >= b->ngroup) return fail(BEEP_BAD_INPUT, "group_of out of range");
	return BEEP_OK;
}

// Packs the caller's current host arrays into the pinned staging buffer.
beep_status stage_inputs(beep_batch *q)
{
	beep_model *m = q->m;
	const beep_sim_batch *b = &q->b;
	const int P = b->nparticle;
	const size_t popsz = (size_t)m->A * m->C * m->DP, pe = m->pop64 ? 8 : 4;   // bytes per population
	const bool fast = b->form == BEEP_FORM_FAST;
	TablePacker pk;
	pk.copy = !fast;
	beep_status st = pack_tables(m, b, pk, q->dirs);
	if (st != BEEP_OK) return st;
	Layout in;
	size_t o_dirs = in.add(sizeof(GroupDir) * q->dirs.size()), o_f = in.add(fast ? 0 : 8 * pk.fsize),
	       o_f32 = in.add(fast ? 4 * pk.fsize : 0),
	       o_i = in.add(4 * pk.i.size()), o_go = in.add(b->group_of ? 4 * (size_t)P : 0),
	       o_so = in.add(b->stream_of ? 4 * (size_t)P : 0), o_pin = in.add(b->ti > 0 && !q->device_io ? pe * popsz * P : 0),
	       o_key = in.add(8 * q->keys.size()),
	       o_sc = in.add(4 * q->scored.size()), o_sp = in.add(4 * q->step_ptr.size()),
	       o_sobs = in.add(4 * q->step_obs.size()), o_tasks = in.add(4 * q->tasks.size());
	CUDA_TRY(q->in_host.reserve(in.size));
	CUDA_TRY(q->in_dev.reserve(in.size));
	q->in_size = in.size;
	char *h = (char *)q->in_host.ptr;
	memcpy(h + o_dirs, q->dirs.data(), sizeof(GroupDir) * q->dirs.size());
	if (!fast) memcpy(h + o_f, pk.f.data(), 8 * pk.fsize);
	if (!pk.i.empty()) memcpy(h + o_i, pk.i.data(), 4 * pk.i.size());
	if (b->group_of) memcpy(h + o_go, b->group_of, 4 * (size_t)P);
	if (b->stream_of) memcpy(h + o_so, b->stream_of, 4 * (size_t)P);
	if (!q->keys.empty()) memcpy(h + o_key, q->keys.data(), 8 * q->keys.size());
	if (b->ti > 0 && !q->device_io)
		memcpy(h + o_pin, m->pop64 ? (const void *)b->pop_in_f64 : (const void *)b->pop_in, pe * popsz * P);
	if (!q->scored.empty()) memcpy(h + o_sc, q->scored.data(), 4 * q->scored.size());
	memcpy(h + o_sp, q->step_ptr.data(), 4 * q->step_ptr.size());
	if (!q->step_obs.empty()) memcpy(h + o_sobs, q->step_obs.data(), 4 * q->step_obs.size());
	if (!q->tasks.empty()) memcpy(h + o_tasks, q->tasks.data(), 4 * q->tasks.size());
	// infectivity difference of each transition, Model::get_infectivity_dif (src/model.cc:820-823)
	if (!fast) {
		double *fpool = (double *)(h + o_f);
		for (int g = 0; g < b->ngroup; g++) {
			const double *inf = b->groups[g].infectivity;
			for (int tr = 0; tr < m->T; tr++)
				fpool[q->dirs[g].infdif + tr] = inf[m->trans_to_h[tr]] - inf[m->trans_from_h[tr]];
		}
	} else {
		// the fast form's FP32 pool, converted from the caller's arrays by up to 8 threads
		float *f32 = (float *)(h + o_f32);
		for (int g = 0; g < b->ngroup; g++) {
			const double *inf = b->groups[g].infectivity;
			for (int tr = 0; tr < m->T; tr++)
				f32[q->dirs[g].infdif + tr] = (float)(inf[m->trans_to_h[tr]] - inf[m->trans_from_h[tr]]);
		}
		auto convert = [&](size_t k0, size_t k1) {
			for (size_t k = k0; k < k1; k++) {
				const TablePacker::Piece &pc = pk.pieces[k];
				float *dst = f32 + pc.off;
				for (size_t j = 0; j < pc.n; j++) dst[j] = (float)pc.src[j];
			}
		};
		const size_t np = pk.pieces.size();
		const unsigned hw = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
		const unsigned nth = pk.fsize > ((size_t)1 << 20) && np >= 2 * hw ? hw : 1;
		if (nth == 1) {
			convert(0, np);
		} else {
			std::vector<std::thread> th;
			for (unsigned t = 0; t < nth; t++) th.emplace_back(convert, np * t / nth, np * (t + 1) / nth);
			for (auto &x : th) x.join();
		}
	}
	char *di = (char *)q->in_dev.ptr;
	BatchDev &bd = q->bd;
	bd.dirs = (const GroupDir *)(di + o_dirs);
	bd.fpool = fast ? nullptr : (const double *)(di + o_f);
	bd.ipool = (const int32_t *)(di + o_i);
	bd.group_of = b->group_of ? (const int32_t *)(di + o_go) : nullptr;
	bd.stream_of = b->stream_of ? (const uint32_t *)(di + o_so) : nullptr;
	bd.key_of = q->keys.empty() ? nullptr : (const uint2 *)(di + o_key);
	bd.pop_in = b->ti > 0 && !q->device_io ? (const int32_t *)(di + o_pin) : nullptr;
	bd.scored = (const int32_t *)(di + o_sc);
	bd.step_ptr = (const int32_t *)(di + o_sp);
	bd.step_obs = (const int32_t *)(di + o_sobs);
	bd.fpool32 = fast ? (const float *)(di + o_f32) : nullptr;
	bd.tasks = (const int4 *)(di + o_tasks);
	return BEEP_OK;
}

}  // namespace

extern "C" {

beep_status beep_batch_create(beep_model *m, const beep_sim_batch *b, beep_batch **out)
{
	if (!m || !b || !out) return fail(BEEP_BAD_INPUT, "null argument");
	*out = nullptr;
	return batch_create_internal(m, b, false, out);
}

}  // extern "C"

beep_status beep::batch_create_internal(beep_model *m, const beep_sim_batch *b, bool device_io, beep_batch **out,
                                        bool device_traj, bool allow_tc, bool allow_ctas, const std::vector<uint2> *keys)
{
	// a count trajectory is written: to the batch's output (transnum_out), or to a
	// device buffer the caller sets in bd.tn_traj before each launch (device_traj)
	const bool traj = b->transnum_out != nullptr || device_traj;
	if (!m || !b || !out) return fail(BEEP_BAD_INPUT, "null argument");
	*out = nullptr;
	beep_status st = check_batch(m, b, device_io);
	if (st != BEEP_OK) return st;
	CUDA_TRY(cudaSetDevice(m->device));
	if (keys && keys->size() != (size_t)b->nparticle) return fail(BEEP_BAD_INPUT, "one key per particle");
	beep_batch *q = new beep_batch();
	q->m = m;
	q->b = *b;
	q->device_io = device_io;
	if (keys) q->keys = *keys;
	const int P = b->nparticle;
	const size_t popsz = (size_t)m->A * m->C * m->DP, tnsz = (size_t)m->A * m->T * m->DP;
	const size_t agsz = (size_t)m->NS * m->A * m->G, pe = m->pop64 ? 8 : 4;   // bytes per population
	const bool want_po = b->pop_out || b->pop_out_f64, want_pt = b->pop_traj_out || b->pop_traj_out_f64;
	const int nsteps = b->tf - b->ti;
	// scored observations and the steps each is active in
	{
		ObsLists ol;
		build_obs_lists(m->obs_sett_i.data(), m->obs_sett_f.data(), m->nobs, b->ti, b->tf, ol);
		q->scored.swap(ol.scored);
		q->step_ptr.swap(ol.step_ptr);
		q->step_obs.swap(ol.step_obs);
	}
	const int nscored = (int)q->scored.size();
	if (b->form == BEEP_FORM_FAST) {
		// accumulator slots: observations whose windows do not overlap share a
		// slot (greedy interval colouring in window-start order)
		q->slot_of.assign(nscored, -1);
		std::vector<int32_t> order(nscored);
		for (int k = 0; k < nscored; k++) order[k] = k;
		std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
			return m->obs_sett_i[q->scored[x]] < m->obs_sett_i[q->scored[y]];
		});
		std::vector<std::pair<int32_t, int32_t>> busy;   // (sett_f, slot) min-heap
		std::vector<int32_t> freeslots;
		int32_t nslots = 0;
		auto cmp = [](const std::pair<int32_t, int32_t> &x, const std::pair<int32_t, int32_t> &y) { return x.first > y.first; };
		for (int k : order) {
			const int o = q->scored[k];
			while (!busy.empty() && busy.front().first <= m->obs_sett_i[o]) {
				freeslots.push_back(busy.front().second);
				std::pop_heap(busy.begin(), busy.end(), cmp);
				busy.pop_back();
			}
			int32_t sl;
			if (!freeslots.empty()) { sl = freeslots.back(); freeslots.pop_back(); }
			else sl = nslots++;
			q->slot_of[k] = sl;
			busy.push_back({m->obs_sett_f[o], sl});
			std::push_heap(busy.begin(), busy.end(), cmp);
		}
		q->bd.nslots = nslots;
		// one 32-byte task per (step, active observation), in step_obs order:
		// {slot, obs, first cell, ncell | last<<31}, {factor bits, spline, cell offset, run}
		// run: 1 when the cells are consecutive counts, 2 consecutive populations (the
		// kernels then read them without the cell list), 0 otherwise
		q->tasks.resize((size_t)8 * q->step_obs.size());
		for (int s2 = 0; s2 < nsteps; s2++)
			for (int k = q->step_ptr[s2]; k < q->step_ptr[s2 + 1]; k++) {
				const int pos = q->step_obs[k], o = q->scored[pos];
				const int c0 = m->obs_cell_ptr_h[o], nc = m->obs_cell_ptr_h[o + 1] - c0;
				const bool last = b->ti + s2 == m->obs_sett_f[o] - 1;
				int32_t *t = &q->tasks[(size_t)8 * k];
				float fac = m->obs_factor_f_h[o];
				int32_t fbits;
				memcpy(&fbits, &fac, 4);
				const std::vector<int32_t> &enc = traj ? m->obs_cells_full_h : m->obs_cells_f_h;
				t[0] = q->slot_of[pos]; t[1] = o; t[2] = nc > 0 ? enc[c0] : 0;
				t[3] = (int32_t)((uint32_t)nc | (last ? 0x80000000u : 0u));
				int32_t run = 0;
				if (nc > 1) {
					const int32_t e0 = enc[c0];
					bool up = e0 >= 0, down = e0 < 0;
					for (int i = 1; i < nc && (up || down); i++) {
						up = up && enc[c0 + i] == e0 + i;
						down = down && enc[c0 + i] == e0 - i;
					}
					run = up ? 1 : down ? 2 : 0;
				}
				t[4] = fbits; t[5] = m->obs_spline[o]; t[6] = c0; t[7] = run;
			}
		const size_t limit = 227 * 1024;
		int nefoi = 1 << 30;
		for (int g = 0; g < b->ngroup; g++) nefoi = std::min(nefoi, (int)b->groups[g].nefoi);
		if (b->ngroup > 1)
			for (int g = 1; g < b->ngroup; g++)
				if (b->groups[g].nefoi != b->groups[0].nefoi) nefoi = 0;
		q->bd.nefoi_stage = nefoi * m->G <= 1024 ? nefoi : 0;
		// counts of unobserved transitions are not stored unless a trajectory is requested; one
		// population buffer suffices when no observation reads populations and strains do not mix
		q->bd.tn_full = traj ? 1 : 0;
		q->bd.pop_single = (!m->dev.pop_obs && m->NS == 1 && !b->pop_traj_out) ? 1 : 0;
		const int tnrows = q->bd.tn_full ? m->T : m->dev.tn_rows;
		const bool ps = q->bd.pop_single != 0;
		// models with more than 8 transitions or 16 age groups: the wide instantiation,
		// one 640-thread CTA per SM with the FOI on FP32 SIMT (sim_fast_wide.cu)
		const bool wide = fast_wide_needed(m->dev);
		const int nt0 = wide ? 640 : 0;
		q->state_global = fast_smem_bytes(m->dev, nslots, false, q->bd.nefoi_stage, false, tnrows, ps, false, nt0) > limit;
		if (fast_smem_bytes(m->dev, nslots, false, q->bd.nefoi_stage, true, tnrows, ps, false, nt0) > limit ||
		    m->NS * m->A > 640 || m->G * m->G > 640 || (wide && !fast_wide_supported(m->dev))) {
			delete q;
			return fail(BEEP_BAD_INPUT, "model too large for the fast form (observation slots or tables exceed shared memory, or more than 16 transitions or 20 age groups)");
		}
		if (wide) q->bd.nt = 640;
		q->bd.m_in_smem = fast_smem_bytes(m->dev, nslots, true, q->bd.nefoi_stage, q->state_global, tnrows, ps, false, nt0) <= limit ? 1 : 0;
		// force of infection on the tensor cores, batched over the particles: every particle
		// advances one step at a time and the contraction is one product over the batch per
		// step (sim_batched.cu); the default for large models
		const int opt = option_fast_foi() != 0 ? option_fast_foi() : m->tuned_foi;
		const bool can_bx = allow_tc && !wide && batched_supported(m->dev) &&
		                    batched_step_smem(m->dev, tnrows) <= limit;
		// the step-synchronous layout by default from 300 areas, and from 100 areas for
		// batches of at least 32 particles per SM (measured on 16384 x 150 areas x 4 ages:
		// 381 ms against 398 ms with four particle-resident CTAs per SM)
		const bool bx_auto = m->A >= 300 || (m->A >= 100 && (long long)P >= 32LL * std::max(1, m->sms));
		if (can_bx && (opt == 3 || (opt == 0 && bx_auto))) {
			q->bd.batched = 1;
			q->state_global = false;
			q->bd.m_in_smem = 0;
		}
		// force of infection on the tensor cores, one particle per CTA: large models (the
		// matrix is streamed from L2 each step; the particle's populations and counts move to
		// global memory to make room for the operand ring)
		const bool can_tc = allow_tc && !wide && m->dev.tc_image != nullptr && fast_pick_threads(m->dev) == 640;
		const bool want_tc = opt == 2 || (opt == 0 && m->A >= 300 && !can_bx);
		if (!q->bd.batched && can_tc && want_tc) {
			// the transition counts stay on chip when they fit beside the operand ring
			for (int tn_on_chip = 1; tn_on_chip >= 0 && !q->bd.foi_tc; tn_on_chip--) {
				const size_t base = fast_smem_bytes(m->dev, nslots, false, q->bd.nefoi_stage, true, tnrows, ps, tn_on_chip != 0);
				const size_t off = (base + 127) & ~(size_t)127;
				if (off + fast_tc_smem_bytes(m->dev) <= limit) {
					q->bd.foi_tc = 1;
					q->bd.tc_smem_off = off;
					q->bd.tn_smem = tn_on_chip;
					q->state_global = true;
					q->bd.m_in_smem = 0;
				}
			}
		}
		// several particles per SM (320-thread CTAs): as many as the SM's shared memory
		// holds, up to four (three above 8 ages), each particle's state on chip -- or only
		// the infectious counts, force of infection and observation slots, with the state
		// in global memory, where the one-CTA layout keeps it there too or the layout is
		// asked for (option) or preferred (autotuner); the matrix is read through L1 unless
		// it fits beside every CTA's share.  Unless the option forces a count, the count
		// comes from the expected time below, and one CTA of 640 threads per SM stays
		// where that is faster.
		const int forced = option_fast_ctas();
		const int pref = forced != 0 ? 0 : m->tuned_ctas;
		const bool asked = forced >= 2 || pref >= 2;
		if (allow_ctas && !wide && !q->bd.foi_tc && !q->bd.batched && forced != 1 && pref != 1 &&
		    fast_pick_threads(m->dev) == 640) {
			const int kmax = std::min(forced >= 2 ? forced : 4, fast_ctas_max(m->G));
			const int kmin = asked ? 2 : 3;
			auto fit = [&](size_t bytes) { return (int)std::min<size_t>((size_t)kmax, kSmemPerSM / (bytes + 1024)); };
			const int nefo = q->bd.nefoi_stage;
			bool glob = false;
			int k = fit(fast_smem_bytes(m->dev, nslots, false, nefo, false, tnrows, ps, false, kDualThreads));
			if (k < kmin && (q->state_global || asked)) {
				glob = true;
				k = fit(fast_smem_bytes(m->dev, nslots, false, nefo, true, tnrows, ps, false, kDualThreads));
			}
			if (forced == 0 && k >= kmin) {
				// expected time in units of one 640-thread wave: ceil(P / SMs) for one CTA per
				// SM; (P / SMs) / gain(r) for 320-thread CTAs, r = min(k, P / SMs) of them
				// resident per SM (the block scheduler spreads a small grid one per SM), gain =
				// the SM throughput of r such CTAs against one 640-thread CTA, measured on the
				// ABC-SMC workload: 0.5 (one alone has half the threads), 1.0, 1.18, 1.26
				const double sms = (double)std::max(1, m->sms), per_sm = (double)P / sms;
				auto gain = [](double r) {
					static const double gt[5] = {0.0, 0.5, 1.0, 1.18, 1.26};
					if (r >= 4.0) return gt[4];
					const int i = (int)r;
					return gt[i] + (r - i) * (gt[i + 1] - gt[i]);
				};
				const double t_one = std::ceil(per_sm);
				int best = 0;
				double t_best = t_one;
				for (int kk = kmin; kk <= k; kk++) {
					const double t = per_sm / gain(std::min((double)kk, per_sm));
					if (t < t_best * 0.999) { t_best = t; best = kk; }
				}
				k = best;
			}
			if (k >= kmin) {
				q->bd.nt = kDualThreads;
				q->bd.ctas = k;
				q->state_global = glob;
				const size_t s1 = fast_smem_bytes(m->dev, nslots, true, nefo, glob, tnrows, ps, false, kDualThreads);
				q->bd.m_in_smem = (size_t)k * (s1 + 1024) <= kSmemPerSM ? 1 : 0;
			}
		}
		// small models in batches too small to fill the GPU (at most four particles per SM):
		// a step's draws one per (transition, column) thread, which shortens the step's
		// sequential chain of draws per thread (the particle filter's sections are this case)
		const int popt = option_parallel_draws();
		const int nt_run = q->bd.nt > 0 ? q->bd.nt : fast_pick_threads(m->dev);
		q->bd.pd = !wide && !q->bd.foi_tc && !q->bd.batched && fast_pd_fits(m->dev, nt_run) && popt != 1 &&
		           (popt == 2 || (long long)P <= 4LL * std::max(1, m->sms)) ? 1 : 0;
		// one pass of 256 threads over the draws instead of two of 128, where the batch
		// leaves room for the larger CTAs (two per SM)
		if (q->bd.pd && popt != 2 && nt_run == 128 && (long long)m->T * m->A * m->DP > 128 &&
		    (long long)P <= 2LL * std::max(1, m->sms))
			q->bd.nt = 256;
	}
	auto bail = [&](beep_status s) { beep_batch_destroy(q); return s; };
	if (b->form == BEEP_FORM_FAST && fast_prepare() != 0) return bail(fail(BEEP_DEVICE_ERROR, "constant tables"));
	st = stage_inputs(q);
	if (st != BEEP_OK) return bail(st);

	Layout wk;
	const size_t PW = b->form == BEEP_FORM_FAST ? 0 : (size_t)P;   // the fast form keeps its state on chip
	const size_t w_gs = wk.add(q->state_global ? fast_gstate_stride(m->dev) * (size_t)P : 0);
	const bool bx = q->bd.batched != 0;
	const size_t w_bxp = wk.add(bx ? (q->bd.pop_single ? 1 : 2) * 4 * popsz * (size_t)P : 0),
	             w_bxi = wk.add(bx ? 2 * 4 * agsz * (size_t)P : 0), w_bxy = wk.add(bx ? 4 * agsz * (size_t)P : 0),
	             w_bxs = wk.add(bx ? 4 * (size_t)q->bd.nslots * P : 0),
	             w_bxk = wk.add(bx ? 8 * (size_t)batched_obs_threads() * P : 0),
	             w_bxt = wk.add(bx ? 4 * (size_t)(q->bd.tn_full ? m->T : m->dev.tn_rows) * m->A * m->DP * P : 0),
	             w_bxw = wk.add(bx ? 4 * (size_t)nsteps : 0),
	             w_bxa = wk.add(bx ? batched_a_bytes(m->dev, P) : 0);
	size_t w_pa = wk.add(pe * popsz * PW), w_pb = wk.add(pe * popsz * PW), w_tn = wk.add(traj ? 0 : 4 * tnsz * PW),
	       w_im = wk.add(8 * agsz * PW), w_id = wk.add(8 * agsz * PW), w_di = wk.add(8 * agsz * PW),
	       w_nmi = wk.add(8 * agsz * PW), w_acc = wk.add(8 * (size_t)nscored * PW);
	Layout ou;
	q->u_st = ou.add(4 * (size_t)P);
	q->u_L = ou.add(b->L_out ? 8 * (size_t)P : 0);
	q->u_po = ou.add(want_po ? pe * popsz * P : 0);
	q->u_tn = ou.add(b->transnum_out ? 4 * tnsz * (size_t)nsteps * P : 0);
	q->u_pt = ou.add(want_pt ? pe * popsz * (size_t)nsteps * P : 0);
	q->out_size = ou.size;
	cudaError_t e = q->work_dev.reserve(wk.size);
	if (e == cudaSuccess) e = q->out_dev.reserve(ou.size);
	if (e == cudaSuccess) e = q->out_host.reserve(ou.size);
	if (e == cudaSuccess) e = cudaEventCreate(&q->ev0);
	if (e == cudaSuccess) e = cudaEventCreate(&q->ev1);
	if (e != cudaSuccess)
		return bail(fail(e == cudaErrorMemoryAllocation ? BEEP_OOM : BEEP_DEVICE_ERROR, cudaGetErrorString(e)));
	char *dw = (char *)q->work_dev.ptr, *dout = (char *)q->out_dev.ptr;
	BatchDev &bd = q->bd;
	bd.P = P; bd.ti = b->ti; bd.tf = b->tf; bd.ngroup = b->ngroup;
	bd.sampler_limit = option_sampler_limit();
	bd.k0 = (uint32_t)b->seed; bd.k1 = (uint32_t)(b->seed >> 32);
	bd.nscored = nscored;
	bd.pop_a = (int32_t *)(dw + w_pa); bd.pop_b = (int32_t *)(dw + w_pb);
	bd.tn = traj ? nullptr : (int32_t *)(dw + w_tn);
	bd.Imap = (double *)(dw + w_im); bd.Idiag = (double *)(dw + w_id); bd.dinf = (double *)(dw + w_di);
	bd.NMI = (double *)(dw + w_nmi); bd.obs_acc = (double *)(dw + w_acc);
	bd.gstate = q->state_global ? (void *)(dw + w_gs) : nullptr;
	if (bx) {
		bd.bx_pop = (int32_t *)(dw + w_bxp);
		bd.bx_ic = (float *)(dw + w_bxi);
		bd.bx_y = (float *)(dw + w_bxy);
		bd.bx_slot = (float *)(dw + w_bxs);
		bd.bx_kahan = (float2 *)(dw + w_bxk);
		bd.bx_tn = (int32_t *)(dw + w_bxt);
		bd.bx_work = (int32_t *)(dw + w_bxw);
		bd.bx_a = (unsigned char *)(dw + w_bxa);
	}
	bd.gstate_stride = q->state_global ? fast_gstate_stride(m->dev) : 0;
	bd.status = (int32_t *)(dout + q->u_st);
	bd.L = b->L_out ? (double *)(dout + q->u_L) : nullptr;
	bd.pop_out = want_po ? (int32_t *)(dout + q->u_po) : nullptr;
	bd.tn_traj = b->transnum_out ? (int32_t *)(dout + q->u_tn) : nullptr;
	bd.pop_traj = want_pt ? (int32_t *)(dout + q->u_pt) : nullptr;
	*out = q;
	return BEEP_OK;
}

extern "C" {

beep_status beep_batch_stage(beep_batch *q)
{
	if (!q) return fail(BEEP_BAD_INPUT, "null batch");
	beep_status st = check_batch(q->m, &q->b, q->device_io);
	if (st != BEEP_OK) return st;
	CUDA_TRY(cudaStreamSynchronize(q->m->stream));   // the staging buffer may still feed a copy
	return stage_inputs(q);
}

beep_status beep_batch_upload(beep_batch *q)
{
	if (!q) return fail(BEEP_BAD_INPUT, "null batch");
	CUDA_TRY(cudaMemcpyAsync(q->in_dev.ptr, q->in_host.ptr, q->in_size, cudaMemcpyHostToDevice, q->m->stream));
	return BEEP_OK;
}

beep_status beep_batch_launch(beep_batch *q)
{
	if (!q) return fail(BEEP_BAD_INPUT, "null batch");
	q->bd.sampler_limit = option_sampler_limit();   // batches kept across calls follow the current option
	CUDA_TRY(cudaMemsetAsync(q->bd.status, 0, 4 * (size_t)q->bd.P, q->m->stream));
	int le = q->b.form != BEEP_FORM_FAST ? launch_sim_plain(q->m->dev, q->bd, q->m->stream)
	         : q->bd.batched              ? launch_sim_batched(q->m->dev, q->bd, q->m->sms, q->m->stream)
	                                      : launch_sim_fast(q->m->dev, q->bd, q->m->stream);
	if (le != 0) return fail(BEEP_DEVICE_ERROR, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)le));
	q->pending = true;
	return BEEP_OK;
}

beep_status beep_batch_download(beep_batch *q)
{
	if (!q) return fail(BEEP_BAD_INPUT, "null batch");
	beep_status st = batch_download_enqueue(q);
	if (st != BEEP_OK) return st;
	CUDA_TRY(cudaStreamSynchronize(q->m->stream));
	return batch_download_finish(q);
}

}  // extern "C"

beep_status beep::batch_download_enqueue(beep_batch *q)
{
	CUDA_TRY(cudaMemcpyAsync(q->out_host.ptr, q->out_dev.ptr, q->out_size, cudaMemcpyDeviceToHost, q->m->stream));
	return BEEP_OK;
}

beep_status beep::batch_download_finish(beep_batch *q)
{
	const beep_sim_batch *b = &q->b;
	q->pending = false;
	const beep_model *m = q->m;
	const int P = b->nparticle, nsteps = b->tf - b->ti;
	const size_t popsz = (size_t)m->A * m->C * m->DP, tnsz = (size_t)m->A * m->T * m->DP;
	const char *ho = (const char *)q->out_host.ptr;
	const int32_t *pst = (const int32_t *)(ho + q->u_st);
	for (int p = 0; p < P; p++)
		if (pst[p] != 0) return fail((beep_status)pst[p], "particle " + std::to_string(p) + " failed on the device");
	if (b->L_out) memcpy(b->L_out, ho + q->u_L, 8 * (size_t)P);
	if (b->pop_out) memcpy(b->pop_out, ho + q->u_po, 4 * popsz * P);
	if (b->pop_out_f64) memcpy(b->pop_out_f64, ho + q->u_po, 8 * popsz * P);
	if (b->transnum_out) memcpy(b->transnum_out, ho + q->u_tn, 4 * tnsz * (size_t)nsteps * P);
	if (b->pop_traj_out) memcpy(b->pop_traj_out, ho + q->u_pt, 4 * popsz * (size_t)nsteps * P);
	if (b->pop_traj_out_f64) memcpy(b->pop_traj_out_f64, ho + q->u_pt, 8 * popsz * (size_t)nsteps * P);
	return BEEP_OK;
}

extern "C" {

beep_status beep_batch_time(beep_batch *q, int32_t iters, double *ms_per_launch)
{
	if (!q || iters <= 0 || !ms_per_launch) return fail(BEEP_BAD_INPUT, "bad argument");
	cudaStream_t s = q->m->stream;
	CUDA_TRY(cudaStreamSynchronize(s));
	CUDA_TRY(cudaEventRecord(q->ev0, s));
	for (int k = 0; k < iters; k++) {
		beep_status st = beep_batch_launch(q);
		if (st != BEEP_OK) return st;
	}
	CUDA_TRY(cudaEventRecord(q->ev1, s));
	CUDA_TRY(cudaEventSynchronize(q->ev1));
	float ms = 0;
	CUDA_TRY(cudaEventElapsedTime(&ms, q->ev0, q->ev1));
	*ms_per_launch = (double)ms / iters;
	return BEEP_OK;
}

beep_status beep_batch_time_kernels(beep_batch *q, int32_t iters, double *ms_per_launch, double *ms_kernels)
{
	if (!q || iters <= 0 || !ms_per_launch || !ms_kernels) return fail(BEEP_BAD_INPUT, "bad argument");
	for (int k = 0; k < 3; k++) ms_kernels[k] = 0.0;
	if (!q->bd.batched) return beep_batch_time(q, iters, ms_per_launch);
	cudaStream_t s = q->m->stream;
	const int nsteps = q->b.tf - q->b.ti;
	if (q->ev_split.size() != (size_t)(4 * nsteps)) {
		for (cudaEvent_t e : q->ev_split) cudaEventDestroy(e);
		q->ev_split.assign(4 * (size_t)nsteps, nullptr);
		for (auto &e : q->ev_split) CUDA_TRY(cudaEventCreate(&e));
	}
	double tot = 0.0, part[3] = {0.0, 0.0, 0.0};
	for (int k = 0; k < iters; k++) {
		CUDA_TRY(cudaStreamSynchronize(s));
		q->bd.sampler_limit = option_sampler_limit();
		CUDA_TRY(cudaMemsetAsync(q->bd.status, 0, 4 * (size_t)q->bd.P, s));
		CUDA_TRY(cudaEventRecord(q->ev0, s));
		const int le = launch_sim_batched(q->m->dev, q->bd, q->m->sms, s, q->ev_split.data());
		if (le != 0) return fail(BEEP_DEVICE_ERROR, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)le));
		CUDA_TRY(cudaEventRecord(q->ev1, s));
		CUDA_TRY(cudaEventSynchronize(q->ev1));
		float ms = 0;
		CUDA_TRY(cudaEventElapsedTime(&ms, q->ev0, q->ev1));
		tot += ms;
		for (int j = 0; j < nsteps; j++)
			for (int kk = 0; kk < 3; kk++) {
				CUDA_TRY(cudaEventElapsedTime(&ms, q->ev_split[4 * j + kk], q->ev_split[4 * j + kk + 1]));
				part[kk] += ms;
			}
	}
	q->pending = true;
	*ms_per_launch = tot / iters;
	for (int kk = 0; kk < 3; kk++) ms_kernels[kk] = part[kk] / iters;
	return BEEP_OK;
}

beep_status beep_batch_time_split(beep_batch *q, int32_t iters, double *ms_per_launch, double *ms_product)
{
	if (!q || iters <= 0 || !ms_per_launch || !ms_product) return fail(BEEP_BAD_INPUT, "bad argument");
	double k3[3];
	const beep_status st = beep_batch_time_kernels(q, iters, ms_per_launch, k3);
	*ms_product = k3[0];
	return st;
}

int32_t beep_batch_launches(const beep_batch *q)
{
	if (!q) return 0;
	return q->bd.batched ? batched_launches(q->b.tf - q->b.ti) : 1;
}

beep_status beep_batch_run_graph(beep_batch *q)
{
	if (!q) return fail(BEEP_BAD_INPUT, "null batch");
	if (q->device_io) return fail(BEEP_BAD_INPUT, "internal batches are not replayed as graphs");
	beep_status st = beep_batch_stage(q);
	if (st != BEEP_OK) return st;
	cudaStream_t s = q->m->stream;
	if (q->graph_exec && q->graph_in_size != q->in_size) {   // the staged inputs changed size: capture again
		cudaGraphExecDestroy(q->graph_exec);
		cudaGraphDestroy(q->graph);
		q->graph_exec = nullptr;
		q->graph = nullptr;
	}
	if (!q->graph_exec) {
		CUDA_TRY(cudaStreamSynchronize(s));
		CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		beep_status cs = beep_batch_upload(q);
		if (cs == BEEP_OK) cs = beep_batch_launch(q);
		if (cs == BEEP_OK) cs = batch_download_enqueue(q);
		cudaGraph_t g = nullptr;
		cudaError_t e = cudaStreamEndCapture(s, &g);
		if (cs != BEEP_OK) {
			if (g) cudaGraphDestroy(g);
			return cs;
		}
		if (e != cudaSuccess) return fail(BEEP_DEVICE_ERROR, std::string("graph capture: ") + cudaGetErrorString(e));
		e = cudaGraphInstantiate(&q->graph_exec, g, 0);
		if (e != cudaSuccess) {
			cudaGraphDestroy(g);
			return fail(BEEP_DEVICE_ERROR, std::string("graph instantiation: ") + cudaGetErrorString(e));
		}
		q->graph = g;
		q->graph_in_size = q->in_size;
	}
	CUDA_TRY(cudaGraphLaunch(q->graph_exec, s));
	CUDA_TRY(cudaStreamSynchronize(s));
	return batch_download_finish(q);
}

beep_status beep_autotune(beep_model *m, const beep_sim_batch *b, int32_t *chosen)
{
	if (!m || !b) return fail(BEEP_BAD_INPUT, "null argument");
	if (b->form != BEEP_FORM_FAST) return fail(BEEP_BAD_INPUT, "the autotuner chooses among fast-form kernels");
	// the sample: the batch's particles up to 64 per SM over a window of up to 90 steps in
	// the middle of its range, started from the populations a run of the first steps leaves
	// there -- the layouts' costs shift as an epidemic grows (draws of larger means, fixed
	// per-step costs weighing less), and a window at the start favoured the
	// particle-resident layouts (398 against 379 ms per 16384-particle generation of the
	// 150-area x 4-age ABC-SMC workload)
	int dev_sms = 152;
	cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, m->device);
	beep_sim_batch t = *b;
	t.nparticle = std::min(b->nparticle, 64 * dev_sms);
	t.L_out = nullptr;
	t.pop_out = nullptr;
	t.pop_out_f64 = nullptr;
	t.transnum_out = nullptr;
	t.pop_traj_out = nullptr;
	t.pop_traj_out_f64 = nullptr;
	if (t.ti > 0 && !t.pop_in) return fail(BEEP_BAD_INPUT, "pop_in is required when ti > 0");
	const int range = b->tf - b->ti, win = std::min(range, 90), t0 = b->ti + (range - win) / 2;
	std::vector<int32_t> pop_mid;
	if (t0 > b->ti) {
		beep_sim_batch pre = t;
		pre.tf = t0;
		pop_mid.resize((size_t)t.nparticle * m->A * m->C * m->DP);
		pre.pop_out = pop_mid.data();
		beep_batch *q = nullptr;
		beep_status st = beep_batch_create(m, &pre, &q);
		if (st == BEEP_OK) st = beep_batch_upload(q);
		if (st == BEEP_OK) st = beep_batch_launch(q);
		if (st == BEEP_OK) st = beep_batch_download(q);
		if (q) beep_batch_destroy(q);
		if (st != BEEP_OK) return st;
		t.ti = t0;
		t.pop_in = pop_mid.data();
	}
	t.tf = t0 + win;
	std::vector<double> L(t.nparticle);
	t.L_out = L.data();
	const int saved_foi = m->tuned_foi, saved_ctas = m->tuned_ctas;
	double best = 1e300;
	int best_foi = 1, best_ctas = 1;
	// candidates (force of infection path, particles per SM): SIMT with one, SIMT with
	// as many as fit (up to four), tensor cores (one particle per CTA), tensor cores
	// batched over the particles (step-synchronous)
	const int cands[4][2] = {{1, 1}, {1, 4}, {2, 1}, {3, 1}};
	for (const auto &c : cands) {
		m->tuned_foi = c[0];
		m->tuned_ctas = c[1];
		beep_batch *q = nullptr;
		beep_status st = beep_batch_create(m, &t, &q);
		if (st != BEEP_OK) { m->tuned_foi = saved_foi; m->tuned_ctas = saved_ctas; return st; }
		const int got = beep_batch_ctas_per_sm(q);
		const bool layout_ok = c[0] == 3 ? got == 0 : (c[1] == 1) == (got == 1);
		if (beep_batch_foi_path(q) != c[0] || !layout_ok) {   // not available for this model
			beep_batch_destroy(q);
			continue;
		}
		double ms = 0;
		st = beep_batch_upload(q);
		if (st == BEEP_OK) st = beep_batch_time(q, 1, &ms);      // warm-up
		if (st == BEEP_OK) st = beep_batch_time(q, 1, &ms);
		beep_batch_destroy(q);
		if (st != BEEP_OK) { m->tuned_foi = saved_foi; m->tuned_ctas = saved_ctas; return st; }
		if (ms < best) { best = ms; best_foi = c[0]; best_ctas = c[1]; }
	}
	m->tuned_foi = best_foi;
	// several per SM won: later batches take that layout where their size makes it
	// faster by the expected-time rule (one per SM for batches too small to fill the
	// SMs several deep)
	m->tuned_ctas = best_ctas;
	if (chosen) *chosen = best_foi;
	return BEEP_OK;
}

int32_t beep_batch_foi_path(const beep_batch *q)
{
	if (!q || q->b.form != BEEP_FORM_FAST) return 0;
	return q->bd.batched ? 3 : q->bd.foi_tc ? 2 : 1;
}

int32_t beep_batch_ctas_per_sm(const beep_batch *q)
{
	if (!q || q->b.form != BEEP_FORM_FAST) return 0;
	if (q->bd.batched) return 0;                  // particles are not pinned to SMs in the step-synchronous layout
	return q->bd.nt == kDualThreads ? q->bd.ctas : 1;
}

beep_status beep_batch_bytes(const beep_batch *q, int64_t *h2d, int64_t *d2h)
{
	if (!q || !h2d || !d2h) return fail(BEEP_BAD_INPUT, "null argument");
	*h2d = (int64_t)q->in_size;
	*d2h = (int64_t)q->out_size;
	return BEEP_OK;
}

beep_status beep_batch_destroy(beep_batch *q)
{
	if (!q) return BEEP_OK;
	if (q->m && q->m->stream) cudaStreamSynchronize(q->m->stream);
	q->in_host.release();
	q->out_host.release();
	q->in_dev.release();
	q->work_dev.release();
	q->out_dev.release();
	if (q->ev0) cudaEventDestroy(q->ev0);
	if (q->ev1) cudaEventDestroy(q->ev1);
	for (cudaEvent_t e : q->ev_split) cudaEventDestroy(e);
	if (q->graph_exec) cudaGraphExecDestroy(q->graph_exec);
	if (q->graph) cudaGraphDestroy(q->graph);
	delete q;
	return BEEP_OK;
}

beep_status beep_simulate(beep_model *m, const beep_sim_batch *b)
{
	if (!m || !b) return fail(BEEP_BAD_INPUT, "null argument");
	std::lock_guard<std::mutex> lock(m->mu);
	beep_batch *q = nullptr;
	beep_status st = beep_batch_create(m, b, &q);
	if (st != BEEP_OK) return st;
	st = beep_batch_upload(q);
	if (st == BEEP_OK) st = beep_batch_launch(q);
	if (st == BEEP_OK) st = beep_batch_download(q);
	std::string err = g_err;
	beep_batch_destroy(q);
	g_err = err;
	return st;
}

}  // extern "C"

size_t beep::model_device_bytes(const beep_model *m) { return m ? m->model_mem.cap : 0; }

size_t beep::batch_device_bytes(const beep_batch *q)
{
	return q ? q->in_dev.cap + q->work_dev.cap + q->out_dev.cap : 0;
}

int beep::option_fast_foi() { return g_fast_foi.load(); }

int beep::option_fast_ctas() { return g_fast_ctas.load(); }

uint32_t beep::option_sampler_limit() { return g_sampler_limit.load(); }
int beep::option_parallel_draws() { return g_parallel_draws.load(); }
