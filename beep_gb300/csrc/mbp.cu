// MBP chains on the device: the reference's Mbp pair of states
// (src/mbp.hh:58-59) for many chains at once.
//
// Each chain owns two trajectory slots in one HBM allocation; plain FP64 form:
//   transnum  int32 [2][nchain][S][A][T][DP]
//   transmean FP64  [2][nchain][S][A][T][DP]
//   Imap, Idiag FP64 [2][nchain][S][NS][A][G]
// fast form (mbp_fast.cu): counts int32 and means FP32 [2][nchain][S][T][A*DP]
// (column-major per step, the fast kernel's layout), no Imap;
// and a host-side record of which slot is its current state (the device
// reads a copy uploaded with every launch).  A proposal is written to the
// other slot; accepting it flips the record (swap_initial_propose_state), so
// no state is ever copied.  The kernels are the plain FP64 form's
// (sim_plain.cu, modes 1-3), which reproduce the reference's counts bit for
// bit under the keyed variate stream.
#include <algorithm>
#include <cuda_runtime.h>
#include <numeric>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace beep;

struct beep_mbp_chains {
	beep_model *m = nullptr;
	int32_t nchain = 0, form = 0;
	DevBuf traj, aux;
	std::vector<uint8_t> cur;            // current slot of each chain
	int32_t *tn = nullptr;
	double *mean = nullptr, *Imap = nullptr, *Idiag = nullptr;
	float *mean_f = nullptr;             // fast form
	bool initialised = false;
	size_t tnsz = 0, agsz = 0;
	// prepared batches, reused while the request keeps its shape (with / without L)
	beep_batch *q[2] = {nullptr, nullptr};
	int32_t q_ngroup[2] = {0, 0};
	bool q_go[2] = {false, false}, q_so[2] = {false, false};
	DevBuf fused_ctr;                    // work counter of fused launches led by this set
};

namespace {

// [S][A][T][DP] (the reference's transnum) -> [S][T][A*DP] (the fast chains' layout)
void to_fast_layout(const beep_mbp_chains *c, const int32_t *src, int32_t *dst)
{
	const int A = c->m->A, T = c->m->T, DP = c->m->DP, S = c->m->S;
	const size_t ncol = (size_t)A * DP;
	for (int s = 0; s < S; s++)
		for (int a = 0; a < A; a++)
			for (int t = 0; t < T; t++)
				for (int dp = 0; dp < DP; dp++)
					dst[((size_t)s * T + t) * ncol + (size_t)a * DP + dp] = src[(((size_t)s * A + a) * T + t) * DP + dp];
}

beep_status check_request(const beep_mbp_chains *c, const beep_mbp_request *r, int mode, bool simu_all)
{
	if (!r || !r->groups || r->ngroup <= 0) return fail(BEEP_BAD_INPUT, "the request needs parameter tables");
	if (r->inf_update != BEEP_INF_UPDATE && r->inf_update != BEEP_INF_DIF_UPDATE)
		return fail(BEEP_BAD_INPUT, "unknown inf_update");
	if (mode == 2 || (mode == 1 && !simu_all))
		if (!c->initialised) return fail(BEEP_BAD_INPUT, "chains are not initialised");
	return BEEP_OK;
}

// The chain batch of a request, staged, with its inputs (tables, current
// slots, SIMU mask) enqueued on the model's stream: mode 1 writes the
// non-current slot (simu_all: State::simulate), mode 3 rebuilds the
// non-current slot from its counts, mode 2 scores the current one.  The
// caller holds the model's lock, with its device current.
beep_status prepare_chains(beep_mbp_chains *c, const beep_mbp_request *r, int mode, bool simu_all, beep_batch **out)
{
	beep_model *m = c->m;
	const int P = c->nchain;
	beep_sim_batch b{};
	b.nparticle = P; b.ngroup = r->ngroup; b.groups = r->groups; b.group_of = r->group_of;
	b.seed = r->seed; b.stream_of = r->stream_of; b.ti = 0; b.tf = m->S;
	b.L_out = mode != 2 ? r->L_out : nullptr;
	b.form = c->form;
	// reuse the prepared batch when the request has the same shape: re-stage its tables
	const int slot = b.L_out ? 1 : 0;
	beep_batch *q = c->q[slot];
	beep_status st = BEEP_OK;
	if (q && c->q_ngroup[slot] == b.ngroup && c->q_go[slot] == (b.group_of != nullptr) &&
	    c->q_so[slot] == (b.stream_of != nullptr)) {
		q->b = b;
		q->bd.k0 = (uint32_t)b.seed;
		q->bd.k1 = (uint32_t)(b.seed >> 32);
		st = beep_batch_stage(q);
		if (st != BEEP_OK) {
			beep_batch_destroy(q);
			c->q[slot] = nullptr;
			return st;
		}
	} else {
		if (q) beep_batch_destroy(q);
		c->q[slot] = nullptr;
		st = batch_create_internal(m, &b, false, &q, false, false, true);
		if (st != BEEP_OK) return st;
		// the chain kernels draw per column thread, in the model's own CTA size
		q->bd.pd = 0;
		if (q->b.form == BEEP_FORM_FAST && q->bd.nt == 256 && fast_pick_threads(m->dev) == 128) q->bd.nt = 0;
		c->q[slot] = q;
		c->q_ngroup[slot] = b.ngroup;
		c->q_go[slot] = b.group_of != nullptr;
		c->q_so[slot] = b.stream_of != nullptr;
	}
	const bool mask = mode == 1 && !simu_all && r->simu;
	Layout L;
	const size_t o_cur = L.add((size_t)P), o_simu = L.add(mask ? (size_t)P * m->S * m->A : 0),
	             o_li = L.add(8 * (size_t)P);
	cudaError_t e = c->aux.reserve(L.size);
	if (e != cudaSuccess) return fail(BEEP_OOM, std::string("chain buffers: ") + cudaGetErrorString(e));
	char *d = (char *)c->aux.ptr;
	e = cudaMemcpyAsync(d + o_cur, c->cur.data(), (size_t)P, cudaMemcpyHostToDevice, m->stream);
	if (e == cudaSuccess && mask)
		e = cudaMemcpyAsync(d + o_simu, r->simu, (size_t)P * m->S * m->A, cudaMemcpyHostToDevice, m->stream);
	if (e != cudaSuccess) return fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e));
	BatchDev &bd = q->bd;
	bd.mode = mode;
	bd.inf_dif = r->inf_update == BEEP_INF_DIF_UPDATE ? 1 : 0;
	bd.simu_all = simu_all ? 1 : 0;
	bd.simu = mask ? (const uint8_t *)(d + o_simu) : nullptr;
	bd.cur = (const uint8_t *)(d + o_cur);
	bd.ch_tn = c->tn; bd.ch_mean = c->mean; bd.ch_Imap = c->Imap; bd.ch_Idiag = c->Idiag;
	bd.ch_mean_f = c->mean_f;
	bd.Li = (double *)(d + o_li);
	st = beep_batch_upload(q);
	if (st == BEEP_OK) *out = q;
	return st;
}

// One launch of the chain kernel over every chain (prepare_chains' modes).
beep_status run_chains(beep_mbp_chains *c, const beep_mbp_request *r, int mode, bool simu_all, double *Li_out)
{
	beep_status st = check_request(c, r, mode, simu_all);
	if (st != BEEP_OK) return st;
	beep_model *m = c->m;
	std::lock_guard<std::mutex> lock(m->mu);
	CUDA_TRY(cudaSetDevice(m->device));
	beep_batch *q = nullptr;
	st = prepare_chains(c, r, mode, simu_all, &q);
	if (st != BEEP_OK) return st;
	st = beep_batch_launch(q);
	if (st == BEEP_OK) st = beep_batch_download(q);   // waits; checks every chain's status
	if (st == BEEP_OK && mode == 2) {
		const cudaError_t e = cudaMemcpy(Li_out, q->bd.Li, 8 * (size_t)c->nchain, cudaMemcpyDeviceToHost);
		if (e != cudaSuccess) st = fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e));
	}
	return st;
}

}  // namespace

extern "C" {

BEEP_API beep_status beep_mbp_create(beep_model *m, int32_t nchain, int32_t form, beep_mbp_chains **out)
{
	if (!m || !out || nchain <= 0) return fail(BEEP_BAD_INPUT, "model, nchain > 0 and out are required");
	*out = nullptr;
	if (form != BEEP_FORM_PLAIN_FP64 && form != BEEP_FORM_FAST) return fail(BEEP_BAD_INPUT, "unknown form");
	if (form == BEEP_FORM_FAST && m->pop64)
		return fail(BEEP_BAD_INPUT, "a model with demographic changes (fractional populations) runs the plain FP64 form only");
	std::lock_guard<std::mutex> lock(m->mu);
	CUDA_TRY(cudaSetDevice(m->device));
	beep_mbp_chains *c = new beep_mbp_chains();
	c->m = m;
	c->nchain = nchain;
	c->form = form;
	c->tnsz = (size_t)m->A * m->T * m->DP;
	c->agsz = (size_t)m->NS * m->A * m->G;
	const size_t slots = 2 * (size_t)nchain * m->S;
	const bool fast = form == BEEP_FORM_FAST;
	Layout L;
	const size_t o_tn = L.add(4 * slots * c->tnsz), o_mean = L.add((fast ? 4 : 8) * slots * c->tnsz),
	             o_im = L.add(fast ? 0 : 8 * slots * c->agsz), o_id = L.add(fast ? 0 : 8 * slots * c->agsz);
	cudaError_t e = c->traj.reserve(L.size);
	if (e != cudaSuccess) {
		delete c;
		return fail(BEEP_OOM, "chain states (" + std::to_string(L.size >> 20) + " MiB): " + cudaGetErrorString(e));
	}
	char *d = (char *)c->traj.ptr;
	c->tn = (int32_t *)(d + o_tn);
	if (fast) c->mean_f = (float *)(d + o_mean);
	else {
		c->mean = (double *)(d + o_mean);
		c->Imap = (double *)(d + o_im);
		c->Idiag = (double *)(d + o_id);
	}
	c->cur.assign(nchain, 0);
	*out = c;
	return BEEP_OK;
}

BEEP_API beep_status beep_mbp_destroy(beep_mbp_chains *c)
{
	if (!c) return BEEP_OK;
	if (c->m) {
		cudaSetDevice(c->m->device);
		cudaStreamSynchronize(c->m->stream);
	}
	for (auto *q : c->q)
		if (q) beep_batch_destroy(q);
	c->traj.release();
	c->aux.release();
	c->fused_ctr.release();
	delete c;
	return BEEP_OK;
}

BEEP_API beep_status beep_mbp_initialise(beep_mbp_chains *c, const beep_mbp_request *r)
{
	if (!c) return fail(BEEP_BAD_INPUT, "null chains");
	beep_status st = run_chains(c, r, 1, true, nullptr);
	if (st != BEEP_OK) return st;
	for (auto &x : c->cur) x ^= 1;
	c->initialised = true;
	return BEEP_OK;
}

BEEP_API beep_status beep_mbp_set_state(beep_mbp_chains *c, const beep_mbp_request *r, const int32_t *transnum)
{
	if (!c || !transnum) return fail(BEEP_BAD_INPUT, "null argument");
	{
		std::lock_guard<std::mutex> lock(c->m->mu);
		CUDA_TRY(cudaSetDevice(c->m->device));
		CUDA_TRY(cudaStreamSynchronize(c->m->stream));
		const size_t S = c->m->S, per = S * c->tnsz;
		std::vector<int32_t> tmp;
		for (int k = 0; k < c->nchain; k++) {
			const size_t off = ((size_t)(1 - c->cur[k]) * c->nchain + k) * per;
			const int32_t *src = transnum + (size_t)k * per;
			if (c->form == BEEP_FORM_FAST) {            // [S][A][T][DP] -> [S][T][A*DP]
				tmp.resize(per);
				to_fast_layout(c, src, tmp.data());
				src = tmp.data();
			}
			// on the model's stream (the chain kernels' stream), completed before the
			// host buffer is reused
			CUDA_TRY(cudaMemcpyAsync(c->tn + off, src, 4 * per, cudaMemcpyHostToDevice, c->m->stream));
			CUDA_TRY(cudaStreamSynchronize(c->m->stream));
		}
	}
	beep_status st = run_chains(c, r, 3, false, nullptr);
	if (st != BEEP_OK) return st;
	for (auto &x : c->cur) x ^= 1;
	c->initialised = true;
	return BEEP_OK;
}

BEEP_API beep_status beep_mbp_propose(beep_mbp_chains *c, const beep_mbp_request *r)
{
	if (!c) return fail(BEEP_BAD_INPUT, "null chains");
	return run_chains(c, r, 1, false, nullptr);
}

BEEP_API beep_status beep_mbp_propose_fused(int32_t nset, beep_mbp_chains *const *sets,
                                            const beep_mbp_request *requests)
{
	if (nset <= 0 || nset > kMaxFusedSets || !sets || !requests)
		return fail(BEEP_BAD_INPUT, "1 to " + std::to_string(kMaxFusedSets) + " chain sets, one request each");
	for (int k = 0; k < nset; k++) {
		const beep_mbp_chains *c = sets[k];
		if (!c) return fail(BEEP_BAD_INPUT, "null chains");
		if (c->form != BEEP_FORM_FAST) return fail(BEEP_BAD_INPUT, "a fused launch takes fast-form chains");
		if (c->m->device != sets[0]->m->device) return fail(BEEP_BAD_INPUT, "the chain sets are on different devices");
		if (!fused_supported(c->m->dev))
			return fail(BEEP_BAD_INPUT, "a fused launch takes models of at most 8 transitions and 16 age groups");
		for (int j = 0; j < k; j++)
			if (sets[j] == c) return fail(BEEP_BAD_INPUT, "a chain set appears twice");
		beep_status st = check_request(c, &requests[k], 1, false);
		if (st != BEEP_OK) return st;
	}
	// every model once, locked in address order
	std::vector<beep_model *> models;
	for (int k = 0; k < nset; k++) models.push_back(sets[k]->m);
	std::sort(models.begin(), models.end());
	models.erase(std::unique(models.begin(), models.end()), models.end());
	std::vector<std::unique_lock<std::mutex>> locks;
	for (beep_model *m : models) locks.emplace_back(m->mu);
	CUDA_TRY(cudaSetDevice(sets[0]->m->device));
	// launch order: the sets whose chains cost most first (steps x columns x transitions)
	std::vector<int> order(nset);
	std::iota(order.begin(), order.end(), 0);
	auto cost = [&](int k) {
		const beep_model *m = sets[k]->m;
		return (double)m->S * m->A * m->DP * m->T;
	};
	std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost(x) > cost(y); });
	beep_mbp_chains *lead = sets[order[0]];
	cudaStream_t st0 = lead->m->stream;
	// on an error once work is enqueued: wait for it, so that no copy is left in flight
	auto drain = [&](beep_status s) {
		for (beep_model *m : models) cudaStreamSynchronize(m->stream);
		return s;
	};
	std::vector<beep_batch *> qs(nset, nullptr);
	for (int i = 0; i < nset; i++) {
		const int k = order[i];
		beep_status st = prepare_chains(sets[k], &requests[k], 1, false, &qs[k]);
		if (st != BEEP_OK) return drain(st);
	}
	// the other models' inputs are on their own streams: complete before the launch on st0
	for (beep_model *m : models)
		if (m->stream != st0 && cudaStreamSynchronize(m->stream) != cudaSuccess)
			return drain(fail(BEEP_DEVICE_ERROR, "chain inputs"));
	ModelDev md[kMaxFusedSets];
	BatchDev bd[kMaxFusedSets];
	for (int i = 0; i < nset; i++) {
		md[i] = sets[order[i]]->m->dev;
		bd[i] = qs[order[i]]->bd;
		bd[i].sampler_limit = option_sampler_limit();
	}
	// one shared-memory layout per set at the launch's thread count and age stride: the
	// area-mixing matrix is read from L2 where its copy no longer fits
	const int mg = fused_mg(md, nset);
	const size_t limit = 227 * 1024;
	for (int i = 0; i < nset; i++) {
		if (bd[i].m_in_smem && fused_smem_bytes(md[i], bd[i], mg) > limit) bd[i].m_in_smem = 0;
		if (fused_smem_bytes(md[i], bd[i], mg) > limit)
			return drain(fail(BEEP_BAD_INPUT, "a model's chain state exceeds the shared memory of a fused launch"));
	}
	cudaError_t e = lead->fused_ctr.reserve(256);
	for (int i = 0; i < nset && e == cudaSuccess; i++)
		e = cudaMemsetAsync(bd[i].status, 0, 4 * (size_t)bd[i].P, st0);
	if (e != cudaSuccess) return drain(fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e)));
	const int le = launch_sim_fast_chain_fused(md, bd, nset, (int32_t *)lead->fused_ctr.ptr, lead->m->sms, st0);
	if (le != 0)
		return drain(fail(BEEP_DEVICE_ERROR, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)le)));
	for (int k = 0; k < nset && e == cudaSuccess; k++)
		e = cudaMemcpyAsync(qs[k]->out_host.ptr, qs[k]->out_dev.ptr, qs[k]->out_size, cudaMemcpyDeviceToHost, st0);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st0);
	if (e != cudaSuccess) return drain(fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e)));
	beep_status st = BEEP_OK;
	for (int k = 0; k < nset; k++) {              // statuses and L of every set
		const beep_status sk = batch_download_finish(qs[k]);
		if (st == BEEP_OK) st = sk;
	}
	return st;
}

BEEP_API beep_status beep_mbp_accept(beep_mbp_chains *c, const uint8_t *accept)
{
	if (!c || !accept) return fail(BEEP_BAD_INPUT, "null argument");
	if (!c->initialised) return fail(BEEP_BAD_INPUT, "chains are not initialised");
	for (int k = 0; k < c->nchain; k++)
		if (accept[k]) c->cur[k] ^= 1;
	return BEEP_OK;
}

BEEP_API beep_status beep_mbp_state_likelihood(beep_mbp_chains *c, const beep_mbp_request *r, double *Li_out)
{
	if (!c || !Li_out) return fail(BEEP_BAD_INPUT, "null argument");
	return run_chains(c, r, 2, false, Li_out);
}

BEEP_API double beep_mbp_acceptance(int32_t cutoff_mode, double invT, double EFcut, double EF_prop, double EF_init,
                                    double Pr_prop, double Pr_init)
{
	double al = 0.0;
	if (cutoff_mode) {
		if (EF_prop < EFcut) al = exp(Pr_prop - Pr_init);
	} else {
		al = exp(-invT * 0.5 * (EF_prop - EF_init) + Pr_prop - Pr_init);
	}
	if (al > 1) al = 1;
	return al;
}

BEEP_API int32_t beep_mbp_ctas_per_sm(const beep_mbp_chains *c)
{
	if (!c) return 0;
	int32_t k = 0;
	for (beep_batch *q : c->q)
		if (q) k = std::max(k, beep_batch_ctas_per_sm(q));
	return k;
}

BEEP_API beep_status beep_mbp_read_state(beep_mbp_chains *c, int32_t chain, int32_t *transnum_out,
                                         double *transmean_out)
{
	if (!c || chain < 0 || chain >= c->nchain) return fail(BEEP_BAD_INPUT, "chain out of range");
	if (!c->initialised) return fail(BEEP_BAD_INPUT, "chains are not initialised");
	std::lock_guard<std::mutex> lock(c->m->mu);
	CUDA_TRY(cudaSetDevice(c->m->device));
	CUDA_TRY(cudaStreamSynchronize(c->m->stream));
	const size_t S = c->m->S, per = S * c->tnsz;
	const size_t off = ((size_t)c->cur[chain] * c->nchain + chain) * per;
	if (c->form != BEEP_FORM_FAST) {
		if (transnum_out) CUDA_TRY(cudaMemcpy(transnum_out, c->tn + off, 4 * per, cudaMemcpyDeviceToHost));
		if (transmean_out) CUDA_TRY(cudaMemcpy(transmean_out, c->mean + off, 8 * per, cudaMemcpyDeviceToHost));
		return BEEP_OK;
	}
	std::vector<int32_t> tn(per), tr(per);
	std::vector<float> mf(per);
	CUDA_TRY(cudaMemcpy(tn.data(), c->tn + off, 4 * per, cudaMemcpyDeviceToHost));
	CUDA_TRY(cudaMemcpy(mf.data(), c->mean_f + off, 4 * per, cudaMemcpyDeviceToHost));
	const int A = c->m->A, T = c->m->T, DP = c->m->DP;
	const size_t ncol = (size_t)A * DP;
	for (size_t s = 0; s < S; s++)
		for (int a = 0; a < A; a++)
			for (int t = 0; t < T; t++)
				for (int dp = 0; dp < DP; dp++) {
					const size_t ref = ((s * A + a) * T + t) * DP + dp, fst = (s * T + t) * ncol + (size_t)a * DP + dp;
					if (transnum_out) transnum_out[ref] = tn[fst];
					if (transmean_out) transmean_out[ref] = (double)mf[fst];
				}
	return BEEP_OK;
}

}  // extern "C"
