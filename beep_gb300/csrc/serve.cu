// Serving loop: continuous batching of simulation and likelihood requests
// of uneven sizes on one GPU.
//
// beep_serve_submit only queues a copy of the request.  One worker thread
//   * retires running requests whose last event completed (status check and
//     copy into the caller's arrays),
//   * admits queued requests in arrival order while fewer than max_inflight
//     run and their device footprint fits the budget -- first fit, holding back
//     the room the oldest waiting request needs, so that later small requests
//     may start early but never starve it,
//   * packs queued simulation requests of the same model (the same model
//     description), form, step range and outputs into one batch: their
//     parameter sets, streams and per-particle keys (each request's seed) are
//     concatenated, so one launch serves them all and each particle draws
//     exactly what it draws alone;
//   * creates each admitted request's (or pack's) device model and batch and
//     enqueues its copies and kernel on the model's own non-blocking stream, so
//     kernels of different requests run side by side on the SMs they leave free.
// Device memory of finished requests is released only while nothing runs (or
// when the oldest request is waiting for that memory): releasing device or
// pinned memory synchronises the whole device and would stall the kernels of
// the other requests.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "capi_internal.h"

using namespace beep;

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
	uint64_t id = 0;
	int32_t kind = 0;
	beep_model_desc desc{};
	beep_sim_batch batch{};
	beep_pf_request pf{};               // BEEP_REQ_PF_LIKELIHOOD
	std::thread pf_thread;              // runs the filter (sections with host steps between them)
	std::atomic<bool> pf_finished{false};
	size_t est = 0, bytes = 0;
	beep_model *m = nullptr;
	beep_batch *q = nullptr;
	cudaEvent_t ev_start = nullptr, ev_end = nullptr;
	int state = 0;                      // 0 queued, 1 running, 2 done
	beep_status status = BEEP_OK;
	std::string err;
	double t_submit = 0, t_admit = 0, t_done = 0, g_start = -1, g_end = -1;
	// a pack: the requests run as one batch (the first is the leader, which holds the
	// device model and batch), and the concatenated inputs and outputs of that batch
	std::vector<Req *> members;
	beep_sim_batch pbatch{};
	std::vector<beep_param_tables> pgroups;
	std::vector<int32_t> pgroup_of, ppop_in, ppop_out;
	std::vector<uint32_t> pstream_of;
	std::vector<uint2> pkeys;
	std::vector<double> pL;
};

constexpr int32_t kPackParticles = 32768;   // particles of one packed batch, at most

// Requests that can share one batch: simulation kinds of the same model description
// (the caller's own arrays), form, step range and outputs; no trajectory outputs.
bool packable(const Req *a, const Req *b)
{
	if (a->kind == BEEP_REQ_PF_LIKELIHOOD || b->kind == BEEP_REQ_PF_LIKELIHOOD) return false;
	if (memcmp(&a->desc, &b->desc, sizeof(beep_model_desc)) != 0) return false;
	if (a->desc.ndemocat_change > 0) return false;      // FP64 populations: not packed
	const beep_sim_batch &x = a->batch, &y = b->batch;
	return x.form == y.form && x.ti == y.ti && x.tf == y.tf && (x.pop_in != nullptr) == (y.pop_in != nullptr) &&
	       !x.transnum_out && !y.transnum_out && !x.pop_traj_out && !y.pop_traj_out &&
	       (x.L_out != nullptr) == (y.L_out != nullptr) && (x.pop_out != nullptr) == (y.pop_out != nullptr);
}

size_t rup(size_t x) { return (x + 255) & ~(size_t)255; }

// Upper estimate of the device bytes a request holds (model + batch); the
// actual figure replaces it once the request is created.
size_t estimate_bytes(const beep_model_desc &d, const beep_sim_batch &b)
{
	const size_t A = d.narea, G = d.nage, DP = d.ndemocatpos, C = d.ncomp, T = d.ntrans, S = d.ndivision;
	const size_t NS = d.nstrain, nobs = d.nobs;
	const size_t ncells = nobs && d.obs_cell_ptr ? (size_t)d.obs_cell_ptr[nobs] : 0;
	const size_t nnz = d.M_rowptr ? (size_t)d.M_rowptr[A] : A * A;
	const size_t popsz = A * C * DP, tnsz = A * T * DP, agsz = NS * A * G, ncol = A * DP;
	const size_t P = b.nparticle, nsteps = b.tf > b.ti ? (size_t)(b.tf - b.ti) : 0;
	size_t model = 4 * A * A + 48 * nnz + 128 * nobs + 24 * ncells + 8 * popsz + 64 * A + 64 * T + 16384;
	size_t tabs = 0;
	for (int g = 0; g < b.ngroup; g++) {
		const beep_param_tables &t = b.groups[g];
		tabs += 12 * (T * DP + DP + C + T + (size_t)t.nbeta_row * S + (size_t)d.period * A + S * G * G + S +
		              (size_t)t.nefoi * (S + G) + (size_t)t.nobs_spline * S) + 8 * NS * A + 256;
	}
	size_t active = 0;   // (step, observation) pairs of the step range
	for (size_t o = 0; o < nobs; o++) {
		const int lo = std::max(d.obs_sett_i[o], b.ti), hi = std::min(d.obs_sett_f[o], b.tf);
		if (hi > lo) active += (size_t)(hi - lo);
	}
	const size_t pe = d.ndemocat_change > 0 ? 8 : 4;   // bytes per population (FP64 with demographic changes)
	if (d.ndemocat_change > 0)
		model += 8 * S * 32 * (size_t)d.ndemocat_change + 4 * (A + DP) * (size_t)d.ndemocat_change;
	size_t in = tabs + 8 * P + (b.ti > 0 ? pe * popsz * P : 0) + 36 * active + 16 * nobs + 4 * nsteps + 4096;
	size_t work;
	if (b.form == BEEP_FORM_FAST) {
		const bool global_state = 4 * (2 * C * ncol + T * ncol) > 150 * 1024;
		work = global_state ? P * rup(4 * (2 * C * ncol + T * ncol)) : 0;
	} else {
		work = P * (2 * pe * popsz + 4 * tnsz + 32 * agsz + 8 * nobs) + 4096;
	}
	size_t out = P * (4 + (b.L_out ? 8 : 0) + (b.pop_out || b.pop_out_f64 ? pe * popsz : 0) +
	                  (b.transnum_out ? 4 * tnsz * nsteps : 0) + (b.pop_traj_out || b.pop_traj_out_f64 ? pe * popsz * nsteps : 0)) +
	             4096;
	return model + in + work + out + 5 * 256;
}

// Device bytes of a particle-filter request: the model, one prepared batch
// per section, the carried populations and weights, and the lineage counts.
size_t estimate_pf_bytes(const beep_model_desc &d, const beep_pf_request &r)
{
	beep_sim_batch b{};
	b.nparticle = r.nparticle;
	b.ngroup = 1;
	b.groups = r.tables;
	b.ti = 0;
	b.tf = d.ndivision;
	b.form = r.form;
	double L = 0;
	b.L_out = &L;
	const size_t N = r.nparticle, popsz = (size_t)d.narea * d.ncomp * d.ndemocatpos;
	const size_t tnsz = (size_t)d.narea * d.ntrans * d.ndemocatpos;
	return 2 * estimate_bytes(d, b) + N * ((d.ndemocat_change > 0 ? 16 : 8) * popsz + 64 + 12 * (size_t)r.nsection) +
	       (r.lineage_transnum_out ? 4 * tnsz * (size_t)d.ndivision * N : 0);
}

}  // namespace

struct beep_server {
	int device = 0;
	size_t budget = 0;
	int max_inflight = 1;
	std::mutex mu;
	std::condition_variable cv_work, cv_done;
	std::deque<Req *> queue;
	std::vector<Req *> running, graveyard;
	std::map<uint64_t, Req *> reqs;
	size_t used = 0, held = 0;          // bytes of running requests / of finished ones not yet released
	uint64_t next_id = 1;
	bool stop = false;
	std::thread worker;
	Clock::time_point t0;
	cudaEvent_t ev0 = nullptr;
	cudaStream_t st0 = nullptr;
	double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void release_request_memory(Req *r)
{
	if (r->pf_thread.joinable()) r->pf_thread.join();
	if (r->q) beep_batch_destroy(r->q);
	if (r->m) beep_model_destroy(r->m);
	if (r->ev_start) cudaEventDestroy(r->ev_start);
	if (r->ev_end) cudaEventDestroy(r->ev_end);
	r->q = nullptr;
	r->m = nullptr;
	r->ev_start = r->ev_end = nullptr;
}

// A particle-filter request runs on its own host thread: the filter steps
// section by section with host work in between (beep_pf_loglik), so it cannot
// be one enqueue; its kernels still run on the request's own stream beside
// the others'.
void run_pf_request(beep_server *s, Req *r)
{
	cudaSetDevice(s->device);
	beep_status st = beep_model_create(&r->desc, &r->m);
	if (st == BEEP_OK) {
		cudaEventCreate(&r->ev_start);
		cudaEventCreate(&r->ev_end);
		cudaEventRecord(r->ev_start, r->m->stream);
		st = beep_pf_loglik(r->m, &r->pf);
		cudaEventRecord(r->ev_end, r->m->stream);
		cudaEventSynchronize(r->ev_end);
		float a = 0, b = 0;
		if (cudaEventElapsedTime(&a, s->ev0, r->ev_start) == cudaSuccess &&
		    cudaEventElapsedTime(&b, s->ev0, r->ev_end) == cudaSuccess) {
			r->g_start = a * 1e-3;
			r->g_end = b * 1e-3;
		}
	}
	if (st != BEEP_OK) {
		r->status = st;
		r->err = beep_last_error();
	}
	r->pf_finished.store(true);
	s->cv_work.notify_all();
}

// Creates the request's model and batch and enqueues its work (worker thread,
// server lock not held).
void start_request(beep_server *s, Req *r)
{
	if (r->kind == BEEP_REQ_PF_LIKELIHOOD) {
		r->bytes = r->est;
		r->pf_thread = std::thread(run_pf_request, s, r);
		return;
	}
	beep_status st = beep_model_create(&r->desc, &r->m);
	if (st == BEEP_OK && r->members.size() > 1) {
		// one batch for the pack: parameter sets, group and stream indices, keys and
		// start populations of the members one after another
		beep_sim_batch &pb = r->pbatch;
		pb = r->batch;
		int32_t P = 0;
		const size_t popsz = (size_t)r->desc.narea * r->desc.ncomp * r->desc.ndemocatpos;
		for (Req *x : r->members) {
			const beep_sim_batch &b = x->batch;
			const int32_t goff = (int32_t)r->pgroups.size();
			for (int g = 0; g < b.ngroup; g++) r->pgroups.push_back(b.groups[g]);
			for (int p = 0; p < b.nparticle; p++) {
				r->pgroup_of.push_back((b.group_of ? b.group_of[p] : 0) + goff);
				r->pstream_of.push_back(b.stream_of ? b.stream_of[p] : (uint32_t)p);
				r->pkeys.push_back(make_uint2((uint32_t)b.seed, (uint32_t)(b.seed >> 32)));
			}
			if (b.pop_in) r->ppop_in.insert(r->ppop_in.end(), b.pop_in, b.pop_in + popsz * b.nparticle);
			P += b.nparticle;
		}
		r->pL.assign(pb.L_out ? (size_t)P : 0, 0.0);
		r->ppop_out.assign(pb.pop_out ? popsz * P : 0, 0);
		pb.nparticle = P;
		pb.ngroup = (int32_t)r->pgroups.size();
		pb.groups = r->pgroups.data();
		pb.group_of = r->pgroup_of.data();
		pb.stream_of = r->pstream_of.data();
		pb.pop_in = pb.pop_in ? r->ppop_in.data() : nullptr;
		pb.L_out = pb.L_out ? r->pL.data() : nullptr;
		pb.pop_out = pb.pop_out ? r->ppop_out.data() : nullptr;
		st = batch_create_internal(r->m, &pb, false, &r->q, false, true, true, &r->pkeys);
	} else if (st == BEEP_OK) {
		st = beep_batch_create(r->m, &r->batch, &r->q);
	}
	if (st == BEEP_OK) {
		cudaStream_t str = r->m->stream;
		cudaError_t e = cudaEventCreate(&r->ev_start);
		if (e == cudaSuccess) e = cudaEventCreate(&r->ev_end);
		if (e == cudaSuccess) e = cudaEventRecord(r->ev_start, str);
		if (e != cudaSuccess) st = fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e));
		if (st == BEEP_OK) st = beep_batch_upload(r->q);
		if (st == BEEP_OK) st = beep_batch_launch(r->q);
		if (st == BEEP_OK) st = batch_download_enqueue(r->q);
		if (st == BEEP_OK) {
			e = cudaEventRecord(r->ev_end, str);
			if (e != cudaSuccess) st = fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e));
		}
	}
	r->bytes = model_device_bytes(r->m) + batch_device_bytes(r->q);
	if (st != BEEP_OK) {
		r->status = st;
		r->err = beep_last_error();
	}
}

// Unpacks a request whose last event completed (worker thread, lock not held).
void finish_request(beep_server *s, Req *r, cudaError_t ev_state)
{
	if (ev_state != cudaSuccess) {
		r->status = BEEP_DEVICE_ERROR;
		r->err = cudaGetErrorString(ev_state);
	} else if (r->members.size() > 1) {
		// the pack's outputs, member by member: statuses, L and final populations
		beep_batch *q = r->q;
		q->pending = false;
		const char *ho = (const char *)q->out_host.ptr;
		const int32_t *pst = (const int32_t *)(ho + q->u_st);
		const double *L = (const double *)(ho + q->u_L);
		const int32_t *pop = (const int32_t *)(ho + q->u_po);
		const size_t popsz = (size_t)r->desc.narea * r->desc.ncomp * r->desc.ndemocatpos;
		size_t off = 0;
		for (Req *x : r->members) {
			const beep_sim_batch &b = x->batch;
			for (int p = 0; p < b.nparticle && x->status == BEEP_OK; p++)
				if (pst[off + p] != 0) {
					x->status = (beep_status)pst[off + p];
					x->err = "particle " + std::to_string(p) + " failed on the device";
				}
			if (x->status == BEEP_OK) {
				if (b.L_out) memcpy(b.L_out, L + off, 8 * (size_t)b.nparticle);
				if (b.pop_out) memcpy(b.pop_out, pop + off * popsz, 4 * popsz * b.nparticle);
			}
			off += (size_t)b.nparticle;
		}
		float a = 0, bt = 0;
		if (cudaEventElapsedTime(&a, s->ev0, r->ev_start) == cudaSuccess &&
		    cudaEventElapsedTime(&bt, s->ev0, r->ev_end) == cudaSuccess) {
			for (Req *x : r->members) {
				x->g_start = a * 1e-3;
				x->g_end = bt * 1e-3;
			}
		}
	} else {
		beep_status st = batch_download_finish(r->q);
		if (st != BEEP_OK) {
			r->status = st;
			r->err = beep_last_error();
		}
		float a = 0, b = 0;
		if (cudaEventElapsedTime(&a, s->ev0, r->ev_start) == cudaSuccess &&
		    cudaEventElapsedTime(&b, s->ev0, r->ev_end) == cudaSuccess) {
			r->g_start = a * 1e-3;
			r->g_end = b * 1e-3;
		}
	}
}

void worker_main(beep_server *s)
{
	cudaSetDevice(s->device);
	std::unique_lock<std::mutex> lk(s->mu);
	while (true) {
		// retire completed requests
		for (size_t i = 0; i < s->running.size();) {
			Req *r = s->running[i];
			const bool pf = r->kind == BEEP_REQ_PF_LIKELIHOOD;
			cudaError_t e = pf ? (r->pf_finished.load() ? cudaSuccess : cudaErrorNotReady)
			                   : r->ev_end ? cudaEventQuery(r->ev_end) : cudaSuccess;
			if (e == cudaErrorNotReady) { i++; continue; }
			s->running.erase(s->running.begin() + i);
			lk.unlock();
			if (pf) r->pf_thread.join();
			else if (r->status == BEEP_OK) finish_request(s, r, e);
			lk.lock();
			r->t_done = s->now();
			r->state = 2;
			for (Req *x : r->members) {
				if (x == r) continue;
				if (r->status != BEEP_OK && x->status == BEEP_OK) { x->status = r->status; x->err = r->err; }
				x->t_done = r->t_done;
				x->state = 2;
			}
			s->used -= r->bytes;
			s->held += r->bytes;
			s->graveyard.push_back(r);
			s->cv_done.notify_all();
		}
		// release finished requests' memory while the device is idle, or when
		// the oldest queued request waits for it
		const bool head_blocked = !s->queue.empty() && !s->running.empty() &&
		                          s->used + s->held + s->queue.front()->est > s->budget &&
		                          s->used + s->queue.front()->est <= s->budget;
		if (!s->graveyard.empty() && (s->running.empty() || head_blocked)) {
			std::vector<Req *> g;
			g.swap(s->graveyard);
			size_t freed = 0;
			for (Req *r : g) freed += r->bytes;
			lk.unlock();
			for (Req *r : g) release_request_memory(r);
			lk.lock();
			s->held -= freed;
		}
		if (s->stop && s->queue.empty() && s->running.empty()) break;
		// admit: first fit in arrival order, the oldest request's room held back
		size_t reserve = 0;
		for (size_t k = 0; k < s->queue.size();) {
			Req *r = s->queue[k];
			const bool alone = s->running.empty() && k == 0;
			const bool fits = (int)s->running.size() < s->max_inflight &&
			                  (s->used + s->held + reserve + r->est <= s->budget || alone);
			if (!fits) {
				if (k == 0) reserve = r->est;
				k++;
				continue;
			}
			s->queue.erase(s->queue.begin() + k);
			r->state = 1;
			r->t_admit = s->now();
			// later queued requests that can share its batch (within the budget and the pack size)
			r->members.assign(1, r);
			int32_t npack = r->batch.nparticle;
			size_t est = r->est;
			for (size_t j = k; j < s->queue.size();) {
				Req *x = s->queue[j];
				if (packable(r, x) && npack + x->batch.nparticle <= kPackParticles &&
				    (s->used + s->held + reserve + est + x->est <= s->budget || alone)) {
					s->queue.erase(s->queue.begin() + j);
					x->state = 1;
					x->t_admit = r->t_admit;
					r->members.push_back(x);
					npack += x->batch.nparticle;
					est += x->est;
				} else {
					j++;
				}
			}
			r->est = est;
			s->used += r->est;
			lk.unlock();
			start_request(s, r);
			lk.lock();
			s->used = s->used - r->est + r->bytes;
			s->running.push_back(r);   // a failed start retires at the next pass
		}
		if (s->running.empty() && s->queue.empty() && s->graveyard.empty() && !s->stop) s->cv_work.wait(lk);
		else s->cv_work.wait_for(lk, std::chrono::microseconds(100));
	}
}

Req *find(beep_server *s, uint64_t t)
{
	auto it = s->reqs.find(t);
	return it == s->reqs.end() ? nullptr : it->second;
}

}  // namespace

extern "C" {

BEEP_API beep_status beep_server_create(int32_t device, int64_t hbm_budget_bytes, int32_t max_inflight,
                                        beep_server **out)
{
	if (!out || hbm_budget_bytes <= 0 || max_inflight <= 0) return fail(BEEP_BAD_INPUT, "bad server arguments");
	*out = nullptr;
	beep_status st = beep_device_init(device);
	if (st != BEEP_OK) return st;
	beep_server *s = new beep_server();
	s->device = device;
	s->budget = (size_t)hbm_budget_bytes;
	s->max_inflight = max_inflight;
	cudaError_t e = cudaStreamCreateWithFlags(&s->st0, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
	if (e == cudaSuccess) e = cudaEventRecord(s->ev0, s->st0);
	if (e == cudaSuccess) e = cudaEventSynchronize(s->ev0);
	if (e != cudaSuccess) {
		delete s;
		return fail(BEEP_DEVICE_ERROR, cudaGetErrorString(e));
	}
	s->t0 = Clock::now();
	s->worker = std::thread(worker_main, s);
	*out = s;
	return BEEP_OK;
}

BEEP_API beep_status beep_server_destroy(beep_server *s)
{
	if (!s) return BEEP_OK;
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_work.notify_all();
	if (s->worker.joinable()) s->worker.join();
	for (Req *r : s->graveyard) release_request_memory(r);
	for (auto &kv : s->reqs) {
		release_request_memory(kv.second);
		delete kv.second;
	}
	if (s->ev0) cudaEventDestroy(s->ev0);
	if (s->st0) cudaStreamDestroy(s->st0);
	delete s;
	return BEEP_OK;
}

BEEP_API beep_status beep_serve_submit(beep_server *s, const beep_request *rq, uint64_t *ticket)
{
	if (!s || !rq || !rq->model || !ticket) return fail(BEEP_BAD_INPUT, "null argument");
	if (rq->kind < BEEP_REQ_LIKELIHOOD || rq->kind > BEEP_REQ_PF_LIKELIHOOD) return fail(BEEP_BAD_INPUT, "unknown request kind");
	if (rq->model->narea <= 0 || rq->model->ndivision <= 0 || !rq->model->M_rowptr)
		return fail(BEEP_BAD_INPUT, "bad model description");
	if (rq->kind == BEEP_REQ_PF_LIKELIHOOD) {
		if (!rq->pf || !rq->pf->tables || rq->pf->nparticle <= 0 || rq->pf->nsection <= 0 || !rq->pf->loglik_out)
			return fail(BEEP_BAD_INPUT, "a particle-filter request needs tables, particles, sections and loglik_out");
		Req *r = new Req();
		r->kind = rq->kind;
		r->desc = *rq->model;
		r->pf = *rq->pf;
		r->est = estimate_pf_bytes(r->desc, r->pf);
		{
			std::lock_guard<std::mutex> lk(s->mu);
			if (s->stop) {
				delete r;
				return fail(BEEP_BAD_INPUT, "the server is shutting down");
			}
			r->id = s->next_id++;
			r->t_submit = s->now();
			s->reqs[r->id] = r;
			s->queue.push_back(r);
			*ticket = r->id;
		}
		s->cv_work.notify_all();
		return BEEP_OK;
	}
	if (!rq->batch) return fail(BEEP_BAD_INPUT, "the request needs a batch");
	const beep_sim_batch &b = *rq->batch;
	if (b.nparticle <= 0 || b.ngroup <= 0 || !b.groups || b.ti < 0 || b.tf <= b.ti)
		return fail(BEEP_BAD_INPUT, "nparticle, groups and a step range are required");
	if (rq->kind == BEEP_REQ_LIKELIHOOD && !b.L_out) return fail(BEEP_BAD_INPUT, "a likelihood request needs L_out");
	if (rq->kind == BEEP_REQ_PREDICTION && (b.ti == 0 || (!b.pop_in && !b.pop_in_f64)))
		return fail(BEEP_BAD_INPUT, "a prediction request continues given populations from ti > 0");
	Req *r = new Req();
	r->kind = rq->kind;
	r->desc = *rq->model;
	r->batch = b;
	r->est = estimate_bytes(r->desc, r->batch);
	{
		std::lock_guard<std::mutex> lk(s->mu);
		if (s->stop) {
			delete r;
			return fail(BEEP_BAD_INPUT, "the server is shutting down");
		}
		r->id = s->next_id++;
		r->t_submit = s->now();
		s->reqs[r->id] = r;
		s->queue.push_back(r);
		*ticket = r->id;
	}
	s->cv_work.notify_all();
	return BEEP_OK;
}

BEEP_API beep_status beep_serve_poll(beep_server *s, uint64_t ticket, int32_t *done)
{
	if (!s || !done) return fail(BEEP_BAD_INPUT, "null argument");
	std::lock_guard<std::mutex> lk(s->mu);
	Req *r = find(s, ticket);
	if (!r) return fail(BEEP_BAD_INPUT, "unknown ticket");
	*done = r->state == 2 ? 1 : 0;
	if (r->state == 2 && r->status != BEEP_OK) return fail(r->status, r->err);
	return BEEP_OK;
}

BEEP_API beep_status beep_serve_wait(beep_server *s, uint64_t ticket, double timeout_s)
{
	if (!s) return fail(BEEP_BAD_INPUT, "null server");
	std::unique_lock<std::mutex> lk(s->mu);
	Req *r = find(s, ticket);
	if (!r) return fail(BEEP_BAD_INPUT, "unknown ticket");
	auto ready = [&] { return r->state == 2; };
	if (timeout_s < 0) s->cv_done.wait(lk, ready);
	else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready))
		return fail(BEEP_TIMEOUT, "request still running");
	if (r->status != BEEP_OK) return fail(r->status, r->err);
	return BEEP_OK;
}

BEEP_API beep_status beep_serve_stats(beep_server *s, uint64_t ticket, beep_request_stats *out)
{
	if (!s || !out) return fail(BEEP_BAD_INPUT, "null argument");
	std::lock_guard<std::mutex> lk(s->mu);
	Req *r = find(s, ticket);
	if (!r) return fail(BEEP_BAD_INPUT, "unknown ticket");
	out->submit_s = r->t_submit;
	out->admit_s = r->t_admit;
	out->done_s = r->t_done;
	out->gpu_start_s = r->g_start;
	out->gpu_end_s = r->g_end;
	out->device_bytes = (int64_t)(r->state == 0 ? r->est : r->bytes);
	out->state = r->state;
	out->status = r->status;
	return BEEP_OK;
}

BEEP_API beep_status beep_serve_release(beep_server *s, uint64_t ticket)
{
	if (!s) return fail(BEEP_BAD_INPUT, "null server");
	std::lock_guard<std::mutex> lk(s->mu);
	Req *r = find(s, ticket);
	if (!r) return fail(BEEP_BAD_INPUT, "unknown ticket");
	if (r->state != 2) return fail(BEEP_BAD_INPUT, "the request has not finished");
	if (std::find(s->graveyard.begin(), s->graveyard.end(), r) != s->graveyard.end())
		return BEEP_OK;   // its memory is released later; the record stays until then
	s->reqs.erase(ticket);
	delete r;
	return BEEP_OK;
}

}  // extern "C"
