// beep_simulate_plain_noalloc: the plain FP64 simulation for callers that must
// not allocate device memory.
//
// Who needs it: a host application that owns every byte of device memory
// through its own allocator or a fixed memory budget (an embedding framework
// with a memory pool, a service that pre-reserves HBM at start-up), where a
// cudaMalloc by a library would fail or take memory the pool counts on.  Such a
// caller allocates the inputs and outputs itself and passes device pointers;
// the kernel's working memory (per-particle populations, counts, infectivity
// maps, observation sums, the packed tables and observation lists) comes from
// one file-scope device array of fixed size, kNoAllocScratchBytes, which every
// GPU that loads this library holds until the process exits.
//
// The array's name is, on the host, only a stand-in for the device object: its
// device address is looked up with cudaGetSymbolAddress, once per device, the
// first time this entry point runs with that device current (so the first call
// on each device should come before any stream capture).  Every call uses the
// same array, which keeps the previous call's contents: the regions that must
// start at zero are cleared by each call, and two calls whose work overlaps on
// the GPU (for example on different streams) race on the array.  The call is
// synchronous: it reads the caller's index tables on the host (in order on the
// caller's stream) and returns once its kernel finished, on every path.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "capi_internal.h"

namespace beep {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;   // 64 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void *g_noalloc_addr[64] = {nullptr};   // device address of the array, per device ordinal

}  // namespace
}  // namespace beep

using namespace beep;

extern "C" BEEP_API beep_status beep_simulate_plain_noalloc(beep_model *m, const beep_param_tables *tab,
                                                             int32_t nparticle, uint64_t seed, int32_t ti,
                                                             int32_t tf, const int32_t *pop_in, double *L_out,
                                                             int32_t *pop_out, void *stream)
{
	if (!m || !tab) return fail(BEEP_BAD_INPUT, "null argument");
	if (nparticle <= 0) return fail(BEEP_BAD_INPUT, "nparticle must be positive");
	if (ti < 0 || tf <= ti || tf > m->S) return fail(BEEP_BAD_INPUT, "step range must satisfy 0 <= ti < tf <= ndivision");
	if (ti > 0 && !pop_in) return fail(BEEP_BAD_INPUT, "pop_in is required when ti > 0");
	if (tab->efoi_mult || tab->transmean_mult)
		return fail(BEEP_BAD_INPUT, "prediction multipliers are not taken by the allocation-free entry point");
	if (m->pop64)
		return fail(BEEP_BAD_INPUT, "models with demographic changes (FP64 populations) are not taken by the allocation-free entry point");
	if (!tab->transrate || !tab->susceptibility || !tab->infectivity || !tab->beta_rows || !tab->beta_row_of ||
	    !tab->areafactor || !tab->Ntime || !tab->geo_spline || !tab->efoi_spline || !tab->efoi_agedist || !tab->efoi_ref)
		return fail(BEEP_BAD_INPUT, "missing table");
	if (tab->nbeta_row <= 0 || tab->nefoi <= 0 || tab->nobs_spline < 0 || m->max_obs_spline >= tab->nobs_spline)
		return fail(BEEP_BAD_INPUT, "bad table counts");
	std::lock_guard<std::mutex> lock(g_noalloc_mu);
	int dev = 0;
	CUDA_TRY(cudaGetDevice(&dev));
	if (dev != m->device) return fail(BEEP_BAD_INPUT, "the current device is not the model's device");
	if (dev < 0 || dev >= 64) return fail(BEEP_BAD_INPUT, "device ordinal out of range");
	if (!g_noalloc_addr[dev]) {
		void *p = nullptr;
		CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
		g_noalloc_addr[dev] = p;
	}
	char *base = (char *)g_noalloc_addr[dev];
	cudaStream_t st = (cudaStream_t)stream;
	// Every return from here on waits for the work this call enqueued, so that no
	// copy into the shared array is still in flight when the next call takes the lock.
	struct StreamDrain {
		cudaStream_t s;
		~StreamDrain() { cudaStreamSynchronize(s); }
	} drain{st};

	const size_t A = m->A, G = m->G, DP = m->DP, NS = m->NS, C = m->C, T = m->T, S = m->S;
	const size_t P = (size_t)nparticle, popsz = A * C * DP, tnsz = A * T * DP, agsz = NS * A * G;
	// the index tables are read on the host to check their ranges (the kernel indexes
	// with them); the reads are ordered on the caller's stream, behind whatever work
	// of the caller's fills the tables there, and complete before the check
	std::vector<int32_t> brow(NS * A), eref(NS * A);
	std::vector<double> inf(C);
	CUDA_TRY(cudaMemcpyAsync(brow.data(), tab->beta_row_of, 4 * NS * A, cudaMemcpyDeviceToHost, st));
	CUDA_TRY(cudaMemcpyAsync(eref.data(), tab->efoi_ref, 4 * NS * A, cudaMemcpyDeviceToHost, st));
	CUDA_TRY(cudaMemcpyAsync(inf.data(), tab->infectivity, 8 * C, cudaMemcpyDeviceToHost, st));
	CUDA_TRY(cudaStreamSynchronize(st));
	for (size_t k = 0; k < NS * A; k++) {
		if (brow[k] < 0 || brow[k] >= tab->nbeta_row) return fail(BEEP_BAD_INPUT, "beta_row_of out of range");
		if (eref[k] < 0 || eref[k] >= tab->nefoi) return fail(BEEP_BAD_INPUT, "efoi_ref out of range");
	}
	ObsLists ol;
	build_obs_lists(m->obs_sett_i.data(), m->obs_sett_f.data(), m->nobs, ti, tf, ol);
	const size_t nscored = ol.scored.size();

	// table pool: the caller's tables copied device-to-device, in the packed
	// layout the kernel addresses through one GroupDir
	GroupDir dir{};
	size_t nf = 0;
	auto fslot = [&](size_t n) { int64_t o = (int64_t)nf; nf += align_up(n, 4); return o; };
	dir.transrate = fslot(T * DP);
	dir.susceptibility = fslot(DP);
	dir.infectivity = fslot(C);
	dir.infdif = fslot(T);
	dir.beta_rows = fslot((size_t)tab->nbeta_row * S);
	dir.areafactor = fslot((size_t)m->period * A);
	dir.Ntime = fslot(S * G * G);
	dir.geo_spline = fslot(S);
	dir.efoi_spline = fslot((size_t)tab->nefoi * S);
	dir.efoi_agedist = fslot((size_t)tab->nefoi * G);
	dir.obs_spline = fslot((size_t)tab->nobs_spline * S);
	dir.efoi_mult = -1;
	dir.tm_mult = -1;
	dir.beta_row_of = 0;
	dir.efoi_ref = (int64_t)align_up(NS * A, 8);
	const size_t ni = (size_t)dir.efoi_ref + NS * A;

	Layout L;
	const size_t o_dir = L.add(sizeof(GroupDir)), o_f = L.add(8 * nf), o_i = L.add(4 * ni), o_sc = L.add(4 * nscored),
	             o_sp = L.add(4 * ol.step_ptr.size()), o_so = L.add(4 * ol.step_obs.size()),
	             o_pa = L.add(4 * popsz * P), o_pb = L.add(4 * popsz * P), o_tn = L.add(4 * tnsz * P),
	             o_im = L.add(8 * agsz * P), o_id = L.add(8 * agsz * P), o_di = L.add(8 * agsz * P),
	             o_nmi = L.add(8 * agsz * P), o_acc = L.add(8 * nscored * P), o_st = L.add(4 * P);
	if (L.size > kNoAllocScratchBytes)
		return fail(BEEP_BAD_INPUT, "batch needs " + std::to_string(L.size) + " bytes of working memory; the no-alloc entry point has " +
		                                std::to_string(kNoAllocScratchBytes) + " (use fewer particles per call)");

	std::vector<double> infdif(T);
	for (size_t tr = 0; tr < T; tr++) infdif[tr] = inf[m->trans_to_h[tr]] - inf[m->trans_from_h[tr]];
	double *fp = (double *)(base + o_f);
	int32_t *ip = (int32_t *)(base + o_i);
	auto d2d = [&](void *dst, const void *src, size_t bytes) {
		return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st) : cudaSuccess;
	};
	CUDA_TRY(cudaMemcpyAsync(base + o_dir, &dir, sizeof dir, cudaMemcpyHostToDevice, st));
	CUDA_TRY(d2d(fp + dir.transrate, tab->transrate, 8 * T * DP));
	CUDA_TRY(d2d(fp + dir.susceptibility, tab->susceptibility, 8 * DP));
	CUDA_TRY(d2d(fp + dir.infectivity, tab->infectivity, 8 * C));
	CUDA_TRY(cudaMemcpyAsync(fp + dir.infdif, infdif.data(), 8 * T, cudaMemcpyHostToDevice, st));
	CUDA_TRY(d2d(fp + dir.beta_rows, tab->beta_rows, 8 * (size_t)tab->nbeta_row * S));
	CUDA_TRY(d2d(fp + dir.areafactor, tab->areafactor, 8 * (size_t)m->period * A));
	CUDA_TRY(d2d(fp + dir.Ntime, tab->Ntime, 8 * S * G * G));
	CUDA_TRY(d2d(fp + dir.geo_spline, tab->geo_spline, 8 * S));
	CUDA_TRY(d2d(fp + dir.efoi_spline, tab->efoi_spline, 8 * (size_t)tab->nefoi * S));
	CUDA_TRY(d2d(fp + dir.efoi_agedist, tab->efoi_agedist, 8 * (size_t)tab->nefoi * G));
	if (tab->nobs_spline > 0) CUDA_TRY(d2d(fp + dir.obs_spline, tab->obs_spline, 8 * (size_t)tab->nobs_spline * S));
	CUDA_TRY(d2d(ip + dir.beta_row_of, tab->beta_row_of, 4 * NS * A));
	CUDA_TRY(d2d(ip + dir.efoi_ref, tab->efoi_ref, 4 * NS * A));
	if (nscored) CUDA_TRY(cudaMemcpyAsync(base + o_sc, ol.scored.data(), 4 * nscored, cudaMemcpyHostToDevice, st));
	CUDA_TRY(cudaMemcpyAsync(base + o_sp, ol.step_ptr.data(), 4 * ol.step_ptr.size(), cudaMemcpyHostToDevice, st));
	if (!ol.step_obs.empty())
		CUDA_TRY(cudaMemcpyAsync(base + o_so, ol.step_obs.data(), 4 * ol.step_obs.size(), cudaMemcpyHostToDevice, st));
	CUDA_TRY(cudaMemsetAsync(base + o_st, 0, 4 * P, st));   // the previous call's statuses

	BatchDev bd{};
	bd.P = (int32_t)P; bd.ti = ti; bd.tf = tf; bd.ngroup = 1;
	bd.k0 = (uint32_t)seed; bd.k1 = (uint32_t)(seed >> 32);
	bd.dirs = (const GroupDir *)(base + o_dir);
	bd.fpool = fp;
	bd.ipool = ip;
	bd.pop_in = ti > 0 ? pop_in : nullptr;
	bd.nscored = (int32_t)nscored;
	bd.scored = (const int32_t *)(base + o_sc);
	bd.step_ptr = (const int32_t *)(base + o_sp);
	bd.step_obs = (const int32_t *)(base + o_so);
	bd.pop_a = (int32_t *)(base + o_pa); bd.pop_b = (int32_t *)(base + o_pb); bd.tn = (int32_t *)(base + o_tn);
	bd.Imap = (double *)(base + o_im); bd.Idiag = (double *)(base + o_id); bd.dinf = (double *)(base + o_di);
	bd.NMI = (double *)(base + o_nmi); bd.obs_acc = (double *)(base + o_acc);
	bd.status = (int32_t *)(base + o_st);
	bd.L = L_out;
	bd.pop_out = pop_out;
	int le = launch_sim_plain(m->dev, bd, st);
	if (le != 0) return fail(BEEP_DEVICE_ERROR, std::string("kernel launch: ") + cudaGetErrorString((cudaError_t)le));
	std::vector<int32_t> status(P);
	CUDA_TRY(cudaMemcpyAsync(status.data(), base + o_st, 4 * P, cudaMemcpyDeviceToHost, st));
	CUDA_TRY(cudaStreamSynchronize(st));
	for (size_t p = 0; p < P; p++)
		if (status[p] != 0) return fail((beep_status)status[p], "particle " + std::to_string(p) + " failed on the device");
	return BEEP_OK;
}
