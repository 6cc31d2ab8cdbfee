// beep_pf_loglik: the bootstrap particle filter of PMCMC on the device
// (PMCMC::obs_prob + bootstrap, src/pmcmc.cc:180-268; Mpi::end_sec_swap,
// src/mpi.cc:215-327).
//
// Per filter section, on the model's stream with no host round trip:
//   1. the simulation kernel (plain or fast form) advances every particle slot
//      from its carried population and writes the section log-likelihood L;
//   2. pf_bootstrap (one CTA) forms w = exp(invT (L - Lmax)), the cumulative
//      sums in slot order, the section's term invT Lmax + log(sum w / N), and the
//      ancestors: N uniforms (word 0 of Philox({j, section, stream, RESAMPLE})),
//      each located in the cumulative sums, then the reference's placement
//      (a selected particle keeps its own slot, the other slots take the
//      surplus selections last-in first-out);
//   3. pf_gather copies each slot's population from its ancestor's.
// With a lineage request every section also writes its slots' transition
// counts, and the sampled particle's trajectory is assembled by walking the
// ancestors back (Mpi::particle_sample, src/mpi.cc:331-389).
// The cumulative sums and the placement are sequential in slot order, as in
// the reference, so the ancestors match it exactly (the FP64 weights of the
// plain form agree with the reference's to the last bits).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "rng_fp64.cuh"

namespace beep {
namespace {

constexpr int kBootThreads = 1024;
constexpr int kBootSmemN = 8192;   // particles whose cumulative sums and placement fit shared memory

// The sequential parts (cumulative sums, placement) read and write one slot after another:
// their arrays are in shared memory for N <= kBootSmemN (launched with 16 N bytes of dynamic
// shared memory), where a load after a store to another slot does not wait for global
// memory; larger filters use the global scratch arrays.
__global__ void __launch_bounds__(kBootThreads) pf_bootstrap(const double *L, int N, double invT, uint32_t k0,
                                                            uint32_t k1, uint32_t rstream, int sec, double *w,
                                                            double *wsum_g, int32_t *sel, int32_t *bp_g,
                                                            int32_t *extra_g, double *ob_sec, int32_t *anc,
                                                            int32_t *status)
{
	extern __shared__ __align__(16) unsigned char boot_smem[];
	__shared__ double red[kBootThreads];
	__shared__ double s_sum;
	const bool sm = N <= kBootSmemN;
	double *wsum = sm ? (double *)boot_smem : wsum_g;
	int32_t *bp = sm ? (int32_t *)(boot_smem + 8 * (size_t)N) : bp_g;
	int32_t *extra = sm ? (int32_t *)(boot_smem + 12 * (size_t)N) : extra_g;
	const int tid = threadIdx.x;
	double mx = -1000000000.0;                       // -LARGE, src/pmcmc.cc:223
	for (int p = tid; p < N; p += kBootThreads) mx = fmax(mx, L[p]);
	red[tid] = mx;
	__syncthreads();
	for (int o = kBootThreads / 2; o > 0; o >>= 1) {
		if (tid < o) red[tid] = fmax(red[tid], red[tid + o]);
		__syncthreads();
	}
	const double Lmax = red[0];
	for (int p = tid; p < N; p += kBootThreads) w[p] = exp(invT * (L[p] - Lmax));
	__syncthreads();
	if (tid == 0) {
		double sum = 0.0;
		for (int p = 0; p < N; p++) {
			sum += w[p];
			wsum[p] = sum;
		}
		s_sum = sum;
		ob_sec[sec] = invT * Lmax + log(sum / N);
	}
	__syncthreads();
	const double sum = s_sum;
	for (int j = tid; j < N; j += kBootThreads) {
		const U4 r = philox10(U4{(uint32_t)j, (uint32_t)sec, rstream, PURPOSE_RESAMPLE << 24}, k0, k1);
		const double z = u01_d(r.x) * sum;
		int lo = 0, hi = N;                          // first slot with wsum >= z
		while (lo < hi) {
			const int mid = (lo + hi) >> 1;
			if (z > wsum[mid]) lo = mid + 1;
			else hi = mid;
		}
		if (lo == N) { atomicCAS(status, 0, BEEP_NAN_RATE); lo = N - 1; }
		sel[j] = lo;
	}
	__syncthreads();
	if (tid == 0) {
		for (int p = 0; p < N; p++) bp[p] = -1;
		int ne = 0;
		for (int j = 0; j < N; j++) {
			const int pp = sel[j];
			if (bp[pp] == -1) bp[pp] = pp;
			else extra[ne++] = pp;
		}
		for (int p = 0; p < N; p++)
			if (bp[p] == -1) bp[p] = extra[--ne];
	}
	__syncthreads();
	for (int p = tid; p < N; p += kBootThreads) {
		if (sm) bp_g[p] = bp[p];
		if (anc) anc[p] = bp[p];
	}
}

__global__ void pf_gather(int32_t *dst, const int32_t *src, const int32_t *bp, int N, int popsz)
{
	const size_t n = (size_t)N * popsz;
	for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
		const size_t p = k / popsz, i = k % popsz;
		dst[k] = src[(size_t)bp[p] * popsz + i];
	}
}

}  // namespace
}  // namespace beep

using namespace beep;

extern "C" BEEP_API beep_status beep_pf_loglik(beep_model *m, const beep_pf_request *r)
{
	if (!m || !r || !r->tables) return fail(BEEP_BAD_INPUT, "null argument");
	const int N = r->nparticle, ns = r->nsection;
	if (N <= 0 || ns <= 0 || !r->section_ti || !r->section_tf || !r->loglik_out)
		return fail(BEEP_BAD_INPUT, "nparticle, sections and loglik_out are required");
	if (r->section_ti[0] != 0 || r->section_tf[ns - 1] != m->S)
		return fail(BEEP_BAD_INPUT, "sections must cover [0, ndivision)");
	for (int k = 0; k < ns; k++) {
		if (r->section_tf[k] <= r->section_ti[k]) return fail(BEEP_BAD_INPUT, "empty section");
		if (k > 0 && r->section_ti[k] != r->section_tf[k - 1]) return fail(BEEP_BAD_INPUT, "sections must be contiguous");
	}
	std::lock_guard<std::mutex> lock(m->mu);
	CUDA_TRY(cudaSetDevice(m->device));
	// populations as 32-bit words: one per population, or two (FP64 populations of a
	// model with demographic changes)
	const size_t popsz = (size_t)m->A * m->C * m->DP * (m->pop64 ? 2 : 1);
	cudaStream_t st = m->stream;

	// one prepared batch per section, kept on the model for later calls of the same
	// shape (then only the tables are staged again and the keys changed)
	const bool lineage = r->lineage_transnum_out != nullptr;
	beep_model::PfCache &pc = m->pf;
	auto drop_cache = [&]() {
		for (auto *x : pc.q) beep_batch_destroy(x);
		pc.q.clear();
		pc.N = 0;
		pc.form = -1;
	};
	const bool same = pc.N == N && pc.form == r->form && pc.lineage == lineage && (int)pc.q.size() == ns &&
	                  std::equal(pc.ti.begin(), pc.ti.end(), r->section_ti) &&
	                  std::equal(pc.tf.begin(), pc.tf.end(), r->section_tf);
	if (!same) {
		drop_cache();
		pc.q.assign(ns, nullptr);
		for (int k = 0; k < ns; k++) {
			beep_sim_batch b{};
			b.nparticle = N; b.ngroup = 1; b.groups = r->tables; b.seed = r->seed;
			b.ti = r->section_ti[k]; b.tf = r->section_tf[k];
			b.form = r->form;
			beep_status s = batch_create_internal(m, &b, true, &pc.q[k], lineage);
			if (s != BEEP_OK) { std::string e = beep_last_error(); drop_cache(); return fail(s, e); }
		}
		pc.N = N;
		pc.form = r->form;
		pc.lineage = lineage;
		pc.ti.assign(r->section_ti, r->section_ti + ns);
		pc.tf.assign(r->section_tf, r->section_tf + ns);
	} else {
		for (int k = 0; k < ns; k++) {
			beep_batch *b = pc.q[k];
			b->b.groups = r->tables;
			b->b.seed = r->seed;
			b->bd.k0 = (uint32_t)r->seed;
			b->bd.k1 = (uint32_t)(r->seed >> 32);
			beep_status s = beep_batch_stage(b);
			if (s != BEEP_OK) { std::string e = beep_last_error(); drop_cache(); return fail(s, e); }
		}
	}
	std::vector<beep_batch *> &q = pc.q;
	const size_t tnsz = (size_t)m->A * m->T * m->DP;
	Layout L;
	const size_t o_tn = L.add(lineage ? 4 * tnsz * (size_t)m->S * N : 0);
	const size_t o_pa = L.add(4 * popsz * N), o_pb = L.add(4 * popsz * N), o_L = L.add(8 * (size_t)ns * N),
	             o_w = L.add(8 * (size_t)N), o_ws = L.add(8 * (size_t)N), o_sel = L.add(4 * (size_t)N),
	             o_bp = L.add(4 * (size_t)N), o_ex = L.add(4 * (size_t)N), o_ob = L.add(8 * (size_t)ns),
	             o_anc = L.add(4 * (size_t)ns * N), o_st = L.add(4), o_pst = L.add(4 * (size_t)ns * N);
	cudaError_t e = pc.work.reserve(L.size);
	if (e != cudaSuccess) { drop_cache(); return fail(BEEP_OOM, std::string("particle filter buffers: ") + cudaGetErrorString(e)); }
	char *d = (char *)pc.work.ptr;
	int32_t *popA = (int32_t *)(d + o_pa), *popB = (int32_t *)(d + o_pb);
	double *Lall = (double *)(d + o_L), *obsec = (double *)(d + o_ob);
	int32_t *anc = (int32_t *)(d + o_anc), *pst = (int32_t *)(d + o_st), *secst = (int32_t *)(d + o_pst);
	beep_status status = BEEP_OK;
	std::string err;
	auto bail = [&](beep_status s, const std::string &msg) { status = s; err = msg; };
	if (cudaMemsetAsync(pst, 0, 4, st) != cudaSuccess) bail(BEEP_DEVICE_ERROR, "memset");
	// the bootstrap's cumulative sums and placement in shared memory (16 N bytes) where they fit
	const size_t boot_smem = N <= kBootSmemN ? 16 * (size_t)N : 0;
	if (status == BEEP_OK && allow_dynamic_smem(pf_bootstrap, boot_smem) != cudaSuccess)
		bail(BEEP_DEVICE_ERROR, "bootstrap shared memory");
	for (int k = 0; k < ns && status == BEEP_OK; k++) {
		beep_batch *b = q[k];
		if (beep_batch_upload(b) != BEEP_OK) { bail(BEEP_DEVICE_ERROR, beep_last_error()); break; }
		b->bd.pop_in = k > 0 ? popA : nullptr;
		b->bd.pop_out = popB;
		b->bd.L = Lall + (size_t)k * N;
		// section k's counts of every slot: [slot][step - ti][cell] at N * ti cells in
		if (lineage) b->bd.tn_traj = (int32_t *)(d + o_tn) + (size_t)N * r->section_ti[k] * tnsz;
		if (beep_batch_launch(b) != BEEP_OK) { bail(BEEP_DEVICE_ERROR, beep_last_error()); break; }
		pf_bootstrap<<<1, kBootThreads, boot_smem, st>>>(Lall + (size_t)k * N, N, r->invT, (uint32_t)r->seed,
		                                         (uint32_t)(r->seed >> 32), r->resample_stream, k,
		                                         (double *)(d + o_w), (double *)(d + o_ws), (int32_t *)(d + o_sel),
		                                         (int32_t *)(d + o_bp), (int32_t *)(d + o_ex), obsec,
		                                         anc + (size_t)k * N, pst);
		if (k + 1 < ns) pf_gather<<<152 * 4, 256, 0, st>>>(popA, popB, (const int32_t *)(d + o_bp), N, (int)popsz);
		if (cudaGetLastError() != cudaSuccess) bail(BEEP_DEVICE_ERROR, "bootstrap launch");
		// the section's per-particle statuses, gathered for one copy at the end
		if (cudaMemcpyAsync(secst + (size_t)k * N, b->bd.status, 4 * (size_t)N, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
			bail(BEEP_DEVICE_ERROR, "status gather");
	}
	std::vector<double> ob(ns);
	std::vector<int32_t> ps((size_t)ns * N);
	int32_t bst = 0;
	if (status == BEEP_OK) {
		e = cudaMemcpyAsync(ob.data(), obsec, 8 * (size_t)ns, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(ps.data(), secst, 4 * (size_t)ns * N, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaMemcpyAsync(&bst, pst, 4, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess && r->L_out) e = cudaMemcpyAsync(r->L_out, Lall, 8 * (size_t)ns * N, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess && r->ancestors_out)
			e = cudaMemcpyAsync(r->ancestors_out, anc, 4 * (size_t)ns * N, cudaMemcpyDeviceToHost, st);
		if (e == cudaSuccess) e = cudaStreamSynchronize(st);
		if (e != cudaSuccess) bail(BEEP_DEVICE_ERROR, cudaGetErrorString(e));
	}
	// per-particle statuses of the simulation launches
	for (int k = 0; k < ns && status == BEEP_OK; k++)
		for (int p = 0; p < N; p++)
			if (ps[(size_t)k * N + p] != 0) {
				bail((beep_status)ps[(size_t)k * N + p], "section " + std::to_string(k) + " particle " + std::to_string(p));
				break;
			}
	if (status == BEEP_OK && bst != 0) bail((beep_status)bst, "resampling found no particle (non-finite weights)");
	if (status == BEEP_OK && lineage) {
		// Mpi::particle_sample: start from the particle the last resampling put in slot
		// 0 and walk the ancestors back, copying each section from the slot its
		// ancestor held then
		std::vector<int32_t> a((size_t)ns * N);
		e = cudaMemcpy(a.data(), anc, 4 * (size_t)ns * N, cudaMemcpyDeviceToHost);
		int32_t pcur = a[(size_t)(ns - 1) * N + 0];
		for (int k = ns - 1; k >= 0 && e == cudaSuccess; k--) {
			const int ti = r->section_ti[k], nst = r->section_tf[k] - ti;
			const int32_t *src = (int32_t *)(d + o_tn) + ((size_t)N * ti + (size_t)pcur * nst) * tnsz;
			e = cudaMemcpy(r->lineage_transnum_out + (size_t)ti * tnsz, src, 4 * (size_t)nst * tnsz, cudaMemcpyDeviceToHost);
			if (k > 0) pcur = a[(size_t)(k - 1) * N + pcur];
		}
		if (e != cudaSuccess) bail(BEEP_DEVICE_ERROR, std::string("lineage copy: ") + cudaGetErrorString(e));
	}
	cudaStreamSynchronize(st);
	if (status != BEEP_OK) {
		drop_cache();
		return fail(status, err);
	}
	double total = 0.0;
	for (int k = 0; k < ns; k++) total += ob[k];
	*r->loglik_out = total;
	if (r->loglik_section_out) memcpy(r->loglik_section_out, ob.data(), 8 * (size_t)ns);
	return BEEP_OK;
}
