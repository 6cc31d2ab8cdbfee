// Host-side definitions shared by the C-ABI translation units: error text,
// growable device/host buffers, buffer layouts and the model handle.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "beep_internal.h"

namespace beep {

// Records the message returned by beep_last_error() on this thread.
beep_status fail(beep_status s, const std::string &msg);

#define CUDA_TRY(expr)                                                                         \
	do {                                                                                       \
		cudaError_t e_ = (expr);                                                               \
		if (e_ != cudaSuccess)                                                                 \
			return ::beep::fail(e_ == cudaErrorMemoryAllocation ? BEEP_OOM : BEEP_DEVICE_ERROR, \
			                    std::string(#expr) + ": " + cudaGetErrorString(e_));           \
	} while (0)

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// A device buffer that only grows.
struct DevBuf {
	void *ptr = nullptr;
	size_t cap = 0;
	cudaError_t reserve(size_t n)
	{
		if (n <= cap) return cudaSuccess;
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		cap = 0;
		cudaError_t e = cudaMalloc(&ptr, n);
		if (e == cudaSuccess) cap = n;
		return e;
	}
	void release()
	{
		if (ptr) cudaFree(ptr);
		ptr = nullptr;
		cap = 0;
	}
};

// A pinned host buffer that only grows.
struct HostBuf {
	void *ptr = nullptr;
	size_t cap = 0;
	cudaError_t reserve(size_t n)
	{
		if (n <= cap) return cudaSuccess;
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		cap = 0;
		cudaError_t e = cudaMallocHost(&ptr, n);
		if (e == cudaSuccess) cap = n;
		return e;
	}
	void release()
	{
		if (ptr) cudaFreeHost(ptr);
		ptr = nullptr;
		cap = 0;
	}
};

// Sequential layout of named regions inside one buffer (256-byte aligned).
struct Layout {
	size_t size = 0;
	size_t add(size_t bytes)
	{
		size_t off = align_up(size, 256);
		size = off + bytes;
		return off;
	}
};

// Scored observations of a step range and the steps each is active in
// (positions into `scored`), as the kernels consume them.
struct ObsLists {
	std::vector<int32_t> scored, step_ptr, step_obs;
};
void build_obs_lists(const int32_t *sett_i, const int32_t *sett_f, int nobs, int ti, int tf, ObsLists &out);

}  // namespace beep

struct beep_model {
	int device = 0;
	int sms = 152;                // SMs of the device
	cudaStream_t stream = nullptr;
	beep::ModelDev dev{};
	beep::DevBuf model_mem;
	// host copies used to prepare batches
	int32_t A, G, DP, NS, C, T, S, period, dpt, nobs;
	std::vector<int32_t> obs_sett_i, obs_sett_f, obs_spline, trans_from_h, trans_to_h, obs_cell_ptr_h, obs_cells_f_h,
	    obs_cells_full_h;
	std::vector<float> obs_factor_f_h;
	int32_t max_obs_spline = -1;
	bool pop64 = false;           // demographic changes: populations are FP64 (plain form only)
	int32_t tuned_foi = 0;        // fast-form FOI path chosen by beep_autotune (0: none)
	int32_t tuned_ctas = 0;       // fast-form particles per SM chosen by beep_autotune (0: none)
	// beep_pf_loglik's prepared section batches and buffers, kept while later calls
	// have the same particles, sections, form and lineage request (PMCMC calls it
	// once per proposal with new tables only)
	struct PfCache {
		int32_t N = 0, form = -1;
		bool lineage = false;
		std::vector<int32_t> ti, tf;
		std::vector<beep_batch *> q;
		beep::DevBuf work;
	} pf;
	std::mutex mu;
};

// A prepared batch: the caller's host arrays (kept by pointer), pinned staging,
// device inputs, work and outputs, and the kernel's view of them.
struct beep_batch {
	bool device_io = false;   // pop_in / L / pop_out are device buffers set by an internal caller
	beep_model *m = nullptr;
	beep_sim_batch b{};
	beep::HostBuf in_host, out_host;
	beep::DevBuf in_dev, work_dev, out_dev;
	size_t in_size = 0, out_size = 0;
	size_t o_f = 0, u_st = 0, u_L = 0, u_po = 0, u_tn = 0, u_pt = 0;
	std::vector<beep::GroupDir> dirs;
	std::vector<uint2> keys;           // per-particle Philox keys (requests packed into one batch), or empty
	std::vector<int32_t> scored, step_ptr, step_obs, slot_of, tasks;
	beep::BatchDev bd{};
	cudaEvent_t ev0 = nullptr, ev1 = nullptr;
	bool pending = false;
	bool state_global = false;   // fast form keeps particle state in global memory
	std::vector<cudaEvent_t> ev_split;   // beep_batch_time_split: around each step's product kernel
	// CUDA graph of upload + status reset + kernel + download (beep_batch_run_graph)
	cudaGraph_t graph = nullptr;
	cudaGraphExec_t graph_exec = nullptr;
	size_t graph_in_size = 0;
};


namespace beep {
// beep_batch_create for internal callers whose start populations and outputs
// live on the device (device_io: pop_in is not read from the host and the
// caller sets bd.pop_in / bd.L / bd.pop_out before each launch).
// With device_traj the kernels write every step's transition counts to a
// device buffer the caller sets in bd.tn_traj ([P][tf-ti][A][T][DP]) before
// each launch.
// allow_tc = false keeps the fast form's force of infection on FP32 SIMT;
// allow_ctas = false keeps it at one particle per SM.
// keys (may be null): one Philox key per particle, for batches that pack the
// particles of requests with different seeds.
beep_status batch_create_internal(beep_model *m, const beep_sim_batch *b, bool device_io, beep_batch **out,
                                  bool device_traj = false, bool allow_tc = true, bool allow_ctas = true,
                                  const std::vector<uint2> *keys = nullptr);
// beep_batch_download in two halves: the device->host copy enqueued on the
// model's stream, and (once that copy completed) the status check and the
// copy into the caller's arrays.
beep_status batch_download_enqueue(beep_batch *q);
beep_status batch_download_finish(beep_batch *q);
// Device bytes held by a model / a batch.
size_t model_device_bytes(const beep_model *m);
size_t batch_device_bytes(const beep_batch *q);
}  // namespace beep
