// MBP chains of several models in ONE persistent launch (fast form).
//
// The chains of up to kMaxFusedSets chain sets -- each its own model, so of
// uneven area, age and horizon sizes -- are work items of a single grid of
// one 640-thread CTA per SM.  A CTA takes the next item from a device
// counter, finds its set in the launch descriptor (every set's ModelDev and
// BatchDev, passed as one __grid_constant__ kernel parameter) and runs that
// chain's coupled proposal with the fast kernel's chain variant
// (sim_fast.cuh, CH = true) over the model's whole horizon; then takes the
// next.  The sets are ordered by their chains' expected cost, largest first,
// so that the long chains start at once and the short ones fill the SMs as
// the long ones end (longest-processing-time-first list scheduling).
//
// Every chain draws from the same keyed variate streams as in its own set's
// launch, with the same arithmetic: the counts are those of beep_mbp_propose.
// Only the order in which a chain's observation log-densities are summed
// over the CTA's threads follows the thread count, so the log-likelihood of
// a set that runs on fewer threads alone can differ in its last FP32 bits.
#include "sim_fast.cuh"

namespace beep {
namespace {

constexpr int kFusedThreads = 640;

struct FusedChains {
	int32_t nset, nitem;
	int32_t *counter;                    // next work item (zero before the launch)
	int32_t first[kMaxFusedSets + 1];    // set k's chains are items [first[k], first[k+1])
	ModelDev m[kMaxFusedSets];
	BatchDev b[kMaxFusedSets];
};
// one kernel parameter: within the 32764 bytes a launch takes (CUDA 12.1 and later)
static_assert(sizeof(FusedChains) <= 32764, "the fused launch descriptor exceeds the kernel parameter limit");

template <int MG>
__global__ void __launch_bounds__(kFusedThreads, 1) sim_fast_fused_kernel(const __grid_constant__ FusedChains f)
{
	__shared__ int item;
	for (;;) {
		__syncthreads();                 // the previous chain is finished with shared memory
		if (threadIdx.x == 0) item = atomicAdd(f.counter, 1);
		__syncthreads();
		const int it = item;
		if (it >= f.nitem) break;
		int k = 0;
		while (k + 1 < f.nset && it >= f.first[k + 1]) k++;
		sim_fast_body<kFusedThreads, MG, false, true, kMaxT>(f.m[k], f.b[k], it - f.first[k]);
	}
}

}  // namespace

int fused_mg(const ModelDev *m, int n)
{
	int g = 0;
	for (int k = 0; k < n; k++) g = std::max(g, m[k].G);
	return (g + 3) & ~3;
}

bool fused_supported(const ModelDev &m) { return m.T <= kMaxT && m.G <= 16 && !fast_wide_needed(m); }

size_t fused_smem_bytes(const ModelDev &m, const BatchDev &b, int mg)
{
	return fast_smem_bytes(m, b.nslots, b.m_in_smem != 0, b.nefoi_stage, b.gstate != nullptr,
	                       b.tn_full ? m.T : m.tn_rows, b.pop_single != 0, b.tn_smem != 0, kFusedThreads, mg);
}

int launch_sim_fast_chain_fused(const ModelDev *m, const BatchDev *b, int n, int32_t *counter, int sms, void *stream)
{
	if (n <= 0 || n > kMaxFusedSets || !counter) return (int)cudaErrorInvalidValue;
	const int e0 = prepare_constants();
	if (e0 != 0) return e0;
	const int mg = fused_mg(m, n);
	FusedChains f{};
	f.nset = n;
	f.counter = counter;
	size_t smem = 0;
	for (int k = 0; k < n; k++) {
		if (!fused_supported(m[k]) || b[k].mode != 1 || b[k].foi_tc || b[k].batched || !b[k].ch_tn || !b[k].ch_mean_f)
			return (int)cudaErrorInvalidValue;
		f.m[k] = m[k];
		f.b[k] = b[k];
		f.first[k + 1] = f.first[k] + b[k].P;
		smem = std::max(smem, fused_smem_bytes(m[k], b[k], mg));
	}
	f.nitem = f.first[n];
	if (f.nitem == 0) return 0;
	auto kern = mg <= 4 ? sim_fast_fused_kernel<4> : mg <= 8 ? sim_fast_fused_kernel<8>
	          : mg <= 12 ? sim_fast_fused_kernel<12> : sim_fast_fused_kernel<16>;
	cudaError_t e = allow_dynamic_smem(kern, smem);
	if (e != cudaSuccess) return (int)e;
	cudaStream_t st = (cudaStream_t)stream;
	e = cudaMemsetAsync(counter, 0, sizeof(int32_t), st);
	if (e != cudaSuccess) return (int)e;
	kern<<<std::min(f.nitem, std::max(1, sms)), kFusedThreads, smem, st>>>(f);
	return (int)cudaGetLastError();
}

}  // namespace beep
