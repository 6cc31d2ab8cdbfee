// MBP chains in the fast (mixed-precision) form: the fast kernel's chain
// variants (sim_fast.cuh with CH = true), compiled in their own translation
// unit.  A chain's two states hold, per step, the transition counts (int32)
// and means (FP32) of every column, [slot][chain][step][transition][column];
// the force of infection is formed from the counts every step, so Imap is not
// stored (INF_UPDATE and INF_DIF_UPDATE give the same map here).
#include "sim_fast.cuh"

namespace beep {

int fast_chain_prepare()
{
	const int e = prepare_constants();
	return e != 0 ? e : fast_chain_ctas_prepare();
}

namespace {

template <int NT>
int launch_chain_nt(const ModelDev &m, const BatchDev &b, size_t smem, cudaStream_t st)
{
	auto kern = m.G <= 4 ? sim_fast_kernel<NT, 4, false, true> : m.G <= 8 ? sim_fast_kernel<NT, 8, false, true>
	          : m.G <= 12 ? sim_fast_kernel<NT, 12, false, true> : sim_fast_kernel<NT, 16, false, true>;
	cudaError_t e = allow_dynamic_smem(kern, smem);
	if (e != cudaSuccess) return (int)e;
	kern<<<b.P, NT, smem, st>>>(m, b);
	return (int)cudaGetLastError();
}

}  // namespace

int launch_sim_fast_chain(const ModelDev &m, const BatchDev &b, void *stream)
{
	if (m.G > 16 || m.T > kMaxT || b.foi_tc || !b.ch_tn || !b.ch_mean_f) return (int)cudaErrorInvalidValue;
	const int nt = b.nt > 0 ? b.nt : fast_pick_threads(m);
	const size_t smem = fast_smem_bytes(m, b.nslots, b.m_in_smem != 0, b.nefoi_stage, b.gstate != nullptr,
	                                    b.tn_full ? m.T : m.tn_rows, b.pop_single != 0, b.tn_smem != 0, nt);
	if (nt == kDualThreads) return launch_sim_fast_chain_ctas(m, b, smem, stream);
	if (nt != fast_pick_threads(m)) return (int)cudaErrorInvalidValue;
	const int e = prepare_constants();
	if (e != 0) return e;
	cudaStream_t st = (cudaStream_t)stream;
	return nt == 128 ? launch_chain_nt<128>(m, b, smem, st) : nt == 256 ? launch_chain_nt<256>(m, b, smem, st)
	                                                                     : launch_chain_nt<640>(m, b, smem, st);
}

}  // namespace beep
