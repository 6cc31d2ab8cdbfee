// MBP chains in the fast form with several chains per SM: the chain variants
// of the fast kernel (sim_fast.cuh, CH = true) in CTAs of kDualThreads (320)
// threads, two to four resident per SM, as sim_fast_ctas.cu does for the
// simulation; own translation unit and constant tables.
#include "sim_fast.cuh"

namespace beep {
namespace {

template <int MG, int MB>
int launch_mb(const ModelDev &m, const BatchDev &b, size_t smem, cudaStream_t st)
{
	auto kern = sim_fast_kernel<kDualThreads, MG, false, true, MB>;
	cudaError_t e = allow_dynamic_smem(kern, smem);
	if (e != cudaSuccess) return (int)e;
	kern<<<b.P, kDualThreads, smem, st>>>(m, b);
	return (int)cudaGetLastError();
}

template <int MG>
int launch_mg(const ModelDev &m, const BatchDev &b, size_t smem, cudaStream_t st)
{
	if constexpr (MG <= 8)
		if (b.ctas >= 4) return launch_mb<MG, 4>(m, b, smem, st);
	return b.ctas >= 3 ? launch_mb<MG, 3>(m, b, smem, st) : launch_mb<MG, 2>(m, b, smem, st);
}

}  // namespace

int fast_chain_ctas_prepare() { return prepare_constants(); }

int launch_sim_fast_chain_ctas(const ModelDev &m, const BatchDev &b, size_t smem, void *stream)
{
	if (b.nt != kDualThreads || b.ctas < 2 || b.ctas > fast_ctas_max(m.G) || b.foi_tc || b.mode == 0)
		return (int)cudaErrorInvalidValue;
	const int e = prepare_constants();
	if (e != 0) return e;
	cudaStream_t st = (cudaStream_t)stream;
	return m.G <= 4 ? launch_mg<4>(m, b, smem, st) : m.G <= 8 ? launch_mg<8>(m, b, smem, st)
	     : m.G <= 12 ? launch_mg<12>(m, b, smem, st) : launch_mg<16>(m, b, smem, st);
}

}  // namespace beep
