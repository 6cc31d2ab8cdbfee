// Fast form for models beyond the usual instantiations: up to 16 transitions
// and 20 age groups (for example Erlang-staged compartments, or 18 five-year
// age bands), one 640-thread CTA per SM, force of infection on FP32 SIMT.
// The device code is sim_fast.cuh's with wider per-column registers; this
// unit has its own copy of the constant tables.
#include "sim_fast.cuh"

namespace beep {
namespace {

template <int MG>
int launch_w(const ModelDev &m, const BatchDev &b, size_t smem, cudaStream_t st)
{
	auto kern = sim_fast_kernel<640, MG, false, false, 1, kWideT>;
	cudaError_t e = allow_dynamic_smem(kern, smem);
	if (e != cudaSuccess) return (int)e;
	kern<<<b.P, 640, smem, st>>>(m, b);
	return (int)cudaGetLastError();
}

}  // namespace

bool fast_wide_needed(const ModelDev &m) { return m.T > kMaxT || m.G > 16; }

bool fast_wide_supported(const ModelDev &m) { return m.T <= kWideT && m.G <= kWideG; }

int fast_wide_prepare() { return prepare_constants(); }

int launch_sim_fast_wide(const ModelDev &m, const BatchDev &b, size_t smem, void *stream)
{
	if (!fast_wide_supported(m) || b.foi_tc || b.nt != 640 || b.mode != 0 || b.batched) return (int)cudaErrorInvalidValue;
	const int e0 = prepare_constants();
	if (e0 != 0) return e0;
	cudaStream_t st = (cudaStream_t)stream;
	return m.G <= 4 ? launch_w<4>(m, b, smem, st) : m.G <= 8 ? launch_w<8>(m, b, smem, st)
	     : m.G <= 12 ? launch_w<12>(m, b, smem, st) : m.G <= 16 ? launch_w<16>(m, b, smem, st)
	     : launch_w<20>(m, b, smem, st);
}

}  // namespace beep
