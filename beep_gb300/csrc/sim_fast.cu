// Fast (mixed-precision) form: host side -- shared-memory sizing, thread
// counts and the launch of the simulation kernels (device code in
// sim_fast.cuh).
#include "sim_fast.cuh"

namespace beep {

static int pick_threads(const ModelDev &m)
{
	const int ncol = m.A * m.DP;
	return ncol <= 128 ? 128 : ncol <= 256 ? 256 : 640;
}

size_t fast_smem_bytes(const ModelDev &m, int nslots, bool m_in_smem, int nefoi_stage, bool state_global,
                       int tnrows, bool pop_single, bool tn_smem, int nt, int mg, bool pd)
{
	auto r = [](size_t x) { return (x + 15) & ~(size_t)15; };
	const size_t A = m.A, G = m.G, DP = m.DP, NS = m.NS, C = m.C, T = m.T, DPS = m.DPS;
	const size_t agsz = NS * A * (size_t)(mg > 0 ? mg : (m.G + 3) & ~3), ncol = A * DP;
	return (m_in_smem ? r(4 * A * ms_lda(m.A)) : 0) + (state_global ? 0 : (pop_single ? 1 : 2) * r(4 * C * ncol)) +
	       (state_global && !tn_smem ? 0 : r(4 * (size_t)tnrows * ncol)) + 3 * r(4 * agsz) +
	       r(4 * (size_t)nslots) + 3 * r(4 * T) + r(4 * DPS) + r(4 * C) + r(4 * T * DP) + r(4 * DP) + r(4 * 64) +
	       r(4 * 32) + 2 * r(4 * NS * A) + r(4 * (size_t)nefoi_stage * G) + 2 * (2 * r(4 * NS * A) + r(4 * G * G)) +
	       r(8) + r(4 * 2 * (size_t)(nt > 0 ? nt : pick_threads(m))) + (nt == kDualThreads ? r(4 * T * (size_t)nt) : 0) +
	       (pd ? r(4 * T * ncol) : 0);
}

int fast_threads() { return kFastThreads; }

int fast_prepare()
{
	int e = prepare_constants();
	if (e == 0) e = fast_chain_prepare();
	if (e == 0) e = batched_prepare();
	if (e == 0) e = fast_wide_prepare();
	return e != 0 ? e : fast_ctas_prepare();
}

int fast_pick_threads(const ModelDev &m) { return pick_threads(m); }

// Draws one per (transition, column) thread: models whose draws of a step take at most
// two passes of the CTA's threads (a 10-area x 3-age model: 180 draws on 128 threads,
// against 6 one after another per column thread)
bool fast_pd_fits(const ModelDev &m, int nt)
{
	return (nt == 128 || nt == 256) && m.T <= kMaxT && (long long)m.T * m.A * m.DP <= 2LL * nt;
}

size_t fast_tc_smem_bytes(const ModelDev &m)
{
	const tc::Geom g = tc::geometry(m.A, m.NS);
	return (size_t)tc::kStages * ((g.chunk_bytes() + 127) & ~(size_t)127) + g.a_bytes();
}

size_t fast_gstate_stride(const ModelDev &m)
{
	auto r = [](size_t x) { return (x + 255) & ~(size_t)255; };
	const size_t ncol = (size_t)m.A * m.DP;
	return 2 * r(4 * m.C * ncol) + r(4 * m.T * ncol);   // upper bound for any row/buffer choice
}

template <int NT, bool TC, int MB = min_ctas(NT), bool PD = false>
static int launch_nt(const ModelDev &m, const BatchDev &b, size_t smem, cudaStream_t st)
{
	// MG: the age count rounded up to a multiple of 4 (the stride of the infectious counts)
	auto kern = m.G <= 4 ? sim_fast_kernel<NT, 4, TC, false, MB, kMaxT, PD>
	          : m.G <= 8 ? sim_fast_kernel<NT, 8, TC, false, MB, kMaxT, PD>
	          : m.G <= 12 ? sim_fast_kernel<NT, 12, TC, false, MB, kMaxT, PD> : sim_fast_kernel<NT, 16, TC, false, MB, kMaxT, PD>;
	cudaError_t e = allow_dynamic_smem(kern, smem);
	if (e != cudaSuccess) return (int)e;
	kern<<<b.P, NT, smem, st>>>(m, b);
	return (int)cudaGetLastError();
}

int launch_sim_fast(const ModelDev &m, const BatchDev &b, void *stream)
{
	if (b.P == 0) return 0;
	if (b.mode != 0) return launch_sim_fast_chain(m, b, stream);
	const int nt = b.nt > 0 ? b.nt : pick_threads(m);
	const bool pd = b.pd != 0 && !b.foi_tc && (nt == 128 || nt == 256) && fast_pd_fits(m, nt);
	size_t smem = fast_smem_bytes(m, b.nslots, b.m_in_smem != 0, b.nefoi_stage, b.gstate != nullptr,
	                              b.tn_full ? m.T : m.tn_rows, b.pop_single != 0, b.tn_smem != 0, nt, 0, pd);
	if (fast_wide_needed(m)) {
		const int e = fast_prepare();
		if (e != 0) return e;
		return launch_sim_fast_wide(m, b, smem, stream);
	}
	if (b.foi_tc) {
		if (!m.tc_image || pick_threads(m) != 640 || b.tc_smem_off < smem) return (int)cudaErrorInvalidValue;
		smem = b.tc_smem_off + fast_tc_smem_bytes(m);
	}
	// (256 threads for a 128-thread model: its draws in one pass, parallel-draw batches)
	if (nt != pick_threads(m) && (nt != kDualThreads || b.foi_tc) && !(pd && nt == 256))
		return (int)cudaErrorInvalidValue;
	{
		const int e = fast_prepare();
		if (e != 0) return e;
	}
	cudaStream_t st = (cudaStream_t)stream;
	if (b.foi_tc) return launch_nt<640, true>(m, b, smem, st);
	if (pd) return nt == 128 ? launch_nt<128, false, min_ctas(128), true>(m, b, smem, st)
	                         : launch_nt<256, false, min_ctas(256), true>(m, b, smem, st);
	switch (nt) {
	case 128: return launch_nt<128, false>(m, b, smem, st);
	case 256: return launch_nt<256, false>(m, b, smem, st);
	case kDualThreads: return launch_sim_fast_ctas(m, b, smem, st);
	default: return launch_nt<640, false>(m, b, smem, st);
	}
}

}  // namespace beep
