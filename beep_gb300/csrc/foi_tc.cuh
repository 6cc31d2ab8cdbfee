// Area-mixing contraction of the force of infection on the tensor cores
// (tcgen05, sm_100 family), for one particle per CTA:
//   Y[st][t][a] = sum_c M[c][t] * I[st][c][a]        (M off-diagonal)
// computed as D[r][t] = sum_c Istack[r][c] * M[c][t] with
//   * N = targets (a chunk of tw <= 256 targets per MMA) -- a tcgen05.mma has
//     a fixed issue cost of about 100 cycles whatever N is, so the targets,
//     the long dimension, go on N;
//   * M = 64 rows r = st*32 + q*16 + a: the counts of strain st split into
//     two BF16 pieces q (Ih + Il, exact for integer counts below 65536), ages
//     a padded to 16; row r lands in tensor-memory lane 32*(r/16) + r%16;
//   * K = sources, 16 per MMA; the matrix is streamed from global memory (L2)
//     as three BF16 pieces Mh + Mm + Ml (24 significant bits) by bulk copies
//     into a ring of shared-memory stages, one MMA per piece and K step.
// The accumulation is FP32 in tensor memory; Y = D[hi rows] + D[lo rows] is
// formed when the accumulators are read out.  Error: a few FP32 ulps of
// sum |M I| (the dropped products are below 2^-24 of each term).
//
// Shared-memory operand layout (no swizzle, K-major, core matrices of 8 rows
// x 16 bytes): element (row r, k) of a tile with R rows sits at
//   (k / 8) * (R * 16) + (r / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
// so the leading-dimension offset (next 8 k) is R*16 bytes and the stride
// offset (next 8 rows) is 128 bytes.
#pragma once

#include <cstdint>

namespace beep {
namespace tc {

#ifndef BEEP_TC_CHUNK_K
#define BEEP_TC_CHUNK_K 32
#endif
#ifndef BEEP_TC_STAGES
#define BEEP_TC_STAGES 3
#endif
constexpr int kRows = 64;                      // MMA M
constexpr int kPieces = 3;                     // M = hi + mid + lo
constexpr int kChunkK = BEEP_TC_CHUNK_K;       // sources per streamed chunk
constexpr int kStages = BEEP_TC_STAGES;        // chunk ring
constexpr int kMaxA = 512;                     // two target chunks of 256
constexpr int kMaxStrains = 2;                 // 32 rows per strain in M = 64
constexpr uint32_t kWaitLimit = 1u << 22;      // mbarrier polls before giving up

// byte offset of element (r, k) in a K-major no-swizzle tile of R rows
__host__ __device__ inline uint32_t kmajor_offset(int r, int k, int R)
{
	return (uint32_t)((k >> 3) * (R * 16) + (r >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// chunking of a model with A areas: nct target chunks of tw targets (a
// multiple of 16, <= 256), nkc source chunks of kChunkK sources
struct Geom {
	int A, NS, nct, tw, nkc;
	__host__ __device__ int kpad() const { return nkc * kChunkK; }
	__host__ __device__ uint32_t piece_bytes() const { return (uint32_t)tw * kChunkK * 2; }
	__host__ __device__ uint32_t chunk_bytes() const { return kPieces * piece_bytes(); }
	__host__ __device__ int nchunks() const { return nct * nkc; }
	__host__ __device__ size_t image_bytes() const { return (size_t)nchunks() * chunk_bytes(); }
	__host__ __device__ int arows() const { return 32 * NS; }                       // stored rows of the counts
	__host__ __device__ uint32_t a_lbo() const { return (uint32_t)arows() * 16; }
	// the M = 64 MMA also reads rows arows()..63: with one strain they alias the next
	// source block (harmless rows of D), so 512 bytes of slack follow the operand
	__host__ __device__ uint32_t a_bytes() const { return (uint32_t)(kpad() / 8) * a_lbo() + 512; }
	__host__ __device__ uint32_t tmem_cols() const
	{
		uint32_t need = (uint32_t)(nct * tw), c = 32;
		while (c < need) c <<= 1;
		return c;
	}
};

__host__ __device__ inline Geom geometry(int A, int NS)
{
	Geom g;
	g.A = A;
	g.NS = NS;
	g.nct = (A + 255) / 256;
	g.tw = ((A + g.nct - 1) / g.nct + 15) / 16 * 16;   // a multiple of 16: valid N for M = 64 and M = 128
	g.nkc = (A + kChunkK - 1) / kChunkK;
	return g;
}

__host__ __device__ inline bool supported(int A, int NS) { return A >= 16 && A <= kMaxA && NS >= 1 && NS <= kMaxStrains; }

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading/stride byte offsets, sm_100 version bits, no swizzle
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
	return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
	       (1ull << 46);
}

// instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major, M = 64, N = n
__device__ __forceinline__ uint32_t idesc_bf16(int n)
{
	return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kRows >> 4) << 24);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// waits for the phase with the given parity to complete; false after kWaitLimit polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
	const uint32_t a = smem_u32(bar);
	for (uint32_t it = 0; it < kWaitLimit; it++) {
		uint32_t ok;
		asm volatile(
		    "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
		    : "=r"(ok)
		    : "r"(a), "r"(parity)
		    : "memory");
		if (ok) return true;
	}
	return false;
}

// bulk copy global -> shared (16-byte aligned, size a multiple of 16), completion on bar
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_u32(dst)),
	             "l"(src), "r"(bytes), "r"(smem_u32(bar))
	             : "memory");
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// whole warp: allocate ncols tensor-memory columns, address written to *slot
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
	             : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, bool acc)
{
	asm volatile(
	    "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
	        d_tmem),
	    "l"(a), "l"(b), "r"(idesc), "r"((uint32_t)acc)
	    : "memory");
}

// arrives once on bar when every tcgen05 operation issued so far by this thread completed
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}

// 16 consecutive FP32 columns of this thread's lane (lane base = 32 * (warp % 4))
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
	uint32_t r[16];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
	    : "r"(taddr));
	asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
	for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// The contraction's shared state inside a kernel.
struct Foi {
	Geom g;
	unsigned char *stage0;           // chunk ring: stage s at stage0 + s * stage_stride (16-byte aligned)
	uint32_t stage_stride;
	unsigned char *a;                // stacked count pieces (a_bytes)
	uint64_t *full, *empty, *done;   // chunk loaded [kStages], chunk consumed [kStages], step's MMAs complete
	const unsigned char *image;      // matrix pieces in global memory, [nct][nkc][piece][tw x kChunkK]
	uint32_t pending, pend_par;      // issuer: stages with a load in flight, and the parity it completes
};

// The chunks of every step are numbered q = step * nchunks + j, chunk j = (target
// chunk j / nkc, source chunk j % nkc); chunk q uses ring stage q % kStages for the
// (q / kStages)-th time, which fixes the phase parity of the stage's barriers.

// Issuer thread: chunk j (number q) into its ring stage, one bulk copy per piece.
__device__ __forceinline__ void load_chunk(Foi &f, uint32_t q, int j)
{
	const uint32_t s = q % kStages, pb = f.g.piece_bytes();
	mbar_expect_tx(&f.full[s], kPieces * pb);
	const unsigned char *src = f.image + (size_t)j * f.g.chunk_bytes();
#pragma unroll
	for (int p = 0; p < kPieces; p++) bulk_load(f.stage0 + s * f.stage_stride + p * pb, src + p * pb, pb, &f.full[s]);
	f.pending |= 1u << s;
	f.pend_par = (f.pend_par & ~(1u << s)) | (((q / kStages) & 1u) << s);
}

// Issuer thread: loads of the first kStages chunks of step step_no (the ring is free).
__device__ __forceinline__ void prefetch(Foi &f, uint32_t step_no)
{
	const int n = f.g.nchunks();
	for (int j = 0; j < kStages && j < n; j++) load_chunk(f, step_no * (uint32_t)n + (uint32_t)j, j);
}

// Issuer thread: every chunk of step step_no -> MMAs into the target-chunk
// accumulators, refilling each stage as its MMAs complete; the step's last
// commit arrives on f.done.  Returns false if a wait timed out.
__device__ __forceinline__ bool issue_step(Foi &f, uint32_t taddr, uint32_t step_no)
{
	const Geom &g = f.g;
	const int n = g.nchunks();
	const uint32_t id = idesc_bf16(g.tw);
	const uint32_t pb = g.piece_bytes(), blbo = (uint32_t)g.tw * 16, albo = g.a_lbo();
	const uint32_t abase = smem_u32(f.a);
	for (int j = 0; j < n; j++) {
		const uint32_t q = step_no * (uint32_t)n + (uint32_t)j;
		const uint32_t s = q % kStages, use = q / kStages;
		if (!mbar_wait(&f.full[s], use & 1u)) return false;
		f.pending &= ~(1u << s);
		tc_after_sync();
		const int ct = j / g.nkc, kc = j % g.nkc;
		const uint32_t d = taddr + (uint32_t)(ct * g.tw);
		const uint32_t b0 = smem_u32(f.stage0) + s * f.stage_stride;
#pragma unroll
		for (int ks = 0; ks < kChunkK / 16; ks++) {
			const uint32_t k0 = (uint32_t)(kc * kChunkK + ks * 16);
			const uint64_t ad = sdesc(abase + (k0 >> 3) * albo, albo, 128);
			const uint32_t boff = (uint32_t)(ks * 2) * blbo;
#pragma unroll
			for (int p = 0; p < kPieces; p++)
				mma_bf16(d, ad, sdesc(b0 + p * pb + boff, blbo, 128), id, !(kc == 0 && ks == 0 && p == 0));
		}
		mma_commit(&f.empty[s]);
		if (j + kStages < n) {                     // refill the stage once its MMAs completed
			if (!mbar_wait(&f.empty[s], use & 1u)) return false;
			load_chunk(f, q + kStages, j + kStages);
		}
	}
	mma_commit(f.done);
	return true;
}

// Issuer thread, after a timeout: waits (bounded) for the loads still in flight,
// so that no bulk copy lands in shared memory after the CTA exits.
__device__ __forceinline__ void drain(Foi &f)
{
	for (uint32_t s = 0; s < (uint32_t)kStages; s++)
		if (f.pending & (1u << s)) mbar_wait(&f.full[s], (f.pend_par >> s) & 1u);
	f.pending = 0;
}

#endif  // __CUDACC__

}  // namespace tc
}  // namespace beep
