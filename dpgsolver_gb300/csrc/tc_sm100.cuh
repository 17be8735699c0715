// Blackwell (sm_100a / sm_103a) tensor-core primitives in inline PTX: TMEM allocation, shared-memory matrix
// descriptors, tcgen05.mma (kind::f16 with BF16 inputs, kind::tf32; A from shared memory or from TMEM),
// tcgen05.commit to an mbarrier, tcgen05.ld / tcgen05.st, bounded mbarrier waits and the async-proxy fences they need.
//
// Operand layout used throughout (both A and B "K-major", no swizzle): a tile of R rows x K elements is stored as
// core matrices of 8 rows x 16 bytes; core matrix (row group g, K chunk c) lives at byte offset
// (g * (K*es/16) + c) * 128 and row r of it at +16*r.  The descriptor's leading-dimension byte offset is the
// distance between K-adjacent core matrices (128 B) and the stride-dimension byte offset the distance between
// row-adjacent core matrices (K*es/16*128 B).  One MMA step consumes 32 bytes of K (16 BF16 or 8 TF32 values).
#pragma once
#include <cstdint>

namespace dpg {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (row, k) in a K-major no-swizzle tile with K elements of es bytes per row.
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int row, int k, int K, int es)
{
	const int kc = (k * es) >> 4, kb = (k * es) & 15;
	return (uint32_t)((((row >> 3) * ((K * es) >> 4) + kc) << 7) + ((row & 7) << 4) + kb);
}

__device__ __forceinline__ uint64_t make_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
	uint64_t d = 0;
	d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
	d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
	d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
	d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
	return d;                // base offset 0, relative LBO, no swizzle
}

// Instruction descriptor: D = F32, A/B K-major.  fmt: 1 = BF16 (kind::f16), 2 = TF32 (kind::tf32).
__host__ __device__ constexpr uint32_t make_idesc(int M, int N, int fmt)
{
	return (1u << 4) | ((uint32_t)fmt << 7) | ((uint32_t)fmt << 10) | ((uint32_t)(N >> 3) << 17) |
	       ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols)
{
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)), "r"(ncols)
	             : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase)
{
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(smem_u32(bar)), "r"(phase)
	    : "memory");
	return ok != 0;
}
// Non-blocking test of an mbarrier phase.
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t phase)
{
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "selp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(smem_u32(bar)), "r"(phase)
	    : "memory");
	return ok != 0;
}
// Bounded wait on an mbarrier phase; false when max_iter polls elapsed without completion.  A completed phase is
// first checked with test_wait: try_wait on a completed phase still costs ~175 cycles of issue latency, which in the
// MMA-issuing warp becomes a bubble of the tensor pipe (its instruction queue is shallow).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase, long long max_iter = (1ll << 22))
{
	if (mbar_test(bar, phase)) return true;
	for (long long it = 0; it < max_iter; ++it)
		if (mbar_try_wait(bar, phase)) return true;
	return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
	    : "memory");
}
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
	    : "memory");
}
// Warp-uniform forms: every lane of the warp executes the call with identical arguments and one elected lane issues
// the instruction (the descriptors stay warp-uniform, so no per-thread to uniform register moves are needed).
__device__ __forceinline__ void mma_bf16_elect(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p, e;\n\t"
	    "elect.sync _|e, 0xffffffff;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "@e tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
	    : "memory");
}
__device__ __forceinline__ void mma_tf32_elect(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p, e;\n\t"
	    "elect.sync _|e, 0xffffffff;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "@e tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
	    : "memory");
}
// A operand from TMEM (lane = row of A, 32-bit columns along K; BF16: two K values per column, the lower K in the
// low half): the MMA then reads only B from shared memory.
__device__ __forceinline__ void mma_bf16_ts_elect(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p, e;\n\t"
	    "elect.sync _|e, 0xffffffff;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "@e tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(acc)
	    : "memory");
}
__device__ __forceinline__ void mma_tf32_ts_elect(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc, uint32_t acc)
{
	asm volatile(
	    "{\n\t.reg .pred p, e;\n\t"
	    "elect.sync _|e, 0xffffffff;\n\t"
	    "setp.ne.b32 p, %4, 0;\n\t"
	    "@e tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
	    "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(acc)
	    : "memory");
}
__device__ __forceinline__ void mma_commit_elect(uint64_t* bar)
{
	asm volatile(
	    "{\n\t.reg .pred e;\n\t"
	    "elect.sync _|e, 0xffffffff;\n\t"
	    "@e tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n\t}" ::"r"(smem_u32(bar))
	    : "memory");
}
// One lane of the (converged) warp returns true.
__device__ __forceinline__ bool elect_one()
{
	uint32_t ok;
	asm volatile(
	    "{\n\t.reg .pred e;\n\t"
	    "elect.sync _|e, 0xffffffff;\n\t"
	    "selp.u32 %0, 1, 0, e;\n\t}"
	    : "=r"(ok));
	return ok != 0;
}
__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}

// 8 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v)
{
	uint32_t r[8];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
	             : "r"(taddr)
	             : "memory");
#pragma unroll
	for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// 4 consecutive 32-bit TMEM columns of this thread's lane.
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float* v)
{
	uint32_t r[4];
	asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
	             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
	             : "r"(taddr)
	             : "memory");
#pragma unroll
	for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
// 4 / 8 consecutive 32-bit TMEM columns of this thread's lane from registers (asynchronous: tmem_st_wait before the
// values are handed to another thread).
__device__ __forceinline__ void tmem_st4(uint32_t taddr, uint4 v)
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr), "r"(v.x), "r"(v.y), "r"(v.z),
	             "r"(v.w)
	             : "memory");
}
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8])
{
	asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(taddr), "r"(v[0]),
	             "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
	             : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// Bulk global -> shared copy completing on an mbarrier (sizes and addresses multiples of 16 bytes).
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_u32(dst)),
	             "l"(src), "r"(bytes), "r"(smem_u32(bar))
	             : "memory");
}

} // namespace tc
} // namespace dpg
