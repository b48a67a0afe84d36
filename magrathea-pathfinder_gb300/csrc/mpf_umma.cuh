// Fifth-generation tensor-core helpers (sm_100 family, tcgen05): TMEM
// allocation, shared-memory matrix descriptors, the kind::f16 MMA with BF16
// operands and FP32 accumulation in TMEM, commit to an mbarrier, and TMEM
// loads.  Inline PTX only; used by the surrogate's MLP layers.
//
// Operand layout in shared memory (SWIZZLE_NONE, K-major): an R x K BF16 tile
// is stored as 8 x 8 core matrices (8 rows of 16 contiguous bytes = 128 B);
// element (r, k) lives at
//     (k / 8) * (R / 8) * 128  +  (r / 8) * 128  +  (r % 8) * 16  +  (k % 8) * 2
// i.e. the core matrices of one 8-column K chunk are contiguous (stride 128 B
// along M/N), and K chunks follow each other (stride R * 16 bytes).  One MMA
// consumes K = 16 (two chunks), so the descriptor of K step s starts at
// 2 s R 16 bytes.
#pragma once
#include <cstdint>

namespace mpf {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in an R-row tile
__host__ __device__ __forceinline__ uint32_t tile_offset(int R, int r, int k)
{
    return (uint32_t)((k >> 3) * (R >> 3) * 128 + (r >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading-dimension byte
// offset (between core matrices adjacent in K), stride-dimension byte offset
// (between core matrices adjacent in M / N), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// descriptor of K step s (16 columns) of an R-row tile at saddr
__device__ __forceinline__ uint64_t tile_desc(uint32_t saddr, int R, int s)
{
    return smem_desc(saddr + (uint32_t)(2 * s * R * 16), (uint32_t)(R * 16), 128u);
}

// Instruction descriptor, kind::f16: D FP32, A and B BF16, both K-major,
// N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- TMEM allocation (one full warp) -------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(ncols)
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

// ---- ordering ---------------------------------------------------------------
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// named barrier over `count` threads
__device__ __forceinline__ void bar_sync(int id, int count)
{
    asm volatile("barrier.cta.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
// named barrier that also ORs a predicate over the participating threads
__device__ __forceinline__ bool bar_or(int id, int count, bool v)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbarrier.cta.red.or.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n}"
                 : "=r"(r)
                 : "r"((uint32_t)v), "r"(id), "r"(count)
                 : "memory");
    return r != 0;
}

// ---- mbarrier -------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar)
{
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Wait for the phase with the given parity to complete; false once
// `timeout_ns` of wall time have passed (each try_wait suspends the thread for
// at most a short, system-dependent time), or after 2^26 tries whatever the
// timer reads.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t timeout_ns)
{
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t tries = 0; tries < (1u << 26); ++tries) {
        if (mbar_try_wait(bar, parity)) return true;
        if (globaltimer_ns() - t0 > timeout_ns) return false;
    }
    return false;
}

// ---- MMA --------------------------------------------------------------------
// D[tmem] (+)= A[smem] * B[smem]^T, one thread issues
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, bool accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
                     d_tmem),
                 "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)accumulate)
                 : "memory");
}
// arrive on the mbarrier once all previously issued MMAs of this thread completed
__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// ---- TMEM -> registers ---------------------------------------------------
// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: warp
// w of a warpgroup reads lanes 32 (w % 4) .. + 31); waits for completion in
// the same statement, so no use of the values can be scheduled before it.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace mpf
