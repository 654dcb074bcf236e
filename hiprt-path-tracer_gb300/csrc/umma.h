// 5th-generation tensor core (tcgen05) helpers for sm_103a: shared-memory matrix descriptors,
// instruction descriptors, TMEM allocation, single-thread MMA issue, commit to an mbarrier,
// bounded waits and TMEM loads. Inline PTX only (no library).
//
// Operand layout: K-major, no swizzle, the canonical "core matrix" layout: a core matrix is 8 rows
// x 16 bytes (8 bf16 along K) stored contiguously; core matrices adjacent along K are LBO = 128
// bytes apart and 8-row groups are SBO = K * 16 bytes apart, so element (r, k) of an R x K tile
// sits at element offset (r / 8) * 8K + (k / 8) * 64 + (r % 8) * 8 + (k % 8). One MMA consumes
// K = 16 (two core matrices along K); step s starts s * 256 bytes into the tile.
// D (M = 128 rows, fp32) lives in TMEM: row r in lane r, column c in TMEM column base + c; warp w
// of the CTA reads lanes 32w..32w+31 with tcgen05.ld.32x32b.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbpt {
namespace umma {

__host__ __device__ __forceinline__ int kmajor_offset(int r, int k, int K)
{
    return (r >> 3) * (K * 8) + (k >> 3) * 64 + (r & 7) * 8 + (k & 7);
}

#ifdef __CUDACC__

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), fixed 0b001 at bits 46-48,
// base offset 0, relative LBO, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | ((uint64_t)1 << 46);
}

// Descriptor of K-step 'ks' of a K-major tile with K columns starting at 'tile'
__device__ __forceinline__ uint64_t tile_desc(const __nv_bfloat16* tile, int K, int ks)
{
    return smem_desc(smem_addr(tile) + (uint32_t)ks * 256u, 128u, (uint32_t)K * 16u);
}

// Instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major, M x N.
__host__ __device__ __forceinline__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Warp-collective TMEM allocation; the base address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }
// generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;"); }

__device__ __forceinline__ void mbar_init(uint64_t* mbar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// D[tmem] (+)= A * B^T over one K = 16 step; issued by one thread.
__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
    asm volatile("{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
                 "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1 : 0));
}

// D(128 x N) (+)= A(128 x K) * B(N x K)^T over all K / 16 steps; accumulate = false overwrites D.
// One thread.
__device__ __forceinline__ void gemm_issue(uint32_t tmem_d, const __nv_bfloat16* A, const __nv_bfloat16* B, int N, int K,
                                           bool accumulate)
{
    const uint32_t id = idesc_bf16(128, N);
    for (int ks = 0; ks < K / 16; ks++) mma(tmem_d, tile_desc(A, K, ks), tile_desc(B, K, ks), id, accumulate || ks > 0);
}

// Arrives on 'mbar' once every MMA issued so far by this thread has completed
__device__ __forceinline__ void commit(uint64_t* mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(mbar)));
}

// D(128 x N) = A(128 x K) * B(N x K)^T, then commit to 'mbar'. One thread.
__device__ __forceinline__ void gemm_commit(uint32_t tmem_d, const __nv_bfloat16* A, const __nv_bfloat16* B, int N, int K,
                                            uint64_t* mbar)
{
    gemm_issue(tmem_d, A, B, N, K, false);
    commit(mbar);
}

// Waits for the mbarrier phase 'parity' with at most 'limit' polls; false if it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, int limit)
{
    const uint32_t a = smem_addr(mbar);
    uint32_t done = 0;
    for (int it = 0; it < limit && !done; it++)
        asm volatile("{\n.reg .pred P;\nmbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\nselp.u32 %0, 1, 0, P;\n}\n"
                     : "=r"(done)
                     : "r"(a), "r"(parity));
    return done != 0;
}

// 16 consecutive fp32 columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* out)
{
    uint32_t v[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                   "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
    for (int j = 0; j < 16; j++) out[j] = __uint_as_float(v[j]);
}

__device__ __forceinline__ uint32_t lane_addr(uint32_t tmem_base, int warp, int col)
{
    return tmem_base + ((uint32_t)(32 * warp) << 16) + (uint32_t)col;
}

#endif  // __CUDACC__

}  // namespace umma
}  // namespace gbpt
