// Inline-PTX helpers for sm_103a: mbarriers, bulk (TMA) copies and the
// 5th-generation tensor core (tcgen05: MMA into tensor memory, TMEM loads).
//
// Every wait is bounded: nn_mbar_wait returns false after `limit` polls so a
// kernel can record an error and leave instead of hanging.
#pragma once

#include <stdint.h>

__device__ __forceinline__ uint32_t nn_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void nn_mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(nn_smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void nn_mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void nn_mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(nn_smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// One arrival (release semantics: this thread's earlier shared-memory reads
// are ordered before the phase it helps complete).
__device__ __forceinline__ void nn_mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(nn_smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool nn_mbar_wait(uint64_t* bar, uint32_t phase, uint32_t limit)
{
    const uint32_t addr = nn_smem_u32(bar);
    for (uint32_t it = 0; it < limit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Contiguous global -> shared copy by the bulk-copy engine; 16-byte aligned
// addresses, size a multiple of 16.
__device__ __forceinline__ void nn_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     nn_smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(nn_smem_u32(bar))
                 : "memory");
}

// Tiled tensor copy global -> shared by the bulk-copy engine (3D tensor map,
// box origin {x, y, z}; x times the element size a multiple of 16 bytes).
__device__ __forceinline__ void nn_tma_load_3d(void* dst, const void* map, int x, int y, int z, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(nn_smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(nn_smem_u32(bar))
        : "memory");
}

// ------------------------------------------------------------- tcgen05 --

// Shared-memory matrix descriptor, no swizzle (canonical layout of 8-row x
// 16-byte core matrices): start address, leading-dimension byte offset (next
// core matrix along K), stride-dimension byte offset (next 8 rows along M/N),
// descriptor version 1.
__device__ __forceinline__ uint64_t nn_umma_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B (both K-major) and
// an FP32 accumulator, shape M x N.
__host__ __device__ constexpr uint32_t nn_umma_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T; issued by one thread.
__device__ __forceinline__ void nn_umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                             uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on the mbarrier once all previously issued MMAs of this thread completed.
__device__ __forceinline__ void nn_umma_commit(uint64_t* bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     nn_smem_u32(bar))
                 : "memory");
}

// Warp-wide: allocate ncols (power of two >= 32) TMEM columns, address to *slot.
__device__ __forceinline__ void nn_tmem_alloc(uint32_t* slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(nn_smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void nn_tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void nn_tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void nn_tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's TMEM lane (32x32b shape: warp
// w of a warpgroup reads lanes 32w .. 32w+31).
__device__ __forceinline__ void nn_tmem_ld16(uint32_t taddr, float* v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
