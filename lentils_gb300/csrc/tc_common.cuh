// Blackwell (sm_100a / sm_103a) tensor-core building blocks in inline PTX: tensor memory (TMEM)
// allocation, shared-memory matrix descriptors, the BF16 instruction descriptor, tcgen05.mma
// issue / commit, TMEM loads, and bounded mbarrier waits.
//
// Shared-memory operand layout used throughout (no swizzle, K-major): the tile is a grid of
// "core matrices" of 8 rows x 16 bytes (8 x 8 BF16 values), each stored as 128 contiguous
// bytes (row r at byte 16 r). LBO is the byte distance between core matrices adjacent along K,
// SBO between core matrices adjacent along M (or N).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace lentils {
namespace tc {

// wait limit for mbarrier polls: far beyond any legitimate wait, small enough that a kernel
// that went wrong returns (with its error flag set) instead of hanging the GPU
constexpr uint32_t kSpinLimit = 1u << 20;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// -- mbarrier --------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Waits until the barrier's phase with parity `parity` has completed. Returns false if the
// wait gave up after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity,
                                          uint32_t limit = kSpinLimit)
{
    const uint32_t addr = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// -- cp.async (16 bytes, zero-filled when src_bytes == 0) ---------------------------------------
__device__ __forceinline__ void cp_async16(void *dst_smem, const void *src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst_smem)),
                 "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// -- fences ------------------------------------------------------------------------------------
// make generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// -- programmatic dependent launch ------------------------------------------------------------
// A kernel launched with programmatic stream serialization may start while the kernel before it
// in the stream is still running; pdl_wait() blocks until that kernel has completed and its
// memory is visible (a no-op for a kernel launched without the attribute), pdl_trigger() lets
// the next such kernel start once every CTA of this grid has triggered or exited. Everything
// before pdl_wait() must neither read what the previous kernel writes nor write what it reads.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// -- TMEM allocation (one full warp) ----------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

// -- descriptors ----------------------------------------------------------------------------------
// Shared-memory matrix descriptor: start address, LBO and SBO in 16-byte units, version 1,
// no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo_bytes, uint32_t sbo_bytes)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo_bytes >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo_bytes >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version
    return d;                // base offset 0, LBO mode 0, layout type 0 (no swizzle)
}

// Shared-memory matrix descriptor for a K-major operand in the 128-byte swizzled layout that a
// TMA load with CU_TENSOR_MAP_SWIZZLE_128B writes: rows of 64 BF16 values (128 bytes), groups
// of 8 rows 1024 bytes apart (SBO), 16-byte chunks permuted within each row by the row index
// modulo 8. The group base must be 1024-byte aligned; a K step of 16 values advances the start
// address by 32 bytes. LBO is unused in this layout (encoded as 1).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                     // LBO (unused)
    d |= (uint64_t)(1024 >> 4) << 32;           // SBO: 8 rows x 128 bytes
    d |= (uint64_t)1 << 46;                     // descriptor version
    d |= (uint64_t)2 << 61;                     // layout: 128-byte swizzle
    return d;
}

// The same for rows of 32 BF16 values (64 bytes) in the 64-byte swizzled layout
// (CU_TENSOR_MAP_SWIZZLE_64B): groups of 8 rows 512 bytes apart; a K step of 16 values advances
// the start address by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                     // LBO (unused)
    d |= (uint64_t)(512 >> 4) << 32;            // SBO: 8 rows x 64 bytes
    d |= (uint64_t)1 << 46;                     // descriptor version
    d |= (uint64_t)4 << 61;                     // layout: 64-byte swizzle
    return d;
}

// Shared-memory matrix descriptor for an MN-major operand in the 64-byte swizzled layout: each
// K row holds 32 consecutive M (or N) values (64 bytes), 8 K rows form a 512-byte swizzle atom,
// atoms adjacent along K are sbo bytes apart and atoms adjacent along M (N) lbo bytes apart. A
// K step of 16 values advances the start address by 2 sbo.
__device__ __forceinline__ uint64_t smem_desc_mn_sw64(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version
    d |= (uint64_t)4 << 61;  // layout: 64-byte swizzle
    return d;
}

template <int SWZ>
__device__ __forceinline__ uint64_t smem_desc_swz(uint32_t saddr)
{
    static_assert(SWZ == 64 || SWZ == 128, "swizzle");
    if constexpr (SWZ == 128) return smem_desc_sw128(saddr);
    else return smem_desc_sw64(saddr);
}

// -- TMA --------------------------------------------------------------------------------------
// mbarrier arrival that also expects `bytes` of asynchronous copies to complete on it
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// 3-D tiled TMA load of the box at (x, y, z) (x innermost)
__device__ __forceinline__ void tma_load_3d(void *dst, const void *map, int x, int y, int z,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// 4-D tiled TMA load of the box at (x, y, z, w) (x innermost; coordinates may be negative or
// past the end, which reads zeros)
__device__ __forceinline__ void tma_load_4d(void *dst, const void *map, int x, int y, int z, int w,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}

// 2-D tiled TMA load of the box at (x, y) (x innermost, in elements) into shared memory;
// completion is signalled on `bar` as transaction bytes. `map` is the generic address of a
// CUtensorMap in parameter (__grid_constant__), constant or global memory.
__device__ __forceinline__ void tma_load_2d(void *dst, const void *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Instruction descriptor for kind::f16 with BF16 A and B, FP32 accumulation, both operands
// K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N)
{
    return (1u << 4)                       // D format: F32
           | (1u << 7)                     // A format: BF16
           | (1u << 10)                    // B format: BF16
           | ((uint32_t)(N >> 3) << 17)    // N / 8
           | ((uint32_t)(M >> 4) << 24);   // M / 16
}

// The same with both operands MN-major (the instruction's transpose bits for A and B)
__host__ __device__ constexpr uint32_t idesc_bf16_f32_mn(int M, int N)
{
    return idesc_bf16_f32(M, N) | (1u << 15) | (1u << 16);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on `bar` once all previously issued tcgen05.mma of this thread have completed
__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// Each thread of a warp reads 8 consecutive 32-bit columns of its TMEM lane
// (warp w of a warpgroup accesses lanes 32(w%4) .. 32(w%4)+31).
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8])
{
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// Each thread of a warp reads 32 consecutive 32-bit columns of its TMEM lane; the registers are
// valid after tmem_wait_ld().
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace tc
}  // namespace lentils
