// Generic BF16 tensor-core GEMM on tcgen05 with pluggable operand loaders and epilogue.
//
//   D[m][n] = sum_k A(m, k) * B(n, k)   (FP32 accumulation in tensor memory)
//
// Operands are produced 16 bytes (8 BF16 along K) at a time by loader functors
// `uint4 LA::operator()(int m, int kpiece)` / `LB::operator()(int n, int kpiece)` returning zero
// outside the problem, so the same kernel serves plain GEMMs and implicit-GEMM convolutions
// (im2col gathered on the fly). One CTA of 128 threads computes a 128 x N tile of D for one
// split of K (blockIdx.z), staging 64-wide K chunks into shared memory in the no-swizzle K-major
// core-matrix layout (cores along K 128 bytes apart, 8-row groups 1024 bytes apart), double
// buffered: while the tensor core works on one chunk (four 128 x N x 16 MMAs issued by one
// thread, completion tracked by an mbarrier), the threads stage the next. The epilogue functor
// `EP::operator()(int m, int n, float v)` receives every element of the tile; each warp reads
// its 32 TMEM lanes (rows) with tcgen05.ld. Waits are bounded: on a timeout *err is set and the
// kernel still frees its tensor memory.
#pragma once

#include <cuda.h>

#include "tc_common.cuh"

namespace lentils {
namespace tc {

constexpr int kChunkK = 64;          // K per shared-memory chunk
constexpr int kPiecesPerChunk = kChunkK / 8;
constexpr int kATileBytes = 128 * kChunkK * 2;  // 16 KB

template <int N>
struct GemmSmem {
    static constexpr int kBTileBytes = N * kChunkK * 2;
    static constexpr int kStageBytes = kATileBytes + kBTileBytes;
    static constexpr int kBytes = 2 * kStageBytes;  // double buffered
};

__device__ __forceinline__ int core_offset(int row, int piece)
{
    return (row >> 3) * 1024 + piece * 128 + (row & 7) * 16;
}

// Piece i of thread t (128 threads) is row r = 16 i + 8 (t / 64) + t % 8, K-piece q = (t / 8) % 8:
// its core-matrix offset is 2048 i + 16 t, so a warp's shared-memory stores are contiguous, and
// eight consecutive threads take eight consecutive rows of one K-piece. All global loads of a
// group are issued before its shared-memory stores (the loaders read through generic pointers,
// which the compiler cannot separate from the stores), so a chunk costs one or two memory
// round trips per thread instead of one per piece.
template <int NP, class L>
__device__ __forceinline__ void stage_rows(const L &ld, int r0, int kp0, int kp_end,
                                           unsigned char *s)
{
    const int t = threadIdx.x;
    const int rr = ((t >> 6) << 3) + (t & 7), q = (t >> 3) & 7, kp = kp0 + q;
    constexpr int kGroup = NP < 8 ? NP : 8;
#pragma unroll
    for (int g = 0; g < NP; g += kGroup) {
        uint4 v[kGroup];
#pragma unroll
        for (int i = 0; i < kGroup; ++i)
            v[i] = (kp < kp_end) ? ld(r0 + 16 * (g + i) + rr, kp) : make_uint4(0, 0, 0, 0);
#pragma unroll
        for (int i = 0; i < kGroup; ++i)
            *reinterpret_cast<uint4 *>(s + 2048 * (g + i) + 16 * t) = v[i];
    }
}

template <int N, class LA, class LB>
__device__ __forceinline__ void stage_chunk(const LA &la, const LB &lb, int m0, int n0, int kp0,
                                            int kp_end, unsigned char *sa, unsigned char *sb)
{
    stage_rows<128 / 16>(la, m0, kp0, kp_end, sa);
    stage_rows<N / 16>(lb, n0, kp0, kp_end, sb);
}

// Epilogues declare `static constexpr bool kRowPerLane = true` when each thread should call them
// for its own row (an output of one column); the others are called through a shared-memory
// transpose, 32 columns at a time, so the 32 lanes of a warp handle 32 consecutive columns of
// one row and row-major stores coalesce.
template <class EP, class = void>
struct row_per_lane {
    static constexpr bool value = false;
};
template <class EP>
struct row_per_lane<EP, decltype((void)EP::kRowPerLane)> {
    static constexpr bool value = EP::kRowPerLane;
};

// kpieces: total K / 8; kp_per_split: pieces handled by one blockIdx.z (multiple of 8)
template <int N, class LA, class LB, class EP>
__global__ void __launch_bounds__(128)
    gemm_kernel(const LA la, const LB lb, const EP ep, int kpieces, int kp_per_split, int *err)
{
    static_assert(N % 16 == 0 && N >= 32 && N <= 256, "N");
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t bar[2];
    __shared__ uint32_t tmem_base;
    constexpr uint32_t ncols = (N <= 32) ? 32 : (N <= 64) ? 64 : (N <= 128) ? 128 : 256;
    const int m0 = blockIdx.x * 128;
    const int n0 = blockIdx.y * N;
    const int kp_begin = blockIdx.z * kp_per_split;
    const int kp_end = min(kpieces, kp_begin + kp_per_split);
    const int warp = threadIdx.x >> 5;

    if (warp == 0) {
        tmem_alloc(&tmem_base, ncols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    constexpr uint32_t idesc = idesc_bf16_f32(128, N);
    const int nchunks = (kp_end > kp_begin) ? (kp_end - kp_begin + kPiecesPerChunk - 1) / kPiecesPerChunk : 0;
    bool ok = true;
    uint32_t phase[2] = {0, 0};
    bool inflight[2] = {false, false};
    for (int ch = 0; ch < nchunks && ok; ++ch) {
        const int buf = ch & 1;
        unsigned char *sa = smem + buf * GemmSmem<N>::kStageBytes;
        unsigned char *sb = sa + kATileBytes;
        if (inflight[buf]) {  // the MMAs that read this buffer two chunks ago must be done
            ok = mbar_wait(&bar[buf], phase[buf]);
            phase[buf] ^= 1;
            inflight[buf] = false;
            if (!ok) break;
        }
        stage_chunk<N>(la, lb, m0, n0, kp_begin + ch * kPiecesPerChunk, kp_end, sa, sb);
        fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < kChunkK / 16; ++s) {
                const uint64_t ad = smem_desc(smem_u32(sa) + s * 256, 128, 1024);
                const uint64_t bd = smem_desc(smem_u32(sb) + s * 256, 128, 1024);
                mma_bf16(tmem, ad, bd, idesc, (ch > 0 || s > 0) ? 1u : 0u);
            }
            mma_commit(&bar[buf]);
        }
        inflight[buf] = true;
    }
    // drain: wait for the MMAs still in flight (both buffers)
    for (int b = 0; b < 2; ++b) {
        if (inflight[b]) {
            const bool w = mbar_wait(&bar[b], phase[b]);
            ok = ok && w;
        }
    }
    tc_fence_after();
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    if (ok && nchunks > 0) {
        const int lane = threadIdx.x & 31;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        if constexpr (row_per_lane<EP>::value || N % 32 != 0) {
            for (int c0 = 0; c0 < N; c0 += 8) {
                float v[8];
                tmem_ld8(taddr + c0, v);
#pragma unroll
                for (int j = 0; j < 8; ++j) ep(m0 + warp * 32 + lane, n0 + c0 + j, v[j]);
            }
        } else {
            // the staging buffers are free: every MMA that read them has completed
            float *tr = reinterpret_cast<float *>(smem) + warp * (32 * 33);
            for (int c0 = 0; c0 < N; c0 += 32) {
#pragma unroll
                for (int j = 0; j < 32; j += 8) {
                    float v[8];
                    tmem_ld8(taddr + c0 + j, v);
#pragma unroll
                    for (int i = 0; i < 8; ++i) tr[lane * 33 + j + i] = v[i];
                }
                __syncwarp();
#pragma unroll 4
                for (int r = 0; r < 32; ++r) ep(m0 + warp * 32 + r, n0 + c0 + lane, tr[r * 33 + lane]);
                __syncwarp();
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

// -- pipelined form ------------------------------------------------------------------------------
// The same GEMM with the operand staging taken off the tensor core's critical path. Loaders
// give the ADDRESS of each 16-byte piece (`const void *LA::ptr(int m, int kpiece)`, null for a
// zero piece). 160 threads: warps 0-3 copy the pieces straight into a ring of STAGES shared-
// memory chunks with cp.async (no register staging), STAGES - 1 chunks ahead, and afterwards
// run the epilogue; warp 4 owns the tensor memory and one of its threads issues the MMAs.
// Chunk c is handed over through two mbarriers: `full` (128 producer arrivals, each after the
// thread's copies of c have landed and been fenced for the async proxy) and `empty` (the
// tcgen05.commit of the MMAs that read it). Waits are bounded; on a timeout *err is set, the
// loops stop, and the kernel waits (bounded) for its MMAs before it frees tensor memory.
constexpr int kPipeThreads = 160;

template <int N, int STAGES>
struct PipeSmem {
    static constexpr int kStageBytes = GemmSmem<N>::kStageBytes;
    static constexpr int kBytes = STAGES * kStageBytes;
};

template <int NP, class L>
__device__ __forceinline__ void stage_rows_async(const L &ld, int r0, int kp0, int kp_end,
                                                 unsigned char *s)
{
    const int t = threadIdx.x;
    const int rr = ((t >> 6) << 3) + (t & 7), q = (t >> 3) & 7, kp = kp0 + q;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        const void *src = (kp < kp_end) ? ld.ptr(r0 + 16 * i + rr, kp) : nullptr;
        cp_async16(s + 2048 * i + 16 * t, src ? src : ld.base(), src ? 16u : 0u);
    }
}

template <int N, int STAGES, class LA, class LB, class EP>
__global__ void __launch_bounds__(kPipeThreads)
    gemm_pipe_kernel(const LA la, const LB lb, const EP ep, int kpieces, int kp_per_split,
                     int *err)
{
    static_assert(N % 16 == 0 && N >= 32 && N <= 256, "N");
    static_assert(STAGES >= 2, "stages");
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t full[STAGES], empty[STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    constexpr uint32_t ncols = (N <= 32) ? 32 : (N <= 64) ? 64 : (N <= 128) ? 128 : 256;
    constexpr int L = STAGES - 1;  // chunks in flight ahead of the one handed over
    const int m0 = blockIdx.x * 128;
    const int n0 = blockIdx.y * N;
    const int kp_begin = blockIdx.z * kp_per_split;
    const int kp_end = min(kpieces, kp_begin + kp_per_split);
    const int warp = threadIdx.x >> 5;
    const int nchunks =
        (kp_end > kp_begin) ? (kp_end - kp_begin + kPiecesPerChunk - 1) / kPiecesPerChunk : 0;

    if (warp == 4) {
        tmem_alloc(&tmem_base, ncols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; ++i) {
            mbar_init(&full[i], 128);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&done, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;
    bool ok = true;

    if (warp < 4) {  // producers
        for (int ch = 0; ch < nchunks + L; ++ch) {
            if (ch < nchunks) {
                const int st = ch % STAGES;
                if (ch >= STAGES) {
                    if (!mbar_wait(&empty[st], ((ch / STAGES) - 1) & 1)) {
                        ok = false;
                        break;
                    }
                }
                unsigned char *sa = smem + st * PipeSmem<N, STAGES>::kStageBytes;
                const int kp0 = kp_begin + ch * kPiecesPerChunk;
                stage_rows_async<128 / 16>(la, m0, kp0, kp_end, sa);
                stage_rows_async<N / 16>(lb, n0, kp0, kp_end, sa + kATileBytes);
            }
            cp_async_commit();
            if (ch >= L) {  // chunk ch - L has landed: hand it to the tensor core
                cp_async_wait_group<L>();
                fence_async_smem();
                mbar_arrive(&full[(ch - L) % STAGES]);
            }
            if (*(volatile int *)&abort_flag) {
                ok = false;
                break;
            }
        }
        cp_async_wait_all();
        if (!ok) atomicExch(&abort_flag, 1);
    } else if (threadIdx.x == 128) {  // the MMA issuer
        constexpr uint32_t idesc = idesc_bf16_f32(128, N);
        for (int ch = 0; ch < nchunks; ++ch) {
            const int st = ch % STAGES;
            if (!mbar_wait(&full[st], (ch / STAGES) & 1) || *(volatile int *)&abort_flag) {
                ok = false;
                break;
            }
            tc_fence_after();
            unsigned char *sa = smem + st * PipeSmem<N, STAGES>::kStageBytes;
            unsigned char *sb = sa + kATileBytes;
#pragma unroll
            for (int k = 0; k < kChunkK / 16; ++k) {
                const uint64_t ad = smem_desc(smem_u32(sa) + k * 256, 128, 1024);
                const uint64_t bd = smem_desc(smem_u32(sb) + k * 256, 128, 1024);
                mma_bf16(tmem, ad, bd, idesc, (ch > 0 || k > 0) ? 1u : 0u);
            }
            mma_commit(&empty[st]);
        }
        if (!ok) atomicExch(&abort_flag, 1);
        mma_commit(&done);  // arrives once every MMA issued above has completed
    }
    if (warp == 4) __syncwarp();  // the issuer's warp-mates wait here, not on the mbarrier
    // every MMA has completed once `done` fires (bounded wait; on a timeout nothing is read)
    const bool fin = mbar_wait(&done, 0);
    tc_fence_after();
    __syncthreads();
    const bool good = fin && !*(volatile int *)&abort_flag && nchunks > 0;
    if (threadIdx.x == 0 && (!fin || *(volatile int *)&abort_flag)) atomicExch(err, 1);
    if (good && warp < 4) {
        const int lane = threadIdx.x & 31;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        if constexpr (row_per_lane<EP>::value || N % 32 != 0) {
            for (int c0 = 0; c0 < N; c0 += 8) {
                float v[8];
                tmem_ld8(taddr + c0, v);
#pragma unroll
                for (int j = 0; j < 8; ++j) ep(m0 + warp * 32 + lane, n0 + c0 + j, v[j]);
            }
        } else {
            float *tr = reinterpret_cast<float *>(smem) + warp * (32 * 33);
            for (int c0 = 0; c0 < N; c0 += 32) {
#pragma unroll
                for (int j = 0; j < 32; j += 8) {
                    float v[8];
                    tmem_ld8(taddr + c0 + j, v);
#pragma unroll
                    for (int i = 0; i < 8; ++i) tr[lane * 33 + j + i] = v[i];
                }
                __syncwarp();
#pragma unroll 4
                for (int r = 0; r < 32; ++r) ep(m0 + warp * 32 + r, n0 + c0 + lane, tr[r * 33 + lane]);
                __syncwarp();
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) tmem_dealloc(tmem, ncols);
}

// -- TMA form ------------------------------------------------------------------------------------
// The GEMM fed by TMA: operands are functors `void LA::load(void *dst, uint64_t *bar, int row0,
// int kp0) const` that issue the tensor-map loads of one K chunk (kChunk values starting at
// piece kp0, in the swizzled layout of kSwz-byte rows: 64 values with 128-byte swizzle or 32
// with 64-byte) of rows row0 .. row0 + 127 (A; LB: N rows) onto the mbarrier `bar`, with
// `static constexpr uint32_t kBytes` the bytes they deliver. One thread issues every load (the
// operands must be passed as __grid_constant__ so that their tensor maps have parameter-space
// addresses), one thread of warp 4 issues the MMAs, warps 0-3 run the epilogue. STAGES chunks
// are in flight; `full` expects the chunk's bytes, `empty` is the MMAs' commit.
template <int N, int STAGES, int KCH = 64>
struct TmaSmem {
    static constexpr int kATile = 128 * KCH * 2;
    static constexpr int kStageBytes = kATile + N * KCH * 2;
    static constexpr int kBytes = STAGES * kStageBytes + 1024;  // + alignment slack
};

template <int N, int STAGES, class LA, class LB, class EP>
__global__ void __launch_bounds__(kPipeThreads)
    gemm_tma_kernel(const __grid_constant__ LA la, const __grid_constant__ LB lb, const EP ep,
                    int kpieces, int kp_per_split, int *err)
{
    static_assert(N % 16 == 0 && N >= 32 && N <= 256, "N");
    constexpr int KCH = LA::kChunk, SWZ = LA::kSwz;
    static_assert(LB::kChunk == KCH && LB::kSwz == SWZ && KCH * 2 == SWZ, "operand layouts");
    constexpr int kATile = TmaSmem<N, STAGES, KCH>::kATile;
    constexpr int kPieces = KCH / 8;  // pieces of 8 values per chunk
    static_assert(LA::kBytes == (uint32_t)kATile && LB::kBytes == (uint32_t)(N * KCH * 2),
                  "operand bytes");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t full[STAGES], empty[STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    // 128-byte swizzle atoms need 1024-byte aligned tiles
    unsigned char *smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    constexpr uint32_t ncols = (N <= 32) ? 32 : (N <= 64) ? 64 : (N <= 128) ? 128 : 256;
    constexpr int kStage = TmaSmem<N, STAGES, KCH>::kStageBytes;
    const int m0 = blockIdx.x * 128;
    const int n0 = blockIdx.y * N;
    const int kp_begin = blockIdx.z * kp_per_split;
    const int kp_end = min(kpieces, kp_begin + kp_per_split);
    const int warp = threadIdx.x >> 5;
    const int nchunks = (kp_end > kp_begin) ? (kp_end - kp_begin + kPieces - 1) / kPieces : 0;

    if (warp == 4) {
        tmem_alloc(&tmem_base, ncols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&done, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    pdl_wait();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    pdl_trigger();
    const uint32_t tmem = tmem_base;
    int last[STAGES];  // producer: the last chunk loaded into each stage (-1: none)
#pragma unroll
    for (int i = 0; i < STAGES; ++i) last[i] = -1;

    // The producer and the MMA issuer are lane 0 of warps 0 and 4; the other lanes of those warps
    // wait at __syncwarp (not polling an mbarrier, which would hold up the lane that works).
    if (threadIdx.x == 0) {  // the TMA producer
        for (int ch = 0; ch < nchunks; ++ch) {
            const int st = ch % STAGES;
            if (ch >= STAGES && !mbar_wait(&empty[st], ((ch / STAGES) - 1) & 1)) {
                atomicExch(&abort_flag, 1);
                break;
            }
            if (*(volatile int *)&abort_flag) break;
            unsigned char *sa = smem + st * kStage;
            const int kp0 = kp_begin + ch * kPieces;
            mbar_arrive_expect_tx(&full[st], LA::kBytes + LB::kBytes);
            la.load(sa, &full[st], m0, kp0);
            lb.load(sa + kATile, &full[st], n0, kp0);
            last[st] = ch;
        }
    } else if (threadIdx.x == 128) {  // the MMA issuer
        constexpr uint32_t idesc = idesc_bf16_f32(128, N);
        for (int ch = 0; ch < nchunks; ++ch) {
            const int st = ch % STAGES;
            if (!mbar_wait(&full[st], (ch / STAGES) & 1) || *(volatile int *)&abort_flag) {
                atomicExch(&abort_flag, 1);
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + st * kStage);
            const uint32_t sb = sa + kATile;
#pragma unroll
            for (int k = 0; k < KCH / 16; ++k)
                mma_bf16(tmem, smem_desc_swz<SWZ>(sa + 32 * k), smem_desc_swz<SWZ>(sb + 32 * k),
                         idesc, (ch > 0 || k > 0) ? 1u : 0u);
            mma_commit(&empty[st]);
        }
        mma_commit(&done);
    }
    if (warp == 0 || warp == 4) __syncwarp();
    const bool fin = mbar_wait(&done, 0);
    if (threadIdx.x == 0) {
        // every load has landed before shared memory is reused or the CTA exits (the MMAs
        // waited for each chunk they read; after an abort a chunk may not have been read)
#pragma unroll
        for (int i = 0; i < STAGES; ++i)
            if (last[i] >= 0 && !mbar_wait(&full[i], (last[i] / STAGES) & 1)) atomicExch(&abort_flag, 1);
    }
    tc_fence_after();
    __syncthreads();
    const bool bad = !fin || *(volatile int *)&abort_flag;
    if (threadIdx.x == 0 && bad) atomicExch(err, 1);
    if (!bad && nchunks > 0 && warp < 4) {
        const int lane = threadIdx.x & 31;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        if constexpr (row_per_lane<EP>::value || N % 32 != 0) {
            for (int c0 = 0; c0 < N; c0 += 8) {
                float v[8];
                tmem_ld8(taddr + c0, v);
#pragma unroll
                for (int j = 0; j < 8; ++j) ep(m0 + warp * 32 + lane, n0 + c0 + j, v[j]);
            }
        } else {
            float *tr = reinterpret_cast<float *>(smem) + warp * (32 * 33);
            for (int c0 = 0; c0 < N; c0 += 32) {
#pragma unroll
                for (int j = 0; j < 32; j += 8) {
                    float v[8];
                    tmem_ld8(taddr + c0 + j, v);
#pragma unroll
                    for (int i = 0; i < 8; ++i) tr[lane * 33 + j + i] = v[i];
                }
                __syncwarp();
#pragma unroll 4
                for (int r = 0; r < 32; ++r) ep(m0 + warp * 32 + r, n0 + c0 + lane, tr[r * 33 + lane]);
                __syncwarp();
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) tmem_dealloc(tmem, ncols);
}

// -- persistent TMA form -----------------------------------------------------------------------
// The TMA-fed GEMM as a persistent kernel: each CTA takes row tiles blockIdx.x, blockIdx.x +
// gridDim.x, ... over the whole K (no split). The accumulator is double buffered in tensor
// memory (2 x N columns), so the epilogue of one tile runs while the MMAs of the next fill the
// other buffer, and the TMA ring runs on across tile boundaries. Six warps: warps 0-3 the
// epilogue (warp w reads TMEM lanes 32w .. 32w + 31, one row per thread), lane 0 of warp 4 the
// TMA producer, warp 5 allocates tensor memory and its lane 0 issues the MMAs.
//   full[s]   : the chunk in stage s has landed (TMA transaction bytes)
//   empty[s]  : the MMAs that read stage s have completed (tcgen05.commit)
//   tfull[b]  : the last MMA of the tile in accumulator b has completed
//   tempty[b] : the four epilogue warps have read accumulator b
// Operands walk K with cursors: `typename L::Cursor L::begin(int row0) const` at the start of a
// tile and `void L::next(void *dst, uint64_t *bar, Cursor &) const`, which issues the loads of
// the next chunk and advances (the producer is one thread, so per-chunk address arithmetic is
// on the critical path). Row epilogues are functors with
//   `void prepare(float *sh, int tid) const` (tid 0..127: stage constants in the 1 KB shared
//   scratch sh, once per CTA),
//   `void row(int m, int n0, const float (&v)[32], float &acc, const float *sh) const`
//   (columns n0 .. n0 + 31 of row m, for n0 = 0, 32, ..., N - 32 in order; acc starts at 0),
//   `void row_end(int m, float acc, const float *sh) const`.
// Every wait is bounded; after a timeout *err is set, each role stops, the producer waits for
// the copies it issued, and the tensor memory is freed.
constexpr int kPersistThreads = 192;

__device__ __forceinline__ void prefetch_tensormap(const void *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

template <int N, int STAGES, class LA, class LB, class EP>
__global__ void __launch_bounds__(kPersistThreads, 1)
    gemm_tma_persist_kernel(const __grid_constant__ LA la, const __grid_constant__ LB lb,
                            const EP ep, int mtiles, int kpieces, int *err)
{
    static_assert(N % 32 == 0 && N >= 32 && N <= 128, "N");
    constexpr int KCH = LA::kChunk, SWZ = LA::kSwz;
    static_assert(LB::kChunk == KCH && LB::kSwz == SWZ && KCH * 2 == SWZ, "operand layouts");
    constexpr int kATile = TmaSmem<N, STAGES, KCH>::kATile;
    constexpr int kStage = TmaSmem<N, STAGES, KCH>::kStageBytes;
    constexpr int kPieces = KCH / 8;
    static_assert(LA::kBytes == (uint32_t)kATile && LB::kBytes == (uint32_t)(N * KCH * 2),
                  "operand bytes");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t full[STAGES], empty[STAGES], tfull[2], tempty[2], mdone;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    __shared__ float scratch[256];
    unsigned char *smem = smem_raw + ((1024 - (smem_u32(smem_raw) & 1023)) & 1023);
    constexpr uint32_t ncols = (2 * N <= 64) ? 64 : (2 * N <= 128) ? 128 : 256;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunks = (kpieces + kPieces - 1) / kPieces;
    const int ntiles =
        (mtiles > (int)blockIdx.x) ? (mtiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x : 0;

    if (warp == 5) {
        tmem_alloc(&tmem_base, ncols);
        tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&tfull[i], 1);
            mbar_init(&tempty[i], 4);
        }
        mbar_init(&mdone, 1);
        abort_flag = 0;
        fence_mbar_init();
    }
    if (threadIdx.x == 128) {
        prefetch_tensormap(&la.map);
        prefetch_tensormap(&lb.map);
    }
    pdl_wait();
    if (warp < 4) ep.prepare(scratch, threadIdx.x);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    pdl_trigger();
    const uint32_t tmem = tmem_base;

    if (warp == 4) {
        if (lane == 0) {  // the TMA producer
            int it = 0;
            for (int j = 0; j < ntiles; ++j) {
                typename LA::Cursor ca = la.begin(((int)blockIdx.x + j * (int)gridDim.x) * 128);
                typename LB::Cursor cb = lb.begin(0);
                int ch = 0;
                for (; ch < nchunks; ++ch, ++it) {
                    const int st = it % STAGES;
                    if (it >= STAGES && !mbar_wait(&empty[st], ((it / STAGES) - 1) & 1)) {
                        atomicExch(&abort_flag, 1);
                        break;
                    }
                    unsigned char *sa = smem + st * kStage;
                    mbar_arrive_expect_tx(&full[st], LA::kBytes + LB::kBytes);
                    la.next(sa, &full[st], ca);
                    lb.next(sa + kATile, &full[st], cb);
                }
                if (ch < nchunks) break;
            }
            // every copy has landed before the CTA exits: stage i last took chunk
            // i + STAGES q for the largest q with that below it
#pragma unroll
            for (int i = 0; i < STAGES; ++i) {
                if (i >= it) continue;
                const int last = i + ((it - 1 - i) / STAGES) * STAGES;
                if (!mbar_wait(&full[i], (last / STAGES) & 1)) atomicExch(&abort_flag, 1);
            }
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {  // the MMA issuer
            constexpr uint32_t idesc = idesc_bf16_f32(128, N);
            int it = 0;
            bool ok = true;
            for (int j = 0; j < ntiles && ok; ++j) {
                const int buf = j & 1;
                if (j >= 2 && !mbar_wait(&tempty[buf], ((j >> 1) - 1) & 1)) {
                    atomicExch(&abort_flag, 1);
                    break;
                }
                tc_fence_after();
                const uint32_t acc = tmem + (uint32_t)(buf * N);
                for (int ch = 0; ch < nchunks; ++ch, ++it) {
                    const int st = it % STAGES;
                    if (!mbar_wait(&full[st], (it / STAGES) & 1)) {
                        atomicExch(&abort_flag, 1);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(smem + st * kStage);
                    const uint32_t sb = sa + kATile;
#pragma unroll
                    for (int k = 0; k < KCH / 16; ++k)
                        mma_bf16(acc, smem_desc_swz<SWZ>(sa + 32 * k), smem_desc_swz<SWZ>(sb + 32 * k),
                                 idesc, (ch > 0 || k > 0) ? 1u : 0u);
                    mma_commit(&empty[st]);
                }
                if (ok) mma_commit(&tfull[buf]);
            }
            // every MMA has completed before the tensor memory is freed
            mma_commit(&mdone);
            if (!mbar_wait(&mdone, 0)) atomicExch(&abort_flag, 1);
        }
        __syncwarp();
    } else {  // the epilogue warps
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        for (int j = 0; j < ntiles; ++j) {
            const int buf = j & 1;
            // lane 0 polls; the warp takes one decision (tcgen05.ld needs the whole warp)
            int go = 0;
            if (lane == 0)
                go = mbar_wait(&tfull[buf], (j >> 1) & 1) && !*(volatile int *)&abort_flag;
            go = __shfl_sync(0xffffffffu, go, 0);
            if (!go) {
                if (lane == 0) atomicExch(&abort_flag, 1);
                break;
            }
            tc_fence_after();
            const int m = ((int)blockIdx.x + j * (int)gridDim.x) * 128 + warp * 32 + lane;
            const uint32_t taddr = tmem + lane_base + (uint32_t)(buf * N);
            float acc = 0.f;
#pragma unroll 1
            for (int n0 = 0; n0 < N; n0 += 32) {
                uint32_t r[32];
                tmem_ld32(taddr + n0, r);
                tmem_wait_ld();
                if (n0 + 32 == N) {  // the accumulator is free for the tile after next
                    tc_fence_before();
                    __syncwarp();
                    if (lane == 0) mbar_arrive(&tempty[buf]);
                }
                float v[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
                ep.row(m, n0, v, acc, scratch);
            }
            ep.row_end(m, acc, scratch);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *(volatile int *)&abort_flag) atomicExch(err, 1);
    if (warp == 5) tmem_dealloc(tmem, ncols);
}

// A row-major [rows][K] BF16 operand through a 2-D tensor map (K innermost, box 64 x ROWS).
template <int ROWS>
struct TmaRowMajor {
    static constexpr int kChunk = 64, kSwz = 128;
    static constexpr uint32_t kBytes = ROWS * 128;
    CUtensorMap map;
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int row0, int kp0) const
    {
        tma_load_2d(dst, &map, kp0 * 8, row0, bar);
    }
};

// -- loaders / epilogues for plain row-major GEMMs ----------------------------------------------
struct RowMajorLoader {  // rows x K bf16, leading dimension ld (multiple of 8)
    const __nv_bfloat16 *p;
    int rows, K, ld;
    __device__ __forceinline__ uint4 operator()(int r, int kp) const
    {
        const int k = kp * 8;
        if (r >= rows || k >= K) return make_uint4(0, 0, 0, 0);
        return *reinterpret_cast<const uint4 *>(p + (size_t)r * ld + k);
    }
    __device__ __forceinline__ const void *ptr(int r, int kp) const
    {
        const int k = kp * 8;
        if (r >= rows || k >= K) return nullptr;
        return p + (size_t)r * ld + k;
    }
    __device__ __forceinline__ const void *base() const { return p; }
};

struct StoreF32 {  // D -> row-major FP32 (M x N), bounds checked
    float *c;
    int M, N, ldc;
    __device__ __forceinline__ void operator()(int m, int n, float v) const
    {
        if (m < M && n < N) c[(size_t)m * ldc + n] = v;
    }
};

}  // namespace tc
}  // namespace lentils
