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

template <int N, class LA, class LB>
__device__ __forceinline__ void stage_chunk(const LA &la, const LB &lb, int m0, int n0, int kp0,
                                            int kp_end, unsigned char *sa, unsigned char *sb)
{
    for (int p = threadIdx.x; p < 128 * kPiecesPerChunk; p += blockDim.x) {
        const int r = p >> 3, q = p & 7;
        const int kp = kp0 + q;
        const uint4 v = (kp < kp_end) ? la(m0 + r, kp) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4 *>(sa + core_offset(r, q)) = v;
    }
    for (int p = threadIdx.x; p < N * kPiecesPerChunk; p += blockDim.x) {
        const int r = p >> 3, q = p & 7;
        const int kp = kp0 + q;
        const uint4 v = (kp < kp_end) ? lb(n0 + r, kp) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4 *>(sb + core_offset(r, q)) = v;
    }
}

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
        const int row = warp * 32 + (threadIdx.x & 31);
        for (int c0 = 0; c0 < N; c0 += 8) {
            float v[8];
            tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
#pragma unroll
            for (int j = 0; j < 8; ++j) ep(m0 + row, n0 + c0 + j, v[j]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

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
