// BF16 tensor-core GEMM on tcgen05 (FP32 accumulation in TMEM): the core of the learned
// preconditioner's convolution kernels, exposed on its own for testing.
//
//   C[M x N] (f32, row-major) = A[M x K] (bf16, row-major) * B[N x K]^T (bf16, row-major)
//
// One CTA of 128 threads computes a 128 x N tile. K advances in chunks of 64: the threads copy
// the A and B chunks from global memory into shared memory in the no-swizzle K-major
// core-matrix layout (8 rows x 16 bytes per core matrix; cores along K 128 bytes apart (LBO),
// 8-row groups 1024 bytes apart (SBO)); one thread then issues four 128 x N x 16 MMAs and a
// commit to an mbarrier, which every thread waits on (bounded) before the next chunk
// overwrites the operands. The accumulator is read back with tcgen05.ld, each warp taking its
// 32 TMEM lanes (rows). A wait that gives up sets *err and the kernel still frees its TMEM.
#include "common.cuh"
#include "tc_common.cuh"

namespace lentils {

constexpr int kTcK = 64;  // K per shared-memory chunk

// Copy a 128-row (or N-row) x 64-column BF16 chunk from row-major global memory (leading
// dimension ld, starting at column k0) into the core-matrix layout; rows beyond `rows` and
// columns beyond K are zero-filled.
__device__ __forceinline__ void load_kmajor_chunk(const __nv_bfloat16 *__restrict__ src, int ld,
                                                  int rows, int K, int k0, int nrows_tile,
                                                  unsigned char *dst)
{
    const int pieces = nrows_tile * (kTcK / 8);  // 16-byte pieces
    for (int p = threadIdx.x; p < pieces; p += blockDim.x) {
        const int r = p / (kTcK / 8), c = p - r * (kTcK / 8);
        const int k = k0 + c * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (r < rows && k + 8 <= K) {
            v = *reinterpret_cast<const uint4 *>(src + (size_t)r * ld + k);
        } else if (r < rows && k < K) {
            unsigned short tmp[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            const unsigned short *s16 = reinterpret_cast<const unsigned short *>(src + (size_t)r * ld);
            for (int e = 0; e < 8 && k + e < K; ++e) tmp[e] = s16[k + e];
            v = *reinterpret_cast<uint4 *>(tmp);
        }
        // core matrix (r/8, c): 8-row groups 1024 B apart, K cores 128 B apart, rows 16 B apart
        *reinterpret_cast<uint4 *>(dst + (r >> 3) * 1024 + c * 128 + (r & 7) * 16) = v;
    }
}

template <int N>
__global__ void __launch_bounds__(128)
    tc_gemm_kernel(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B,
                   float *__restrict__ C, int M, int K, int swap_lbo_sbo, int *err)
{
    static_assert(N % 16 == 0 && N >= 32 && N <= 256, "N");
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *sa = smem;               // 128 x 64 bf16 = 16 KB
    unsigned char *sb = smem + 16384;       // N x 64 bf16
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    const int m0 = blockIdx.x * 128;
    const int warp = threadIdx.x >> 5;
    constexpr uint32_t ncols = (N <= 32) ? 32 : (N <= 64) ? 64 : (N <= 128) ? 128 : 256;

    if (warp == 0) {
        tc::tmem_alloc(&tmem_base, ncols);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        tc::fence_mbar_init();
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = tc::idesc_bf16_f32(128, N);
    const uint32_t lbo = swap_lbo_sbo ? 1024u : 128u;
    const uint32_t sbo = swap_lbo_sbo ? 128u : 1024u;
    bool ok = true;
    uint32_t phase = 0;
    const int nchunks = (K + kTcK - 1) / kTcK;
    for (int ch = 0; ch < nchunks && ok; ++ch) {
        load_kmajor_chunk(A + (size_t)m0 * K, K, min(128, M - m0), K, ch * kTcK, 128, sa);
        load_kmajor_chunk(B, K, N, K, ch * kTcK, N, sb);
        tc::fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0) {
            tc::tc_fence_after();
#pragma unroll
            for (int s = 0; s < kTcK / 16; ++s) {
                const uint64_t ad = tc::smem_desc(tc::smem_u32(sa) + s * 256, lbo, sbo);
                const uint64_t bd = tc::smem_desc(tc::smem_u32(sb) + s * 256, lbo, sbo);
                tc::mma_bf16(tmem, ad, bd, idesc, (ch > 0 || s > 0) ? 1u : 0u);
            }
            tc::mma_commit(&bar);
        }
        ok = tc::mbar_wait(&bar, phase);
        phase ^= 1;
        tc::tc_fence_after();
    }
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    if (ok) {
        const int row = m0 + warp * 32 + (threadIdx.x & 31);
        for (int c0 = 0; c0 < N; c0 += 8) {
            float v[8];
            tc::tmem_ld8(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
            if (row < M)
#pragma unroll
                for (int j = 0; j < 8; ++j) C[(size_t)row * N + c0 + j] = v[j];
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

template <int N>
static int launch_tc_gemm(const void *A, const void *B, float *C, int M, int K, int swap,
                          int *err, cudaStream_t s)
{
    const size_t smem = 16384 + (size_t)N * 128;
    LENTILS_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_kernel<N>,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    tc_gemm_kernel<N><<<(M + 127) / 128, 128, smem, s>>>((const __nv_bfloat16 *)A,
                                                         (const __nv_bfloat16 *)B, C, M, K, swap,
                                                         err);
    LENTILS_CHECK_LAUNCH("tc_gemm_kernel");
    return LENTILS_OK;
}

}  // namespace lentils

using namespace lentils;

extern "C" {

// C = A * B^T with A (M x K) and B (N x K) BF16 row-major on the device and C (M x N) FP32;
// N in {32, 64, 128, 256}, K a multiple of 8. swap_lbo_sbo selects the alternative
// orientation of the shared-memory descriptor offsets (diagnostic). *err_dev (device int) is
// set to 1 if a bounded wait gave up.
int lentils_tc_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K,
                         int swap_lbo_sbo, int *err_dev, void *stream)
{
    clear_error();
    if (!A || !B || !C || !err_dev || M < 1 || K < 8 || (K % 8) != 0)
        return set_error(LENTILS_ERR_INVALID, "tc_gemm_bf16: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    switch (N) {
    case 32: return launch_tc_gemm<32>(A, B, C, M, K, swap_lbo_sbo, err_dev, s);
    case 64: return launch_tc_gemm<64>(A, B, C, M, K, swap_lbo_sbo, err_dev, s);
    case 128: return launch_tc_gemm<128>(A, B, C, M, K, swap_lbo_sbo, err_dev, s);
    case 256: return launch_tc_gemm<256>(A, B, C, M, K, swap_lbo_sbo, err_dev, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "tc_gemm_bf16: N=%d", N);
}

}  // extern "C"
