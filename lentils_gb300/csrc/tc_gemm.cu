// BF16 tensor-core GEMM entry point (tcgen05, FP32 accumulation in TMEM) on the generic kernels
// of tc_gemm.cuh -- the core of the learned preconditioner's convolutions, exposed for tests:
//   C[M x N] (f32, row-major) = A[M x K] (bf16, row-major) * B[N x K]^T (bf16, row-major)
#include "common.cuh"
#include "tc_gemm.cuh"
#include "tma.cuh"

namespace lentils {

template <int N>
static int launch_tc_gemm(const void *A, const void *B, float *C, int M, int K, int form,
                          int *err, cudaStream_t s)
{
    using namespace tc;
    RowMajorLoader la{(const __nv_bfloat16 *)A, M, K, K};
    RowMajorLoader lb{(const __nv_bfloat16 *)B, N, K, K};
    StoreF32 ep{C, M, N, N};
    const int kpieces = (K + 7) / 8;
    dim3 grid((M + 127) / 128, 1, 1);
    if (form == 2) {
        constexpr int kStages = 4;
        TmaRowMajor<128> ta;
        TmaRowMajor<N> tb;
        const uint64_t da[2] = {(uint64_t)K, (uint64_t)M}, db[2] = {(uint64_t)K, (uint64_t)N};
        const uint64_t stride[1] = {(uint64_t)K * 2};
        const uint32_t ba[2] = {64, 128}, bb[2] = {64, (uint32_t)N};
        if (int st = tma_map_bf16(&ta.map, A, 2, da, stride, ba)) return st;
        if (int st = tma_map_bf16(&tb.map, B, 2, db, stride, bb)) return st;
        const size_t smem = TmaSmem<N, kStages>::kBytes;
        auto kern = gemm_tma_kernel<N, kStages, TmaRowMajor<128>, TmaRowMajor<N>, StoreF32>;
        LENTILS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, kPipeThreads, smem, s>>>(ta, tb, ep, kpieces, kpieces, err);
        LENTILS_CHECK_LAUNCH("tc gemm_tma_kernel");
        return LENTILS_OK;
    }
    if (form == 1) {
        constexpr int kStages = 3;
        const size_t smem = PipeSmem<N, kStages>::kBytes;
        auto kern = gemm_pipe_kernel<N, kStages, RowMajorLoader, RowMajorLoader, StoreF32>;
        LENTILS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<grid, kPipeThreads, smem, s>>>(la, lb, ep, kpieces, kpieces, err);
        LENTILS_CHECK_LAUNCH("tc gemm_pipe_kernel");
        return LENTILS_OK;
    }
    const size_t smem = GemmSmem<N>::kBytes;
    auto kern = gemm_kernel<N, RowMajorLoader, RowMajorLoader, StoreF32>;
    LENTILS_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, 128, smem, s>>>(la, lb, ep, kpieces, kpieces, err);
    LENTILS_CHECK_LAUNCH("tc gemm_kernel");
    return LENTILS_OK;
}

// Self-test of the bounded wait: one CTA allocates tensor memory, waits on an mbarrier that
// nothing arrives on (with a short poll limit), records the timeout like the GEMM kernels do,
// frees its tensor memory and returns.
__global__ void __launch_bounds__(32) tc_timeout_selftest_kernel(int *err, uint32_t limit)
{
    using namespace tc;
    __shared__ uint64_t bar;
    __shared__ uint32_t tmem_base;
    tmem_alloc(&tmem_base, 32);
    tmem_relinquish();
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    tc_fence_before();
    __syncwarp();
    tc_fence_after();
    const bool ok = mbar_wait(&bar, 0, limit);  // phase 0 never completes
    if (!ok && threadIdx.x == 0) atomicExch(err, 1);
    tc_fence_before();
    __syncwarp();
    tmem_dealloc(tmem_base, 32);
}

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_tc_timeout_selftest(int *err_dev, int poll_limit, void *stream)
{
    clear_error();
    if (!err_dev || poll_limit < 1 || poll_limit > (1 << 20))
        return set_error(LENTILS_ERR_INVALID, "tc_timeout_selftest: bad arguments");
    tc_timeout_selftest_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(err_dev, (uint32_t)poll_limit);
    LENTILS_CHECK_LAUNCH("tc_timeout_selftest_kernel");
    return LENTILS_OK;
}

int lentils_tc_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K,
                         int form, int *err_dev, void *stream)
{
    clear_error();
    if (!A || !B || !C || !err_dev || M < 1 || K < 8 || (K % 8) != 0 || form < 0 || form > 2)
        return set_error(LENTILS_ERR_INVALID, "tc_gemm_bf16: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    switch (N) {
    case 32: return launch_tc_gemm<32>(A, B, C, M, K, form, err_dev, s);
    case 64: return launch_tc_gemm<64>(A, B, C, M, K, form, err_dev, s);
    case 128: return launch_tc_gemm<128>(A, B, C, M, K, form, err_dev, s);
    case 256: return launch_tc_gemm<256>(A, B, C, M, K, form, err_dev, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "tc_gemm_bf16: N=%d", N);
}

}  // extern "C"
