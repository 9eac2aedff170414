// Tensor-map encoding for the TMA loads of the tcgen05 GEMMs (see tma.cuh).
#include <mutex>

#include "common.cuh"
#include "tma.cuh"

namespace lentils {

using PfnEncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                    const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                    const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static int encoder(PfnEncodeTiled *out)
{
    static PfnEncodeTiled fn = nullptr;
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        LENTILS_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                                          cudaEnableDefault, &q));
        if (q != cudaDriverEntryPointSuccess || !f)
            return set_error(LENTILS_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        fn = (PfnEncodeTiled)f;
    }
    *out = fn;
    return LENTILS_OK;
}

int tma_map_bf16(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                 const uint64_t *strides, const uint32_t *box, int swizzle)
{
    if (swizzle != 64 && swizzle != 128)
        return set_error(LENTILS_ERR_INVALID, "tma_map_bf16: swizzle %d", swizzle);
    if (rank < 1 || rank > 5 || !map || !base || ((uintptr_t)base & 15) != 0)
        return set_error(LENTILS_ERR_INVALID, "tma_map_bf16: rank %d or unaligned base", rank);
    if (box[0] * 2 > (uint32_t)swizzle)
        return set_error(LENTILS_ERR_INVALID, "tma_map_bf16: inner box %u values", box[0]);
    for (int i = 0; i + 1 < rank; ++i)
        if (strides[i] % 16 != 0)
            return set_error(LENTILS_ERR_INVALID, "tma_map_bf16: stride %llu",
                             (unsigned long long)strides[i]);
    PfnEncodeTiled enc;
    if (int st = encoder(&enc)) return st;
    cuuint64_t gd[5], gs[4];
    cuuint32_t bx[5], es[5];
    for (int i = 0; i < rank; ++i) {
        gd[i] = dims[i];
        bx[i] = box[i];
        es[i] = 1;
    }
    for (int i = 0; i + 1 < rank; ++i) gs[i] = strides[i];
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank,
                           const_cast<void *>(base), gd, gs, bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           swizzle == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(LENTILS_ERR_CUDA, "cuTensorMapEncodeTiled: %d", (int)r);
    return LENTILS_OK;
}

}  // namespace lentils
