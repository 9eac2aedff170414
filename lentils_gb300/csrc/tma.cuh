// Host side of the TMA (tensor memory accelerator) loads: tensor maps for BF16 operands in the
// 128-byte swizzled layout the tcgen05 GEMMs read (tc::smem_desc_sw128). The encoder is the
// driver's cuTensorMapEncodeTiled, fetched through the runtime (the library does not link
// libcuda).
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace lentils {

// A BF16 tensor of `rank` (1..5) dimensions, innermost first: dims[i] elements, strides[i]
// bytes between consecutive indices of dimension i + 1 (rank - 1 entries, multiples of 16),
// box[i] elements per load, swizzle 128 or 64 (bytes; box[0] * 2 <= swizzle). Loads outside
// the tensor read zeros.
int tma_map_bf16(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                 const uint64_t *strides, const uint32_t *box, int swizzle = 128);

}  // namespace lentils
