// Bilinear lens operator L (image pixels <- regular source grid) and its transpose, on device.
//
// The reference builds its lens operators as CSR matrices on the CPU (barycentric Delaunay
// interpolation, lentils/backend/triangles.c:105-140, and rasterised overlaps,
// lentils/backend/raster.c:272-395). The CG source inversion here uses bilinear interpolation
// onto a regular source grid, which has no reference implementation; its definition (and the
// FP64 oracle it is checked against) is: an unmasked image pixel whose deflected position
// (x, y) lies inside the source node lattice (nodes at xmin + j*dx, ymin + k*dy, the pixel
// corners of the reference's ImageSpace.points) interpolates from the four surrounding nodes
// with weights (1-tx)(1-ty), tx(1-ty), (1-tx)ty, tx*ty; other pixels give empty rows.
//
// Storage: L as ELL (4 entries per image pixel, column -1 when absent) for the gather L s;
// L^T as CSR over source nodes, built once by a stable radix sort of the entries by column, so
// L^T r is a deterministic gather (no atomics).
#include <cub/cub.cuh>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"

struct lentils_lensop {
    int nimg;         // image pixels (rows)
    int nsrc;         // source nodes (columns)
    int nnz;          // stored entries of L^T
    int *ell_col;     // 4 * nimg
    double *ell_val64;
    float *ell_val32;
    int *f_ptr;       // general CSR form (nimg + 1; null for the 4-wide bilinear form)
    int *f_col;
    double *f_val64;
    float *f_val32;
    int *t_ptr;       // nsrc + 1
    int *t_row;       // nnz (image pixel of each entry)
    double *t_val64;
    float *t_val32;
};

namespace lentils {

static int blocks_for(long long n)
{
    long long b = (n + 255) / 256;
    if (b > 152LL * 32) b = 152LL * 32;
    return (int)std::max(1LL, b);
}

__global__ void bilinear_build_kernel(const double *__restrict__ pts,
                                      const unsigned char *__restrict__ mask, int nimg, int nsx,
                                      int nsy, double sxmin, double symin, double sdx, double sdy,
                                      int *__restrict__ col, double *__restrict__ v64,
                                      float *__restrict__ v32, unsigned *__restrict__ keys,
                                      int *__restrict__ ids, int *__restrict__ counts)
{
    const int nsrc = nsx * nsy;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nimg;
         p += (long long)gridDim.x * blockDim.x) {
        const double fx = (pts[2 * p] - sxmin) / sdx;
        const double fy = (pts[2 * p + 1] - symin) / sdy;
        bool ok = (mask == nullptr || mask[p] != 0) && isfinite(fx) && isfinite(fy);
        double j0 = 0, k0 = 0;
        if (ok) {
            j0 = floor(fx);
            k0 = floor(fy);
            ok = j0 >= 0 && j0 <= nsx - 2 && k0 >= 0 && k0 <= nsy - 2;
        }
        int c[4] = {-1, -1, -1, -1};
        double w[4] = {0, 0, 0, 0};
        if (ok) {
            const int j = (int)j0, k = (int)k0;
            const double tx = fx - j0, ty = fy - k0;
            c[0] = j * nsy + k;
            c[1] = (j + 1) * nsy + k;
            c[2] = j * nsy + k + 1;
            c[3] = (j + 1) * nsy + k + 1;
            w[0] = (1 - tx) * (1 - ty);
            w[1] = tx * (1 - ty);
            w[2] = (1 - tx) * ty;
            w[3] = tx * ty;
        }
        for (int q = 0; q < 4; ++q) {
            const long long e = 4 * p + q;
            col[e] = c[q];
            v64[e] = w[q];
            v32[e] = (float)w[q];
            keys[e] = (c[q] >= 0) ? (unsigned)c[q] : (unsigned)nsrc;  // absent entries sort last
            ids[e] = (int)e;
            if (c[q] >= 0) atomicAdd(&counts[c[q]], 1);
        }
    }
}

__global__ void transpose_fill_kernel(const int *__restrict__ ids, const double *__restrict__ v64,
                                      int *__restrict__ trow, double *__restrict__ tv64,
                                      float *__restrict__ tv32, int nnz)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nnz;
         i += (long long)gridDim.x * blockDim.x) {
        const int e = ids[i];
        trow[i] = e >> 2;
        tv64[i] = v64[e];
        tv32[i] = (float)v64[e];
    }
}

template <typename R>
__global__ void lens_apply_kernel(const int *__restrict__ col, const R *__restrict__ val,
                                  const R *__restrict__ src, R *__restrict__ img, int nimg)
{
    pdl_entry();
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nimg;
         p += (long long)gridDim.x * blockDim.x) {
        const int4 c = reinterpret_cast<const int4 *>(col)[p];
        R acc = (R)0;
        if (c.x >= 0) acc += val[4 * p + 0] * src[c.x];
        if (c.y >= 0) acc += val[4 * p + 1] * src[c.y];
        if (c.z >= 0) acc += val[4 * p + 2] * src[c.z];
        if (c.w >= 0) acc += val[4 * p + 3] * src[c.w];
        img[p] = acc;
    }
}

template <typename R>
__global__ void lens_apply_csr_kernel(const int *__restrict__ ptr, const int *__restrict__ col,
                                      const R *__restrict__ val, const R *__restrict__ src,
                                      R *__restrict__ img, int nimg)
{
    pdl_entry();
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nimg;
         p += (long long)gridDim.x * blockDim.x) {
        R acc = (R)0;
        for (int e = ptr[p]; e < ptr[p + 1]; ++e) acc += val[e] * src[col[e]];
        img[p] = acc;
    }
}

// CSR entry -> row; per-column counts; FP32 copy of the values
__global__ void csr_rows_kernel(const int *__restrict__ ptr, const int *__restrict__ col,
                                const double *__restrict__ v64, int *__restrict__ rowof,
                                unsigned *__restrict__ keys, int *__restrict__ ids,
                                int *__restrict__ counts, float *__restrict__ v32, int nimg)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < nimg;
         p += (long long)gridDim.x * blockDim.x) {
        for (int e = ptr[p]; e < ptr[p + 1]; ++e) {
            rowof[e] = (int)p;
            keys[e] = (unsigned)col[e];
            ids[e] = e;
            v32[e] = (float)v64[e];
            atomicAdd(&counts[col[e]], 1);
        }
    }
}

__global__ void csr_transpose_fill_kernel(const int *__restrict__ ids, const int *__restrict__ rowof,
                                          const double *__restrict__ v64, int *__restrict__ trow,
                                          double *__restrict__ tv64, float *__restrict__ tv32,
                                          int nnz)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nnz;
         i += (long long)gridDim.x * blockDim.x) {
        const int e = ids[i];
        trow[i] = rowof[e];
        tv64[i] = v64[e];
        tv32[i] = (float)v64[e];
    }
}

// src = L^T img from the transposed CSR: one warp per source node. Row lengths are very uneven
// (no image pixel maps to most of the outer source grid; hundreds do near the critical curves),
// so the lanes stride a row's entries (coalesced loads) and combine with shuffles.
template <typename R>
__global__ void lens_apply_t_kernel(const int *__restrict__ ptr, const int *__restrict__ row,
                                    const R *__restrict__ val, const R *__restrict__ img,
                                    R *__restrict__ src, int nsrc)
{
    pdl_entry();
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long j = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; j < nsrc;
         j += nwarps) {
        R acc = (R)0;
        const int e1 = ptr[j + 1];
        for (int e = ptr[j] + lane; e < e1; e += 32) acc += val[e] * img[row[e]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) src[j] = acc;
    }
}

__global__ void lens_diag_kernel(const int *__restrict__ ptr, const double *__restrict__ val,
                                 double *__restrict__ d, int nsrc)
{
    for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nsrc;
         j += (long long)gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int e = ptr[j]; e < ptr[j + 1]; ++e) acc += val[e] * val[e];
        d[j] = acc;
    }
}

}  // namespace lentils

using namespace lentils;

static void lensop_free(lentils_lensop *op)
{
    cudaFree(op->f_ptr);
    cudaFree(op->f_col);
    cudaFree(op->f_val64);
    cudaFree(op->f_val32);
    cudaFree(op->ell_col);
    cudaFree(op->ell_val64);
    cudaFree(op->ell_val32);
    cudaFree(op->t_ptr);
    cudaFree(op->t_row);
    cudaFree(op->t_val64);
    cudaFree(op->t_val32);
}

extern "C" {

int lentils_lensop_create(lentils_lensop **out, const double *src_points, const unsigned char *mask,
                          int nimg, int nsx, int nsy, double sxmin, double symin, double sdx,
                          double sdy, void *stream)
{
    clear_error();
    if (!out || !src_points || nimg < 1 || nsx < 2 || nsy < 2 || !(sdx > 0) || !(sdy > 0))
        return set_error(LENTILS_ERR_INVALID, "lensop_create: bad arguments");
    *out = nullptr;
    const long long nent = 4LL * nimg;
    if (nent >= (1LL << 31) || (long long)nsx * nsy >= (1LL << 31))
        return set_error(LENTILS_ERR_UNSUPPORTED, "lensop_create: too many entries");
    cudaStream_t s = (cudaStream_t)stream;
    lentils_lensop *op = new (std::nothrow) lentils_lensop();
    if (!op) return set_error(LENTILS_ERR_ALLOC, "lensop_create: host allocation");
    memset(op, 0, sizeof(*op));
    op->nimg = nimg;
    op->nsrc = nsx * nsy;
    unsigned *keys = nullptr, *keys_sorted = nullptr;
    int *ids = nullptr, *ids_sorted = nullptr, *counts = nullptr;
    void *tmp = nullptr;
    int st = LENTILS_OK;
    cudaError_t e = cudaMalloc(&op->ell_col, sizeof(int) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&op->ell_val64, sizeof(double) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&op->ell_val32, sizeof(float) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&op->t_ptr, sizeof(int) * (op->nsrc + 1));
    if (e == cudaSuccess) e = cudaMalloc(&keys, sizeof(unsigned) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&keys_sorted, sizeof(unsigned) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&ids, sizeof(int) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&ids_sorted, sizeof(int) * nent);
    if (e == cudaSuccess) e = cudaMalloc(&counts, sizeof(int) * (op->nsrc + 1));
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * (op->nsrc + 1), s);
    if (e != cudaSuccess) st = cuda_status(e, "lensop_create alloc");
    if (!st) {
        bilinear_build_kernel<<<blocks_for(nimg), 256, 0, s>>>(
            src_points, mask, nimg, nsx, nsy, sxmin, symin, sdx, sdy, op->ell_col, op->ell_val64,
            op->ell_val32, keys, ids, counts);
        e = cudaGetLastError();
        if (e != cudaSuccess) st = cuda_status(e, "bilinear_build_kernel");
    }
    int bits = 1;
    while ((1LL << bits) <= op->nsrc) ++bits;
    size_t tmp_bytes = 0, scan_bytes = 0;
    if (!st) {
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys_sorted, ids, ids_sorted,
                                            (int64_t)nent, 0, bits, s);
        if (e == cudaSuccess)
            e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, counts, op->t_ptr,
                                              op->nsrc + 1, s);
        if (e == cudaSuccess) e = cudaMalloc(&tmp, std::max(tmp_bytes, scan_bytes));
        if (e == cudaSuccess)
            e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_sorted, ids, ids_sorted,
                                                (int64_t)nent, 0, bits, s);
        if (e == cudaSuccess)
            e = cub::DeviceScan::ExclusiveSum(tmp, scan_bytes, counts, op->t_ptr, op->nsrc + 1, s);
        int nnz = 0;
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&nnz, op->t_ptr + op->nsrc, sizeof(int), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) {
            op->nnz = nnz;
            e = cudaMalloc(&op->t_row, sizeof(int) * std::max(1, nnz));
            if (e == cudaSuccess) e = cudaMalloc(&op->t_val64, sizeof(double) * std::max(1, nnz));
            if (e == cudaSuccess) e = cudaMalloc(&op->t_val32, sizeof(float) * std::max(1, nnz));
        }
        if (e == cudaSuccess && nnz > 0) {
            transpose_fill_kernel<<<blocks_for(nnz), 256, 0, s>>>(ids_sorted, op->ell_val64,
                                                                 op->t_row, op->t_val64,
                                                                 op->t_val32, nnz);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_status(e, "lensop_create transpose");
    }
    cudaFree(keys);
    cudaFree(keys_sorted);
    cudaFree(ids);
    cudaFree(ids_sorted);
    cudaFree(counts);
    cudaFree(tmp);
    if (st) {
        lensop_free(op);
        delete op;
        return st;
    }
    *out = op;
    return LENTILS_OK;
}

// A general lens matrix in CSR form (device arrays, copied): nimg rows, nsrc columns, FP64
// values; the transpose is built by a stable sort on the column.
int lentils_lensop_create_csr(lentils_lensop **out, const int *row_ptr, const int *cols,
                              const double *vals, int nimg, int nsrc, int nnz, void *stream)
{
    clear_error();
    if (!out || !row_ptr || (nnz > 0 && (!cols || !vals)) || nimg < 1 || nsrc < 1 || nnz < 0)
        return set_error(LENTILS_ERR_INVALID, "lensop_create_csr: bad arguments");
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    lentils_lensop *op = new (std::nothrow) lentils_lensop();
    if (!op) return set_error(LENTILS_ERR_ALLOC, "lensop_create_csr: host allocation");
    memset(op, 0, sizeof(*op));
    op->nimg = nimg;
    op->nsrc = nsrc;
    op->nnz = nnz;
    const size_t nz = (size_t)std::max(1, nnz);
    unsigned *keys = nullptr, *keys_sorted = nullptr;
    int *ids = nullptr, *ids_sorted = nullptr, *counts = nullptr, *rowof = nullptr;
    void *tmp = nullptr;
    int st = LENTILS_OK;
    cudaError_t e = cudaMalloc(&op->f_ptr, sizeof(int) * (nimg + 1));
    if (e == cudaSuccess) e = cudaMalloc(&op->f_col, sizeof(int) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&op->f_val64, sizeof(double) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&op->f_val32, sizeof(float) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&op->t_ptr, sizeof(int) * (nsrc + 1));
    if (e == cudaSuccess) e = cudaMalloc(&op->t_row, sizeof(int) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&op->t_val64, sizeof(double) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&op->t_val32, sizeof(float) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&keys, sizeof(unsigned) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&keys_sorted, sizeof(unsigned) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&ids, sizeof(int) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&ids_sorted, sizeof(int) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&rowof, sizeof(int) * nz);
    if (e == cudaSuccess) e = cudaMalloc(&counts, sizeof(int) * (nsrc + 1));
    if (e == cudaSuccess) e = cudaMemcpyAsync(op->f_ptr, row_ptr, sizeof(int) * (nimg + 1), cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && nnz > 0)
        e = cudaMemcpyAsync(op->f_col, cols, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && nnz > 0)
        e = cudaMemcpyAsync(op->f_val64, vals, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * (nsrc + 1), s);
    if (e == cudaSuccess) {
        csr_rows_kernel<<<blocks_for(nimg), 256, 0, s>>>(op->f_ptr, op->f_col, op->f_val64, rowof,
                                                         keys, ids, counts, op->f_val32, nimg);
        e = cudaGetLastError();
    }
    int bits = 1;
    while ((1LL << bits) <= nsrc) ++bits;
    size_t tmp_bytes = 0, scan_bytes = 0;
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, keys, keys_sorted, ids, ids_sorted,
                                            (int64_t)nnz, 0, bits, s);
    if (e == cudaSuccess)
        e = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, counts, op->t_ptr, nsrc + 1, s);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, std::max<size_t>(1, std::max(tmp_bytes, scan_bytes)));
    if (e == cudaSuccess && nnz > 0)
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, keys, keys_sorted, ids, ids_sorted,
                                            (int64_t)nnz, 0, bits, s);
    if (e == cudaSuccess)
        e = cub::DeviceScan::ExclusiveSum(tmp, scan_bytes, counts, op->t_ptr, nsrc + 1, s);
    if (e == cudaSuccess && nnz > 0) {
        csr_transpose_fill_kernel<<<blocks_for(nnz), 256, 0, s>>>(ids_sorted, rowof, op->f_val64,
                                                                 op->t_row, op->t_val64,
                                                                 op->t_val32, nnz);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) st = cuda_status(e, "lensop_create_csr");
    cudaFree(keys);
    cudaFree(keys_sorted);
    cudaFree(ids);
    cudaFree(ids_sorted);
    cudaFree(rowof);
    cudaFree(counts);
    cudaFree(tmp);
    if (st) {
        lensop_free(op);
        delete op;
        return st;
    }
    *out = op;
    return LENTILS_OK;
}

int lentils_lensop_destroy(lentils_lensop *op)
{
    clear_error();
    if (!op) return LENTILS_OK;
    lensop_free(op);
    delete op;
    return LENTILS_OK;
}

int lentils_lensop_nnz(const lentils_lensop *op) { return op ? op->nnz : -1; }

int lentils_lensop_apply(const lentils_lensop *op, const float *src, float *img, void *stream)
{
    clear_error();
    if (!op || !src || !img) return set_error(LENTILS_ERR_INVALID, "lensop_apply: null argument");
    if (op->f_ptr)
        LENTILS_CUDA_TRY(pdl_launch(lens_apply_csr_kernel<float>, dim3(blocks_for(op->nimg)), dim3(256), 0, (cudaStream_t)stream, op->f_ptr, op->f_col, op->f_val32, src, img, op->nimg));
    else
        LENTILS_CUDA_TRY(pdl_launch(lens_apply_kernel<float>, dim3(blocks_for(op->nimg)), dim3(256), 0, (cudaStream_t)stream, op->ell_col, op->ell_val32, src, img, op->nimg));
    LENTILS_CHECK_LAUNCH("lens_apply_kernel");
    return LENTILS_OK;
}

int lentils_lensop_apply_t(const lentils_lensop *op, const float *img, float *src, void *stream)
{
    clear_error();
    if (!op || !src || !img) return set_error(LENTILS_ERR_INVALID, "lensop_apply_t: null argument");
    LENTILS_CUDA_TRY(pdl_launch(lens_apply_t_kernel<float>, dim3(blocks_for(32LL * op->nsrc)), dim3(256), 0, (cudaStream_t)stream, op->t_ptr, op->t_row, op->t_val32, img, src, op->nsrc));
    LENTILS_CHECK_LAUNCH("lens_apply_t_kernel");
    return LENTILS_OK;
}

int lentils_lensop_apply64(const lentils_lensop *op, const double *src, double *img, void *stream)
{
    clear_error();
    if (!op || !src || !img) return set_error(LENTILS_ERR_INVALID, "lensop_apply64: null argument");
    if (op->f_ptr)
        LENTILS_CUDA_TRY(pdl_launch(lens_apply_csr_kernel<double>, dim3(blocks_for(op->nimg)), dim3(256), 0, (cudaStream_t)stream, op->f_ptr, op->f_col, op->f_val64, src, img, op->nimg));
    else
        LENTILS_CUDA_TRY(pdl_launch(lens_apply_kernel<double>, dim3(blocks_for(op->nimg)), dim3(256), 0, (cudaStream_t)stream, op->ell_col, op->ell_val64, src, img, op->nimg));
    LENTILS_CHECK_LAUNCH("lens_apply_kernel");
    return LENTILS_OK;
}

int lentils_lensop_apply_t64(const lentils_lensop *op, const double *img, double *src,
                             void *stream)
{
    clear_error();
    if (!op || !src || !img)
        return set_error(LENTILS_ERR_INVALID, "lensop_apply_t64: null argument");
    LENTILS_CUDA_TRY(pdl_launch(lens_apply_t_kernel<double>, dim3(blocks_for(32LL * op->nsrc)), dim3(256), 0, (cudaStream_t)stream, op->t_ptr, op->t_row, op->t_val64, img, src, op->nsrc));
    LENTILS_CHECK_LAUNCH("lens_apply_t_kernel");
    return LENTILS_OK;
}

// diag(L^T L): sum of squared weights per source node (FP64, device output)
int lentils_lensop_diag_ltl(const lentils_lensop *op, double *diag, void *stream)
{
    clear_error();
    if (!op || !diag) return set_error(LENTILS_ERR_INVALID, "lensop_diag_ltl: null argument");
    lens_diag_kernel<<<blocks_for(op->nsrc), 256, 0, (cudaStream_t)stream>>>(op->t_ptr, op->t_val64,
                                                                             diag, op->nsrc);
    LENTILS_CHECK_LAUNCH("lens_diag_kernel");
    return LENTILS_OK;
}

}  // extern "C"
