// The NUFFT operator F = Degrid . rFFT2 . ZeroPad . Apod and its transpose
// F^T = Crop-Apod . irFFT2 . Grid (lentils/operators/fourier_operators.py:96-126), on device
// buffers, in FP32 (the solver's matvec) or FP64 (refinement residuals).
//
//   forward: image (nx, ny) --apod, zero-pad--> padded (nu, nv) --R2C--> grid (nu, nv/2+1)
//            --degrid--> visibilities (plan order)
//   adjoint: visibilities --grid--> grid --Hermitian edge projection, C2R--> padded
//            --crop, apod--> image
//
// The apodisation 1/(sinhc_x outer sinhc_y) (ApodizationCorrectionOperator,
// fourier_operators.py:54-68) is separable and is passed as its two factors. Zero padding
// follows ZeroPaddingOperator (fourier_operators.py:27-52). The FFT normalisations are the
// reference's: rfft2(norm='backward') is cuFFT's unnormalised R2C and irfft2(norm='forward')
// its unnormalised C2R. numpy's irfft2 keeps only the Hermitian part of the columns the last
// axis's real transform treats as self-conjugate (column 0 and, for even nv, column nv/2);
// the adjoint projects those two columns onto their Hermitian part before cuFFT's C2R so the
// result is the same whatever order cuFFT applies its passes in.
#include <cufft.h>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"

struct lentils_nufft {
    const lentils_plan *plan;
    int nx, ny, padx, pady, nu, nv, half_nv;
    int precisions;  // bit 0: FP32 buffers/plans, bit 1: FP64
    float *apx32, *apy32;
    double *apx64, *apy64;
    float *pad32;
    float2 *grid32;
    double *pad64;
    double2 *grid64;
    cufftHandle r2c32, c2r32, d2z64, z2d64;
    bool have32, have64;
};

namespace lentils {

int launch_degrid(const lentils_plan *p, const float2 *grid, float2 *vis, cudaStream_t s,
                  const float *vscale = nullptr);
int launch_grid(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s);
int launch_degrid64(const lentils_plan *p, const double2 *grid, double2 *vis, cudaStream_t s,
                    const double *vscale = nullptr);
int nufft_forward_scaled(lentils_nufft *op, const float *image, float *vis_plan,
                         const float *vscale, void *stream);
int nufft_forward_scaled64(lentils_nufft *op, const double *image, double *vis_plan,
                           const double *vscale, void *stream);
int launch_grid64(const lentils_plan *p, const double2 *vis, double2 *grid, cudaStream_t s);

static int cufft_status(cufftResult r, const char *what)
{
    if (r == CUFFT_SUCCESS) return LENTILS_OK;
    if (r == CUFFT_ALLOC_FAILED) return set_error(LENTILS_ERR_ALLOC, "%s: cuFFT alloc failed", what);
    return set_error(LENTILS_ERR_CUDA, "%s: cuFFT error %d", what, (int)r);
}

#define LENTILS_CUFFT_TRY(expr)                                                   \
    do {                                                                          \
        cufftResult _r = (expr);                                                  \
        if (_r != CUFFT_SUCCESS) return ::lentils::cufft_status(_r, #expr);       \
    } while (0)

static int nblocks(long long n)
{
    long long b = (n + 255) / 256;
    if (b > 152LL * 32) b = 152LL * 32;
    return (int)std::max(1LL, b);
}

// padded[i, j] = apx[i-padx] * apy[j-pady] * img[i-padx, j-pady] inside the image, else 0
template <typename R>
__global__ void apod_pad_kernel(const R *__restrict__ img, R *__restrict__ pad,
                                const R *__restrict__ apx, const R *__restrict__ apy, int nx,
                                int ny, int padx, int pady, int nu, int nv)
{
    pdl_entry();
    const long long total = (long long)nu * nv;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / nv), j = (int)(e - (long long)i * nv);
        const int ii = i - padx, jj = j - pady;
        R v = (R)0;
        if (ii >= 0 && ii < nx && jj >= 0 && jj < ny) v = apx[ii] * apy[jj] * img[(long long)ii * ny + jj];
        pad[e] = v;
    }
}

// img[i, j] (+)= apx[i] * apy[j] * padded[i+padx, j+pady]
template <typename R>
__global__ void crop_apod_kernel(const R *__restrict__ pad, R *__restrict__ img,
                                 const R *__restrict__ apx, const R *__restrict__ apy, int nx,
                                 int ny, int padx, int pady, int nv)
{
    pdl_entry();
    const long long total = (long long)nx * ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / ny), j = (int)(e - (long long)i * ny);
        img[e] = apx[i] * apy[j] * pad[(long long)(i + padx) * nv + (j + pady)];
    }
}

// Hermitian part of the self-conjugate columns (0, and nv/2 when nv is even) along u:
// G[a, c] <- (G[a, c] + conj(G[-a, c])) / 2. One thread per pair (a, nu-a).
template <typename C>
__global__ void hermitian_edges_kernel(C *grid, int nu, int half_nv, int ncols_edge, int last)
{
    pdl_entry();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int pairs = nu / 2 + 1;  // a = 0 .. nu/2 (a and nu-a coincide at 0 and nu/2)
    if (t >= pairs * ncols_edge) return;
    const int col = (t >= pairs) ? last : 0;
    const int a = t % pairs;
    const int b = (nu - a) % nu;
    C *pa = grid + (long long)a * half_nv + col;
    C *pb = grid + (long long)b * half_nv + col;
    const C va = *pa, vb = *pb;
    C h;
    h.x = 0.5 * (va.x + vb.x);
    h.y = 0.5 * (va.y - vb.y);
    *pa = h;
    if (b != a) {
        C hb;
        hb.x = h.x;
        hb.y = -h.y;
        *pb = hb;
    }
}

}  // namespace lentils

using namespace lentils;

static void nufft_free(lentils_nufft *op)
{
    cudaFree(op->apx32);
    cudaFree(op->apy32);
    cudaFree(op->apx64);
    cudaFree(op->apy64);
    cudaFree(op->pad32);
    cudaFree(op->grid32);
    cudaFree(op->pad64);
    cudaFree(op->grid64);
    if (op->have32) {
        cufftDestroy(op->r2c32);
        cufftDestroy(op->c2r32);
    }
    if (op->have64) {
        cufftDestroy(op->d2z64);
        cufftDestroy(op->z2d64);
    }
}

extern "C" {

int lentils_nufft_create(lentils_nufft **out, const lentils_plan *plan, int nx, int ny, int padx,
                         int pady, const double *apod_x, const double *apod_y, int precisions,
                         void *stream)
{
    clear_error();
    if (!out || !plan || !apod_x || !apod_y)
        return set_error(LENTILS_ERR_INVALID, "nufft_create: null argument");
    *out = nullptr;
    if (nx < 1 || ny < 1 || padx < 0 || pady < 0 || (precisions & 3) == 0)
        return set_error(LENTILS_ERR_INVALID, "nufft_create: bad sizes/precisions");
    if (nx + 2 * padx != plan->geom.nu || ny + 2 * pady != plan->geom.nv)
        return set_error(LENTILS_ERR_INVALID,
                         "nufft_create: padded image %dx%d does not match the plan grid %dx%d",
                         nx + 2 * padx, ny + 2 * pady, plan->geom.nu, plan->geom.nv);
    lentils_nufft *op = new (std::nothrow) lentils_nufft();
    if (!op) return set_error(LENTILS_ERR_ALLOC, "nufft_create: host allocation");
    memset(op, 0, sizeof(*op));
    op->plan = plan;
    op->nx = nx;
    op->ny = ny;
    op->padx = padx;
    op->pady = pady;
    op->nu = plan->geom.nu;
    op->nv = plan->geom.nv;
    op->half_nv = plan->geom.half_nv;
    op->precisions = precisions;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t npad = (size_t)op->nu * op->nv, ngrid = (size_t)op->nu * op->half_nv;
    int st = LENTILS_OK;
    auto fail = [&](int code) {
        const int c = lentils_last_error();
        char msg[512];
        strncpy(msg, lentils_last_error_message(), sizeof(msg) - 1);
        msg[sizeof(msg) - 1] = 0;
        nufft_free(op);
        delete op;
        return set_error(c ? c : code, "%s", msg);
    };
    cudaError_t e = cudaSuccess;
    if (precisions & 1) {
        e = cudaMalloc(&op->apx32, sizeof(float) * nx);
        if (e == cudaSuccess) e = cudaMalloc(&op->apy32, sizeof(float) * ny);
        if (e == cudaSuccess) e = cudaMalloc(&op->pad32, sizeof(float) * npad);
        if (e == cudaSuccess) e = cudaMalloc(&op->grid32, sizeof(float2) * ngrid);
        if (e == cudaSuccess) {
            std::vector<float> fx(nx), fy(ny);
            for (int i = 0; i < nx; ++i) fx[i] = (float)apod_x[i];
            for (int j = 0; j < ny; ++j) fy[j] = (float)apod_y[j];
            e = cudaMemcpy(op->apx32, fx.data(), sizeof(float) * nx, cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = cudaMemcpy(op->apy32, fy.data(), sizeof(float) * ny, cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) {
            cuda_status(e, "nufft_create (FP32 buffers)");
            return fail(LENTILS_ERR_CUDA);
        }
        if (cufftPlan2d(&op->r2c32, op->nu, op->nv, CUFFT_R2C) != CUFFT_SUCCESS) {
            set_error(LENTILS_ERR_CUDA, "nufft_create: cufftPlan2d R2C");
            return fail(LENTILS_ERR_CUDA);
        }
        if (cufftPlan2d(&op->c2r32, op->nu, op->nv, CUFFT_C2R) != CUFFT_SUCCESS) {
            cufftDestroy(op->r2c32);
            set_error(LENTILS_ERR_CUDA, "nufft_create: cufftPlan2d C2R");
            return fail(LENTILS_ERR_CUDA);
        }
        op->have32 = true;
    }
    if (precisions & 2) {
        e = cudaMalloc(&op->apx64, sizeof(double) * nx);
        if (e == cudaSuccess) e = cudaMalloc(&op->apy64, sizeof(double) * ny);
        if (e == cudaSuccess) e = cudaMalloc(&op->pad64, sizeof(double) * npad);
        if (e == cudaSuccess) e = cudaMalloc(&op->grid64, sizeof(double2) * ngrid);
        if (e == cudaSuccess)
            e = cudaMemcpy(op->apx64, apod_x, sizeof(double) * nx, cudaMemcpyHostToDevice);
        if (e == cudaSuccess)
            e = cudaMemcpy(op->apy64, apod_y, sizeof(double) * ny, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cuda_status(e, "nufft_create (FP64 buffers)");
            return fail(LENTILS_ERR_CUDA);
        }
        if (cufftPlan2d(&op->d2z64, op->nu, op->nv, CUFFT_D2Z) != CUFFT_SUCCESS) {
            set_error(LENTILS_ERR_CUDA, "nufft_create: cufftPlan2d D2Z");
            return fail(LENTILS_ERR_CUDA);
        }
        if (cufftPlan2d(&op->z2d64, op->nu, op->nv, CUFFT_Z2D) != CUFFT_SUCCESS) {
            cufftDestroy(op->d2z64);
            set_error(LENTILS_ERR_CUDA, "nufft_create: cufftPlan2d Z2D");
            return fail(LENTILS_ERR_CUDA);
        }
        op->have64 = true;
    }
    (void)s;
    (void)st;
    *out = op;
    return LENTILS_OK;
}

int lentils_nufft_destroy(lentils_nufft *op)
{
    clear_error();
    if (!op) return LENTILS_OK;
    nufft_free(op);
    delete op;
    return LENTILS_OK;
}

int lentils_nufft_forward(lentils_nufft *op, const float *image, float *vis_plan, void *stream)
{
    return lentils::nufft_forward_scaled(op, image, vis_plan, nullptr, stream);
}

int lentils_nufft_forward64(lentils_nufft *op, const double *image, double *vis_plan,
                            void *stream)
{
    return lentils::nufft_forward_scaled64(op, image, vis_plan, nullptr, stream);
}

}  // extern "C"

namespace lentils {

// The forward operator with each visibility multiplied by vscale (plan order; null: none),
// folded into the degridding kernel's output.
int nufft_forward_scaled(lentils_nufft *op, const float *image, float *vis_plan,
                         const float *vscale, void *stream)
{
    clear_error();
    if (!op || !op->have32 || !image || !vis_plan)
        return set_error(LENTILS_ERR_INVALID, "nufft_forward: bad arguments (FP32 not created?)");
    cudaStream_t s = (cudaStream_t)stream;
    LENTILS_CUDA_TRY(pdl_launch(apod_pad_kernel<float>, dim3(nblocks((long long)op->nu * op->nv)), dim3(256), 0, s, image, op->pad32, op->apx32, op->apy32, op->nx, op->ny, op->padx, op->pady, op->nu, op->nv));
    LENTILS_CHECK_LAUNCH("apod_pad_kernel");
    LENTILS_CUFFT_TRY(cufftSetStream(op->r2c32, s));
    LENTILS_CUFFT_TRY(cufftExecR2C(op->r2c32, op->pad32, (cufftComplex *)op->grid32));
    return launch_degrid(op->plan, op->grid32, (float2 *)vis_plan, s, vscale);
}

int nufft_forward_scaled64(lentils_nufft *op, const double *image, double *vis_plan,
                           const double *vscale, void *stream)
{
    clear_error();
    if (!op || !op->have64 || !image || !vis_plan)
        return set_error(LENTILS_ERR_INVALID, "nufft_forward64: bad arguments (FP64 not created?)");
    cudaStream_t s = (cudaStream_t)stream;
    LENTILS_CUDA_TRY(pdl_launch(apod_pad_kernel<double>, dim3(nblocks((long long)op->nu * op->nv)), dim3(256), 0, s, image, op->pad64, op->apx64, op->apy64, op->nx, op->ny, op->padx, op->pady, op->nu, op->nv));
    LENTILS_CHECK_LAUNCH("apod_pad_kernel");
    LENTILS_CUFFT_TRY(cufftSetStream(op->d2z64, s));
    LENTILS_CUFFT_TRY(cufftExecD2Z(op->d2z64, op->pad64, (cufftDoubleComplex *)op->grid64));
    return launch_degrid64(op->plan, op->grid64, (double2 *)vis_plan, s, vscale);
}

}  // namespace lentils

extern "C" {

int lentils_nufft_adjoint(lentils_nufft *op, const float *vis_plan, float *image, void *stream)
{
    clear_error();
    if (!op || !op->have32 || !image || !vis_plan)
        return set_error(LENTILS_ERR_INVALID, "nufft_adjoint: bad arguments (FP32 not created?)");
    cudaStream_t s = (cudaStream_t)stream;
    LENTILS_CUDA_TRY(cudaMemsetAsync(op->grid32, 0, sizeof(float2) * (size_t)op->nu * op->half_nv, s));
    if (int st = launch_grid(op->plan, (const float2 *)vis_plan, op->grid32, s)) return st;
    const int ncols = (op->nv % 2 == 0) ? 2 : 1;
    const int pairs = op->nu / 2 + 1;
    LENTILS_CUDA_TRY(pdl_launch(hermitian_edges_kernel<float2>, dim3((pairs * ncols + 255) / 256), dim3(256), 0, s, op->grid32, op->nu, op->half_nv, ncols, op->half_nv - 1));
    LENTILS_CHECK_LAUNCH("hermitian_edges_kernel");
    LENTILS_CUFFT_TRY(cufftSetStream(op->c2r32, s));
    LENTILS_CUFFT_TRY(cufftExecC2R(op->c2r32, (cufftComplex *)op->grid32, op->pad32));
    LENTILS_CUDA_TRY(pdl_launch(crop_apod_kernel<float>, dim3(nblocks((long long)op->nx * op->ny)), dim3(256), 0, s, op->pad32, image, op->apx32, op->apy32, op->nx, op->ny, op->padx, op->pady, op->nv));
    LENTILS_CHECK_LAUNCH("crop_apod_kernel");
    return LENTILS_OK;
}

int lentils_nufft_adjoint64(lentils_nufft *op, const double *vis_plan, double *image,
                            void *stream)
{
    clear_error();
    if (!op || !op->have64 || !image || !vis_plan)
        return set_error(LENTILS_ERR_INVALID, "nufft_adjoint64: bad arguments (FP64 not created?)");
    cudaStream_t s = (cudaStream_t)stream;
    LENTILS_CUDA_TRY(cudaMemsetAsync(op->grid64, 0, sizeof(double2) * (size_t)op->nu * op->half_nv, s));
    if (int st = launch_grid64(op->plan, (const double2 *)vis_plan, op->grid64, s)) return st;
    const int ncols = (op->nv % 2 == 0) ? 2 : 1;
    const int pairs = op->nu / 2 + 1;
    LENTILS_CUDA_TRY(pdl_launch(hermitian_edges_kernel<double2>, dim3((pairs * ncols + 255) / 256), dim3(256), 0, s, op->grid64, op->nu, op->half_nv, ncols, op->half_nv - 1));
    LENTILS_CHECK_LAUNCH("hermitian_edges_kernel");
    LENTILS_CUFFT_TRY(cufftSetStream(op->z2d64, s));
    LENTILS_CUFFT_TRY(cufftExecZ2D(op->z2d64, (cufftDoubleComplex *)op->grid64, op->pad64));
    LENTILS_CUDA_TRY(pdl_launch(crop_apod_kernel<double>, dim3(nblocks((long long)op->nx * op->ny)), dim3(256), 0, s, op->pad64, image, op->apx64, op->apy64, op->nx, op->ny, op->padx, op->pady, op->nv));
    LENTILS_CHECK_LAUNCH("crop_apod_kernel");
    return LENTILS_OK;
}

// FP64 degrid / grid on plan-order buffers (the double-precision operator).
int lentils_degrid64(const lentils_plan *p, const double *grid, double *vis, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!grid || !vis)))
        return set_error(LENTILS_ERR_INVALID, "degrid64: null argument");
    return launch_degrid64(p, (const double2 *)grid, (double2 *)vis, (cudaStream_t)stream);
}

int lentils_grid64(const lentils_plan *p, const double *vis, double *grid, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!grid || !vis)))
        return set_error(LENTILS_ERR_INVALID, "grid64: null argument");
    return launch_grid64(p, (const double2 *)vis, (double2 *)grid, (cudaStream_t)stream);
}

}  // extern "C"
