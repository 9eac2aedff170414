// Blurred covariance F^T C^-1 F as a convolution with the dirty beam, the reference's
// production form of the CG data term (RadioDataset.blurred_covariance_operator,
// lentils/common/data_base.py:115-129, dirty_beam :160-172):
//
//   beam   = NUFFT_beam^T C^-1 1  on the beam space (2nx x 2ny pixels, bounds +-(n dx))
//   FCF x  = crop( irfft2_unscaled( rfft2(roll(beam)) / (2nx 2ny) * rfft2(pad(x)) ) )
//
// i.e. the circular convolution of the zero-padded image (padding n/2 on each side,
// ZeroPaddingOperator, fourier_operators.py:27-52) with the beam rolled so that zero offset
// sits at index 0. The beam itself is computed once by the caller with the NUFFT adjoint;
// this operator keeps its spectrum (FP64 and FP32) and applies the convolution with cuFFT
// (R2C / C2R in FP32 for the CG inner iterations, D2Z / Z2D in FP64 for the refinement).
#include <cufft.h>

#include <algorithm>
#include <new>

#include "common.cuh"

struct lentils_bcb {
    int nx, ny;      // image
    int px, py;      // padded / beam (2 nx, 2 ny)
    int hy;          // py / 2 + 1
    int padx, pady;  // n / 2
    double centre;   // beam at zero offset
    cufftHandle r2c = 0, c2r = 0, d2z = 0, z2d = 0;
    double2 *spec64 = nullptr;  // rfft2(roll(beam)) / (px py)
    float2 *spec32 = nullptr;
    double *real64 = nullptr;   // padded image (px x py)
    float *real32 = nullptr;
    double2 *work64 = nullptr;  // spectrum of the padded image
    float2 *work32 = nullptr;
};

namespace lentils {

static int cufft_status(cufftResult r, const char *what)
{
    return set_error(LENTILS_ERR_CUDA, "%s: cuFFT error %d", what, (int)r);
}

#define LENTILS_CUFFT_TRY(expr)                                                   \
    do {                                                                          \
        cufftResult _r = (expr);                                                  \
        if (_r != CUFFT_SUCCESS) return cufft_status(_r, #expr);                  \
    } while (0)

static int nblk(long long n)
{
    long long b = (n + 255) / 256;
    return (int)std::max(1LL, std::min(b, 152LL * 32));
}

// out (px x py) = roll(beam, (nx, ny)): out[i][j] = beam[(i + nx) % px][(j + ny) % py]
__global__ void roll_kernel(const double *__restrict__ beam, double *__restrict__ out, int px,
                            int py, int sx, int sy)
{
    const long long n = (long long)px * py;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / py), j = (int)(e - (long long)i * py);
        out[e] = beam[(long long)((i + sx) % px) * py + (j + sy) % py];
    }
}

__global__ void scale_spec_kernel(double2 *__restrict__ s64, float2 *__restrict__ s32, long long n,
                                  double scale)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const double2 v = make_double2(s64[e].x * scale, s64[e].y * scale);
        s64[e] = v;
        s32[e] = make_float2((float)v.x, (float)v.y);
    }
}

// padded (px x py) <- image (nx x ny) at offset (padx, pady), zeros elsewhere
template <typename R>
__global__ void pad_kernel(const R *__restrict__ x, R *__restrict__ out, int nx, int ny, int px,
                           int py, int padx, int pady)
{
    const long long n = (long long)px * py;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / py) - padx, j = (int)(e - (long long)(e / py) * py) - pady;
        out[e] = (i >= 0 && i < nx && j >= 0 && j < ny) ? x[(long long)i * ny + j] : (R)0;
    }
}

template <typename C>
__global__ void mul_spec_kernel(C *__restrict__ w, const C *__restrict__ s, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const C a = w[e], b = s[e];
        C o;
        o.x = a.x * b.x - a.y * b.y;
        o.y = a.x * b.y + a.y * b.x;
        w[e] = o;
    }
}

template <typename R>
__global__ void crop_kernel(const R *__restrict__ in, R *__restrict__ out, int nx, int ny, int py,
                            int padx, int pady)
{
    const long long n = (long long)nx * ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / ny), j = (int)(e - (long long)i * ny);
        out[e] = in[(long long)(i + padx) * py + (j + pady)];
    }
}

static void bcb_free(lentils_bcb *op)
{
    if (op->r2c) cufftDestroy(op->r2c);
    if (op->c2r) cufftDestroy(op->c2r);
    if (op->d2z) cufftDestroy(op->d2z);
    if (op->z2d) cufftDestroy(op->z2d);
    cudaFree(op->spec64);
    cudaFree(op->spec32);
    cudaFree(op->real64);
    cudaFree(op->real32);
    cudaFree(op->work64);
    cudaFree(op->work32);
}

static int bcb_init(lentils_bcb *op, const double *beam, cudaStream_t s)
{
    const long long nr = (long long)op->px * op->py, nc = (long long)op->px * op->hy;
    LENTILS_CUDA_TRY(cudaMalloc(&op->spec64, sizeof(double2) * nc));
    LENTILS_CUDA_TRY(cudaMalloc(&op->spec32, sizeof(float2) * nc));
    LENTILS_CUDA_TRY(cudaMalloc(&op->real64, sizeof(double) * nr));
    LENTILS_CUDA_TRY(cudaMalloc(&op->real32, sizeof(float) * nr));
    LENTILS_CUDA_TRY(cudaMalloc(&op->work64, sizeof(double2) * nc));
    LENTILS_CUDA_TRY(cudaMalloc(&op->work32, sizeof(float2) * nc));
    LENTILS_CUFFT_TRY(cufftPlan2d(&op->r2c, op->px, op->py, CUFFT_R2C));
    LENTILS_CUFFT_TRY(cufftPlan2d(&op->c2r, op->px, op->py, CUFFT_C2R));
    LENTILS_CUFFT_TRY(cufftPlan2d(&op->d2z, op->px, op->py, CUFFT_D2Z));
    LENTILS_CUFFT_TRY(cufftPlan2d(&op->z2d, op->px, op->py, CUFFT_Z2D));
    roll_kernel<<<nblk(nr), 256, 0, s>>>(beam, op->real64, op->px, op->py, op->nx, op->ny);
    LENTILS_CHECK_LAUNCH("roll_kernel");
    LENTILS_CUFFT_TRY(cufftSetStream(op->d2z, s));
    LENTILS_CUFFT_TRY(cufftExecD2Z(op->d2z, op->real64, (cufftDoubleComplex *)op->spec64));
    scale_spec_kernel<<<nblk(nc), 256, 0, s>>>(op->spec64, op->spec32, nc, 1.0 / (double)nr);
    LENTILS_CHECK_LAUNCH("scale_spec_kernel");
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&op->centre, beam + (long long)op->nx * op->py + op->ny,
                                     sizeof(double), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    return LENTILS_OK;
}

template <typename R, typename C>
static int bcb_apply_t(lentils_bcb *op, const R *x, R *out, R *real, C *work, const C *spec,
                       cufftHandle fwd, cufftHandle inv, cudaStream_t s)
{
    const long long nr = (long long)op->px * op->py, nc = (long long)op->px * op->hy;
    pad_kernel<R><<<nblk(nr), 256, 0, s>>>(x, real, op->nx, op->ny, op->px, op->py, op->padx,
                                           op->pady);
    LENTILS_CHECK_LAUNCH("pad_kernel");
    LENTILS_CUFFT_TRY(cufftSetStream(fwd, s));
    LENTILS_CUFFT_TRY(cufftSetStream(inv, s));
    if constexpr (sizeof(R) == 4) {
        LENTILS_CUFFT_TRY(cufftExecR2C(fwd, (cufftReal *)real, (cufftComplex *)work));
    } else {
        LENTILS_CUFFT_TRY(cufftExecD2Z(fwd, (cufftDoubleReal *)real, (cufftDoubleComplex *)work));
    }
    mul_spec_kernel<C><<<nblk(nc), 256, 0, s>>>(work, spec, nc);
    LENTILS_CHECK_LAUNCH("mul_spec_kernel");
    if constexpr (sizeof(R) == 4) {
        LENTILS_CUFFT_TRY(cufftExecC2R(inv, (cufftComplex *)work, (cufftReal *)real));
    } else {
        LENTILS_CUFFT_TRY(cufftExecZ2D(inv, (cufftDoubleComplex *)work, (cufftDoubleReal *)real));
    }
    crop_kernel<R><<<nblk((long long)op->nx * op->ny), 256, 0, s>>>(real, out, op->nx, op->ny,
                                                                    op->py, op->padx, op->pady);
    LENTILS_CHECK_LAUNCH("crop_kernel");
    return LENTILS_OK;
}

int bcb_apply32(lentils_bcb *op, const float *x, float *out, cudaStream_t s)
{
    return bcb_apply_t<float, float2>(op, x, out, op->real32, op->work32, op->spec32, op->r2c,
                                      op->c2r, s);
}

int bcb_apply64(lentils_bcb *op, const double *x, double *out, cudaStream_t s)
{
    return bcb_apply_t<double, double2>(op, x, out, op->real64, op->work64, op->spec64, op->d2z,
                                        op->z2d, s);
}

double bcb_centre(const lentils_bcb *op) { return op->centre; }
int bcb_image_size(const lentils_bcb *op) { return op->nx * op->ny; }

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_bcb_create(lentils_bcb **out, const double *beam, int nx, int ny, void *stream)
{
    clear_error();
    if (!out || !beam || nx < 2 || ny < 2 || (nx % 2) || (ny % 2))
        return set_error(LENTILS_ERR_INVALID, "bcb_create: even nx, ny >= 2 and a beam required");
    *out = nullptr;
    lentils_bcb *op = new (std::nothrow) lentils_bcb();
    if (!op) return set_error(LENTILS_ERR_ALLOC, "bcb_create: host allocation");
    op->nx = nx;
    op->ny = ny;
    op->px = 2 * nx;
    op->py = 2 * ny;
    op->hy = op->py / 2 + 1;
    op->padx = nx / 2;
    op->pady = ny / 2;
    const int st = bcb_init(op, beam, (cudaStream_t)stream);
    if (st) {
        bcb_free(op);
        delete op;
        return st;
    }
    *out = op;
    return LENTILS_OK;
}

int lentils_bcb_destroy(lentils_bcb *op)
{
    clear_error();
    if (!op) return LENTILS_OK;
    bcb_free(op);
    delete op;
    return LENTILS_OK;
}

int lentils_bcb_apply(lentils_bcb *op, const float *x, float *out, void *stream)
{
    clear_error();
    if (!op || !x || !out) return set_error(LENTILS_ERR_INVALID, "bcb_apply: null");
    return bcb_apply32(op, x, out, (cudaStream_t)stream);
}

int lentils_bcb_apply64(lentils_bcb *op, const double *x, double *out, void *stream)
{
    clear_error();
    if (!op || !x || !out) return set_error(LENTILS_ERR_INVALID, "bcb_apply64: null");
    return bcb_apply64(op, x, out, (cudaStream_t)stream);
}

double lentils_bcb_centre(const lentils_bcb *op) { return op ? op->centre : 0.0; }

}  // extern "C"
