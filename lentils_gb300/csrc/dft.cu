// Direct Fourier sum (DFTOperator, lentils/operators/fourier_operators.py:130-145, with the
// matrix of dft_matrix_csr, lentils/backend/nufft.c:128-161) as a GPU validator, FP64:
//
//   forward:  V_k = sum_{unmasked p} x_p (cos a_kp + i sin a_kp)
//   adjoint:  x_p = sum_k Re V_k cos a_kp + Im V_k sin a_kp   (the real transpose)
//   a_kp = -2 pi ARCSEC_TO_RADIANS (u_k x_p + v_k y_p),  u = uv[0] ch[0], v = -uv[1] ch[0],
//   x_p = xmin + i dx, y_p = ymin + j dy (pixel p = i ny + j)
//
// Only the first channel enters (the reference's ch_vis = 0). The forward sum walks each image
// row with a complex rotation by the step phase, re-anchored with an exact sincos every 32
// pixels, so its rounding stays at the level of a few ulp of the terms.
#include <math.h>

#include "common.cuh"

namespace lentils {


struct DftGeom {
    int nx, ny;
    double xmin, ymin, dx, dy, ch;
};

__global__ void __launch_bounds__(128)
    dft_forward_kernel(const double *__restrict__ uvw, int nrows, DftGeom g,
                       const unsigned char *__restrict__ mask, const double *__restrict__ img,
                       double2 *__restrict__ vis)
{
    const double c = -2.0 * M_PI * kArcsecToRad;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nrows; k += gridDim.x * blockDim.x) {
        const double u = uvw[3 * k] * g.ch, v = -uvw[3 * k + 1] * g.ch;
        double sr, si;
        sincos(c * v * g.dy, &si, &sr);  // step along a row (j -> j + 1)
        double re = 0.0, im = 0.0;
        for (int i = 0; i < g.nx; ++i) {
            const double x = i * g.dx + g.xmin;
            double pr = 0.0, pi = 0.0;
            for (int j = 0; j < g.ny; ++j) {
                if ((j & 31) == 0) {
                    const double y = j * g.dy + g.ymin;
                    sincos(c * (u * x + v * y), &pi, &pr);
                } else {
                    const double t = pr * sr - pi * si;
                    pi = pr * si + pi * sr;
                    pr = t;
                }
                const long long p = (long long)i * g.ny + j;
                if (!mask[p]) continue;
                re += img[p] * pr;
                im += img[p] * pi;
            }
        }
        vis[k] = make_double2(re, im);
    }
}

__global__ void __launch_bounds__(128)
    dft_adjoint_kernel(const double *__restrict__ uvw, int nrows, DftGeom g,
                       const unsigned char *__restrict__ mask, const double2 *__restrict__ vis,
                       double *__restrict__ img)
{
    const double c = -2.0 * M_PI * kArcsecToRad;
    const long long npix = (long long)g.nx * g.ny;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        if (!mask[p]) {
            img[p] = 0.0;
            continue;
        }
        const int i = (int)(p / g.ny), j = (int)(p - (long long)i * g.ny);
        const double x = i * g.dx + g.xmin, y = j * g.dy + g.ymin;
        double acc = 0.0;
        for (int k = 0; k < nrows; ++k) {
            const double u = uvw[3 * k] * g.ch, v = -uvw[3 * k + 1] * g.ch;
            double s, co;
            sincos(c * (u * x + v * y), &s, &co);
            const double2 vk = vis[k];
            acc += vk.x * co + vk.y * s;
        }
        img[p] = acc;
    }
}

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_dft_forward(const double *uvw, int nrows, const double *channels,
                        const lentils_image_space *im, const unsigned char *mask,
                        const double *image, double *vis, void *stream)
{
    clear_error();
    if (!uvw || nrows < 0 || !channels || !im || !mask || !image || !vis || im->nx < 1 ||
        im->ny < 1)
        return set_error(LENTILS_ERR_INVALID, "dft_forward: bad arguments");
    double ch = 0.0;  // read on the caller's stream, after whatever wrote it there
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&ch, channels, sizeof(double), cudaMemcpyDeviceToHost,
                                     (cudaStream_t)stream));
    LENTILS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    DftGeom g{im->nx, im->ny, im->xmin, im->ymin, im->dx, im->dy, ch};
    const int blocks = std::max(1, std::min((nrows + 127) / 128, 152 * 16));
    dft_forward_kernel<<<blocks, 128, 0, (cudaStream_t)stream>>>(uvw, nrows, g, mask, image,
                                                                 (double2 *)vis);
    LENTILS_CHECK_LAUNCH("dft_forward_kernel");
    return LENTILS_OK;
}

int lentils_dft_adjoint(const double *uvw, int nrows, const double *channels,
                        const lentils_image_space *im, const unsigned char *mask,
                        const double *vis, double *image, void *stream)
{
    clear_error();
    if (!uvw || nrows < 0 || !channels || !im || !mask || !image || !vis || im->nx < 1 ||
        im->ny < 1)
        return set_error(LENTILS_ERR_INVALID, "dft_adjoint: bad arguments");
    double ch = 0.0;  // read on the caller's stream, after whatever wrote it there
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&ch, channels, sizeof(double), cudaMemcpyDeviceToHost,
                                     (cudaStream_t)stream));
    LENTILS_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    DftGeom g{im->nx, im->ny, im->xmin, im->ymin, im->dx, im->dy, ch};
    const long long npix = (long long)im->nx * im->ny;
    const int blocks = (int)std::max(1LL, std::min((npix + 127) / 128, 152LL * 16));
    dft_adjoint_kernel<<<blocks, 128, 0, (cudaStream_t)stream>>>(uvw, nrows, g, mask,
                                                                 (const double2 *)vis, image);
    LENTILS_CHECK_LAUNCH("dft_adjoint_kernel");
    return LENTILS_OK;
}

}  // extern "C"
