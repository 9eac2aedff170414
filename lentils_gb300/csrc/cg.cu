// Normal-equation operator of the CG source inversion and the iterative-refinement CG solver.
//
//   A s = L^T F^T C^-1 F L s + lambda R^T R s,      b = L^T F^T C^-1 d
//
// L is the bilinear lens operator (lens_ops.cu), F the NUFFT operator (nufft_op.cu), C^-1 the
// per-visibility inverse variances (RadioDataset.covariance_operator,
// lentils/common/data_base.py:36-44) and lambda R^T R the 'gradient' prior of
// PriorCovarianceOperator (lentils/operators/operator_base.py:225-242) with R the forward
// differences of grad_matrix_findiff_csr (lentils/backend/nufft.c:163-194), applied here as a
// matrix-free stencil. The solve restates the reference's CG pattern
// (lentils/tests/solver_tests.py:97-114) as mixed-precision iterative refinement:
//
//   outer (FP64): r = b - A64 x; stop when ||r|| / ||b|| <= tol (the true FP64 residual)
//   inner (FP32 operator, FP64 scalars): Jacobi-preconditioned CG on A e = r to a relative
//          reduction inner_tol; x += e.
//
// Every inner-iteration scalar (alpha, beta, the dot products) lives in device memory, so one
// iteration is a fixed sequence of kernel launches and cuFFT calls that is captured once into a
// CUDA graph and replayed; the host reads the residual norm every `check_every` iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <new>
#include <vector>

#include "common.cuh"
#include "unet.cuh"

namespace lentils {
int nufft_forward_scaled(lentils_nufft *op, const float *image, float *vis_plan,
                         const float *vscale, void *stream);
int nufft_forward_scaled64(lentils_nufft *op, const double *image, double *vis_plan,
                           const double *vscale, void *stream);
int bcb_apply32(lentils_bcb *op, const float *x, float *out, cudaStream_t s);
int bcb_apply64(lentils_bcb *op, const double *x, double *out, cudaStream_t s);
double bcb_centre(const lentils_bcb *op);
int bcb_image_size(const lentils_bcb *op);
}  // namespace lentils

struct lentils_normal_op {
    lentils_lensop *L;
    lentils_nufft *F;
    lentils_bcb *bcb;  // dirty-beam form of F^T C^-1 F (then F is unused)
    int nsx, nsy, nsrc, nimg;
    long long nvis;
    double lambda, idx2, idy2;
    double wsum;
    float *w32;
    double *w64;
    float *img32a, *img32b;
    float2 *vis32;
    double *img64a, *img64b;
    double2 *vis64;
};

namespace lentils {

constexpr int kRedBlocks = 120;  // partial sums per reduction (deterministic two-stage)

static int nb(long long n)
{
    long long b = (n + 255) / 256;
    if (b > 152LL * 32) b = 152LL * 32;
    return (int)std::max(1LL, b);
}

template <typename C, typename R>
__global__ void scale_vis_kernel(C *__restrict__ v, const R *__restrict__ w, long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const R s = w[k];
        C x = v[k];
        x.x *= s;
        x.y *= s;
        v[k] = x;
    }
}

// out (+)= lambda * R^T R s for the forward-difference gradient on an nx x ny grid (x-major).
template <typename R>
__global__ void rtr_kernel(const R *__restrict__ s, R *__restrict__ out, int nx, int ny, R idx2,
                           R idy2, R lam, int accumulate)
{
    pdl_entry();
    const long long n = (long long)nx * ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(e / ny), j = (int)(e - (long long)i * ny);
        const R v = s[e];
        R acc = (R)0;
        if (i >= 1) acc += (v - s[e - ny]) * idx2;
        if (i <= nx - 2) acc -= (s[e + ny] - v) * idx2;
        if (j >= 1) acc += (v - s[e - 1]) * idy2;
        if (j <= ny - 2) acc -= (s[e + 1] - v) * idy2;
        out[e] = (accumulate ? out[e] : (R)0) + lam * acc;
    }
}

__device__ __forceinline__ double block_sum(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;  // valid in thread 0
}

// partial[block] = sum a[i]*b[i] over the block's grid-stride share, accumulated in FP64
template <typename A, typename B>
__global__ void __launch_bounds__(256)
    dot_partial_kernel(const A *__restrict__ a, const B *__restrict__ b, long long n,
                       double *__restrict__ partial)
{
    pdl_entry();
    __shared__ double sh[8];
    double acc = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        acc += (double)a[i] * (double)b[i];
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void sum_partials_kernel(const double *__restrict__ partial, int np,
                                    double *__restrict__ out)
{
    pdl_entry();
    __shared__ double sh[8];
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc += partial[i];
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) *out = t;
}

// Scalars of the inner CG, in device memory.
struct CGScalars {
    double rz, pap, alpha, beta, rr, rz_new, rr0, pad;
};

__global__ void cg_alpha_kernel(const double *__restrict__ partial, int np, CGScalars *sc)
{
    pdl_entry();
    __shared__ double sh[8];
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc += partial[i];
    const double t = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        sc->pap = t;
        sc->alpha = (t != 0.0) ? sc->rz / t : 0.0;
    }
}

// e += alpha p; r -= alpha Ap; z = minv * r; partials of r.z and r.r
__global__ void __launch_bounds__(256)
    cg_update_kernel(float *__restrict__ e, float *__restrict__ r, float *__restrict__ z,
                     const float *__restrict__ p, const float *__restrict__ ap,
                     const float *__restrict__ minv, const CGScalars *__restrict__ sc, int n,
                     double *__restrict__ partial)
{
    pdl_entry();
    __shared__ double sh[8];
    const float alpha = (float)sc->alpha;
    double rz = 0.0, rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        e[i] = fmaf(alpha, p[i], e[i]);
        const float ri = fmaf(-alpha, ap[i], r[i]);
        r[i] = ri;
        const float zi = minv ? ri * minv[i] : ri;
        z[i] = zi;
        rz += (double)ri * (double)zi;
        rr += (double)ri * (double)ri;
    }
    const double a = block_sum(rz, sh);
    const double b = block_sum(rr, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = a;
        partial[gridDim.x + blockIdx.x] = b;
    }
}

__global__ void cg_beta_kernel(const double *__restrict__ partial, int np, CGScalars *sc)
{
    pdl_entry();
    __shared__ double sh[8];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        a += partial[i];
        b += partial[np + i];
    }
    const double ta = block_sum(a, sh);
    const double tb = block_sum(b, sh);
    if (threadIdx.x == 0) {
        sc->beta = (sc->rz != 0.0) ? ta / sc->rz : 0.0;
        sc->rz_new = ta;
        sc->rz = ta;
        sc->rr = tb;
    }
}

__global__ void cg_p_kernel(float *__restrict__ p, const float *__restrict__ z,
                            const CGScalars *__restrict__ sc, int n)
{
    pdl_entry();
    const float beta = (float)sc->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = fmaf(beta, p[i], z[i]);
}

// start of an inner solve: r32 = (float) r64, e = 0, z = minv r, p = z, partial sums of r.z, r.r
__global__ void cg_start_kernel(const double *__restrict__ r64, float *__restrict__ r,
                                float *__restrict__ e, float *__restrict__ z,
                                float *__restrict__ p, const float *__restrict__ minv, int n,
                                double *__restrict__ partial)
{
    pdl_entry();
    __shared__ double sh[8];
    double rz = 0.0, rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float ri = (float)r64[i];
        r[i] = ri;
        e[i] = 0.f;
        const float zi = minv ? ri * minv[i] : ri;
        z[i] = zi;
        p[i] = zi;
        rz += (double)ri * (double)zi;
        rr += (double)ri * (double)ri;
    }
    const double a = block_sum(rz, sh);
    const double b = block_sum(rr, sh);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = a;
        partial[gridDim.x + blockIdx.x] = b;
    }
}

__global__ void cg_start_finish_kernel(const double *__restrict__ partial, int np, CGScalars *sc)
{
    pdl_entry();
    __shared__ double sh[8];
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        a += partial[i];
        b += partial[np + i];
    }
    const double ta = block_sum(a, sh);
    const double tb = block_sum(b, sh);
    if (threadIdx.x == 0) {
        sc->rz = ta;
        sc->rr = tb;
        sc->rr0 = tb;
    }
}

// x64 += e32 ; r64 = b - ax64 handled separately
__global__ void add_f32_to_f64_kernel(double *__restrict__ x, const float *__restrict__ e, int n)
{
    pdl_entry();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] += (double)e[i];
}

__global__ void sub_kernel(const double *__restrict__ b, const double *__restrict__ a,
                           double *__restrict__ r, int n)
{
    pdl_entry();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        r[i] = b[i] - a[i];
}

__global__ void jacobi_kernel(const double *__restrict__ dltl, double wsum, double lam,
                              double idx2, double idy2, int nx, int ny, double *__restrict__ inv,
                              float *__restrict__ inv32)
{
    const int n = nx * ny;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const int i = e / ny, j = e - i * ny;
        const double drtr = idx2 * ((i >= 1) + (i <= nx - 2)) + idy2 * ((j >= 1) + (j <= ny - 2));
        const double d = wsum * dltl[e] + lam * drtr;
        const double v = (d > 0.0) ? 1.0 / d : 1.0;
        if (inv) inv[e] = v;
        if (inv32) inv32[e] = (float)v;
    }
}

// -- flexible CG (learned preconditioner) --------------------------------------------------------
struct FCGScalars {
    double pap, pr, alpha, beta, rr, rr0, use_net, fallbacks, net_iters, pad;
};

__global__ void fcg_rr_kernel(const double *__restrict__ partial, int np, FCGScalars *sc, int start)
{
    pdl_entry();
    __shared__ double sh[8];
    double a = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) a += partial[i];
    const double t = block_sum(a, sh);
    if (threadIdx.x == 0) {
        sc->rr = t;
        if (start) sc->rr0 = t;
    }
}

// Truncated flexible CG keeps the last `m` directions P[j] and their images Q[j] = A P[j]
// (ring buffers, fixed device addresses so that one iteration replays as a CUDA graph; the
// ring position lives in device memory).
constexpr int kMaxWindow = 8;
struct FCGWindow {
    double pq[kMaxWindow];    // P[j] . Q[j]
    double beta[kMaxWindow];  // coefficients of the current orthogonalisation
    int slot, count, m, pad;
};

// start of an inner solve: r32 = (float) r64, e = p = ap = 0; partials of r.r
__global__ void __launch_bounds__(256)
    fcg_start_kernel(const double *__restrict__ r64, float *__restrict__ r, float *__restrict__ e,
                     float *__restrict__ p, float *__restrict__ ap, int n,
                     double *__restrict__ partial)
{
    pdl_entry();
    __shared__ double sh[8];
    double rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float ri = (float)r64[i];
        r[i] = ri;
        e[i] = 0.f;
        p[i] = 0.f;
        ap[i] = 0.f;
        rr += (double)ri * (double)ri;
    }
    const double t = block_sum(rr, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// -- fused flexible-CG steps: grid-wide passes whose last block finishes the reduction ----------
// Each block writes its FP64 partials; the block that arrives last (atomic counter, reset by it
// for the next replay) sums them in block order and derives the step's scalars, so one
// iteration needs three launches besides the matvec instead of nine. Nothing waits on another
// block. Per element the arithmetic is that of the separate kernels.
constexpr int kFusedRows = 24;  // partial rows: K1 2, K2 1 + window, select 1 + 2 x window

// thread 0 (after writing its block's partials) learns whether its block arrived last
__device__ __forceinline__ bool arrive_last(unsigned *counter, int *flag)
{
    if (threadIdx.x == 0) {
        __threadfence();
        *flag = (atomicAdd(counter, 1u) == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    return *flag != 0;
}

// sum of row k of the partials, in block order (valid in thread 0 of the last block)
__device__ __forceinline__ double sum_row(const double *part, int k, double *sh)
{
    double a = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) a += __ldcg(&part[k * gridDim.x + i]);
    return block_sum(a, sh);
}

// K1: p.ap and p.r; the last block sets pap, pr and alpha = p.r / p.ap
__global__ void __launch_bounds__(256)
    fcg_alpha_fused_kernel(const float *__restrict__ p, const float *__restrict__ ap,
                           const float *__restrict__ r, int n, double *__restrict__ part,
                           unsigned *__restrict__ counter, FCGScalars *__restrict__ sc)
{
    pdl_entry();
    __shared__ double sh[8];
    __shared__ int last;
    double a = 0.0, b = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        a += (double)p[i] * (double)ap[i];
        b += (double)p[i] * (double)r[i];
    }
    const double ta = block_sum(a, sh), tb = block_sum(b, sh);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = ta;
        part[gridDim.x + blockIdx.x] = tb;
    }
    if (!arrive_last(counter, &last)) return;
    const double A = sum_row(part, 0, sh), B = sum_row(part, 1, sh);
    if (threadIdx.x == 0) {
        sc->pap = A;
        sc->pr = B;
        sc->alpha = (A != 0.0) ? B / A : 0.0;
        *counter = 0u;
    }
}

// beta_j = -(d.Q[j]) / pq[j] over the valid window entries, then the ring advances
__device__ __forceinline__ void window_finish(const double *dots, int valid, int first,
                                              FCGWindow *win)
{
    const int m = win->m;
    for (int j = 0; j < kMaxWindow; ++j)
        win->beta[j] = (j < valid && win->pq[j] != 0.0) ? -dots[j] / win->pq[j] : 0.0;
    if (first) {
        win->count = 0;
        win->slot = 0;
    } else {
        win->count = valid;
        win->slot = (win->slot + 1) % m;
    }
}

// K2: e += alpha p, r -= alpha ap, r.r, P[slot] = p, Q[slot] = ap; with_dir: the window dots of
// the Jacobi direction d = dinv r (not stored). The last block sets rr and pq[slot] and, with_dir,
// the window coefficients.
__global__ void __launch_bounds__(256)
    fcg_update_fused_kernel(float *__restrict__ e, float *__restrict__ r,
                            const float *__restrict__ p, const float *__restrict__ ap,
                            float *__restrict__ P, float *__restrict__ Q,
                            const float *__restrict__ dinv, int n, FCGScalars *__restrict__ sc,
                            FCGWindow *__restrict__ win, double *__restrict__ part,
                            unsigned *__restrict__ counter, int with_dir)
{
    pdl_entry();
    __shared__ double sh[8];
    __shared__ int last;
    const float alpha = (float)sc->alpha;
    const int slot = win->slot;
    const int valid = with_dir ? min(win->count + 1, win->m) : 0;
    float *ps = P + (size_t)slot * n;
    float *qs = Q + (size_t)slot * n;
    double rr = 0.0, acc[kMaxWindow];
#pragma unroll
    for (int j = 0; j < kMaxWindow; ++j) acc[j] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float pi = p[i], api = ap[i];
        e[i] = fmaf(alpha, pi, e[i]);
        const float ri = fmaf(-alpha, api, r[i]);
        r[i] = ri;
        rr += (double)ri * (double)ri;
        ps[i] = pi;
        qs[i] = api;
        if (valid > 0) {
            const double di = (double)(dinv[i] * ri);
#pragma unroll
            for (int j = 0; j < kMaxWindow; ++j)
                if (j < valid) acc[j] += di * (double)((j == slot) ? api : Q[(size_t)j * n + i]);
        }
    }
    const double t = block_sum(rr, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    for (int j = 0; j < valid; ++j) {
        const double tj = block_sum(acc[j], sh);
        if (threadIdx.x == 0) part[(1 + j) * gridDim.x + blockIdx.x] = tj;
    }
    if (!arrive_last(counter, &last)) return;
    const double R = sum_row(part, 0, sh);
    double dots[kMaxWindow];
    for (int j = 0; j < valid; ++j) dots[j] = sum_row(part, 1 + j, sh);
    if (threadIdx.x == 0) {
        sc->rr = R;
        win->pq[slot] = sc->pap;
        if (with_dir) window_finish(dots, valid, 0, win);
        *counter = 0u;
    }
}

// The direction choice with the network's z (z may be null: Jacobi only): partials of z.r and
// of the window dots of both candidates, z and d = dinv r; the last block keeps z where it
// descends (z.r > 0; counted in sc), else d, and sets the window coefficients. first: start of
// an inner solve (empty window).
__global__ void __launch_bounds__(256)
    fcg_select_fused_kernel(const float *__restrict__ z, const float *__restrict__ r,
                            const float *__restrict__ dinv, const float *__restrict__ Q, int n,
                            FCGScalars *__restrict__ sc, FCGWindow *__restrict__ win,
                            double *__restrict__ part, unsigned *__restrict__ counter, int first)
{
    pdl_entry();
    __shared__ double sh[8];
    __shared__ int last;
    const int valid = first ? 0 : min(win->count + 1, win->m);
    double zr = 0.0, az[kMaxWindow], aj[kMaxWindow];
#pragma unroll
    for (int j = 0; j < kMaxWindow; ++j) az[j] = aj[j] = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float ri = r[i];
        const double ji = (double)(dinv[i] * ri);
        const double zi = z ? (double)z[i] : 0.0;
        zr += zi * (double)ri;
#pragma unroll
        for (int j = 0; j < kMaxWindow; ++j)
            if (j < valid) {
                const double q = (double)Q[(size_t)j * n + i];
                az[j] += zi * q;
                aj[j] += ji * q;
            }
    }
    const double t = block_sum(zr, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
    for (int j = 0; j < valid; ++j) {
        const double a = block_sum(az[j], sh), b = block_sum(aj[j], sh);
        if (threadIdx.x == 0) {
            part[(1 + j) * gridDim.x + blockIdx.x] = a;
            part[(1 + kMaxWindow + j) * gridDim.x + blockIdx.x] = b;
        }
    }
    if (!arrive_last(counter, &last)) return;
    const double ZR = sum_row(part, 0, sh);
    __shared__ int use_z;
    if (threadIdx.x == 0) {
        const bool ok = z && ZR > 0.0 && ZR < 1e300;
        if (z) {
            sc->use_net = ok ? 1.0 : 0.0;
            if (ok) sc->net_iters += 1.0;
            else sc->fallbacks += 1.0;
        } else {
            sc->use_net = 0.0;
        }
        use_z = ok ? 1 : 0;
    }
    __syncthreads();
    double dots[kMaxWindow];
    for (int j = 0; j < valid; ++j) dots[j] = sum_row(part, (use_z ? 1 : 1 + kMaxWindow) + j, sh);
    if (threadIdx.x == 0) {
        window_finish(dots, valid, first, win);
        *counter = 0u;
    }
}

// K3: p = d + sum_j beta_j P[j], d = z where the network's direction was kept, else dinv r
__global__ void __launch_bounds__(256)
    fcg_p_fused_kernel(float *__restrict__ p, const float *__restrict__ z,
                       const float *__restrict__ r, const float *__restrict__ dinv,
                       const float *__restrict__ P, const FCGScalars *__restrict__ sc,
                       const FCGWindow *__restrict__ win, int n)
{
    pdl_entry();
    __shared__ float beta[kMaxWindow];
    const int m = win->m;
    if (threadIdx.x < kMaxWindow) beta[threadIdx.x] = (threadIdx.x < m) ? (float)win->beta[threadIdx.x] : 0.f;
    __syncthreads();
    const bool zdir = z && sc->use_net != 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float v = zdir ? z[i] : dinv[i] * r[i];
        for (int j = 0; j < m; ++j) v = fmaf(beta[j], P[(size_t)j * n + i], v);
        p[i] = v;
    }
}

static double host_dot64(const double *a, const double *b, int n, double *partial, double *out,
                         cudaStream_t s)
{
    LENTILS_CUDA_TRY(pdl_launch(dot_partial_kernel<double, double>, dim3(kRedBlocks), dim3(256), 0, s, a, b, n, partial));
    LENTILS_CUDA_TRY(pdl_launch(sum_partials_kernel, dim3(1), dim3(256), 0, s, partial, kRedBlocks, out));
    double h = 0.0;
    cudaMemcpyAsync(&h, out, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return h;
}

// r = b - A x in FP64. A zero x (the usual start) needs no matvec, whose FP64 form costs
// about twenty FP32 ones: r = b.
static int initial_residual(lentils_normal_op *op, const double *b, const double *x,
                            double *ax64, double *r64, int n, double *partial, double *scal,
                            cudaStream_t s)
{
    if (host_dot64(x, x, n, partial, scal, s) == 0.0) {
        LENTILS_CUDA_TRY(cudaMemcpyAsync(r64, b, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        return LENTILS_OK;
    }
    if (int st = lentils_normal_op_apply64(op, x, ax64, s)) return st;
    LENTILS_CUDA_TRY(pdl_launch(sub_kernel, dim3(nb(n)), dim3(256), 0, s, b, ax64, r64, n));
    LENTILS_CHECK_LAUNCH("sub_kernel");
    return LENTILS_OK;
}

}  // namespace lentils

using namespace lentils;

static void normal_op_free(lentils_normal_op *op)
{
    cudaFree(op->w32);
    cudaFree(op->w64);
    cudaFree(op->img32a);
    cudaFree(op->img32b);
    cudaFree(op->vis32);
    cudaFree(op->img64a);
    cudaFree(op->img64b);
    cudaFree(op->vis64);
}

extern "C" {

// weights_plan: C^-1 per visibility in plan order (device, f64). nimg = image pixels of L.
int lentils_normal_op_create(lentils_normal_op **out, lentils_lensop *L, lentils_nufft *F,
                             const double *weights_plan, long long nvis, int nimg, int nsx,
                             int nsy, double src_dx, double src_dy, double lambda, void *stream)
{
    clear_error();
    if (!out || !L || !F || !weights_plan || nvis < 0 || nimg < 1 || nsx < 1 || nsy < 1 ||
        !(src_dx > 0) || !(src_dy > 0))
        return set_error(LENTILS_ERR_INVALID, "normal_op_create: bad arguments");
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    lentils_normal_op *op = new (std::nothrow) lentils_normal_op();
    if (!op) return set_error(LENTILS_ERR_ALLOC, "normal_op_create: host allocation");
    memset(op, 0, sizeof(*op));
    op->L = L;
    op->F = F;
    op->nsx = nsx;
    op->nsy = nsy;
    op->nsrc = nsx * nsy;
    op->nimg = nimg;
    op->nvis = nvis;
    op->lambda = lambda;
    op->idx2 = 1.0 / (src_dx * src_dx);
    op->idy2 = 1.0 / (src_dy * src_dy);
    const size_t nv = (size_t)std::max(1LL, nvis);
    cudaError_t e = cudaMalloc(&op->w32, sizeof(float) * nv);
    if (e == cudaSuccess) e = cudaMalloc(&op->w64, sizeof(double) * nv);
    if (e == cudaSuccess) e = cudaMalloc(&op->img32a, sizeof(float) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->img32b, sizeof(float) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->vis32, sizeof(float2) * nv);
    if (e == cudaSuccess) e = cudaMalloc(&op->img64a, sizeof(double) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->img64b, sizeof(double) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->vis64, sizeof(double2) * nv);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(op->w64, weights_plan, sizeof(double) * nvis, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) {
        const int st = cuda_status(e, "normal_op_create");
        normal_op_free(op);
        delete op;
        return st;
    }
    // FP32 copy of the weights and their sum (the dirty-beam peak) for the Jacobi scaling
    {
        std::vector<double> hw(nvis);
        e = cudaMemcpyAsync(hw.data(), weights_plan, sizeof(double) * nvis, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        std::vector<float> hf(nvis);
        double sum = 0.0;
        for (long long k = 0; k < nvis; ++k) {
            hf[k] = (float)hw[k];
            sum += hw[k];
        }
        op->wsum = sum;
        if (e == cudaSuccess)
            e = cudaMemcpy(op->w32, hf.data(), sizeof(float) * nvis, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            const int st = cuda_status(e, "normal_op_create weights");
            normal_op_free(op);
            delete op;
            return st;
        }
    }
    *out = op;
    return LENTILS_OK;
}

// The same operator with the dirty-beam form of the data term: A = L^T B L + lambda R^T R with
// B the blurred covariance (lentils_bcb); no visibilities in the matvec.
int lentils_normal_op_create_bcb(lentils_normal_op **out, lentils_lensop *L, lentils_bcb *B,
                                 int nimg, int nsx, int nsy, double src_dx, double src_dy,
                                 double lambda, void *stream)
{
    clear_error();
    if (!out || !L || !B || nimg < 1 || nsx < 1 || nsy < 1 || !(src_dx > 0) || !(src_dy > 0))
        return set_error(LENTILS_ERR_INVALID, "normal_op_create_bcb: bad arguments");
    if (bcb_image_size(B) != nimg)
        return set_error(LENTILS_ERR_INVALID, "normal_op_create_bcb: beam image %d != %d pixels",
                         bcb_image_size(B), nimg);
    (void)stream;
    *out = nullptr;
    lentils_normal_op *op = new (std::nothrow) lentils_normal_op();
    if (!op) return set_error(LENTILS_ERR_ALLOC, "normal_op_create_bcb: host allocation");
    memset(op, 0, sizeof(*op));
    op->L = L;
    op->bcb = B;
    op->nsx = nsx;
    op->nsy = nsy;
    op->nsrc = nsx * nsy;
    op->nimg = nimg;
    op->lambda = lambda;
    op->idx2 = 1.0 / (src_dx * src_dx);
    op->idy2 = 1.0 / (src_dy * src_dy);
    op->wsum = bcb_centre(B);  // diagonal of B: the beam at zero offset
    cudaError_t e = cudaMalloc(&op->img32a, sizeof(float) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->img32b, sizeof(float) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->img64a, sizeof(double) * nimg);
    if (e == cudaSuccess) e = cudaMalloc(&op->img64b, sizeof(double) * nimg);
    if (e != cudaSuccess) {
        const int st = cuda_status(e, "normal_op_create_bcb");
        normal_op_free(op);
        delete op;
        return st;
    }
    *out = op;
    return LENTILS_OK;
}

// b = L^T d_img in FP64 for an image-plane data vector (the dirty image F^T C^-1 d)
int lentils_normal_op_rhs_image64(lentils_normal_op *op, const double *d_img, double *b,
                                  void *stream)
{
    clear_error();
    if (!op || !d_img || !b) return set_error(LENTILS_ERR_INVALID, "normal_op_rhs_image64: null");
    return lentils_lensop_apply_t64(op->L, d_img, b, stream);
}

int lentils_normal_op_destroy(lentils_normal_op *op)
{
    clear_error();
    if (!op) return LENTILS_OK;
    normal_op_free(op);
    delete op;
    return LENTILS_OK;
}

int lentils_normal_op_apply(lentils_normal_op *op, const float *s_in, float *out, void *stream)
{
    clear_error();
    if (!op || !s_in || !out) return set_error(LENTILS_ERR_INVALID, "normal_op_apply: null");
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if ((st = lentils_lensop_apply(op->L, s_in, op->img32a, stream))) return st;
    if (op->bcb) {
        if ((st = bcb_apply32(op->bcb, op->img32a, op->img32b, s))) return st;
    } else {
        // C^-1 F L s, the data weights applied by the degridding kernel
        if ((st = nufft_forward_scaled(op->F, op->img32a, (float *)op->vis32, op->w32, stream)))
            return st;
        if ((st = lentils_nufft_adjoint(op->F, (const float *)op->vis32, op->img32b, stream)))
            return st;
    }
    if ((st = lentils_lensop_apply_t(op->L, op->img32b, out, stream))) return st;
    LENTILS_CUDA_TRY(pdl_launch(rtr_kernel<float>, dim3(nb(op->nsrc)), dim3(256), 0, s, s_in, out, op->nsx, op->nsy, (float)op->idx2,
                                                   (float)op->idy2, (float)op->lambda, 1));
    LENTILS_CHECK_LAUNCH("rtr_kernel");
    return LENTILS_OK;
}

int lentils_normal_op_apply64(lentils_normal_op *op, const double *s_in, double *out,
                              void *stream)
{
    clear_error();
    if (!op || !s_in || !out) return set_error(LENTILS_ERR_INVALID, "normal_op_apply64: null");
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if ((st = lentils_lensop_apply64(op->L, s_in, op->img64a, stream))) return st;
    if (op->bcb) {
        if ((st = bcb_apply64(op->bcb, op->img64a, op->img64b, s))) return st;
    } else {
        if ((st = nufft_forward_scaled64(op->F, op->img64a, (double *)op->vis64, op->w64,
                                         stream)))
            return st;
        if ((st = lentils_nufft_adjoint64(op->F, (const double *)op->vis64, op->img64b, stream)))
            return st;
    }
    if ((st = lentils_lensop_apply_t64(op->L, op->img64b, out, stream))) return st;
    LENTILS_CUDA_TRY(pdl_launch(rtr_kernel<double>, dim3(nb(op->nsrc)), dim3(256), 0, s, s_in, out, op->nsx, op->nsy, op->idx2,
                                                    op->idy2, op->lambda, 1));
    LENTILS_CHECK_LAUNCH("rtr_kernel");
    return LENTILS_OK;
}

// b = L^T F^T C^-1 d in FP64; d: plan-order plan-frame visibilities (c128, device)
int lentils_normal_op_rhs64(lentils_normal_op *op, const double *d_plan, double *b, void *stream)
{
    clear_error();
    if (!op || !d_plan || !b) return set_error(LENTILS_ERR_INVALID, "normal_op_rhs64: null");
    if (op->bcb)
        return set_error(LENTILS_ERR_INVALID,
                         "normal_op_rhs64: dirty-beam operator; use normal_op_rhs_image64");
    cudaStream_t s = (cudaStream_t)stream;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(op->vis64, d_plan, sizeof(double2) * op->nvis,
                                     cudaMemcpyDeviceToDevice, s));
    scale_vis_kernel<double2, double><<<nb(op->nvis), 256, 0, s>>>(op->vis64, op->w64, op->nvis);
    LENTILS_CHECK_LAUNCH("scale_vis_kernel");
    int st;
    if ((st = lentils_nufft_adjoint64(op->F, (const double *)op->vis64, op->img64b, stream)))
        return st;
    return lentils_lensop_apply_t64(op->L, op->img64b, b, stream);
}

// inverse Jacobi diagonal: 1 / (wsum * diag(L^T L) + lambda * diag(R^T R)); either output may
// be null.
int lentils_normal_op_jacobi(lentils_normal_op *op, double *inv_diag, float *inv_diag32,
                             void *stream)
{
    clear_error();
    if (!op) return set_error(LENTILS_ERR_INVALID, "normal_op_jacobi: null");
    cudaStream_t s = (cudaStream_t)stream;
    double *d = nullptr;
    LENTILS_CUDA_TRY(cudaMalloc(&d, sizeof(double) * op->nsrc));
    int st = lentils_lensop_diag_ltl(op->L, d, stream);
    if (!st) {
        jacobi_kernel<<<nb(op->nsrc), 256, 0, s>>>(d, op->wsum, op->lambda, op->idx2, op->idy2,
                                                   op->nsx, op->nsy, inv_diag, inv_diag32);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_status(e, "jacobi_kernel");
    }
    cudaFree(d);
    return st;
}

double lentils_normal_op_weight_sum(const lentils_normal_op *op) { return op ? op->wsum : 0.0; }

int lentils_cg_solve(lentils_normal_op *op, const double *b, double *x, const float *inv_diag32,
                     const lentils_cg_options *opt, lentils_cg_result *res, void *stream)
{
    clear_error();
    if (!op || !b || !x || !opt || !res) return set_error(LENTILS_ERR_INVALID, "cg_solve: null");
    memset(res, 0, sizeof(*res));
    cudaStream_t s = (cudaStream_t)stream;
    const int n = op->nsrc;
    float *e32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *ap32 = nullptr;
    double *r64 = nullptr, *ax64 = nullptr, *partial = nullptr, *scal = nullptr;
    CGScalars *sc = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int st = LENTILS_OK;
    cudaError_t e = cudaMalloc(&e32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&r32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&z32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&p32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&ap32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&r64, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&ax64, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&partial, sizeof(double) * 2 * kRedBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&scal, sizeof(double) * 2);
    if (e == cudaSuccess) e = cudaMalloc(&sc, sizeof(CGScalars));
    if (e == cudaSuccess) e = cudaMemsetAsync(sc, 0, sizeof(CGScalars), s);
    if (e != cudaSuccess) st = cuda_status(e, "cg_solve alloc");

    // one inner iteration (everything on stream s, scalars on the device)
    auto inner_iteration = [&]() -> int {
        int q = lentils_normal_op_apply(op, p32, ap32, s);
        if (q) return q;
        LENTILS_CUDA_TRY(pdl_launch(dot_partial_kernel<float, float>, dim3(kRedBlocks), dim3(256), 0, s, p32, ap32, n, partial));
        LENTILS_CUDA_TRY(pdl_launch(cg_alpha_kernel, dim3(1), dim3(256), 0, s, partial, kRedBlocks, sc));
        LENTILS_CUDA_TRY(pdl_launch(cg_update_kernel, dim3(kRedBlocks), dim3(256), 0, s, e32, r32, z32, p32, ap32, inv_diag32, sc, n,
                                                   partial));
        LENTILS_CUDA_TRY(pdl_launch(cg_beta_kernel, dim3(1), dim3(256), 0, s, partial, kRedBlocks, sc));
        LENTILS_CUDA_TRY(pdl_launch(cg_p_kernel, dim3(nb(n)), dim3(256), 0, s, p32, z32, sc, n));
        cudaError_t le = cudaGetLastError();
        return le == cudaSuccess ? LENTILS_OK : cuda_status(le, "cg inner iteration");
    };

    const auto t0 = std::chrono::steady_clock::now();
    double bnorm = 0.0, rel = 0.0;
    if (!st) {
        bnorm = sqrt(host_dot64(b, b, n, partial, scal, s));
        // r = b - A x (the FP64 matvec is skipped for the zero initial guess: r = b)
        st = initial_residual(op, b, x, ax64, r64, n, partial, scal, s);
        if (!st)
            rel = (bnorm > 0) ? sqrt(host_dot64(r64, r64, n, partial, scal, s)) / bnorm : 0.0;
    }
    if (!st && opt->use_graph) {
        // capture one inner iteration
        e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const int q = inner_iteration();
            cudaError_t ee = cudaStreamEndCapture(s, &graph);
            if (q) st = q;
            else if (ee != cudaSuccess) st = cuda_status(ee, "cudaStreamEndCapture");
        } else {
            st = cuda_status(e, "cudaStreamBeginCapture");
        }
        if (!st) {
            e = cudaGraphInstantiate(&gexec, graph, 0);
            if (e != cudaSuccess) st = cuda_status(e, "cudaGraphInstantiate");
        }
    }
    int outer = 0, inner_total = 0;
    const int check = std::max(1, opt->check_every);
    while (!st && rel > opt->tol && outer < opt->max_outer) {
        ++outer;
        LENTILS_CUDA_TRY(pdl_launch(cg_start_kernel, dim3(kRedBlocks), dim3(256), 0, s, r64, r32, e32, z32, p32, inv_diag32, n, partial));
        LENTILS_CUDA_TRY(pdl_launch(cg_start_finish_kernel, dim3(1), dim3(256), 0, s, partial, kRedBlocks, sc));
        CGScalars hs;
        int k = 0;
        while (k < opt->max_inner) {
            for (int c = 0; c < check && k < opt->max_inner; ++c, ++k) {
                if (gexec) {
                    e = cudaGraphLaunch(gexec, s);
                    if (e != cudaSuccess) {
                        st = cuda_status(e, "cudaGraphLaunch");
                        break;
                    }
                } else if ((st = inner_iteration())) {
                    break;
                }
            }
            if (st) break;
            e = cudaMemcpyAsync(&hs, sc, sizeof(CGScalars), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                st = cuda_status(e, "cg residual read");
                break;
            }
            if (!(hs.rr == hs.rr)) {
                st = set_error(LENTILS_ERR_NONFINITE, "cg_solve: NaN in the inner residual");
                break;
            }
            if (hs.rr <= opt->inner_tol * opt->inner_tol * hs.rr0) break;
        }
        inner_total += k;
        if (st) break;
        LENTILS_CUDA_TRY(pdl_launch(add_f32_to_f64_kernel, dim3(nb(n)), dim3(256), 0, s, x, e32, n));
        if ((st = lentils_normal_op_apply64(op, x, ax64, s))) break;
        LENTILS_CUDA_TRY(pdl_launch(sub_kernel, dim3(nb(n)), dim3(256), 0, s, b, ax64, r64, n));
        rel = (bnorm > 0) ? sqrt(host_dot64(r64, r64, n, partial, scal, s)) / bnorm : 0.0;
    }
    if (!st) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_status(e, "cg_solve sync");
    }
    const auto t1 = std::chrono::steady_clock::now();
    res->converged = (!st && rel <= opt->tol) ? 1 : 0;
    res->outer = outer;
    res->inner_total = inner_total;
    res->rel_residual = rel;
    res->seconds = std::chrono::duration<double>(t1 - t0).count();
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    cudaFree(e32);
    cudaFree(r32);
    cudaFree(z32);
    cudaFree(p32);
    cudaFree(ap32);
    cudaFree(r64);
    cudaFree(ax64);
    cudaFree(partial);
    cudaFree(scal);
    cudaFree(sc);
    return st;
}

// Flexible CG inside the FP64 iterative refinement (see the header for the iteration). With
// p = ap = 0 at the start of an inner solve, the direction step below yields p = dir.
int lentils_fcg_solve(lentils_normal_op *op, const double *b, double *x, const float *inv_diag32,
                      lentils_unet *net, const lentils_cg_options *opt, lentils_cg_result *res,
                      void *stream)
{
    clear_error();
    if (!op || !b || !x || !inv_diag32 || !opt || !res)
        return set_error(LENTILS_ERR_INVALID, "fcg_solve: null");
    if (net && unet_size(net) != op->nsrc)
        return set_error(LENTILS_ERR_INVALID, "fcg_solve: network grid %d != source grid %d",
                         unet_size(net), op->nsrc);
    memset(res, 0, sizeof(*res));
    cudaStream_t s = (cudaStream_t)stream;
    const int n = op->nsrc;
    const int m = std::min(kMaxWindow, std::max(1, opt->window));
    float *e32 = nullptr, *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *ap32 = nullptr,
          *feat = nullptr, *Pw = nullptr, *Qw = nullptr;
    double *r64 = nullptr, *ax64 = nullptr, *partial = nullptr, *scal = nullptr,
           *fpart = nullptr;
    unsigned *counter = nullptr;
    FCGScalars *sc = nullptr;
    FCGWindow *win = nullptr;
    cudaGraph_t graph[2] = {nullptr, nullptr};  // one inner iteration: [0] Jacobi, [1] network
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int st = LENTILS_OK;
    cudaError_t e = cudaMalloc(&e32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&r32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&z32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&p32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&ap32, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&feat, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&Pw, sizeof(float) * n * m);
    if (e == cudaSuccess) e = cudaMalloc(&Qw, sizeof(float) * n * m);
    if (e == cudaSuccess) e = cudaMalloc(&r64, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&ax64, sizeof(double) * n);
    if (e == cudaSuccess) e = cudaMalloc(&partial, sizeof(double) * kMaxWindow * kRedBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&fpart, sizeof(double) * kFusedRows * kRedBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&counter, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaMalloc(&scal, sizeof(double) * 2);
    if (e == cudaSuccess) e = cudaMalloc(&sc, sizeof(FCGScalars));
    if (e == cudaSuccess) e = cudaMalloc(&win, sizeof(FCGWindow));
    if (e == cudaSuccess) e = cudaMemsetAsync(sc, 0, sizeof(FCGScalars), s);
    // unused ring slots enter the direction update with a zero coefficient: keep them finite
    if (e == cudaSuccess) e = cudaMemsetAsync(Pw, 0, sizeof(float) * n * m, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(Qw, 0, sizeof(float) * n * m, s);
    if (e == cudaSuccess) {
        FCGWindow hw;
        memset(&hw, 0, sizeof(hw));
        hw.m = m;
        e = cudaMemcpy(win, &hw, sizeof(hw), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) st = cuda_status(e, "fcg_solve alloc");
    if (!st && net) st = lentils_unet_features(inv_diag32, feat, n, stream);
    if (!st && net) st = unet_prepare(net);
    bool use_net = net != nullptr;  // false after a stagnation fallback
    const int every = std::max(1, opt->net_every);

    // direction step: z = M(r) (with_net) and d = z or the Jacobi direction;
    // p = d - sum_j (d.Q[j] / pq[j]) P[j]
    auto direction = [&](bool first, bool with_net) -> int {
        float *zdir = with_net ? z32 : nullptr;
        if (with_net)
            if (int q = unet_precondition(net, r32, inv_diag32, feat, z32, s)) return q;
        LENTILS_CUDA_TRY(pdl_launch(fcg_select_fused_kernel, dim3(kRedBlocks), dim3(256), 0, s, zdir, r32, inv_diag32, Qw, n, sc, win,
                                                            fpart, counter, first ? 1 : 0));
        LENTILS_CUDA_TRY(pdl_launch(fcg_p_fused_kernel, dim3(nb(n)), dim3(256), 0, s, p32, zdir, r32, inv_diag32, Pw, sc, win, n));
        cudaError_t le = cudaGetLastError();
        return le == cudaSuccess ? LENTILS_OK : cuda_status(le, "fcg direction");
    };
    // one inner iteration: ap = A p; alpha; the updates, ring store and (Jacobi direction) the
    // window coefficients in one pass; then p -- three launches besides the matvec
    auto inner_iteration = [&](bool with_net) -> int {
        int q = lentils_normal_op_apply(op, p32, ap32, s);
        if (q) return q;
        LENTILS_CUDA_TRY(pdl_launch(fcg_alpha_fused_kernel, dim3(kRedBlocks), dim3(256), 0, s, p32, ap32, r32, n, fpart, counter, sc));
        LENTILS_CUDA_TRY(pdl_launch(fcg_update_fused_kernel, dim3(kRedBlocks), dim3(256), 0, s, e32, r32, p32, ap32, Pw, Qw,
                                                            inv_diag32, n, sc, win, fpart,
                                                            counter, with_net ? 0 : 1));
        if (with_net) return direction(false, true);
        LENTILS_CUDA_TRY(pdl_launch(fcg_p_fused_kernel, dim3(nb(n)), dim3(256), 0, s, p32, nullptr, r32, inv_diag32, Pw, sc, win, n));
        cudaError_t le = cudaGetLastError();
        return le == cudaSuccess ? LENTILS_OK : cuda_status(le, "fcg step");
    };

    const auto t0 = std::chrono::steady_clock::now();
    double bnorm = 0.0, rel = 0.0;
    if (!st) {
        bnorm = sqrt(host_dot64(b, b, n, partial, scal, s));
        st = initial_residual(op, b, x, ax64, r64, n, partial, scal, s);
        if (!st)
            rel = (bnorm > 0) ? sqrt(host_dot64(r64, r64, n, partial, scal, s)) / bnorm : 0.0;
    }
    // one inner iteration captured as a graph, with and/or without the network (again after a
    // fallback changes the iteration)
    auto capture_one = [&](int w) -> int {
        cudaError_t ce = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (ce != cudaSuccess) return cuda_status(ce, "cudaStreamBeginCapture");
        const int q = inner_iteration(w == 1);
        ce = cudaStreamEndCapture(s, &graph[w]);
        if (q) return q;
        if (ce != cudaSuccess) return cuda_status(ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&gexec[w], graph[w], 0);
        return ce == cudaSuccess ? LENTILS_OK : cuda_status(ce, "cudaGraphInstantiate");
    };
    auto capture = [&]() -> int {
        for (int w = 0; w < 2; ++w) {
            if (gexec[w]) cudaGraphExecDestroy(gexec[w]);
            if (graph[w]) cudaGraphDestroy(graph[w]);
            gexec[w] = nullptr;
            graph[w] = nullptr;
        }
        if (use_net)
            if (int q = capture_one(1)) return q;
        if (!use_net || every > 1) return capture_one(0);
        return LENTILS_OK;
    };
    if (!st && opt->use_graph) st = capture();
    int outer = 0, inner_total = 0, fallback = 0;
    const int check = std::max(1, opt->check_every);
    const int stall_checks = 20;
    while (!st && rel > opt->tol && outer < opt->max_outer) {
        ++outer;
        LENTILS_CUDA_TRY(pdl_launch(fcg_start_kernel, dim3(kRedBlocks), dim3(256), 0, s, r64, r32, e32, p32, ap32, n, partial));
        LENTILS_CUDA_TRY(pdl_launch(fcg_rr_kernel, dim3(1), dim3(256), 0, s, partial, kRedBlocks, sc, 1));
        if ((st = direction(true, use_net))) break;
        FCGScalars hs;
        int k = 0;
        double mark_rr = -1.0;
        int mark_k = 0;
        while (k < opt->max_inner) {
            for (int c = 0; c < check && k < opt->max_inner; ++c, ++k) {
                // the direction this iteration ends with is the (k + 2)-th of the inner solve
                const int w = (use_net && (k + 1) % every == 0) ? 1 : 0;
                if (gexec[w]) {
                    e = cudaGraphLaunch(gexec[w], s);
                    if (e != cudaSuccess) {
                        st = cuda_status(e, "cudaGraphLaunch");
                        break;
                    }
                } else if ((st = inner_iteration(w == 1))) {
                    break;
                }
            }
            if (st) break;
            e = cudaMemcpyAsync(&hs, sc, sizeof(FCGScalars), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) {
                st = cuda_status(e, "fcg residual read");
                break;
            }
            if (!(hs.rr == hs.rr)) {
                st = set_error(LENTILS_ERR_NONFINITE, "fcg_solve: NaN in the inner residual");
                break;
            }
            if (hs.rr <= opt->inner_tol * opt->inner_tol * hs.rr0) break;
            // stagnation: the residual norm has not halved over the last stall_checks checks
            if (mark_rr < 0.0 || hs.rr <= 0.25 * mark_rr) {
                mark_rr = hs.rr;
                mark_k = k;
            } else if (use_net && k - mark_k >= stall_checks * check) {
                use_net = false;
                fallback = 1;
                mark_k = k;
                if (opt->use_graph && (st = capture())) break;
            }
        }
        inner_total += k;
        if (st) break;
        LENTILS_CUDA_TRY(pdl_launch(add_f32_to_f64_kernel, dim3(nb(n)), dim3(256), 0, s, x, e32, n));
        if ((st = lentils_normal_op_apply64(op, x, ax64, s))) break;
        LENTILS_CUDA_TRY(pdl_launch(sub_kernel, dim3(nb(n)), dim3(256), 0, s, b, ax64, r64, n));
        rel = (bnorm > 0) ? sqrt(host_dot64(r64, r64, n, partial, scal, s)) / bnorm : 0.0;
    }
    if (!st) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_status(e, "fcg_solve sync");
    }
    const auto t1 = std::chrono::steady_clock::now();
    FCGScalars hs_end;
    memset(&hs_end, 0, sizeof(hs_end));
    if (!st) {
        e = cudaMemcpy(&hs_end, sc, sizeof(FCGScalars), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_status(e, "fcg_solve scalars");
    }
    if (!st && net) {
        int flag = 0;
        st = unet_error_flag_device(net, &flag);
        if (!st && flag) st = set_error(LENTILS_ERR_TIMEOUT, "fcg_solve: a tensor-core wait gave up");
    }
    res->net_iterations = (int)hs_end.net_iters;
    res->fallback = fallback;
    res->converged = (!st && rel <= opt->tol) ? 1 : 0;
    res->outer = outer;
    res->inner_total = inner_total;
    res->rel_residual = rel;
    res->seconds = std::chrono::duration<double>(t1 - t0).count();
    for (int w = 0; w < 2; ++w) {
        if (gexec[w]) cudaGraphExecDestroy(gexec[w]);
        if (graph[w]) cudaGraphDestroy(graph[w]);
    }
    cudaFree(e32);
    cudaFree(r32);
    cudaFree(z32);
    cudaFree(p32);
    cudaFree(ap32);
    cudaFree(feat);
    cudaFree(fpart);
    cudaFree(counter);
    cudaFree(Pw);
    cudaFree(Qw);
    cudaFree(win);
    cudaFree(r64);
    cudaFree(ax64);
    cudaFree(partial);
    cudaFree(scal);
    cudaFree(sc);
    return st;
}

// lambda R^T R s for the forward-difference gradient on an (nx, ny) grid (overwrites out)
int lentils_prior_gradient_apply(const float *s_in, float *out, int nx, int ny, double dx,
                                 double dy, double lambda, void *stream)
{
    clear_error();
    if (!s_in || !out || nx < 1 || ny < 1 || !(dx > 0) || !(dy > 0))
        return set_error(LENTILS_ERR_INVALID, "prior_gradient_apply: bad arguments");
    LENTILS_CUDA_TRY(pdl_launch(rtr_kernel<float>, dim3(nb((long long)nx * ny)), dim3(256), 0, (cudaStream_t)stream, s_in, out, nx, ny, (float)(1.0 / (dx * dx)), (float)(1.0 / (dy * dy)), (float)lambda, 0));
    LENTILS_CHECK_LAUNCH("rtr_kernel");
    return LENTILS_OK;
}

int lentils_prior_gradient_apply64(const double *s_in, double *out, int nx, int ny, double dx,
                                   double dy, double lambda, void *stream)
{
    clear_error();
    if (!s_in || !out || nx < 1 || ny < 1 || !(dx > 0) || !(dy > 0))
        return set_error(LENTILS_ERR_INVALID, "prior_gradient_apply64: bad arguments");
    LENTILS_CUDA_TRY(pdl_launch(rtr_kernel<double>, dim3(nb((long long)nx * ny)), dim3(256), 0, (cudaStream_t)stream, s_in, out, nx, ny, 1.0 / (dx * dx), 1.0 / (dy * dy), lambda, 0));
    LENTILS_CHECK_LAUNCH("rtr_kernel");
    return LENTILS_OK;
}

// FP64 dot product of two device vectors (host result; synchronises the stream)
int lentils_dot64(const double *a, const double *b, int n, double *out, void *stream)
{
    clear_error();
    if (!a || !b || !out || n < 0) return set_error(LENTILS_ERR_INVALID, "dot64: bad arguments");
    double *partial = nullptr, *scal = nullptr;
    cudaError_t e = cudaMalloc(&partial, sizeof(double) * kRedBlocks);
    if (e == cudaSuccess) e = cudaMalloc(&scal, sizeof(double));
    if (e != cudaSuccess) {
        cudaFree(partial);
        return cuda_status(e, "dot64 alloc");
    }
    *out = host_dot64(a, b, n, partial, scal, (cudaStream_t)stream);
    e = cudaGetLastError();
    cudaFree(partial);
    cudaFree(scal);
    return e == cudaSuccess ? LENTILS_OK : cuda_status(e, "dot64");
}

}  // extern "C"
