// Lens-equation kernel: beta = theta - sum_l alpha_l(theta) for a batch of points,
// one thread per point, FP32 arithmetic with FP64 kept for the input offsets, the output sum
// and the tail of the 2F1 series when |u| nears 1.
//
// Mass models follow the reference's packing (lentils/models/lens_models.py:102-172) and
// formulas:
//   type 0 PEMD  -- deflect_PEMD_series + hyp2f1_series, lentils/backend/deflect.c:179-301;
//   type 1 shear -- deflect_external_potential, deflect.c:70-108;
//   type 2 multipoles -- deflect_internal_multipoles, deflect.c:126-175.
// Per-lens constants that depend only on the parameters (the Einstein-radius normalisation
// b' = (b/2 q^(t-1/2) (3-t)/(2-t))^(1/t), the series coefficients a_n, cos 2sa / sin 2sa)
// are computed once on the host in FP64.
#include <math.h>

#include <algorithm>

#include "common.cuh"
#include <type_traits>

#include "deflect_device.cuh"

namespace lentils {

template <typename P>
__global__ void __launch_bounds__(256)
    deflect_kernel(const P *__restrict__ pin, P *__restrict__ pout, long long n,
                   const __grid_constant__ DevLensSet lenses, int accumulate)
{
    if constexpr (std::is_same<P, float2>::value) {  // FP32 points: FP32 arithmetic only
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
             i += (long long)gridDim.x * blockDim.x) {
            const float2 v = pin[i];
            float axs = 0.f, ays = 0.f;
            for (int l = 0; l < lenses.n; ++l) {
                const DevLens &L = lenses.l[l];
                float ax, ay;
                lens_alpha(L, offset_f32(v.x, L.x0h, L.x0l), offset_f32(v.y, L.y0h, L.y0l),
                           ax, ay);
                axs += ax;
                ays += ay;
            }
            const float2 base = accumulate ? pout[i] : v;
            pout[i] = make_float2(base.x - axs, base.y - ays);
        }
        return;
    }
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        double x, y;
        load_point(pin, i, x, y);
        float axs = 0.f, ays = 0.f;
        for (int l = 0; l < lenses.n; ++l) {
            const DevLens &L = lenses.l[l];
            const float sx = (float)(x - L.x0);
            const float sy = (float)(y - L.y0);
            float ax, ay;
            lens_alpha(L, sx, sy, ax, ay);
            axs += ax;
            ays += ay;
        }
        double ox, oy;
        if (accumulate) {
            load_point(pout, i, ox, oy);
        } else {
            ox = x;
            oy = y;
        }
        P o;
        o.x = (decltype(o.x))(ox - (double)axs);
        o.y = (decltype(o.y))(oy - (double)ays);
        pout[i] = o;
    }
}

int build_lens(const lentils_mass_model &m, DevLens &L)
{
    memset(&L, 0, sizeof(L));
    const double *p = m.fpars;
    L.type = (int)m.type;
    L.x0 = p[0];
    L.y0 = p[1];
    L.x0h = (float)p[0];
    L.x0l = (float)(p[0] - (double)L.x0h);
    L.y0h = (float)p[1];
    L.y0l = (float)(p[1] - (double)L.y0h);
    if (m.type == 0) {
        const double t = 2.0 * p[7];
        const double q = p[2];
        const double b = pow(0.5 * p[6] * pow(q, t - 0.5) * (3.0 - t) / (2.0 - t), 1.0 / t);
        L.q = (float)q;
        L.sth = (float)p[4];
        L.cth = (float)p[5];
        L.t = (float)t;
        L.bnorm = (float)b;
        L.bnorm2 = (float)(b * b);
        L.qp = (float)((1 - q * q) / (q * q));
        double an = 1.0;
        for (int n = 0; n < kSeriesTerms; ++n) {
            L.an[n] = (float)an;
            L.an64[n] = an;
            const double ntf = 2 * n + 4 - t;
            an *= (ntf - t) / ntf;
        }
    } else if (m.type == 1) {
        L.ss = (float)p[2];
        L.c2 = (float)(-p[5] * p[5] + p[4] * p[4]);
        L.s2 = (float)(-2 * p[4] * p[5]);
        L.gks = (float)p[6];
        L.sgka = (float)p[8];
        L.cgka = (float)p[9];
        L.gss = (float)p[10];
        L.sgsa = (float)p[12];
        L.cgsa = (float)p[13];
    } else if (m.type == 2) {
        const int order = m.ipars[0];
        if (order > kMaxMultipoleOrder)
            return set_error(LENTILS_ERR_UNSUPPORTED, "deflect: multipole order %d (max %d)",
                             order, kMaxMultipoleOrder);
        L.order = order;
        const double al = 2.0 * p[2];
        L.alpha = (float)al;
        for (int mm = 3; mm <= order; ++mm) {
            L.am[mm] = (float)p[3 + 2 * (mm - 3)];
            L.bm[mm] = (float)p[3 + 2 * (mm - 3) + 1];
            L.mnorm[mm] = (float)(2.0 * pow(1.0, al) / (mm * mm - (al - 2) * (al - 2)));
        }
    } else {
        return set_error(LENTILS_ERR_INVALID, "deflect: unknown mass-model type %u", m.type);
    }
    return LENTILS_OK;
}

template <typename P>
static int deflect_launch(const lentils_mass_model *lenses, int nlenses, const P *pin, P *pout,
                          long long n, cudaStream_t s)
{
    if (nlenses < 0 || n < 0 || (n > 0 && (!pin || !pout)) || (nlenses > 0 && !lenses))
        return set_error(LENTILS_ERR_INVALID, "deflect: bad arguments");
    if (n == 0) return LENTILS_OK;
    long long blocks = (n + 255) / 256;
    if (blocks > 152LL * 64) blocks = 152LL * 64;
    int done = 0;
    do {
        DevLensSet set;
        memset(&set, 0, sizeof(set));
        set.n = std::min(kMaxLensesPerLaunch, nlenses - done);
        for (int l = 0; l < set.n; ++l) {
            int st = build_lens(lenses[done + l], set.l[l]);
            if (st) return st;
        }
        // later launches evaluate the lenses at the original positions and subtract from pout
        deflect_kernel<P><<<(int)blocks, 256, 0, s>>>(pin, pout, n, set, done > 0 ? 1 : 0);
        LENTILS_CHECK_LAUNCH("deflect_kernel");
        done += set.n;
    } while (done < nlenses);
    return LENTILS_OK;
}

// ------------------------------------------------------------------------------------------------
// Parameter derivatives (want_deriv), FP64.
//
// PEMD: d alpha / d (b, qh, q, x, y, th) as deflect_PEMD_series computes them
// (lentils/backend/deflect.c:243-339, with the 2F1 series derivatives of hyp2f1_series
// :179-239): the series derivative in t and u, the chain rule through
// w^2 = q' r_s^2 / z^2, the radial factor A's derivatives, the rotation back, the factor 2 of
// t = 2 qh and the degree-to-radian factor of th. External shear: d alpha / d (x, y, ss, sa) as
// the derivative block of deflect_external_potential states it (deflect.c:110-119), which the
// reference leaves compiled out. Per point the 8 parameters (b, qh, q, x, y, th, ss, sa) give
// 16 numbers (real, imaginary = x, y component).
// ------------------------------------------------------------------------------------------------
struct DerivLens {
    int type;
    double x0, y0;
    double q, sth, cth, b, t;   // PEMD (b: the normalised b' of deflect.c:284)
    double ss, cs2, sn2;        // shear
};

struct DerivLensSet {
    int n;
    DerivLens l[kMaxLensesPerLaunch];
};

struct dcx {
    double x, y;
};
__device__ __forceinline__ dcx dc(double a, double b) { return {a, b}; }
__device__ __forceinline__ dcx operator+(dcx a, dcx b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ dcx operator-(dcx a, dcx b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ dcx operator-(dcx a) { return {-a.x, -a.y}; }
__device__ __forceinline__ dcx operator*(dcx a, dcx b)
{
    return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ dcx operator*(double s, dcx a) { return {s * a.x, s * a.y}; }
__device__ __forceinline__ dcx operator*(dcx a, double s) { return {s * a.x, s * a.y}; }
__device__ __forceinline__ dcx operator/(dcx a, dcx b)
{
    const double d = b.x * b.x + b.y * b.y;
    return {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d};
}
__device__ __forceinline__ dcx operator/(dcx a, double s) { return {a.x / s, a.y / s}; }
__device__ __forceinline__ dcx operator/(double a, dcx b) { return dc(a, 0.0) / b; }
__device__ __forceinline__ dcx dconj(dcx a) { return {a.x, -a.y}; }
// principal square root (branch cut on the negative real axis, as C's csqrt)
__device__ __forceinline__ dcx dcsqrt(dcx z)
{
    const double r = hypot(z.x, z.y);
    if (r == 0.0) return {0.0, 0.0};
    double re = sqrt(0.5 * (r + fabs(z.x)));
    double im = z.y / (2.0 * re);
    if (z.x < 0.0) {
        const double t = fabs(im);
        im = copysign(re, z.y);
        re = t;
    }
    return {re, im};
}

// PEMD alpha and its 6 parameter derivatives (complex: x + i y components) at offset (dx, dy)
__device__ void pemd_derivs(const DerivLens &L, double px, double py, dcx &alpha, dcx (&d)[6])
{
    const double t = L.t, q = L.q, b = L.b;
    const dcx I = dc(0.0, 1.0);
    const dcx crot = dc(L.cth, -L.sth);
    const dcx z = dc(px - L.x0, py - L.y0) * crot;
    const double x = z.x, y = z.y;
    const double rs2 = q * q * x * x + y * y;
    const double rs = sqrt(rs2);
    const dcx A = (b * b) * pow(b / rs, t - 2.0) / (q * z);
    // hyp2f1_series with derivatives
    const double qq = (1.0 - q * q) / (q * q);
    const dcx w2 = (qq * rs2) / (z * z);
    const dcx sq = dcsqrt(dc(1.0, 0.0) - w2);
    const dcx u = 0.5 * (dc(1.0, 0.0) - sq);
    dcx F = dc(0, 0), un = dc(1, 0), un1 = dc(0, 0), dfdu = dc(0, 0), dfdt = dc(0, 0);
    double an = 1.0, dadt = 0.0;
    for (int n = 0; n < kSeriesTerms; ++n) {
        F = F + an * un;
        const double ntf = 2 * n + 4 - t;
        dfdt = dfdt + dadt * un;
        dfdu = dfdu + (an * n) * un1;
        un1 = un;
        dadt = -2.0 * (2 + n) / (ntf * ntf) * an + 2.0 * (2 + n - t) / ntf * dadt;
        un = un * u;
        an *= (ntf - t) / ntf;
    }
    const dcx z2 = z * z, z3 = z2 * z;
    const dcx dudw2 = dc(1.0, 0.0) / (4.0 * sq);
    const dcx dfdw2 = dfdu * dudw2;
    const dcx dw2dq = (-2.0 * (q * q * q * q * x * x + y * y)) / (q * q * q * z2);
    const dcx dw2dx = (-2.0 * qq * y) * (dc(y, 0.0) - (q * q * x) * I) / z3;
    const dcx dw2dy = ((-2.0 * qq * x) * I) * (dc(q * q * x, 0.0) + y * I) / z3;
    const dcx dFdt = dfdt, dFdq = dfdw2 * dw2dq, dFdx = dfdw2 * dw2dx, dFdy = dfdw2 * dw2dy;
    const dcx dAdb = A * (t / b);
    const dcx dAdt = A * log(b / rs);
    const dcx dAdq = -(A * (((t - 1.0) * q * q * x * x + y * y) / (q * rs2)));
    const dcx dAdx = -(A * (dc(y * y + q * q * x * x * (t - 1.0), q * q * x * (t - 2.0) * y)) /
                       (z * rs2));
    const dcx dAdy = -(A * (dc(y * (t - 2.0) * x, q * q * x * x + (t - 1.0) * y * y)) /
                       (z * rs2));
    alpha = dconj(A * F * crot);
    const dcx dab = dconj((F * dAdb) * crot);
    const dcx dat = 2.0 * dconj((F * dAdt + A * dFdt) * crot);
    const dcx daq = dconj((F * dAdq + A * dFdq) * crot);
    const dcx daxs = dconj((F * dAdx + A * dFdx) * crot);
    const dcx days = dconj((F * dAdy + A * dFdy) * crot);
    const dcx dax = -(daxs * L.cth - days * L.sth);
    const dcx day = -(daxs * L.sth + days * L.cth);
    const dcx dath = (3.14159265358979323846 / 180.0) * (daxs * y - days * x + I * alpha);
    d[0] = dab;
    d[1] = dat;
    d[2] = daq;
    d[3] = dax;
    d[4] = day;
    d[5] = dath;
}

// per-point derivatives (8 parameters) summed over the lenses; grads (8, n, 2) and/or the
// per-block partial sums of the 12 PEMD numbers (the reference's want_deriv accumulation)
__global__ void __launch_bounds__(256)
    deflect_deriv_kernel(const double2 *__restrict__ pts, double *__restrict__ grads,
                         double *__restrict__ sum12, long long n,
                         const __grid_constant__ DerivLensSet lenses)
{
    double acc[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) acc[k] = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double2 p = pts[i];
        dcx g[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) g[k] = dc(0.0, 0.0);
        for (int l = 0; l < lenses.n; ++l) {
            const DerivLens &L = lenses.l[l];
            if (L.type == 0) {
                dcx alpha, d[6];
                pemd_derivs(L, p.x, p.y, alpha, d);
#pragma unroll
                for (int k = 0; k < 6; ++k) g[k] = g[k] + d[k];
            } else if (L.type == 1) {
                const double sx = p.x - L.x0, sy = p.y - L.y0;
                const double pi180 = 3.14159265358979323846 / 180.0;
                g[3] = g[3] + dc(-L.ss * L.cs2, -L.ss * L.sn2);
                g[4] = g[4] + dc(-L.ss * L.sn2, L.ss * L.cs2);
                g[6] = g[6] + dc(L.cs2 * sx + L.sn2 * sy, L.sn2 * sx - L.cs2 * sy);
                g[7] = g[7] + dc(pi180 * L.ss * (2 * sy * L.cs2 - 2 * sx * L.sn2),
                                 pi180 * L.ss * (2 * sx * L.cs2 + 2 * sy * L.sn2));
            }
        }
        if (grads) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                grads[2 * (k * n + i)] = g[k].x;
                grads[2 * (k * n + i) + 1] = g[k].y;
            }
        }
        if (sum12) {  // the PEMD part only, as the reference accumulates it
            for (int l = 0; l < lenses.n; ++l) {
                if (lenses.l[l].type != 0) continue;
                dcx alpha, d[6];
                pemd_derivs(lenses.l[l], p.x, p.y, alpha, d);
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    acc[2 * k] += d[k].x;
                    acc[2 * k + 1] += d[k].y;
                }
            }
        }
    }
    if (!sum12) return;
    __shared__ double sh[12][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
        double v = acc[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) sh[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < 12) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += sh[threadIdx.x][w];
        atomicAdd(&sum12[threadIdx.x], v);
    }
}

static int build_deriv_lens(const lentils_mass_model &m, DerivLens &L)
{
    memset(&L, 0, sizeof(L));
    const double *p = m.fpars;
    L.type = (int)m.type;
    L.x0 = p[0];
    L.y0 = p[1];
    if (m.type == 0) {
        const double t = 2.0 * p[7], q = p[2];
        L.t = t;
        L.q = q;
        L.sth = p[4];
        L.cth = p[5];
        L.b = pow(0.5 * p[6] * pow(q, t - 0.5) * (3.0 - t) / (2.0 - t), 1.0 / t);
    } else if (m.type == 1) {
        L.ss = p[2];
        L.cs2 = -p[5] * p[5] + p[4] * p[4];
        L.sn2 = -2 * p[4] * p[5];
    } else if (m.type != 2) {
        return set_error(LENTILS_ERR_INVALID, "deflect: unknown mass-model type %u", m.type);
    }
    return LENTILS_OK;
}

// grads (8, n, 2) and/or sum12 (device, accumulated)
int deflect_derivatives(const lentils_mass_model *lenses, int nlenses, const double *points,
                        double *grads, double *sum12, long long n, cudaStream_t s)
{
    if (n == 0) return LENTILS_OK;
    for (int l0 = 0; l0 < std::max(1, nlenses); l0 += kMaxLensesPerLaunch) {
        DerivLensSet set;
        memset(&set, 0, sizeof(set));
        set.n = std::min(kMaxLensesPerLaunch, nlenses - l0);
        for (int l = 0; l < set.n; ++l)
            if (int st = build_deriv_lens(lenses[l0 + l], set.l[l])) return st;
        if (l0 > 0 && grads)
            return set_error(LENTILS_ERR_UNSUPPORTED,
                             "deflect gradients: at most %d lenses", kMaxLensesPerLaunch);
        const long long blocks = std::min<long long>((n + 255) / 256, 152LL * 16);
        deflect_deriv_kernel<<<(int)std::max(1LL, blocks), 256, 0, s>>>(
            (const double2 *)points, grads, sum12, n, set);
        LENTILS_CHECK_LAUNCH("deflect_deriv_kernel");
        if (nlenses == 0) break;
    }
    return LENTILS_OK;
}

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_deflect_f32(const lentils_mass_model *lenses, int nlenses, const float *points,
                        float *out, long long npoints, void *stream)
{
    clear_error();
    return deflect_launch<float2>(lenses, nlenses, (const float2 *)points, (float2 *)out,
                                  npoints, (cudaStream_t)stream);
}

int lentils_deflect_f64io(const lentils_mass_model *lenses, int nlenses, const double *points,
                          double *out, long long npoints, void *stream)
{
    clear_error();
    return deflect_launch<double2>(lenses, nlenses, (const double2 *)points, (double2 *)out,
                                   npoints, (cudaStream_t)stream);
}

// Per-point derivatives of the deflection for the 8 parameters (b, qh, q, x, y, th, ss, sa)
// summed over the lenses: grads (device) (8, n, 2) float64, OVERWRITTEN.
int lentils_deflect_grad(const lentils_mass_model *lenses, int nlenses, const double *points,
                         double *grads, long long npoints, void *stream)
{
    clear_error();
    if (!lenses || nlenses < 1 || nlenses > kMaxLensesPerLaunch || !points || !grads ||
        npoints < 0)
        return set_error(LENTILS_ERR_INVALID, "deflect_grad: bad arguments");
    return deflect_derivatives(lenses, nlenses, points, grads, nullptr, npoints,
                               (cudaStream_t)stream);
}

}  // extern "C"
