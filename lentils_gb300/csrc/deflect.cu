// Lens-equation kernel ("K4"): beta = theta - sum_l alpha_l(theta) for a batch of points,
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

namespace lentils {

constexpr int kMaxLensesPerLaunch = 8;
constexpr int kSeriesTerms = 20;  // fixed 20-term series (deflect.c:212)
constexpr int kMaxMultipoleOrder = 12;

struct DevLens {
    int type;
    int order;    // multipoles: highest order
    double x0, y0;
    // PEMD
    float q, cth, sth, t, bnorm2, bnorm, qp;  // qp = (1-q^2)/q^2
    float an[kSeriesTerms];
    double an64[kSeriesTerms];
    // shear
    float ss, c2, s2, gks, cgka, sgka, gss, cgsa, sgsa;
    // multipoles
    float alpha, mnorm[kMaxMultipoleOrder + 1], am[kMaxMultipoleOrder + 1],
        bm[kMaxMultipoleOrder + 1];
};

struct DevLensSet {
    int n;
    DevLens l[kMaxLensesPerLaunch];
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__device__ __forceinline__ float2 cdiv(float2 a, float2 b)
{
    const float d = b.x * b.x + b.y * b.y;
    const float inv = 1.0f / d;
    return make_float2((a.x * b.x + a.y * b.y) * inv, (a.y * b.x - a.x * b.y) * inv);
}

// principal square root, branch cut on the negative real axis (C99 csqrt convention)
__device__ __forceinline__ float2 csqrtf_(float2 z)
{
    const float r = hypotf(z.x, z.y);
    float re = sqrtf(0.5f * (r + fabsf(z.x)));
    float im;
    if (re == 0.f) return make_float2(0.f, z.y);
    im = 0.5f * z.y / re;
    if (z.x >= 0.f) return make_float2(re, im);
    return make_float2(fabsf(im), copysignf(re, z.y));
}

__device__ __forceinline__ void pemd_alpha(const DevLens &L, float dx, float dy, float &ax,
                                           float &ay)
{
    // z = ((x-x0) + i(y-y0)) * (cos th' - i sin th')
    const float2 rot = make_float2(L.cth, -L.sth);
    const float2 z = cmul(make_float2(dx, dy), rot);
    const float X = z.x, Y = z.y;
    const float rs2 = L.q * L.q * X * X + Y * Y;
    const float rs = sqrtf(rs2);
    // A = b'^2 / (q z) * (b'/rs)^(t-2)
    const float pw = powf(L.bnorm / rs, L.t - 2.0f);
    const float2 A0 = cdiv(make_float2(L.bnorm2, 0.f), make_float2(L.q * z.x, L.q * z.y));
    const float2 A = make_float2(A0.x * pw, A0.y * pw);
    // w^2 = q' rs^2 / z^2 ; u = (1 - sqrt(1 - w^2)) / 2
    const float2 z2 = cmul(z, z);
    const float2 w2 = cdiv(make_float2(L.qp * rs2, 0.f), z2);
    const float2 sq = csqrtf_(make_float2(1.0f - w2.x, -w2.y));
    const float2 u = make_float2(0.5f * (1.0f - sq.x), -0.5f * sq.y);
    float2 F;
    if (u.x * u.x + u.y * u.y < 0.5625f) {  // |u| < 0.75: FP32 Horner
        F = make_float2(L.an[kSeriesTerms - 1], 0.f);
#pragma unroll
        for (int n = kSeriesTerms - 2; n >= 0; --n) {
            F = cmul(F, u);
            F.x += L.an[n];
        }
    } else {  // tail near |u| = 1: series in FP64
        double fr = L.an64[kSeriesTerms - 1], fi = 0.0;
        const double ur = u.x, ui = u.y;
        for (int n = kSeriesTerms - 2; n >= 0; --n) {
            const double tr = fr * ur - fi * ui;
            fi = fr * ui + fi * ur;
            fr = tr + L.an64[n];
        }
        F = make_float2((float)fr, (float)fi);
    }
    const float2 al = cmul(cmul(A, F), rot);
    ax = al.x;
    ay = -al.y;  // conj
}

__device__ __forceinline__ void shear_alpha(const DevLens &L, float sx, float sy, float &ax,
                                            float &ay)
{
    ax = L.ss * (L.c2 * sx + L.s2 * sy);
    ay = L.ss * (L.s2 * sx - L.c2 * sy);
    if (L.gks != 0.f) {
        const float rx = sx * L.cgka + sy * L.sgka;
        const float ry = -sx * L.sgka + sy * L.cgka;
        const float dx = -0.25f * L.gks * (3.f * rx * rx + ry * ry);
        const float dy = -0.5f * L.gks * rx * ry;
        ax += dx * L.cgka - dy * L.sgka;
        ay += dx * L.sgka + dy * L.cgka;
    }
    if (L.gss != 0.f) {
        const float rx = sx * L.cgsa + sy * L.sgsa;
        const float ry = -sx * L.sgsa + sy * L.cgsa;
        const float dx = -0.5f * L.gss * (rx * rx - ry * ry);
        const float dy = L.gss * rx * ry;
        ax += dx * L.cgsa - dy * L.sgsa;
        ay += dx * L.sgsa + dy * L.cgsa;
    }
}

__device__ __forceinline__ void multipole_alpha(const DevLens &L, float sx, float sy, float &ax,
                                                float &ay)
{
    const float r = sqrtf(sx * sx + sy * sy);
    const float th = atan2f(sy, sx);
    const float cn = sx / r, sn = sy / r;
    const float rp = powf(r, 1.0f - L.alpha);
    ax = 0.f;
    ay = 0.f;
    for (int m = 3; m <= L.order; ++m) {
        float sm, cm;
        sincosf((float)m * th, &sm, &cm);
        const float dr = -L.mnorm[m] * (2.0f - L.alpha) * rp * (L.bm[m] * sm + L.am[m] * cm);
        const float dt = L.mnorm[m] * (float)m * rp * (-L.bm[m] * cm + L.am[m] * sm);
        ax += cn * dr - sn * dt;
        ay += sn * dr + cn * dt;
    }
}

template <typename P>
__device__ __forceinline__ void load_point(const P *pts, long long i, double &x, double &y);
template <>
__device__ __forceinline__ void load_point<float2>(const float2 *pts, long long i, double &x,
                                                   double &y)
{
    const float2 v = pts[i];
    x = v.x;
    y = v.y;
}
template <>
__device__ __forceinline__ void load_point<double2>(const double2 *pts, long long i, double &x,
                                                    double &y)
{
    const double2 v = pts[i];
    x = v.x;
    y = v.y;
}

template <typename P>
__global__ void __launch_bounds__(256)
    deflect_kernel(const P *__restrict__ pin, P *__restrict__ pout, long long n,
                   const __grid_constant__ DevLensSet lenses, int accumulate)
{
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
            if (L.type == 0) pemd_alpha(L, sx, sy, ax, ay);
            else if (L.type == 1) shear_alpha(L, sx, sy, ax, ay);
            else multipole_alpha(L, sx, sy, ax, ay);
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

static int build_lens(const lentils_mass_model &m, DevLens &L)
{
    memset(&L, 0, sizeof(L));
    const double *p = m.fpars;
    L.type = (int)m.type;
    L.x0 = p[0];
    L.y0 = p[1];
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

}  // extern "C"
