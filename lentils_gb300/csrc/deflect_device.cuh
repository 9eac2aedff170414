// Device-side lens-equation pieces (per-lens constants and deflection formulas), shared by the
// deflection kernel (deflect.cu) and the persistent batched sweep (sweep.cu). The formulas and
// their reference sources are documented in deflect.cu.
#pragma once

#include "common.cuh"

namespace lentils {

constexpr int kMaxLensesPerLaunch = 8;
constexpr int kSeriesTerms = 20;  // fixed 20-term series (deflect.c:212)
constexpr int kMaxMultipoleOrder = 12;

struct DevLens {
    int type;
    int order;    // multipoles: highest order
    double x0, y0;
    float x0h, x0l, y0h, y0l;  // the centre as FP32 pairs: x0 = x0h + x0l to ~2^-48 relative
    float gxh, gxl, gyh, gyl;  // batched sweep: its sample's pixel-grid origin minus the centre
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

// x - (hi + lo) for FP32 x and a pair (hi, lo), rounded once: Knuth's two-sum gives
// x - hi = s + e exactly, then s + (e - lo). Exact offsets from a lens centre matter near the
// centre, where the angle of the offset sets the direction of the deflection; this keeps the
// FP32 path off the FP64 units, which on GB300 run at a small fraction of the FP32 rate.
__device__ __forceinline__ float offset_f32(float x, float hi, float lo)
{
    const float s = x - hi;
    const float bp = s - x;
    const float e = (x - (s - bp)) + (-hi - bp);
    return s + (e - lo);
}

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

// per-lens constants from the reference's packed parameters (host, FP64)
int build_lens(const lentils_mass_model &m, DevLens &L);

// alpha of one lens at offset (sx, sy) from its centre
__device__ __forceinline__ void lens_alpha(const DevLens &L, float sx, float sy, float &ax,
                                           float &ay)
{
    if (L.type == 0) pemd_alpha(L, sx, sy, ax, ay);
    else if (L.type == 1) shear_alpha(L, sx, sy, ax, ay);
    else multipole_alpha(L, sx, sy, ax, ay);
}

}  // namespace lentils
