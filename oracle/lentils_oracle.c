/*
 * CPU oracle: a plain-C restatement of the reference's FP64 hot path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
 * reference arm may load this library, and only to compare results against or as the timed
 * CPU baseline.
 * Nothing in lentils_gb300/ links, loads or calls it.
 *
 * Each function restates one reference routine (cited per function) with the same
 * arithmetic, the same constants (including the reference's truncated 2*pi) and the same
 * evaluation order, so that with one OpenMP thread it reproduces the compiled reference bit
 * for bit (pinned by tests/test_oracle.py against oracle/_ref and tests/golden/).
 * Build: oracle/Makefile (gcc -O2 -fopenmp -ffp-contract=off).
 */
#include <math.h>
#include <complex.h>
#include <string.h>
#include <stdlib.h>
#include <stdio.h>
#include "gsl/gsl_sf_bessel.h" /* oracle/shim: power-series I0 */
#include "lentils_gb300.h"     /* by-value struct layouts shared with the reference ABI */

/* Constants as the reference defines them (lentils/backend/common.h:8-11). */
#define ORC_ARCSEC_TO_RAD 4.8481368111e-6
#define ORC_PI_TRUNC 3.14159265359
#define ORC_TWO_PI_TRUNC 6.28318530718

/* Separable Kaiser-Bessel weight of one 2-D tap: zero outside the square [-w, w]^2,
 * else I0(beta*sqrt(1-(a/w)^2)) * I0(beta*sqrt(1-(b/w)^2)) / (4 w^2).
 * Restates kb_g, lentils/backend/nufft.c:11-21 (same product order). */
double oracle_kb_tap(double a, double b, double beta, double w)
{
    if (!(a >= -w && a <= w && b >= -w && b <= w)) return 0.0;
    double ra = 1.0 - (a / w) * (a / w);
    double rb = 1.0 - (b / w) * (b / w);
    if (ra < 0.0) ra = 0.0;
    if (rb < 0.0) rb = 0.0;
    const double norm = 1.0 / (4.0 * w * w);
    return norm * gsl_sf_bessel_I0(beta * sqrt(ra)) * gsl_sf_bessel_I0(beta * sqrt(rb));
}

/* Apodisation (grid-correction) factor sinhc(x)*sinhc(y) with
 * sinhc(c) = sinh(s)/s, s = sqrt(beta^2 - (2 pi w c)^2). Restates kb_w, nufft.c:23-33. */
double oracle_kb_apod(double cx, double cy, double beta, double w)
{
    const double sx = sqrt(beta * beta - (ORC_TWO_PI_TRUNC * w * cx) * (ORC_TWO_PI_TRUNC * w * cx));
    const double sy = sqrt(beta * beta - (ORC_TWO_PI_TRUNC * w * cy) * (ORC_TWO_PI_TRUNC * w * cy));
    const double fx = (fabs(sx) < 1.0e-6) ? 1.0 : sinh(sx) / sx;
    const double fy = (fabs(sy) < 1.0e-6) ? 1.0 : sinh(sy) / sy;
    return fx * fy;
}

/* Beatty et al. (2005) shape parameter, restating kb_optimal_beta, nufft.c:36-38. */
double oracle_kb_beta(double pad, double w)
{
    return ORC_PI_TRUNC * sqrt(((2.0 * w) / pad) * ((2.0 * w) / pad) * (pad - 0.5) * (pad - 0.5) - 0.8);
}

static inline int orc_wrap(int i, int n)
{
    while (i < 0) i += n;
    while (i >= n) i -= n;
    return i;
}

/* Kaiser-Bessel degridding (direction 0) and gridding (direction 1) between visibilities and
 * the r2c half-plane grid. Restates grid_cpu, lentils/backend/nufft.c:42-122:
 *  - coordinates u = uv[0]*ch, v = -uv[1]*ch (nufft.c:60-61);
 *  - phase 2pi*(u*gcx + v*gcy) with the truncated 2pi (nufft.c:63-64);
 *  - taps round(u/du)-w .. round(u/du)+w inclusive per axis (nufft.c:65-68);
 *  - checkerboard sign (-1)^(iu+iv) on unwrapped indices (nufft.c:78);
 *  - wrap mod (nu, nv), then fold i_v >= nv/2+1 onto the half plane with conjugation
 *    (nufft.c:83-93);
 *  - degrid: vis += 2*(0.5*k*p) * e^{-i phase} * G (nufft.c:98-105);
 *  - grid: G += 0.5*k*p * e^{+i phase} * V, conjugated on folded taps, doubled on column 0
 *    (nufft.c:106-118).
 * Rows run in parallel under OpenMP with atomic updates, as in the reference. */
void oracle_grid(lentils_visibility_space vs, double *vis, lentils_fourier_space gs,
                 double *grid, int wsup, double beta, int direction)
{
    const double wd = (double)wsup;
    for (int ch = 0; ch < vs.nchannels; ++ch) {
        const double scale = vs.channels[ch];
#pragma omp parallel for schedule(static)
        for (int row = 0; row < vs.nrows; ++row) {
            const double u = vs.uv[3 * row + 0] * scale;
            const double v = -vs.uv[3 * row + 1] * scale;
            const double cph = cos(ORC_TWO_PI_TRUNC * (u * gs.gcx + v * gs.gcy));
            const double sph = sin(ORC_TWO_PI_TRUNC * (u * gs.gcx + v * gs.gcy));
            const int cu = (int)round(u / gs.du);
            const int cv = (int)round(v / gs.dv);
            const long vidx = (long)vs.nrows * ch + row;
            double *vout = vis + 2 * vidx;
            for (int tu = cu - wsup; tu <= cu + wsup; ++tu) {
                for (int tv = cv - wsup; tv <= cv + wsup; ++tv) {
                    const double k = oracle_kb_tap(u / gs.du - tu, v / gs.dv - tv, beta, wd);
                    const int sign = 1 - 2 * ((tu + tv) & 1);
                    double wre = 0.5 * k * sign;
                    double wim = 0.5 * k * sign;
                    int gu = orc_wrap(tu, gs.nu);
                    int gv = orc_wrap(tv, gs.nv);
                    if (gv >= gs.half_nv) { /* Hermitian fold onto the stored half plane */
                        gu = (gs.nu - gu) % gs.nu;
                        gv = gs.nv - gv;
                        wim = -wim;
                    }
                    const long cell = (long)gs.half_nv * gu + gv;
                    if (direction == 0) {
                        const double gre = wre * grid[2 * cell + 0];
                        const double gim = wim * grid[2 * cell + 1];
#pragma omp atomic
                        vout[0] += 2 * (cph * gre + sph * gim);
#pragma omp atomic
                        vout[1] += 2 * (-sph * gre + cph * gim);
                    } else if (direction == 1) {
                        if (gv == 0) {
                            wre *= 2;
                            wim *= 2;
                        }
                        const double vre = vout[0];
                        const double vim = vout[1];
#pragma omp atomic
                        grid[2 * cell + 0] += wre * (cph * vre - sph * vim);
#pragma omp atomic
                        grid[2 * cell + 1] += wim * (sph * vre + cph * vim);
                    }
                }
            }
        }
    }
}

/* 2F1 series of O'Riordan et al. for the PEMD deflection, fixed 20 terms.
 * Restates hyp2f1_series, lentils/backend/deflect.c:179-225 (value only). */
static double complex orc_hyp2f1(double t, double q, double complex z)
{
    const double x = creal(z), y = cimag(z);
    const double r2 = q * q * x * x + y * y;
    const double qp = (1 - q * q) / (q * q);
    const double complex w2 = qp * r2 / (z * z);
    const double complex u = 0.5 * (1.0 - csqrt(1.0 - w2));
    double complex f = 0.0;
    double complex un = 1.0;
    double an = 1.0;
    for (int n = 0; n < 20; ++n) {
        f += an * un;
        const double ntf = 2 * n + 4 - t;
        un *= u;
        an *= (ntf - t) / ntf;
    }
    return f;
}

/* PEMD deflection. fpars: x, y, f(=q), th, sin(th+90), cos(th+90), b, qh, rc.
 * Restates deflect_PEMD_series, lentils/backend/deflect.c:243-301 (value only). */
static void orc_pemd(const lentils_mass_model *m, const double *xin, double *a)
{
    const double *p = m->fpars;
    const double t = 2 * p[7];
    const double q = p[2];
    const double b = pow(0.5 * p[6] * pow(q, t - 0.5) * (3.0 - t) / (2.0 - t), 1.0 / t);
    const double complex rot = p[5] - I * p[4];
    const double complex z = ((xin[0] - p[0]) + I * (xin[1] - p[1])) * rot;
    const double x = creal(z), y = cimag(z);
    const double rs = sqrt(q * q * x * x + y * y);
    const double complex A = b * b / (q * z) * pow(b / rs, t - 2);
    const double complex F = orc_hyp2f1(t, q, z);
    const double complex al = conj(A * F * rot);
    a[0] += creal(al);
    a[1] += cimag(al);
}

/* External shear + convergence/shear gradients (Keeton 2001).
 * fpars: x, y, ss, sa, sin(sa+90), cos(sa+90), gks, gka, sin(gka+90), cos(gka+90), gss, gsa,
 * sin(gsa+90), cos(gsa+90). Restates deflect_external_potential, deflect.c:70-108. */
static void orc_shear(const lentils_mass_model *m, const double *xin, double *a)
{
    const double *p = m->fpars;
    const double sx = xin[0] - p[0], sy = xin[1] - p[1];
    const double c2 = -p[5] * p[5] + p[4] * p[4];
    const double s2 = -2 * p[4] * p[5];
    a[0] += p[2] * (c2 * sx + s2 * sy);
    a[1] += p[2] * (s2 * sx - c2 * sy);
    double rx = sx * p[9] + sy * p[8];
    double ry = -sx * p[8] + sy * p[9];
    double dx = -0.25 * p[6] * (3 * rx * rx + ry * ry);
    double dy = -0.5 * p[6] * rx * ry;
    a[0] += dx * p[9] - dy * p[8];
    a[1] += dx * p[8] + dy * p[9];
    rx = sx * p[13] + sy * p[12];
    ry = -sx * p[12] + sy * p[13];
    dx = -0.5 * p[10] * (rx * rx - ry * ry);
    dy = 1.0 * p[10] * rx * ry;
    a[0] += dx * p[13] - dy * p[12];
    a[1] += dx * p[12] + dy * p[13];
}

/* Internal multipoles of order 3..ipars[0]. fpars: x, y, qh, then (a_m, b_m) pairs.
 * Restates deflect_internal_multipoles, deflect.c:126-175. */
static void orc_multipoles(const lentils_mass_model *m, const double *xin, double *a)
{
    const double *p = m->fpars;
    const double sx = xin[0] - p[0], sy = xin[1] - p[1];
    const double r = sqrt(sx * sx + sy * sy);
    const double th = atan2(sy, sx);
    const double cn = sx / r, sn = sy / r;
    for (int mm = 3; mm <= m->ipars[0]; ++mm) {
        const double am = p[3 + 2 * (mm - 3) + 0];
        const double bm = p[3 + 2 * (mm - 3) + 1];
        const double al = 2.0 * p[2];
        const double bs = 1.0;
        const double norm = 2.0 * pow(bs, al) / (mm * mm - (al - 2) * (al - 2));
        const double cm = cos(mm * th), sm = sin(mm * th);
        const double dr = -norm * (2.0 - al) * pow(r, 1.0 - al) * (bm * sm + am * cm);
        const double dt = norm * mm * pow(r, 1.0 - al) * (-bm * cm + am * sm);
        a[0] += cn * dr - sn * dt;
        a[1] += sn * dr + cn * dt;
    }
}

/* x_out = x_in - sum_l alpha_l(x_in) for each point (single plane: every lens sees x_in).
 * Restates deflect / deflect_points, lentils/backend/deflect.c:26-66. */
void oracle_deflect_points(lentils_global_lens_model glm, const double *pin, int npoints,
                           double *pout)
{
    for (int i = 0; i < npoints; ++i) {
        const double *xin = pin + 2 * i;
        double *xo = pout + 2 * i;
        xo[0] = xin[0];
        xo[1] = xin[1];
        for (int l = 0; l < glm.num_lenses; ++l) {
            double al[2] = {0.0, 0.0};
            const lentils_mass_model *m = &glm.lenses[l];
            if (m->type == 0) orc_pemd(m, xin, al);
            else if (m->type == 1) orc_shear(m, xin, al);
            else if (m->type == 2) orc_multipoles(m, xin, al);
            xo[0] -= al[0];
            xo[1] -= al[1];
        }
    }
}

/* Forward-difference gradient CSR: rows 0..nx*ny-1 hold d/dx (zero rows at ix = nx-1), rows
 * nx*ny..2*nx*ny-1 hold d/dy (zero rows at iy = ny-1), entries -1/h then +1/h.
 * Restates grad_matrix_findiff_csr, lentils/backend/nufft.c:163-194. */
void oracle_grad_findiff_csr(lentils_image_space im, int *rows, int *cols, double *vals)
{
    int r = 0, k = 0;
    for (int ix = 0; ix < im.nx; ++ix)
        for (int iy = 0; iy < im.ny; ++iy, ++r) {
            rows[r] = k;
            if (ix < im.nx - 1) {
                vals[k] = -1.0 / im.dx; cols[k++] = im.ny * ix + iy;
                vals[k] = 1.0 / im.dx;  cols[k++] = im.ny * (ix + 1) + iy;
            }
        }
    for (int ix = 0; ix < im.nx; ++ix)
        for (int iy = 0; iy < im.ny; ++iy, ++r) {
            rows[r] = k;
            if (iy < im.ny - 1) {
                vals[k] = -1.0 / im.dy; cols[k++] = im.ny * ix + iy;
                vals[k] = 1.0 / im.dy;  cols[k++] = im.ny * ix + iy + 1;
            }
        }
    rows[r] = k;
}

/* Direct Fourier transform as a dense real matrix with 2*nrows rows (cos, sin) over the
 * unmasked pixels, pixel positions at the lower-left corners x = xmin + i*dx.
 * Restates dft_matrix_csr, lentils/backend/nufft.c:128-161, densely (row-major, nrows*2 x
 * npix; masked columns are zero). */
void oracle_dft_dense(lentils_visibility_space vs, lentils_image_space im, double *mat)
{
    const long npix = (long)im.nx * im.ny;
    for (int row = 0; row < 2 * vs.nrows; ++row) {
        const int iv = row / 2, odd = row % 2;
        const double u = vs.uv[3 * iv + 0] * vs.channels[0];
        const double v = -vs.uv[3 * iv + 1] * vs.channels[0];
        double *out = mat + (long)row * npix;
        for (int ix = 0, col = 0; ix < im.nx; ++ix)
            for (int iy = 0; iy < im.ny; ++iy, ++col) {
                if (!im.mask[col]) { out[col] = 0.0; continue; }
                const double x = ix * im.dx + im.xmin;
                const double y = iy * im.dy + im.ymin;
                const double arg = -2.0 * M_PI * ORC_ARCSEC_TO_RAD * (u * x + v * y);
                out[col] = odd ? sin(arg) : cos(arg);
            }
    }
}

double oracle_bessel_i0(double x) { return gsl_sf_bessel_I0(x); }
