// Host-side runtime of lentils_gb300: per-thread error state, the Kaiser-Bessel polynomial
// fit used by the gridding kernels, and small exported utilities.
#include <math.h>
#include <stdarg.h>

#include "common.cuh"

namespace lentils {

namespace {
thread_local int t_err = LENTILS_OK;
thread_local char t_msg[512] = {0};
}  // namespace

int set_error(int code, const char *fmt, ...)
{
    t_err = code;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
    va_end(ap);
    return code;
}

int clear_error()
{
    t_err = LENTILS_OK;
    t_msg[0] = 0;
    return LENTILS_OK;
}

int cuda_status(cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation)
        return set_error(LENTILS_ERR_ALLOC, "%s: %s", what, cudaGetErrorString(e));
    if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
        return set_error(LENTILS_ERR_NO_DEVICE, "%s: %s", what, cudaGetErrorString(e));
    return set_error(LENTILS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// Modified Bessel function I0 from its defining power series
// sum_k (x^2/4)^k / (k!)^2 (Abramowitz & Stegun 9.6.12); all terms are positive, so the
// running sum is accurate to a few ulp. Used only on the host, to fit the kernel polynomials.
double host_bessel_i0(double x)
{
    const double q = 0.25 * x * x;
    double sum = 1.0, term = 1.0;
    for (int k = 1; k < 100000; ++k) {
        term *= q / ((double)k * (double)k);
        sum += term;
        if (term < 1e-18 * sum) break;
    }
    return sum;
}

// Kaiser-Bessel profile on one axis, I0(beta*sqrt(1-(a/w)^2)), zero outside [-w, w]
// (the per-axis factor of kb_g, lentils/backend/nufft.c:11-21).
static double kb_profile(double a, double w, double beta)
{
    if (!(a >= -w && a <= w)) return 0.0;
    double r = 1.0 - (a / w) * (a / w);
    if (r < 0.0) r = 0.0;
    return host_bessel_i0(beta * sqrt(r));
}

// Chebyshev interpolation (at the n Chebyshev points of the first kind) of each tap's weight
// as a function of t = 2f - 1, converted to monomial coefficients in t.
void kb_poly_build(int w, double beta, KBPoly *out, double *fit_err, KBPoly64 *out64)
{
    memset(out, 0, sizeof(*out));
    if (out64) memset(out64, 0, sizeof(*out64));
    const int n = kPolyCoef;
    const double norm = 1.0 / (2.0 * w);
    double worst = 0.0;
    const double peak = kb_profile(0.0, w, beta) * norm;
    double mono_all[kMaxTaps][kPolyCoef];
    for (int i = 0; i < w; ++i) {
        const double sgn = (i & 1) ? -1.0 : 1.0;
        double fval[kPolyCoef];
        for (int j = 0; j < n; ++j) {
            const double t = cos(M_PI * (j + 0.5) / n);
            const double f = 0.5 * (t + 1.0);
            fval[j] = sgn * norm * kb_profile(f + w - 1 - i, w, beta);
        }
        double cheb[kPolyCoef];
        for (int k = 0; k < n; ++k) {
            double s = 0.0;
            for (int j = 0; j < n; ++j) s += fval[j] * cos(M_PI * k * (j + 0.5) / n);
            cheb[k] = 2.0 * s / n;
        }
        cheb[0] *= 0.5;
        // monomial coefficients: accumulate c_k * T_k(t), T_k built by the three-term rule
        double mono[kPolyCoef] = {0};
        double tkm1[kPolyCoef] = {0}, tk[kPolyCoef] = {0}, tkp1[kPolyCoef];
        tkm1[0] = 1.0;  // T_0
        tk[1] = 1.0;    // T_1
        mono[0] += cheb[0];
        if (n > 1)
            for (int d = 0; d < n; ++d) mono[d] += cheb[1] * tk[d];
        for (int k = 2; k < n; ++k) {
            for (int d = 0; d < n; ++d)
                tkp1[d] = 2.0 * (d > 0 ? tk[d - 1] : 0.0) - tkm1[d];
            for (int d = 0; d < n; ++d) {
                mono[d] += cheb[k] * tkp1[d];
                tkm1[d] = tk[d];
                tk[d] = tkp1[d];
            }
        }
        for (int d = 0; d < n; ++d) {
            mono_all[i][d] = mono[d];
            // reflected tap 2w-1-i: P(t) = -P_i(-t)
            mono_all[2 * w - 1 - i][d] = ((d & 1) ? 1.0 : -1.0) * mono[d];
        }
        // even/odd tables, FP32 and FP64 (highest power of t^2 first)
        for (int k = 0; k < kHalfCoef; ++k) {
            if (out64) {
                out64->ce[k][i] = mono[2 * (kHalfCoef - 1 - k)];
                out64->co[k][i] = mono[2 * (kHalfCoef - 1 - k) + 1];
            }
            const float e = (float)mono[2 * (kHalfCoef - 1 - k)];
            const float o = (float)mono[2 * (kHalfCoef - 1 - k) + 1];
            if (i & 1) {
                out->ce[k][i >> 1].y = e;
                out->co[k][i >> 1].y = o;
            } else {
                out->ce[k][i >> 1].x = e;
                out->co[k][i >> 1].x = o;
            }
        }
    }
    for (int i = 0; i < 2 * w; ++i) {
        const double sgn = (i & 1) ? -1.0 : 1.0;
        if (fit_err) {
            for (int s = 0; s <= 400; ++s) {
                const double t = -1.0 + s / 200.0;
                double acc = 0.0;
                for (int d = n - 1; d >= 0; --d) acc = acc * t + mono_all[i][d];
                const double ref = sgn * norm * kb_profile(0.5 * (t + 1.0) + w - 1 - i, w, beta);
                const double e = fabs(acc - ref) / peak;
                if (e > worst) worst = e;
            }
        }
    }
    // extra tap at argument exactly +w (frac == 0): profile I0(0) = 1, tap index -1 -> sign -1
    out->edge = (float)(-norm * kb_profile((double)w, w, beta));
    if (out64) out64->edge = -norm * kb_profile((double)w, w, beta);
    if (fit_err) *fit_err = worst;
}

// Full per-tap monomial table (highest degree first) reconstructed from the FP32 even/odd
// table, as the kernels evaluate it.
void kb_poly_taps(const KBPoly &p, int w, float *coef /* 2w x kPolyCoef */)
{
    for (int i = 0; i < w; ++i) {
        float mono[kPolyCoef];
        for (int k = 0; k < kHalfCoef; ++k) {
            const float e = (i & 1) ? p.ce[k][i >> 1].y : p.ce[k][i >> 1].x;
            const float o = (i & 1) ? p.co[k][i >> 1].y : p.co[k][i >> 1].x;
            mono[2 * (kHalfCoef - 1 - k)] = e;
            mono[2 * (kHalfCoef - 1 - k) + 1] = o;
        }
        for (int d = 0; d < kPolyCoef; ++d) {
            coef[i * kPolyCoef + (kPolyCoef - 1 - d)] = mono[d];
            coef[(2 * w - 1 - i) * kPolyCoef + (kPolyCoef - 1 - d)] = ((d & 1) ? 1.f : -1.f) * mono[d];
        }
    }
}

}  // namespace lentils

extern "C" {

int lentils_last_error(void) { return lentils::t_err; }
const char *lentils_last_error_message(void) { return lentils::t_msg; }
int lentils_version(void) { return 10000; }

// copy `bytes` from a device array to host memory once all device work has finished (the
// producer may have run on any stream, including a non-blocking one)
int lentils_copy_to_host(void *dst, const void *src, long long bytes)
{
    lentils::clear_error();
    if (bytes < 0 || (bytes > 0 && (!dst || !src)))
        return lentils::set_error(LENTILS_ERR_INVALID, "copy_to_host: bad arguments");
    if (!bytes) return LENTILS_OK;
    LENTILS_CUDA_TRY(cudaDeviceSynchronize());
    LENTILS_CUDA_TRY(cudaMemcpy(dst, src, (size_t)bytes, cudaMemcpyDeviceToHost));
    return LENTILS_OK;
}

// release a device array that an entry point allocated for the caller
int lentils_device_free(void *ptr)
{
    lentils::clear_error();
    LENTILS_CUDA_TRY(cudaFree(ptr));
    return LENTILS_OK;
}

// Host-only helper (no GPU needed): the per-tap polynomial table for (w, beta), as
// kPolyCoef x 2w floats, tap-major (coef[i*kPolyCoef + k], highest degree first), and the
// FP64 fit error relative to the kernel peak. Exposed for tests and diagnostics.
int lentils_kb_poly_table(int w, double beta, float *coef, int ncoef_capacity, double *fit_err)
{
    lentils::clear_error();
    if (w < 1 || w > lentils::kMaxW || !coef)
        return lentils::set_error(LENTILS_ERR_INVALID, "kb_poly_table: bad w=%d", w);
    if (ncoef_capacity < 2 * w * lentils::kPolyCoef)
        return lentils::set_error(LENTILS_ERR_INVALID, "kb_poly_table: capacity too small");
    lentils::KBPoly p;
    lentils::kb_poly_build(w, beta, &p, fit_err);
    lentils::kb_poly_taps(p, w, coef);
    return LENTILS_OK;
}

int lentils_kb_poly_ncoef(void) { return lentils::kPolyCoef; }

}  // extern "C"
