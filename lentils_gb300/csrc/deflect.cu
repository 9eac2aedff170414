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
#include "deflect_device.cuh"

namespace lentils {

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
