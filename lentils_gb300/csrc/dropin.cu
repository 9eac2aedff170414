// Drop-in entry points with the reference's exact C signatures (host pointers, by-value
// structs, void return). Each stages its inputs on the current CUDA device, runs the GPU
// kernels and copies the results back; failures are reported through lentils_last_error()
// and printed to stderr, since the reference's signatures have no error channel.
#include <stdio.h>

#include <mutex>
#include <vector>

#include "common.cuh"

namespace lentils {
int deflect_derivatives(const lentils_mass_model *lenses, int nlenses, const double *points,
                        double *grads, double *sum12, long long n, cudaStream_t s);
}  // namespace lentils

using namespace lentils;

namespace {

void report(const char *fn)
{
    fprintf(stderr, "lentils_gb300 %s failed (status %d): %s\n", fn, lentils_last_error(),
            lentils_last_error_message());
}

// Forward-difference gradient CSR, closed form per row (so rows fill in parallel):
// x-rows r < nx*ny have entries iff ix < nx-1; y-rows have entries iff iy < ny-1.
// Same layout and values as grad_matrix_findiff_csr, lentils/backend/nufft.c:163-194.
__global__ void grad_csr_kernel(int nx, int ny, double dx, double dy, int *rows, int *cols,
                                double *vals)
{
    const long long n = (long long)nx * ny;
    const long long nx_entries = 2LL * (nx - 1) * ny;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r <= 2 * n;
         r += (long long)gridDim.x * blockDim.x) {
        if (r == 2 * n) {
            rows[r] = (int)(nx_entries + 2LL * nx * (ny - 1));
            continue;
        }
        if (r < n) {
            const int ix = (int)(r / ny), iy = (int)(r % ny);
            const long long k = 2LL * std::min<long long>(r, (long long)(nx - 1) * ny);
            rows[r] = (int)k;
            if (ix < nx - 1) {
                vals[k] = -1.0 / dx;
                cols[k] = ny * ix + iy;
                vals[k + 1] = 1.0 / dx;
                cols[k + 1] = ny * (ix + 1) + iy;
            }
        } else {
            const long long rr = r - n;
            const int ix = (int)(rr / ny), iy = (int)(rr % ny);
            const long long k = nx_entries + 2LL * ((long long)ix * (ny - 1) + std::min(iy, ny - 1));
            rows[r] = (int)k;
            if (iy < ny - 1) {
                vals[k] = -1.0 / dy;
                cols[k] = ny * ix + iy;
                vals[k + 1] = 1.0 / dy;
                cols[k + 1] = ny * ix + iy + 1;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------
// Plan cache of the drop-in grid_cpu.
//
// The reference calls grid_cpu on every operator application with the same visibility space
// (GriddingOperator._matrixfree_forward/_transpose, fourier_operators.py:85-93), so binning the
// uv set (lentils_plan_create: FP64 coordinates, radix sort, device arrays) on every call would
// cost more than the gridding itself. Plans are kept, least recently used first out, keyed by
// the device, the uv buffer's address, nrows, the channel values, the grid geometry (nu, nv,
// du, dv, gcx, gcy), wsup and beta, and a digest of the uv contents:
//   mode 1 (default): the digest covers 4096 rows spread evenly over the buffer plus its last
//                     row -- microseconds, and it catches a new uv set at a reused address;
//   mode 2:           the digest covers every byte of uv (about 30 ms per 1e7 rows);
//   mode 0:           no cache: every call bins the uv set anew.
// A caller that rewrites a uv buffer in place between calls, keeping the sampled rows, must
// use mode 2 or clear the cache (lentils_dropin_cache_clear). Calls are serialised by one
// mutex, since a cached plan's staging buffers are shared.
// ---------------------------------------------------------------------------------------
constexpr int kCacheSlots = 4;
constexpr int kDigestRows = 4096;

struct CachedPlan {
    int device;
    const double *uv;
    int nrows;
    std::vector<double> chans;
    int nu, nv;
    double du, dv, gcx, gcy;
    int wsup;
    double beta;
    unsigned long long digest;
    unsigned long long last_use;
    lentils_plan *plan;
};

std::mutex g_cache_mu;
std::vector<CachedPlan> g_cache;
unsigned long long g_tick = 0;
int g_cache_mode = 1;

unsigned long long mix_word(unsigned long long h, unsigned long long x)
{
    h ^= x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
    return h * 0x100000001b3ull;
}

unsigned long long uv_digest(const double *uv, int nrows, int mode)
{
    unsigned long long h = 0xcbf29ce484222325ull ^ (unsigned long long)nrows;
    auto row = [&](long long r) {
        unsigned long long w[3];
        memcpy(w, uv + 3 * r, sizeof(w));
        h = mix_word(mix_word(mix_word(h, w[0]), w[1]), w[2]);
    };
    if (mode == 2 || nrows <= kDigestRows) {
        for (long long r = 0; r < nrows; ++r) row(r);
    } else {
        for (long long k = 0; k < kDigestRows; ++k) row(k * (long long)nrows / kDigestRows);
        row(nrows - 1);
    }
    return h;
}

void destroy_cached(CachedPlan &c)
{
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != c.device) cudaSetDevice(c.device);
    lentils_plan_destroy(c.plan);
    if (cur >= 0 && cur != c.device) cudaSetDevice(cur);
    c.plan = nullptr;
}

// The plan for this call: a cached one when every key matches, else a new one (cached unless
// mode 0). *owned is set when the caller must destroy the returned plan itself.
int cached_plan(const lentils_visibility_space &vs, const lentils_fourier_space &gs, int wsup,
                double beta, lentils_plan **out, bool *owned)
{
    int dev = 0;
    LENTILS_CUDA_TRY(cudaGetDevice(&dev));
    *owned = false;
    const unsigned long long dig = g_cache_mode ? uv_digest(vs.uv, vs.nrows, g_cache_mode) : 0;
    if (g_cache_mode) {
        for (CachedPlan &c : g_cache) {
            if (c.device == dev && c.uv == vs.uv && c.nrows == vs.nrows &&
                (int)c.chans.size() == vs.nchannels &&
                memcmp(c.chans.data(), vs.channels, sizeof(double) * vs.nchannels) == 0 &&
                c.nu == gs.nu && c.nv == gs.nv && c.du == gs.du && c.dv == gs.dv &&
                c.gcx == gs.gcx && c.gcy == gs.gcy && c.wsup == wsup && c.beta == beta &&
                c.digest == dig) {
                c.last_use = ++g_tick;
                *out = c.plan;
                return LENTILS_OK;
            }
        }
    }
    lentils_grid_desc gd;
    memset(&gd, 0, sizeof(gd));
    gd.nu = gs.nu;
    gd.nv = gs.nv;
    gd.du = gs.du;
    gd.dv = gs.dv;
    gd.gcx = gs.gcx;
    gd.gcy = gs.gcy;
    gd.wsup = wsup;
    gd.kb_beta = beta;
    lentils_plan *plan = nullptr;
    if (int st = lentils_plan_create(&plan, &gd, vs.uv, vs.nrows, vs.channels, vs.nchannels, 0,
                                     nullptr))
        return st;
    if (!g_cache_mode) {
        *out = plan;
        *owned = true;
        return LENTILS_OK;
    }
    for (size_t i = 0; i < g_cache.size();) {  // same buffer, other contents: stale
        if (g_cache[i].device == dev && g_cache[i].uv == vs.uv) {
            destroy_cached(g_cache[i]);
            g_cache.erase(g_cache.begin() + i);
        } else {
            ++i;
        }
    }
    if ((int)g_cache.size() >= kCacheSlots) {  // evict the least recently used plan
        size_t lru = 0;
        for (size_t i = 1; i < g_cache.size(); ++i)
            if (g_cache[i].last_use < g_cache[lru].last_use) lru = i;
        destroy_cached(g_cache[lru]);
        g_cache.erase(g_cache.begin() + lru);
    }
    CachedPlan c;
    c.device = dev;
    c.uv = vs.uv;
    c.nrows = vs.nrows;
    c.chans.assign(vs.channels, vs.channels + vs.nchannels);
    c.nu = gs.nu;
    c.nv = gs.nv;
    c.du = gs.du;
    c.dv = gs.dv;
    c.gcx = gs.gcx;
    c.gcy = gs.gcy;
    c.wsup = wsup;
    c.beta = beta;
    c.digest = dig;
    c.last_use = ++g_tick;
    c.plan = plan;
    g_cache.push_back(c);
    *out = plan;
    return LENTILS_OK;
}

int grid_cpu_impl(lentils_visibility_space vs, double *vis, lentils_fourier_space gs,
                  double *grid, int wsup, double beta, int direction)
{
    if (direction != 0 && direction != 1)
        return set_error(LENTILS_ERR_INVALID, "grid_cpu: direction %d (0 or 1)", direction);
    if (vs.nrows < 0 || vs.nchannels < 1 || !vis || !grid)
        return set_error(LENTILS_ERR_INVALID, "grid_cpu: bad visibility space or buffers");
    if (vs.nrows > 0 && (!vs.uv || !vs.channels))
        return set_error(LENTILS_ERR_INVALID, "grid_cpu: null uv or channels");
    if (gs.half_nv != gs.nv / 2 + 1)
        return set_error(LENTILS_ERR_UNSUPPORTED, "grid_cpu: half_nv=%d, expected nv/2+1",
                         gs.half_nv);
    if (vs.nrows == 0) return LENTILS_OK;
    std::lock_guard<std::mutex> lock(g_cache_mu);
    lentils_plan *plan = nullptr;
    bool owned = false;
    int st = cached_plan(vs, gs, wsup, beta, &plan, &owned);
    if (st) return st;
    if (direction == 0) st = lentils_degrid_host(plan, grid, vis, 1, nullptr);
    else st = lentils_grid_host(plan, vis, grid, 1, nullptr);
    if (!owned) return st;
    const int code = st ? lentils_last_error() : LENTILS_OK;
    char msg[512] = {0};
    if (st) strncpy(msg, lentils_last_error_message(), sizeof(msg) - 1);
    lentils_plan_destroy(plan);
    if (st) return set_error(code, "%s", msg);
    return LENTILS_OK;
}

// want_deriv != 0: deriv[0..11] += the PEMD derivatives d alpha / d (b, qh, q, x, y, th)
// (x, y components) summed over all points and PEMD lenses, which is what the reference's
// deflect_points does with its single deriv pointer (deflect.c:26-66, 330-338).
int deflect_points_impl(lentils_global_lens_model glm, double *pin, int n, double *pout,
                        int want_deriv, double *deriv)
{
    if (n < 0 || (n > 0 && (!pin || !pout)) || glm.num_lenses < 0 ||
        (glm.num_lenses > 0 && !glm.lenses) || (want_deriv && !deriv))
        return set_error(LENTILS_ERR_INVALID, "deflect_points: bad arguments");
    if (n == 0) return LENTILS_OK;
    double *din = nullptr, *dout = nullptr;
    const size_t bytes = sizeof(double) * 2 * (size_t)n;
    int st = LENTILS_OK;
    cudaError_t e = cudaMalloc(&din, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dout, bytes);
    if (e == cudaSuccess) e = cudaMemcpy(din, pin, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) st = cuda_status(e, "deflect_points staging");
    if (!st) st = lentils_deflect_f64io(glm.lenses, glm.num_lenses, din, dout, n, nullptr);
    if (!st) {
        e = cudaMemcpy(pout, dout, bytes, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_status(e, "deflect_points copy back");
    }
    if (!st && want_deriv) {
        double *dsum = nullptr;
        double hsum[12];
        e = cudaMalloc(&dsum, sizeof(hsum));
        if (e == cudaSuccess) e = cudaMemset(dsum, 0, sizeof(hsum));
        if (e != cudaSuccess) st = cuda_status(e, "deflect_points derivatives");
        if (!st) st = deflect_derivatives(glm.lenses, glm.num_lenses, din, nullptr, dsum, n, nullptr);
        if (!st) {
            e = cudaMemcpy(hsum, dsum, sizeof(hsum), cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) st = cuda_status(e, "deflect_points derivatives copy back");
        }
        if (!st)
            for (int k = 0; k < 12; ++k) deriv[k] += hsum[k];
        cudaFree(dsum);
    }
    cudaFree(din);
    cudaFree(dout);
    return st;
}

int grad_csr_impl(lentils_image_space im, int *rows, int *cols, double *vals)
{
    if (im.nx < 1 || im.ny < 1 || !rows || !cols || !vals)
        return set_error(LENTILS_ERR_INVALID, "grad_matrix_findiff_csr: bad arguments");
    const long long n = (long long)im.nx * im.ny;
    const long long nnz = 2LL * (im.nx - 1) * im.ny + 2LL * im.nx * (im.ny - 1);
    int *drows = nullptr, *dcols = nullptr;
    double *dvals = nullptr;
    int st = LENTILS_OK;
    cudaError_t e = cudaMalloc(&drows, sizeof(int) * (2 * n + 1));
    if (e == cudaSuccess) e = cudaMalloc(&dcols, sizeof(int) * std::max(nnz, 1LL));
    if (e == cudaSuccess) e = cudaMalloc(&dvals, sizeof(double) * std::max(nnz, 1LL));
    if (e != cudaSuccess) st = cuda_status(e, "grad_matrix_findiff_csr alloc");
    if (!st) {
        long long blocks = (2 * n + 1 + 255) / 256;
        if (blocks > 152 * 32) blocks = 152 * 32;
        grad_csr_kernel<<<(int)blocks, 256>>>(im.nx, im.ny, im.dx, im.dy, drows, dcols, dvals);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpy(rows, drows, sizeof(int) * (2 * n + 1), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && nnz > 0) e = cudaMemcpy(cols, dcols, sizeof(int) * nnz, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess && nnz > 0) e = cudaMemcpy(vals, dvals, sizeof(double) * nnz, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) st = cuda_status(e, "grad_matrix_findiff_csr");
    }
    cudaFree(drows);
    cudaFree(dcols);
    cudaFree(dvals);
    return st;
}

}  // namespace

extern "C" {

void grid_cpu(lentils_visibility_space vs, double *vis, lentils_fourier_space gs, double *grid,
              int wsup, double kb_beta, int direction)
{
    clear_error();
    if (grid_cpu_impl(vs, vis, gs, grid, wsup, kb_beta, direction)) report("grid_cpu");
}

int lentils_dropin_cache_mode(int mode)
{
    clear_error();
    if (mode < 0 || mode > 2)
        return set_error(LENTILS_ERR_INVALID, "dropin_cache_mode: %d (0, 1 or 2)", mode);
    std::lock_guard<std::mutex> lock(g_cache_mu);
    if (mode != g_cache_mode) {  // digests of another mode do not compare
        for (CachedPlan &c : g_cache) destroy_cached(c);
        g_cache.clear();
    }
    g_cache_mode = mode;
    return LENTILS_OK;
}

int lentils_dropin_cache_clear(void)
{
    clear_error();
    std::lock_guard<std::mutex> lock(g_cache_mu);
    for (CachedPlan &c : g_cache) destroy_cached(c);
    g_cache.clear();
    return LENTILS_OK;
}

int lentils_dropin_cache_size(void)
{
    std::lock_guard<std::mutex> lock(g_cache_mu);
    return (int)g_cache.size();
}

void deflect_points(lentils_global_lens_model glm, double *p_in, int npoints, double *p_out,
                    int want_deriv, double *deriv)
{
    clear_error();
    if (deflect_points_impl(glm, p_in, npoints, p_out, want_deriv, deriv))
        report("deflect_points");
}

void grad_matrix_findiff_csr(lentils_image_space imspace, int *row_inds, int *cols, double *vals)
{
    clear_error();
    if (grad_csr_impl(imspace, row_inds, cols, vals)) report("grad_matrix_findiff_csr");
}

}  // extern "C"
