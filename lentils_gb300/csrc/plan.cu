// Gridding plan: one-time binning of visibilities by uv tile, the frame
// transforms between the reference's row order and plan order, and the host-buffer forms of
// degrid/grid.
//
// Plan construction, per visibility (FP64, reference conventions of grid_cpu,
// lentils/backend/nufft.c:60-66):
//   u = uv[0]*ch, v = -uv[1]*ch, (ug, vg) = (u/du, v/dv)
//   wrap (ug, vg) into the canonical window [-nu/2, nu-nu/2) x [-nv/2, nv-nv/2) by whole grid
//   periods (ku, kv); the tap cells then equal the reference's wrapped cells, and the
//   reference's checkerboard sign on unwrapped indices becomes s = (-1)^(ku*nu + kv*nv);
//   quantise to 24-bit fixed point, split into tile, cell-in-tile and fraction;
//   phase = s * e^{-i 2pi (u*gcx + v*gcy)} (truncated 2pi as in nufft.c:63-64).
// Visibilities are then stably sorted by (tile, cell) and the tiles are cut into work items of
// at most `chunk` visibilities.
#include <cub/cub.cuh>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"

namespace lentils {

// flags bits
constexpr int kFlagGuard = 1;
constexpr int kFlagNonFinite = 2;

// Canonical tile / cell / fraction of one axis, and the reference's edge-tap membership.
// g is the reference's grid coordinate u/du (unwrapped). Tap i is in the reference's set iff
// |g - i| <= w evaluated in FP64 (kb_g, nufft.c:12); with b the floor of the quantised
// coordinate (in the unwrapped frame) the candidates are b-w .. b+w.
__device__ __forceinline__ void canon_axis(double g, int n, int H, int logT, int T, int w,
                                           long long &k, int &tile, int &cell, uint32_t &word,
                                           float &res)
{
    const double g0 = g;
    k = (long long)floor((g + (double)H) / (double)n);
    g -= (double)k * (double)n;
    long long q = llrint(ldexp(g, kFracBits));
    long long c = (q >> kFracBits) + H;
    if (c < 0) {
        q += (long long)n << kFracBits;
        k -= 1;
        c += n;
    } else if (c >= n) {
        q -= (long long)n << kFracBits;
        k += 1;
        c -= n;
    }
    const uint32_t frac = (uint32_t)(q & (long long)kFracMask);
    res = (float)(g - ldexp((double)q, -kFracBits));  // |res| <= 2^-25, exact difference
    tile = (int)(c >> logT);
    cell = (int)(c & (T - 1));
    const double b = (double)((q >> kFracBits) + k * (long long)n);  // floor, unwrapped frame
    const bool extra = (g0 - (b - w)) <= (double)w;
    const bool top_off = !((g0 - (b + w)) >= -(double)w);
    word = ((uint32_t)cell << kFracBits) | frac | (extra ? kExtraTapBit : 0u) |
           (top_off ? kTopOffBit : 0u);
}

__global__ void canon_kernel(const double *__restrict__ uvw, const double *__restrict__ chans,
                             CanonParams p, unsigned *__restrict__ keys, int *__restrict__ idx,
                             uint2 *__restrict__ coords, float2 *__restrict__ phase,
                             int *__restrict__ tile_counts, int *__restrict__ flags,
                             float2 *__restrict__ res)
{
    const long long total = (long long)p.nrows * p.nch;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        const int ch = (int)(n / p.nrows);
        const int row = (int)(n - (long long)ch * p.nrows);
        const double scale = chans[ch];
        const double u = uvw[3 * (long long)row + 0] * scale;
        const double v = -uvw[3 * (long long)row + 1] * scale;
        const double ug = u / p.du, vg = v / p.dv;
        if (!isfinite(ug) || !isfinite(vg)) {
            atomicOr(flags, kFlagNonFinite);
            keys[n] = 0xffffffffu;
            idx[n] = (int)n;
            coords[n] = make_uint2(0, 0);
            phase[n] = make_float2(0.f, 0.f);
            if (res) res[n] = make_float2(0.f, 0.f);
            continue;
        }
        if (p.guard && (fabs(ug) + p.w + 1 > 0.5 * p.nu || fabs(vg) + p.w + 1 > 0.5 * p.nv))
            atomicOr(flags, kFlagGuard);
        long long ku, kv;
        int tu, tv, lu, lv;
        uint32_t wu, wv;
        float ru, rv;
        canon_axis(ug, p.nu, p.Hu, p.logT, p.T, p.w, ku, tu, lu, wu, ru);
        canon_axis(vg, p.nv, p.Hv, p.logT, p.T, p.w, kv, tv, lv, wv, rv);
        if (res) res[n] = make_float2(ru, rv);
        const int tile = tu * p.ntv + tv;
        keys[n] = ((unsigned)tile << (2 * p.logT)) | ((unsigned)lu << p.logT) | (unsigned)lv;
        idx[n] = (int)n;
        coords[n] = make_uint2(wu, wv);
        const long long par = (ku * (long long)p.nu + kv * (long long)p.nv) & 1LL;
        double sn, cs;
        sincos(kTwoPiTrunc * (u * p.gcx + v * p.gcy), &sn, &cs);
        const float s = par ? -1.f : 1.f;
        phase[n] = make_float2(s * (float)cs, -s * (float)sn);
        atomicAdd(&tile_counts[tile], 1);
    }
}

__global__ void gather_plan_kernel(const int *__restrict__ perm, const uint2 *__restrict__ cin,
                                   const float2 *__restrict__ pin, uint2 *__restrict__ cout,
                                   float2 *__restrict__ pout, long long n,
                                   const float2 *__restrict__ rin, float2 *__restrict__ rout)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const int s = perm[k];
        cout[k] = cin[s];
        pout[k] = pin[s];
        if (rin) rout[k] = rin[s];
    }
}

// plan order <- user order:  x[k] = conj(phase[k]) * V[perm[k]]
template <typename TU>
__global__ void to_plan_kernel(const int *__restrict__ perm, const float2 *__restrict__ phase,
                               const TU *__restrict__ vu, float2 *__restrict__ vp, long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const TU v = vu[perm[k]];
        const float2 ph = phase[k];
        const float re = (float)v.x, im = (float)v.y;
        vp[k] = make_float2(ph.x * re + ph.y * im, ph.x * im - ph.y * re);
    }
}

// user order <- plan order:  V[perm[k]] (+)= phase[k] * y[k]
template <typename TU>
__global__ void from_plan_kernel(const int *__restrict__ perm, const float2 *__restrict__ phase,
                                 const float2 *__restrict__ vp, TU *__restrict__ vu, long long n,
                                 int accumulate)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const float2 y = vp[k];
        const float2 ph = phase[k];
        const float re = ph.x * y.x - ph.y * y.y;
        const float im = ph.x * y.y + ph.y * y.x;
        TU &dst = vu[perm[k]];
        if (accumulate) {
            dst.x += re;
            dst.y += im;
        } else {
            dst.x = re;
            dst.y = im;
        }
    }
}

// Host-buffer forms on page-locked host memory read and write the user-order (host) side
// directly from the kernels, so the host side must be the coalesced one:
// plan order <- user order, by user index:  x[iperm[u]] = conj(phase) * V[u]
template <typename TU>
__global__ void to_plan_scatter_kernel(const int *__restrict__ iperm,
                                       const float2 *__restrict__ phase,
                                       const TU *__restrict__ vu, float2 *__restrict__ vp,
                                       long long n)
{
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < n;
         u += (long long)gridDim.x * blockDim.x) {
        const int k = iperm[u];
        const TU v = vu[u];
        const float2 ph = phase[k];
        const float re = (float)v.x, im = (float)v.y;
        vp[k] = make_float2(ph.x * re + ph.y * im, ph.x * im - ph.y * re);
    }
}

// user order <- plan order, by user index:  V[u] (+)= phase * y[iperm[u]]
template <typename TU>
__global__ void from_plan_gather_kernel(const int *__restrict__ iperm,
                                        const float2 *__restrict__ phase,
                                        const float2 *__restrict__ vp, TU *__restrict__ vu,
                                        long long n, int accumulate)
{
    for (long long u = blockIdx.x * (long long)blockDim.x + threadIdx.x; u < n;
         u += (long long)gridDim.x * blockDim.x) {
        const int k = iperm[u];
        const float2 y = vp[k];
        const float2 ph = phase[k];
        TU out;
        out.x = ph.x * y.x - ph.y * y.y;
        out.y = ph.x * y.y + ph.y * y.x;
        if (accumulate) {
            const TU old = vu[u];
            out.x += old.x;
            out.y += old.y;
        }
        vu[u] = out;
    }
}

__global__ void invert_perm_kernel(const int *__restrict__ perm, int *__restrict__ iperm,
                                   long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        iperm[perm[k]] = (int)k;
}

// plan order <- user order in FP64 (c128 both sides)
__global__ void to_plan64_kernel(const int *__restrict__ perm, const float2 *__restrict__ phase,
                                 const double2 *__restrict__ vu, double2 *__restrict__ vp,
                                 long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const double2 v = vu[perm[k]];
        const double px = phase[k].x, py = phase[k].y;
        vp[k] = make_double2(px * v.x + py * v.y, px * v.y - py * v.x);
    }
}

// user order <- plan order in FP64: V[perm[k]] (+)= phase[k] * y[k]
__global__ void from_plan64_kernel(const int *__restrict__ perm, const float2 *__restrict__ phase,
                                   const double2 *__restrict__ vp, double2 *__restrict__ vu,
                                   long long n, int accumulate)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const double2 y = vp[k];
        const double px = phase[k].x, py = phase[k].y;
        const double re = px * y.x - py * y.y, im = px * y.y + py * y.x;
        double2 &d = vu[perm[k]];
        if (accumulate) {
            d.x += re;
            d.y += im;
        } else {
            d = make_double2(re, im);
        }
    }
}

__global__ void gather_real_kernel(const int *__restrict__ perm, const double *__restrict__ u,
                                   double *__restrict__ out, long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        out[k] = u[perm[k]];
}

__global__ void c128_to_c64_kernel(const double2 *__restrict__ in, float2 *__restrict__ out,
                                   long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const double2 v = in[k];
        out[k] = make_float2((float)v.x, (float)v.y);
    }
}

__global__ void c64_to_c128_kernel(const float2 *__restrict__ in, double2 *__restrict__ out,
                                   long long n, int accumulate)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const float2 v = in[k];
        if (accumulate) {
            double2 o = out[k];
            o.x += (double)v.x;
            o.y += (double)v.y;
            out[k] = o;
        } else {
            out[k] = make_double2((double)v.x, (double)v.y);
        }
    }
}

static int grid_blocks(long long n, int threads = 256)
{
    long long b = (n + threads - 1) / threads;
    if (b > 152LL * 32) b = 152LL * 32;
    if (b < 1) b = 1;
    return (int)b;
}

int launch_c128_to_c64(const void *in, float2 *out, long long n, cudaStream_t s)
{
    if (n <= 0) return LENTILS_OK;
    c128_to_c64_kernel<<<grid_blocks(n), 256, 0, s>>>((const double2 *)in, out, n);
    LENTILS_CHECK_LAUNCH("c128_to_c64");
    return LENTILS_OK;
}

int launch_c64_to_c128(const float2 *in, void *out, long long n, int accumulate,
                       cudaStream_t s)
{
    if (n <= 0) return LENTILS_OK;
    c64_to_c128_kernel<<<grid_blocks(n), 256, 0, s>>>(in, (double2 *)out, n, accumulate);
    LENTILS_CHECK_LAUNCH("c64_to_c128");
    return LENTILS_OK;
}

// Launchers of the binning kernels for callers that own their buffers.
int launch_canon(const double *uvw, const double *chans, const CanonParams &p, unsigned *keys,
                 int *idx, uint2 *coords, float2 *phase, int *tile_counts, int *flags,
                 long long nvis, cudaStream_t s)
{
    if (nvis <= 0) return LENTILS_OK;
    canon_kernel<<<grid_blocks(nvis), 256, 0, s>>>(uvw, chans, p, keys, idx, coords, phase,
                                                   tile_counts, flags, nullptr);
    LENTILS_CHECK_LAUNCH("canon_kernel");
    return LENTILS_OK;
}

int launch_gather_plan(const int *perm, const uint2 *cin, const float2 *pin, uint2 *cout,
                       float2 *pout, long long n, cudaStream_t s)
{
    if (n <= 0) return LENTILS_OK;
    gather_plan_kernel<<<grid_blocks(n), 256, 0, s>>>(perm, cin, pin, cout, pout, n, nullptr,
                                                      nullptr);
    LENTILS_CHECK_LAUNCH("gather_plan_kernel");
    return LENTILS_OK;
}

int launch_to_plan_c64(const int *perm, const float2 *phase, const float2 *vu, float2 *vp,
                       long long n, cudaStream_t s)
{
    if (n <= 0) return LENTILS_OK;
    to_plan_kernel<float2><<<grid_blocks(n), 256, 0, s>>>(perm, phase, vu, vp, n);
    LENTILS_CHECK_LAUNCH("to_plan_kernel");
    return LENTILS_OK;
}

// defined in gridding.cu
// Same-cell chunks. mark[k] = k where a run of equal sort keys (one cell of one tile) or a
// work item starts, else 0; an inclusive max-scan then gives every visibility the start of its
// run, and a chunk starts every chunk_k visibilities from there.
__global__ void run_start_kernel(const unsigned *__restrict__ keys, int *__restrict__ mark,
                                 long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        mark[k] = (k == 0 || keys[k] != keys[k - 1]) ? (int)k : 0;
}

__global__ void item_start_kernel(const WorkItem *__restrict__ items, int nitems,
                                  int *__restrict__ mark)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x)
        mark[items[i].begin] = items[i].begin;
}

__global__ void chunk_start_kernel(const int *__restrict__ last, int *__restrict__ cflag,
                                   long long n, int K)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x)
        cflag[k] = ((k - last[k]) % K == 0) ? 1 : 0;
}

__global__ void chunk_write_kernel(const int *__restrict__ cflag, const int *__restrict__ cidx,
                                   int *__restrict__ chunk_begin, long long n)
{
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        if (cflag[k]) chunk_begin[cidx[k]] = (int)k;
        if (k == n - 1) chunk_begin[cidx[k] + cflag[k]] = (int)n;  // end of the last chunk
    }
}

__global__ void item_chunk_kernel(const WorkItem *__restrict__ items, int nitems,
                                  const int *__restrict__ cidx, long long n, int nchunks,
                                  int2 *__restrict__ out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += gridDim.x * blockDim.x) {
        const WorkItem it = items[i];
        const long long end = (long long)it.begin + it.count;
        out[i] = make_int2(cidx[it.begin], end < n ? cidx[end] : nchunks);
    }
}

struct MaxInt {
    __device__ int operator()(int a, int b) const { return a > b ? a : b; }
};

int launch_degrid(const lentils_plan *p, const float2 *grid, float2 *vis, cudaStream_t s,
                  const float *vscale = nullptr);
int launch_grid(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s);

static int ilog2_exact(int v)
{
    int l = 0;
    while ((1 << l) < v) ++l;
    return ((1 << l) == v) ? l : -1;
}

template <typename T>
static int dev_alloc(T **ptr, size_t count, long long *acct = nullptr)
{
    *ptr = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc((void **)ptr, count * sizeof(T));
    if (e != cudaSuccess) {
        *ptr = nullptr;
        return cuda_status(e, "cudaMalloc");
    }
    if (acct) *acct += (long long)(count * sizeof(T));
    return LENTILS_OK;
}

static void free_plan_arrays(lentils_plan *p)
{
    cudaFree(p->coords);
    cudaFree(p->perm);
    cudaFree(p->iperm);
    cudaFree(p->phase);
    cudaFree(p->coords_res);
    cudaFree(p->items);
    cudaFree(p->chunk_begin);
    cudaFree(p->item_chunks);
    cudaFree(p->stage_vis64);
    cudaFree(p->stage_grid64);
    cudaFree(p->stage_vis32);
    cudaFree(p->stage_grid32);
}

// RAII holder of temporaries used during plan construction.
struct DevTemps {
    std::vector<void *> ptrs;
    ~DevTemps()
    {
        for (void *q : ptrs) cudaFree(q);
    }
    template <typename T>
    int alloc(T **ptr, size_t count)
    {
        int st = dev_alloc(ptr, count);
        if (st == LENTILS_OK) ptrs.push_back((void *)*ptr);
        return st;
    }
};

// Visibilities per same-cell chunk of the degridding kernel for half-width w (0: none). The
// chunk's weights stay in registers, 4 * 2 * 2w floats; wider kernels keep one visibility per
// thread.
static int chunk_width(int w) { return w <= 4 ? 4 : 0; }

// Builds p->chunk_begin / p->item_chunks from the sorted keys (after p->items is on the
// device). Synchronises once, for the chunk count.
static int build_chunks(lentils_plan *p, const unsigned *keys_sorted, DevTemps &tmp,
                        cudaStream_t s)
{
    const long long n = p->nvis;
    const int K = chunk_width(p->geom.w);
    int *mark, *last, *cflag, *cidx;
    int st;
    if ((st = tmp.alloc(&mark, n))) return st;
    if ((st = tmp.alloc(&last, n))) return st;
    if ((st = tmp.alloc(&cflag, n))) return st;
    if ((st = tmp.alloc(&cidx, n))) return st;
    run_start_kernel<<<grid_blocks(n), 256, 0, s>>>(keys_sorted, mark, n);
    LENTILS_CHECK_LAUNCH("run_start_kernel");
    item_start_kernel<<<grid_blocks(p->nitems), 256, 0, s>>>(p->items, p->nitems, mark);
    LENTILS_CHECK_LAUNCH("item_start_kernel");
    size_t b1 = 0, b2 = 0;
    LENTILS_CUDA_TRY(cub::DeviceScan::InclusiveScan(nullptr, b1, mark, last, MaxInt(), n, s));
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, b2, cflag, cidx, n, s));
    unsigned char *temp;
    if ((st = tmp.alloc(&temp, std::max(b1, b2)))) return st;
    LENTILS_CUDA_TRY(cub::DeviceScan::InclusiveScan(temp, b1, mark, last, MaxInt(), n, s));
    chunk_start_kernel<<<grid_blocks(n), 256, 0, s>>>(last, cflag, n, K);
    LENTILS_CHECK_LAUNCH("chunk_start_kernel");
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(temp, b2, cflag, cidx, n, s));
    int tail[2] = {0, 0};
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&tail[0], cidx + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&tail[1], cflag + n - 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    const long long nchunks = (long long)tail[0] + tail[1];
    if ((st = dev_alloc(&p->chunk_begin, (size_t)nchunks + 1, &p->device_bytes))) return st;
    if ((st = dev_alloc(&p->item_chunks, (size_t)p->nitems, &p->device_bytes))) return st;
    chunk_write_kernel<<<grid_blocks(n), 256, 0, s>>>(cflag, cidx, p->chunk_begin, n);
    LENTILS_CHECK_LAUNCH("chunk_write_kernel");
    item_chunk_kernel<<<grid_blocks(p->nitems), 256, 0, s>>>(p->items, p->nitems, cidx, n,
                                                             (int)nchunks, p->item_chunks);
    LENTILS_CHECK_LAUNCH("item_chunk_kernel");
    p->chunk_k = K;
    p->nchunks = nchunks;
    return LENTILS_OK;
}

static int plan_build(lentils_plan *p, const double *uvw, const double *chans, int flags,
                      cudaStream_t s)
{
    GridGeom &g = p->geom;
    const long long nvis = p->nvis;
    const int ntiles = g.ntu * g.ntv;
    DevTemps tmp;
    const double *d_uvw = uvw;
    const double *d_ch = chans;
    int st;
    if (!(flags & LENTILS_PLAN_UVW_ON_DEVICE)) {
        double *a, *b;
        if ((st = tmp.alloc(&a, (size_t)p->nrows * 3))) return st;
        if ((st = tmp.alloc(&b, (size_t)p->nchannels))) return st;
        LENTILS_CUDA_TRY(cudaMemcpyAsync(a, uvw, sizeof(double) * 3 * (size_t)p->nrows,
                                         cudaMemcpyHostToDevice, s));
        LENTILS_CUDA_TRY(cudaMemcpyAsync(b, chans, sizeof(double) * (size_t)p->nchannels,
                                         cudaMemcpyHostToDevice, s));
        d_uvw = a;
        d_ch = b;
    }
    unsigned *keys, *keys_sorted;
    int *idx, *tile_counts, *d_flags;
    uint2 *coords_user;
    float2 *phase_user, *res_user;
    if ((st = tmp.alloc(&keys, nvis))) return st;
    if ((st = tmp.alloc(&keys_sorted, nvis))) return st;
    if ((st = tmp.alloc(&idx, nvis))) return st;
    if ((st = tmp.alloc(&coords_user, nvis))) return st;
    if ((st = tmp.alloc(&phase_user, nvis))) return st;
    if ((st = tmp.alloc(&res_user, nvis))) return st;
    if ((st = tmp.alloc(&tile_counts, ntiles))) return st;
    if ((st = tmp.alloc(&d_flags, 1))) return st;
    if ((st = dev_alloc(&p->coords, nvis, &p->device_bytes))) return st;
    if ((st = dev_alloc(&p->perm, nvis, &p->device_bytes))) return st;
    if ((st = dev_alloc(&p->iperm, nvis, &p->device_bytes))) return st;
    if ((st = dev_alloc(&p->phase, nvis, &p->device_bytes))) return st;
    if ((st = dev_alloc(&p->coords_res, nvis, &p->device_bytes))) return st;
    LENTILS_CUDA_TRY(cudaMemsetAsync(tile_counts, 0, sizeof(int) * ntiles, s));
    LENTILS_CUDA_TRY(cudaMemsetAsync(d_flags, 0, sizeof(int), s));

    CanonParams cp;
    cp.nu = g.nu; cp.nv = g.nv; cp.T = g.T; cp.logT = g.logT; cp.Hu = g.Hu; cp.Hv = g.Hv;
    cp.ntu = g.ntu; cp.ntv = g.ntv; cp.w = g.w; cp.nrows = p->nrows; cp.nch = p->nchannels;
    cp.guard = (flags & LENTILS_PLAN_NYQUIST_GUARD) ? 1 : 0;
    cp.du = p->desc.du; cp.dv = p->desc.dv; cp.gcx = p->desc.gcx; cp.gcy = p->desc.gcy;
    canon_kernel<<<grid_blocks(nvis), 256, 0, s>>>(d_uvw, d_ch, cp, keys, idx, coords_user,
                                                   phase_user, tile_counts, d_flags, res_user);
    LENTILS_CHECK_LAUNCH("canon_kernel");

    // stable radix sort of (key, user index) pairs
    int tile_bits = 1;
    while ((1 << tile_bits) < ntiles) ++tile_bits;
    const int key_bits = 2 * g.logT + tile_bits;
    size_t temp_bytes = 0;
    LENTILS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, keys, keys_sorted,
                                                     idx, p->perm, (int64_t)nvis, 0,
                                                     std::min(32, key_bits), s));
    unsigned char *temp;
    if ((st = tmp.alloc(&temp, temp_bytes))) return st;
    LENTILS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys, keys_sorted, idx,
                                                     p->perm, (int64_t)nvis, 0,
                                                     std::min(32, key_bits), s));
    gather_plan_kernel<<<grid_blocks(nvis), 256, 0, s>>>(p->perm, coords_user, phase_user,
                                                         p->coords, p->phase, nvis, res_user,
                                                         p->coords_res);
    LENTILS_CHECK_LAUNCH("gather_plan_kernel");
    invert_perm_kernel<<<grid_blocks(nvis), 256, 0, s>>>(p->perm, p->iperm, nvis);
    LENTILS_CHECK_LAUNCH("invert_perm_kernel");

    std::vector<int> counts(ntiles);
    int hflags = 0;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(counts.data(), tile_counts, sizeof(int) * ntiles,
                                     cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&hflags, d_flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    if (hflags & kFlagNonFinite)
        return set_error(LENTILS_ERR_NONFINITE, "plan_create: non-finite uv coordinate");
    if (hflags & kFlagGuard)
        return set_error(LENTILS_ERR_NYQUIST,
                         "plan_create: visibility space contains points higher than the "
                         "Nyquist frequency of the grid");

    // work items: tiles cut into chunks of at most `chunk` visibilities, largest first
    const int chunk = p->desc.chunk;
    std::vector<WorkItem> items;
    long long begin = 0;
    int heaviest = 0;
    for (int t = 0; t < ntiles; ++t) {
        const int c = counts[t];
        heaviest = std::max(heaviest, c);
        for (int off = 0; off < c; off += chunk) {
            WorkItem it;
            it.tu = t / g.ntv;
            it.tv = t - it.tu * g.ntv;
            it.begin = (int)(begin + off);
            it.count = std::min(chunk, c - off);
            items.push_back(it);
        }
        begin += c;
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const WorkItem &a, const WorkItem &b) { return a.count > b.count; });
    p->nitems = (int)items.size();
    p->max_item = items.empty() ? 0 : items[0].count;
    p->heaviest_tile = heaviest;
    if ((st = dev_alloc(&p->items, items.size(), &p->device_bytes))) return st;
    if (!items.empty())
        LENTILS_CUDA_TRY(cudaMemcpyAsync(p->items, items.data(), sizeof(WorkItem) * items.size(),
                                         cudaMemcpyHostToDevice, s));
    if (chunk_width(g.w) > 0 && !items.empty())
        if ((st = build_chunks(p, keys_sorted, tmp, s))) return st;
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    return LENTILS_OK;
}

// Page-locked (or device) memory that kernels can address directly: its device address, else
// null (pageable memory goes through the staging copies).
static void *kernel_address(const void *ptr)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeDevice ||
        a.type == cudaMemoryTypeManaged)
        return a.devicePointer;
    return nullptr;
}

static int ensure_device_staging(lentils_plan *p)
{
    const long long ng = (long long)p->geom.nu * p->geom.half_nv;
    int st;
    if (!p->stage_vis32 && (st = dev_alloc(&p->stage_vis32, p->nvis))) return st;
    if (!p->stage_grid32 && (st = dev_alloc(&p->stage_grid32, ng))) return st;
    return LENTILS_OK;
}

static int ensure_staging(lentils_plan *p)
{
    const long long ng = (long long)p->geom.nu * p->geom.half_nv;
    int st;
    if (!p->stage_vis64 && (st = dev_alloc((double2 **)&p->stage_vis64, p->nvis))) return st;
    if (!p->stage_grid64 && (st = dev_alloc((double2 **)&p->stage_grid64, ng))) return st;
    if (!p->stage_vis32 && (st = dev_alloc(&p->stage_vis32, p->nvis))) return st;
    if (!p->stage_grid32 && (st = dev_alloc(&p->stage_grid32, ng))) return st;
    return LENTILS_OK;
}

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_plan_create(lentils_plan **out, const lentils_grid_desc *gd, const double *uvw,
                        int nrows, const double *channels, int nchannels, int flags,
                        void *stream)
{
    clear_error();
    if (!out || !gd) return set_error(LENTILS_ERR_INVALID, "plan_create: null argument");
    *out = nullptr;
    if (nrows < 0 || nchannels < 1 || (nrows > 0 && (!uvw || !channels)))
        return set_error(LENTILS_ERR_INVALID, "plan_create: bad rows/channels");
    if (gd->nu < 2 || gd->nv < 2 || gd->nu > 65536 || gd->nv > 65536)
        return set_error(LENTILS_ERR_INVALID, "plan_create: grid %dx%d out of range", gd->nu,
                         gd->nv);
    if (gd->wsup < 1 || gd->wsup > kMaxW)
        return set_error(LENTILS_ERR_UNSUPPORTED, "plan_create: wsup=%d (supported 1..%d)",
                         gd->wsup, kMaxW);
    if (!(gd->du > 0) || !(gd->dv > 0) || !isfinite(gd->kb_beta))
        return set_error(LENTILS_ERR_INVALID, "plan_create: bad du/dv/beta");
    const long long nvis = (long long)nrows * nchannels;
    if (nvis >= (1LL << 31))
        return set_error(LENTILS_ERR_UNSUPPORTED, "plan_create: %lld visibilities (max 2^31-1)",
                         nvis);

    lentils_plan *p = new (std::nothrow) lentils_plan();
    if (!p) return set_error(LENTILS_ERR_ALLOC, "plan_create: host allocation");
    memset(p, 0, sizeof(*p));
    p->desc = *gd;
    cudaGetDevice(&p->device);
    int T = gd->tile;
    if (T == 0) T = 16;  // measured best for both kernels (degrid and the row-owner gridder)
    const int logT = ilog2_exact(T);
    if (logT < 3 || logT > 6) {
        delete p;
        return set_error(LENTILS_ERR_INVALID, "plan_create: tile %d (use 8, 16, 32 or 64)", T);
    }
    int chunk = gd->chunk;
    if (chunk <= 0) {
        long long c = nvis / (4LL * 152);
        chunk = (int)std::max(256LL, std::min(4096LL, c));
    }
    p->desc.tile = T;
    p->desc.chunk = chunk;
    GridGeom &g = p->geom;
    g.nu = gd->nu;
    g.nv = gd->nv;
    g.half_nv = gd->nv / 2 + 1;
    g.w = gd->wsup;
    g.T = T;
    g.logT = logT;
    g.E = T + 2 * g.w;
    g.stride = g.E | 1;
    g.Hu = gd->nu / 2;
    g.Hv = gd->nv / 2;
    g.ntu = (gd->nu + T - 1) / T;
    g.ntv = (gd->nv + T - 1) / T;
    if ((unsigned long long)g.ntu * g.ntv * T * T > 0xffffffffull) {
        delete p;
        return set_error(LENTILS_ERR_UNSUPPORTED, "plan_create: grid too large for 32-bit keys");
    }
    p->nvis = nvis;
    p->nrows = nrows;
    p->nchannels = nchannels;
    p->has_phase = (gd->gcx != 0.0 || gd->gcy != 0.0) ? 1 : 0;
    p->grid_variant = 0;
    p->degrid_variant = 0;
    kb_poly_build(g.w, gd->kb_beta, &p->kb, nullptr, &p->kb64);

    int st = LENTILS_OK;
    if (nvis > 0) st = plan_build(p, uvw, channels, flags, (cudaStream_t)stream);
    if (st != LENTILS_OK) {
        const int code = lentils_last_error();
        char msg[512];
        strncpy(msg, lentils_last_error_message(), sizeof(msg) - 1);
        msg[sizeof(msg) - 1] = 0;
        free_plan_arrays(p);
        delete p;
        return set_error(code, "%s", msg);
    }
    *out = p;
    return LENTILS_OK;
}

int lentils_plan_destroy(lentils_plan *p)
{
    clear_error();
    if (!p) return LENTILS_OK;
    free_plan_arrays(p);
    delete p;
    return LENTILS_OK;
}

int lentils_plan_set_grid_variant(lentils_plan *p, int variant)
{
    clear_error();
    if (!p || variant < 0 || variant > 12)
        return set_error(LENTILS_ERR_INVALID, "plan_set_grid_variant: variant 0 to 12");
    p->grid_variant = variant;
    return LENTILS_OK;
}

int lentils_plan_set_degrid_variant(lentils_plan *p, int variant)
{
    clear_error();
    if (!p || variant < 0 || variant > 2)
        return set_error(LENTILS_ERR_INVALID, "plan_set_degrid_variant: variant 0 to 2");
    p->degrid_variant = variant;
    return LENTILS_OK;
}

int lentils_plan_get_stats(const lentils_plan *p, lentils_plan_stats *s)
{
    clear_error();
    if (!p || !s) return set_error(LENTILS_ERR_INVALID, "plan_get_stats: null argument");
    s->nvis = p->nvis;
    s->ntiles_u = p->geom.ntu;
    s->ntiles_v = p->geom.ntv;
    s->tile = p->geom.T;
    s->nitems = p->nitems;
    s->max_item_vis = p->max_item;
    s->heaviest_tile_vis = p->heaviest_tile;
    s->wsup = p->geom.w;
    s->has_phase = p->has_phase;
    s->device_bytes = p->device_bytes;
    return LENTILS_OK;
}

int lentils_degrid(const lentils_plan *p, const float *grid, float *vis, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!grid || !vis)))
        return set_error(LENTILS_ERR_INVALID, "degrid: null argument");
    return launch_degrid(p, (const float2 *)grid, (float2 *)vis, (cudaStream_t)stream);
}

int lentils_grid(const lentils_plan *p, const float *vis, float *grid, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!grid || !vis)))
        return set_error(LENTILS_ERR_INVALID, "grid: null argument");
    return launch_grid(p, (const float2 *)vis, (float2 *)grid, (cudaStream_t)stream);
}

int lentils_vis_to_plan(const lentils_plan *p, const void *vu, int c128, float *vp, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!vu || !vp)))
        return set_error(LENTILS_ERR_INVALID, "vis_to_plan: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (c128)
        to_plan_kernel<double2><<<grid_blocks(p->nvis), 256, 0, s>>>(
            p->perm, p->phase, (const double2 *)vu, (float2 *)vp, p->nvis);
    else
        to_plan_kernel<float2><<<grid_blocks(p->nvis), 256, 0, s>>>(
            p->perm, p->phase, (const float2 *)vu, (float2 *)vp, p->nvis);
    LENTILS_CHECK_LAUNCH("to_plan_kernel");
    return LENTILS_OK;
}

int lentils_vis_from_plan(const lentils_plan *p, const float *vp, void *vu, int c128,
                          int accumulate, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!vu || !vp)))
        return set_error(LENTILS_ERR_INVALID, "vis_from_plan: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    if (c128)
        from_plan_kernel<double2><<<grid_blocks(p->nvis), 256, 0, s>>>(
            p->perm, p->phase, (const float2 *)vp, (double2 *)vu, p->nvis, accumulate);
    else
        from_plan_kernel<float2><<<grid_blocks(p->nvis), 256, 0, s>>>(
            p->perm, p->phase, (const float2 *)vp, (float2 *)vu, p->nvis, accumulate);
    LENTILS_CHECK_LAUNCH("from_plan_kernel");
    return LENTILS_OK;
}

int lentils_vis_to_plan64(const lentils_plan *p, const double *vu, double *vp, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!vu || !vp)))
        return set_error(LENTILS_ERR_INVALID, "vis_to_plan64: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    to_plan64_kernel<<<grid_blocks(p->nvis), 256, 0, (cudaStream_t)stream>>>(
        p->perm, p->phase, (const double2 *)vu, (double2 *)vp, p->nvis);
    LENTILS_CHECK_LAUNCH("to_plan64_kernel");
    return LENTILS_OK;
}

int lentils_vis_from_plan64(const lentils_plan *p, const double *vp, double *vu, int accumulate,
                            void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!vu || !vp)))
        return set_error(LENTILS_ERR_INVALID, "vis_from_plan64: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    from_plan64_kernel<<<grid_blocks(p->nvis), 256, 0, (cudaStream_t)stream>>>(
        p->perm, p->phase, (const double2 *)vp, (double2 *)vu, p->nvis, accumulate);
    LENTILS_CHECK_LAUNCH("from_plan64_kernel");
    return LENTILS_OK;
}

int lentils_plan_gather_real(const lentils_plan *p, const double *u, double *out, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!u || !out)))
        return set_error(LENTILS_ERR_INVALID, "plan_gather_real: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    gather_real_kernel<<<grid_blocks(p->nvis), 256, 0, (cudaStream_t)stream>>>(p->perm, u, out,
                                                                               p->nvis);
    LENTILS_CHECK_LAUNCH("gather_real_kernel");
    return LENTILS_OK;
}

int lentils_degrid_host(lentils_plan *p, const double *grid_host, double *vis_host,
                        int accumulate, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!grid_host || !vis_host)))
        return set_error(LENTILS_ERR_INVALID, "degrid_host: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    int st;
    cudaStream_t s = (cudaStream_t)stream;
    const long long ng = (long long)p->geom.nu * p->geom.half_nv;
    const double2 *grid_k = (const double2 *)kernel_address(grid_host);
    double2 *vis_k = (double2 *)kernel_address(vis_host);
    if (grid_k && vis_k) {  // page-locked: the kernels read and write host memory directly
        if ((st = ensure_device_staging(p))) return st;
        if ((st = launch_c128_to_c64(grid_k, p->stage_grid32, ng, s))) return st;
        if ((st = launch_degrid(p, p->stage_grid32, p->stage_vis32, s))) return st;
        from_plan_gather_kernel<double2><<<grid_blocks(p->nvis), 256, 0, s>>>(
            p->iperm, p->phase, p->stage_vis32, vis_k, p->nvis, accumulate);
        LENTILS_CHECK_LAUNCH("from_plan_gather_kernel");
        LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
        return LENTILS_OK;
    }
    if ((st = ensure_staging(p))) return st;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(p->stage_grid64, grid_host, sizeof(double2) * ng,
                                     cudaMemcpyHostToDevice, s));
    if ((st = launch_c128_to_c64(p->stage_grid64, p->stage_grid32, ng, s))) return st;
    if ((st = launch_degrid(p, p->stage_grid32, p->stage_vis32, s))) return st;
    if (accumulate)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(p->stage_vis64, vis_host, sizeof(double2) * p->nvis,
                                         cudaMemcpyHostToDevice, s));
    if ((st = lentils_vis_from_plan(p, (const float *)p->stage_vis32, p->stage_vis64, 1,
                                    accumulate, stream)))
        return st;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(vis_host, p->stage_vis64, sizeof(double2) * p->nvis,
                                     cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    return LENTILS_OK;
}

int lentils_grid_host(lentils_plan *p, const double *vis_host, double *grid_host,
                      int accumulate, void *stream)
{
    clear_error();
    if (!p || (p->nvis > 0 && (!grid_host || !vis_host)))
        return set_error(LENTILS_ERR_INVALID, "grid_host: null argument");
    if (p->nvis == 0) return LENTILS_OK;
    int st;
    cudaStream_t s = (cudaStream_t)stream;
    const long long ng = (long long)p->geom.nu * p->geom.half_nv;
    const double2 *vis_k = (const double2 *)kernel_address(vis_host);
    double2 *grid_k = (double2 *)kernel_address(grid_host);
    if (grid_k && vis_k) {  // page-locked: the kernels read and write host memory directly
        if ((st = ensure_device_staging(p))) return st;
        to_plan_scatter_kernel<double2><<<grid_blocks(p->nvis), 256, 0, s>>>(
            p->iperm, p->phase, vis_k, p->stage_vis32, p->nvis);
        LENTILS_CHECK_LAUNCH("to_plan_scatter_kernel");
        LENTILS_CUDA_TRY(cudaMemsetAsync(p->stage_grid32, 0, sizeof(float2) * ng, s));
        if ((st = launch_grid(p, p->stage_vis32, p->stage_grid32, s))) return st;
        if ((st = launch_c64_to_c128(p->stage_grid32, grid_k, ng, accumulate, s))) return st;
        LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
        return LENTILS_OK;
    }
    if ((st = ensure_staging(p))) return st;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(p->stage_vis64, vis_host, sizeof(double2) * p->nvis,
                                     cudaMemcpyHostToDevice, s));
    if ((st = lentils_vis_to_plan(p, p->stage_vis64, 1, (float *)p->stage_vis32, stream)))
        return st;
    LENTILS_CUDA_TRY(cudaMemsetAsync(p->stage_grid32, 0, sizeof(float2) * ng, s));
    if ((st = launch_grid(p, p->stage_vis32, p->stage_grid32, s))) return st;
    if (accumulate)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(p->stage_grid64, grid_host, sizeof(double2) * ng,
                                         cudaMemcpyHostToDevice, s));
    if ((st = launch_c64_to_c128(p->stage_grid32, p->stage_grid64, ng, accumulate, s)))
        return st;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(grid_host, p->stage_grid64, sizeof(double2) * ng,
                                     cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    return LENTILS_OK;
}

}  // extern "C"
