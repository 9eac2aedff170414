// Kaiser-Bessel degridding ("K1") and gridding ("K2") on plan-ordered visibilities.
//
// One CTA per work item (a tile of T x T uv cells and up to `chunk` of its visibilities,
// sorted by cell). The CTA stages the tile plus a w-cell halo ("extended tile", E x E cells,
// E = T + 2w) in shared memory:
//   degrid: gathered from the stored r2c half-plane grid with the reference's wrap and
//           Hermitian fold applied on the way in (lentils/backend/nufft.c:83-93), so the
//           inner loop reads a plain full-plane patch. Consecutive threads take consecutive
//           (sorted) visibilities, so a warp's loads fall on one or a few neighbouring cells
//           and are served by broadcast without bank conflicts.
//   grid:   zeroed, accumulated, and flushed once through the fold (conjugate on folded
//           cells, x2 on column 0, nufft.c:107-111) with one 8-byte global atomic per touched
//           cell. Weights are evaluated one visibility per thread into a shared batch; each
//           warp then walks consecutive (sorted) visibilities with its lanes owning the taps
//           of the window, summing in registers while the visibilities stay in one cell, so
//           shared-memory atomics happen once per cell run and never collide within a warp.
// Weights: 2w separable weights per axis from degree-9 polynomials of the fixed-point
// fraction (packed FP32x2 FMAs); the checkerboard sign (-1)^(i_u+i_v) (nufft.c:78) is folded
// into the table per tap plus one parity per visibility; the factors 2*0.5 (degrid) and 0.5
// (grid) of nufft.c:79-80,102-104 are applied here.
//
// Tap set. The reference visits round(g)-w .. round(g)+w per axis (nufft.c:65-68) and zeroes
// taps with |g - i| > w (nufft.c:12-13), so its non-zero taps are floor(g)-w+1 .. floor(g)+w
// (2w regular taps) plus, when g is (within FP64) an integer, floor(g)-w at argument +w. The
// plan records that extra tap, and the rare exclusion of the top tap, as flag bits decided in
// FP64; the extra tap (weight I0(0)/(2w)) runs on a separate, rarely taken path.
#include <type_traits>

#include "common.cuh"

namespace lentils {

__device__ __forceinline__ int wrap_index(int a, int n)
{
    int r = a % n;
    return r < 0 ? r + n : r;
}

template <int W2>
__device__ __forceinline__ void kb_weights(const KBPoly &kb, uint32_t word, float (&wt)[W2],
                                           float /*res: FP64 kernels only*/ = 0.f)
{
    const float f = (float)(word & kFracMask) * (1.0f / (float)(1u << kFracBits));
    const float t = fmaf(2.0f, f, -1.0f);
    const float2 tt = make_float2(t, t);
#pragma unroll
    for (int p = 0; p < W2 / 2; ++p) {
        float2 acc = kb.cp[0][p];
#pragma unroll
        for (int k = 1; k < kPolyCoef; ++k) acc = __ffma2_rn(acc, tt, kb.cp[k][p]);
        wt[2 * p] = acc.x;
        wt[2 * p + 1] = acc.y;
    }
    if (word & kTopOffBit) wt[W2 - 1] = 0.f;
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

__device__ __forceinline__ int cell_of(uint32_t word) { return (int)((word >> kFracBits) & kCellMask); }

// Precision traits: the float kernels are the hot path (packed FP32x2 FMAs, float2 global
// atomics); the double kernels apply the FP64 operator used for refinement residuals.
template <typename R>
struct Prec;
template <>
struct Prec<float> {
    using C = float2;
    using Table = KBPoly;
    __device__ static C zero() { return make_float2(0.f, 0.f); }
    __device__ static C fma(float w, C a, C acc) { return __ffma2_rn(f2(w), a, acc); }
    __device__ static C scale(float w, C a) { return make_float2(w * a.x, w * a.y); }
    __device__ static void gadd(C *dst, C v) { atomicAdd(dst, v); }
};
template <>
struct Prec<double> {
    using C = double2;
    using Table = KBPoly64;
    __device__ static C zero() { return make_double2(0.0, 0.0); }
    __device__ static C fma(double w, C a, C acc)
    {
        return make_double2(fma_(w, a.x, acc.x), fma_(w, a.y, acc.y));
    }
    __device__ static double fma_(double a, double b, double c) { return ::fma(a, b, c); }
    __device__ static C scale(double w, C a) { return make_double2(w * a.x, w * a.y); }
    __device__ static void gadd(C *dst, C v)
    {
        atomicAdd(&dst->x, v.x);
        atomicAdd(&dst->y, v.y);
    }
};

template <int W2>
__device__ __forceinline__ void kb_weights(const KBPoly64 &kb, uint32_t word, double (&wt)[W2],
                                           float res)
{
    const double f = (double)(word & kFracMask) * (1.0 / (double)(1u << kFracBits)) + (double)res;
    const double t = 2.0 * f - 1.0;
#pragma unroll
    for (int i = 0; i < W2; ++i) {
        double acc = kb.cd[0][i];
#pragma unroll
        for (int k = 1; k < kPolyCoef; ++k) acc = ::fma(acc, t, kb.cd[k][i]);
        wt[i] = acc;
    }
    if (word & kTopOffBit) wt[W2 - 1] = 0.0;
}

// Parity of the first regular tap (canonical cell index) of a visibility in the item's tile.
__device__ __forceinline__ int tap_parity(const WorkItem &it, const GridGeom &g, int lu, int lv)
{
    return (it.tu * g.T - g.Hu + lu - g.w + 1 + it.tv * g.T - g.Hv + lv - g.w + 1) & 1;
}

template <int W2, typename R>
__global__ void __launch_bounds__(256)
    degrid_kernel(const typename Prec<R>::C *__restrict__ grid, const uint2 *__restrict__ coords,
                  typename Prec<R>::C *__restrict__ out, const WorkItem *__restrict__ items,
                  const __grid_constant__ typename Prec<R>::Table kb, const GridGeom g,
                  const float2 *__restrict__ cres)
{
    using P = Prec<R>;
    using C = typename P::C;
    extern __shared__ __align__(16) unsigned char smraw[];
    C *sm = reinterpret_cast<C *>(smraw);
    const WorkItem it = items[blockIdx.x];
    constexpr int w = W2 / 2;
    const int a0 = it.tu * g.T - g.Hu - w;  // canonical index of extended row 0
    const int b0 = it.tv * g.T - g.Hv - w;
    const int E = g.E, S = g.stride;
    for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
        const int ea = e / E, eb = e - ea * E;
        int au = wrap_index(a0 + ea, g.nu);
        int bv = wrap_index(b0 + eb, g.nv);
        C val;
        if (bv >= g.half_nv) {
            au = (g.nu - au) % g.nu;
            bv = g.nv - bv;
            val = grid[(long long)au * g.half_nv + bv];
            val.y = -val.y;
        } else {
            val = grid[(long long)au * g.half_nv + bv];
        }
        sm[ea * S + eb] = val;
    }
    __syncthreads();

    for (int k = threadIdx.x; k < it.count; k += blockDim.x) {
        const uint2 c = coords[it.begin + k];
        const int lu = cell_of(c.x), lv = cell_of(c.y);
        const float2 rr = cres ? cres[it.begin + k] : make_float2(0.f, 0.f);
        R wu[W2], wv[W2];
        kb_weights<W2>(kb, c.x, wu, rr.x);
        kb_weights<W2>(kb, c.y, wv, rr.y);
        const C *p = sm + (lu + 1) * S + (lv + 1);
        C acc = P::zero();
#pragma unroll
        for (int i = 0; i < W2; ++i) {
            C r = P::zero();
#pragma unroll
            for (int j = 0; j < W2; ++j) r = P::fma(wv[j], p[i * S + j], r);
            acc = P::fma(wu[i], r, acc);
        }
        if ((c.x | c.y) & kExtraTapBit) {
            // extra taps at argument +w: extended row lu (u) / column lv (v)
            const R eu = (c.x & kExtraTapBit) ? (R)kb.edge : (R)0;
            const R ev = (c.y & kExtraTapBit) ? (R)kb.edge : (R)0;
            const C *q = sm + lu * S + lv;
            C r = P::zero();
            for (int j = 0; j < W2; ++j) r = P::fma(wv[j], q[j + 1], r);
            r = P::fma(ev, q[0], r);
            acc = P::fma(eu, r, acc);
            C cs = P::zero();
            for (int i = 0; i < W2; ++i) cs = P::fma(wu[i], q[(i + 1) * S], cs);
            acc = P::fma(ev, cs, acc);
        }
        if (tap_parity(it, g, lu, lv)) {
            acc.x = -acc.x;
            acc.y = -acc.y;
        }
        out[it.begin + k] = acc;
    }
}

// Extra taps of one visibility (rare): added to shared memory directly.
template <int W2, typename R>
__device__ __forceinline__ void grid_extra_taps(typename Prec<R>::C *sm, int S, int lu, int lv,
                                                uint2 c, const R (&wu)[W2], const R (&wv)[W2],
                                                R edge, typename Prec<R>::C x)
{
    using C = typename Prec<R>::C;
    const R eu = (c.x & kExtraTapBit) ? edge : (R)0;
    const R ev = (c.y & kExtraTapBit) ? edge : (R)0;
    C *q = sm + lu * S + lv;
    if (eu != (R)0) {
        const C t = Prec<R>::scale(eu, x);
        for (int j = 0; j < W2; ++j) {
            atomicAdd(&q[j + 1].x, wv[j] * t.x);
            atomicAdd(&q[j + 1].y, wv[j] * t.y);
        }
        atomicAdd(&q[0].x, ev * t.x);
        atomicAdd(&q[0].y, ev * t.y);
    }
    if (ev != (R)0) {
        for (int i = 0; i < W2; ++i) {
            atomicAdd(&q[(i + 1) * S].x, wu[i] * ev * x.x);
            atomicAdd(&q[(i + 1) * S].y, wu[i] * ev * x.y);
        }
    }
}

template <int W2, typename R>
__device__ __forceinline__ void grid_flush_extended(const typename Prec<R>::C *sm,
                                                    typename Prec<R>::C *__restrict__ grid,
                                                    const WorkItem &it, const GridGeom &g)
{
    using C = typename Prec<R>::C;
    constexpr int w = W2 / 2;
    const int a0 = it.tu * g.T - g.Hu - w;
    const int b0 = it.tv * g.T - g.Hv - w;
    const int E = g.E, S = g.stride;
    for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
        const int ea = e / E, eb = e - ea * E;
        C val = sm[ea * S + eb];
        if (val.x == (R)0 && val.y == (R)0) continue;
        int au = wrap_index(a0 + ea, g.nu);
        int bv = wrap_index(b0 + eb, g.nv);
        if (bv >= g.half_nv) {
            au = (g.nu - au) % g.nu;
            bv = g.nv - bv;
            val.y = -val.y;
        } else if (bv == 0) {
            val.x *= (R)2;
            val.y *= (R)2;
        }
        Prec<R>::gadd(&grid[(long long)au * g.half_nv + bv], val);
    }
}

// Taps per lane in the warp-cooperative gridder: the smallest divisor of 2w whose 32 lanes
// cover all (2w)^2 taps, so each lane's taps lie in one row of the window.
template <int W2>
struct LaneTaps {
    static constexpr int per()
    {
        for (int d = 1; d <= W2; ++d)
            if (W2 % d == 0 && 32 * d >= W2 * W2) return d;
        return W2;
    }
    static constexpr int PER = per();
    static constexpr int STR = 2 * W2 + 1;  // floats per visibility in the weight batch (odd)
};

constexpr int kGridBatch = 256;  // visibilities per weight batch (= threads per CTA)

// Gridding: per batch of 256 sorted visibilities, each thread evaluates one visibility's 2w+2w
// weights into shared memory; then each warp walks 32 consecutive visibilities, its lanes
// owning PER taps of the 2w x 2w window (one row, PER adjacent columns) and accumulating them
// in registers while the visibilities stay in one cell. A change of cell (or the end of the
// warp's 32) flushes the lane's taps to the shared extended tile with PER*2 atomics on distinct
// addresses; the whole warp flushes together.
template <int W2, typename R>
__global__ void __launch_bounds__(kGridBatch)
    grid_kernel(const typename Prec<R>::C *__restrict__ vis, const uint2 *__restrict__ coords,
                typename Prec<R>::C *__restrict__ grid, const WorkItem *__restrict__ items,
                const __grid_constant__ typename Prec<R>::Table kb, const GridGeom g,
                const float2 *__restrict__ cres)
{
    using P = Prec<R>;
    using C = typename P::C;
    using LT = LaneTaps<W2>;
    constexpr int PER = LT::PER, STR = LT::STR;
    extern __shared__ __align__(16) unsigned char smraw[];
    const WorkItem it = items[blockIdx.x];
    const int E = g.E, S = g.stride;
    C *sm = reinterpret_cast<C *>(smraw);                       // E x S extended tile
    const size_t tile_bytes = ((sizeof(C) * (size_t)E * S) + 15) & ~size_t(15);
    C *sx = reinterpret_cast<C *>(smraw + tile_bytes);           // per vis: weighted value
    int *skey = reinterpret_cast<int *>(sx + kGridBatch);        // per vis: cell key
    R *swt = reinterpret_cast<R *>(skey + kGridBatch);           // per vis: wu[W2] | wv[W2]
    for (int e = threadIdx.x; e < E * S; e += blockDim.x) sm[e] = P::zero();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int t0 = lane * PER;
    const bool active = t0 < W2 * W2;
    const int ti = active ? t0 / W2 : 0;
    const int tj = active ? t0 % W2 : 0;

    for (int base = 0; base < it.count; base += kGridBatch) {
        const int n = min(kGridBatch, it.count - base);
        __syncthreads();  // tile zeroed / previous batch consumed
        if ((int)threadIdx.x < n) {
            const int k = threadIdx.x;
            const uint2 c = coords[it.begin + base + k];
            const int lu = cell_of(c.x), lv = cell_of(c.y);
            const float2 rr = cres ? cres[it.begin + base + k] : make_float2(0.f, 0.f);
            R wu[W2], wv[W2];
            kb_weights<W2>(kb, c.x, wu, rr.x);
            kb_weights<W2>(kb, c.y, wv, rr.y);
            C x = vis[it.begin + base + k];
            const R h = tap_parity(it, g, lu, lv) ? (R)-0.5 : (R)0.5;
            x = P::scale(h, x);
            R *wrow = swt + k * STR;
#pragma unroll
            for (int i = 0; i < W2; ++i) wrow[i] = wu[i];
#pragma unroll
            for (int j = 0; j < W2; ++j) wrow[W2 + j] = wv[j];
            sx[k] = x;
            skey[k] = (lu << 6) | lv;
            if ((c.x | c.y) & kExtraTapBit)
                grid_extra_taps<W2, R>(sm, S, lu, lv, c, wu, wv, (R)kb.edge, x);
        }
        __syncthreads();
        const int k0 = warp * 32, k1 = min(n, k0 + 32);
        C acc[PER];
#pragma unroll
        for (int r = 0; r < PER; ++r) acc[r] = P::zero();
        int cur = -1;
        for (int k = k0; k < k1; ++k) {
            const int key = skey[k];
            if (key != cur) {
                if (cur >= 0 && active) {
                    C *p = sm + ((cur >> 6) + 1 + ti) * S + (cur & 63) + 1 + tj;
#pragma unroll
                    for (int r = 0; r < PER; ++r) {
                        atomicAdd(&p[r].x, acc[r].x);
                        atomicAdd(&p[r].y, acc[r].y);
                        acc[r] = P::zero();
                    }
                }
                cur = key;
            }
            const R *wrow = swt + k * STR;
            const C t = P::scale(wrow[ti], sx[k]);
#pragma unroll
            for (int r = 0; r < PER; ++r) acc[r] = P::fma(wrow[W2 + tj + r], t, acc[r]);
        }
        if (cur >= 0 && active) {
            C *p = sm + ((cur >> 6) + 1 + ti) * S + (cur & 63) + 1 + tj;
#pragma unroll
            for (int r = 0; r < PER; ++r) {
                atomicAdd(&p[r].x, acc[r].x);
                atomicAdd(&p[r].y, acc[r].y);
            }
        }
    }
    __syncthreads();
    grid_flush_extended<W2, R>(sm, grid, it, g);
}

template <typename K>
static int set_smem(K kernel, size_t smem)
{
    if (smem > 48 * 1024)
        LENTILS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
    return LENTILS_OK;
}

template <typename R>
static const typename Prec<R>::Table &table_of(const lentils_plan *p);
template <>
const KBPoly &table_of<float>(const lentils_plan *p) { return p->kb; }
template <>
const KBPoly64 &table_of<double>(const lentils_plan *p) { return p->kb64; }

template <int W2, typename R>
static int launch_degrid_t(const lentils_plan *p, const typename Prec<R>::C *grid,
                           typename Prec<R>::C *vis, cudaStream_t s)
{
    const GridGeom &g = p->geom;
    const size_t smem = sizeof(typename Prec<R>::C) * (size_t)g.E * g.stride;
    if (int st = set_smem(degrid_kernel<W2, R>, smem)) return st;
    const float2 *cres = std::is_same<R, double>::value ? p->coords_res : nullptr;
    degrid_kernel<W2, R><<<p->nitems, 256, smem, s>>>(grid, p->coords, vis, p->items,
                                                     table_of<R>(p), g, cres);
    LENTILS_CHECK_LAUNCH("degrid_kernel");
    return LENTILS_OK;
}

template <int W2, typename R>
static int launch_grid_t(const lentils_plan *p, const typename Prec<R>::C *vis,
                         typename Prec<R>::C *grid, cudaStream_t s)
{
    using C = typename Prec<R>::C;
    const GridGeom &g = p->geom;
    const size_t tile_bytes = ((sizeof(C) * (size_t)g.E * g.stride) + 15) & ~size_t(15);
    const size_t smem = tile_bytes + (sizeof(C) + sizeof(int)) * kGridBatch +
                        sizeof(R) * (size_t)kGridBatch * LaneTaps<W2>::STR;
    if (int st = set_smem(grid_kernel<W2, R>, smem)) return st;
    const float2 *cres = std::is_same<R, double>::value ? p->coords_res : nullptr;
    grid_kernel<W2, R><<<p->nitems, kGridBatch, smem, s>>>(vis, p->coords, grid, p->items,
                                                          table_of<R>(p), g, cres);
    LENTILS_CHECK_LAUNCH("grid_kernel");
    return LENTILS_OK;
}

template <typename R>
static int launch_degrid_r(const lentils_plan *p, const typename Prec<R>::C *grid,
                           typename Prec<R>::C *vis, cudaStream_t s)
{
    if (p->nitems == 0) return LENTILS_OK;
    switch (p->geom.w) {
    case 1: return launch_degrid_t<2, R>(p, grid, vis, s);
    case 2: return launch_degrid_t<4, R>(p, grid, vis, s);
    case 3: return launch_degrid_t<6, R>(p, grid, vis, s);
    case 4: return launch_degrid_t<8, R>(p, grid, vis, s);
    case 5: return launch_degrid_t<10, R>(p, grid, vis, s);
    case 6: return launch_degrid_t<12, R>(p, grid, vis, s);
    case 7: return launch_degrid_t<14, R>(p, grid, vis, s);
    case 8: return launch_degrid_t<16, R>(p, grid, vis, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "degrid: w=%d", p->geom.w);
}

template <typename R>
static int launch_grid_r(const lentils_plan *p, const typename Prec<R>::C *vis,
                         typename Prec<R>::C *grid, cudaStream_t s)
{
    if (p->nitems == 0) return LENTILS_OK;
    switch (p->geom.w) {
    case 1: return launch_grid_t<2, R>(p, vis, grid, s);
    case 2: return launch_grid_t<4, R>(p, vis, grid, s);
    case 3: return launch_grid_t<6, R>(p, vis, grid, s);
    case 4: return launch_grid_t<8, R>(p, vis, grid, s);
    case 5: return launch_grid_t<10, R>(p, vis, grid, s);
    case 6: return launch_grid_t<12, R>(p, vis, grid, s);
    case 7: return launch_grid_t<14, R>(p, vis, grid, s);
    case 8: return launch_grid_t<16, R>(p, vis, grid, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "grid: w=%d", p->geom.w);
}

int launch_degrid(const lentils_plan *p, const float2 *grid, float2 *vis, cudaStream_t s)
{
    return launch_degrid_r<float>(p, grid, vis, s);
}

int launch_grid(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s)
{
    return launch_grid_r<float>(p, vis, grid, s);
}

int launch_degrid64(const lentils_plan *p, const double2 *grid, double2 *vis, cudaStream_t s)
{
    return launch_degrid_r<double>(p, grid, vis, s);
}

int launch_grid64(const lentils_plan *p, const double2 *vis, double2 *grid, cudaStream_t s)
{
    return launch_grid_r<double>(p, vis, grid, s);
}

}  // namespace lentils
