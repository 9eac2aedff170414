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
#include "common.cuh"

namespace lentils {

__device__ __forceinline__ int wrap_index(int a, int n)
{
    int r = a % n;
    return r < 0 ? r + n : r;
}

template <int W2>
__device__ __forceinline__ void kb_weights(const KBPoly &kb, uint32_t word, float (&wt)[W2])
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

// Parity of the first regular tap (canonical cell index) of a visibility in the item's tile.
__device__ __forceinline__ int tap_parity(const WorkItem &it, const GridGeom &g, int lu, int lv)
{
    return (it.tu * g.T - g.Hu + lu - g.w + 1 + it.tv * g.T - g.Hv + lv - g.w + 1) & 1;
}

template <int W2>
__global__ void __launch_bounds__(256)
    degrid_kernel(const float2 *__restrict__ grid, const uint2 *__restrict__ coords,
                  float2 *__restrict__ out, const WorkItem *__restrict__ items,
                  const __grid_constant__ KBPoly kb, const GridGeom g)
{
    extern __shared__ float2 sm[];
    const WorkItem it = items[blockIdx.x];
    constexpr int w = W2 / 2;
    const int a0 = it.tu * g.T - g.Hu - w;  // canonical index of extended row 0
    const int b0 = it.tv * g.T - g.Hv - w;
    const int E = g.E, S = g.stride;
    for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
        const int ea = e / E, eb = e - ea * E;
        int au = wrap_index(a0 + ea, g.nu);
        int bv = wrap_index(b0 + eb, g.nv);
        float2 val;
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
        float wu[W2], wv[W2];
        kb_weights<W2>(kb, c.x, wu);
        kb_weights<W2>(kb, c.y, wv);
        const float2 *p = sm + (lu + 1) * S + (lv + 1);
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < W2; ++i) {
            float2 r = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < W2; ++j) r = __ffma2_rn(f2(wv[j]), p[i * S + j], r);
            acc = __ffma2_rn(f2(wu[i]), r, acc);
        }
        if ((c.x | c.y) & kExtraTapBit) {
            // extra taps at argument +w: extended row lu (u) / column lv (v)
            const float eu = (c.x & kExtraTapBit) ? kb.edge : 0.f;
            const float ev = (c.y & kExtraTapBit) ? kb.edge : 0.f;
            const float2 *q = sm + lu * S + lv;
            float2 r = make_float2(0.f, 0.f);
            for (int j = 0; j < W2; ++j) r = __ffma2_rn(f2(wv[j]), q[j + 1], r);
            r = __ffma2_rn(f2(ev), q[0], r);
            acc = __ffma2_rn(f2(eu), r, acc);
            float2 cs = make_float2(0.f, 0.f);
            for (int i = 0; i < W2; ++i) cs = __ffma2_rn(f2(wu[i]), q[(i + 1) * S], cs);
            acc = __ffma2_rn(f2(ev), cs, acc);
        }
        if (tap_parity(it, g, lu, lv)) acc = make_float2(-acc.x, -acc.y);
        out[it.begin + k] = acc;
    }
}

// Extra taps of one visibility (rare): added to shared memory directly.
template <int W2>
__device__ __forceinline__ void grid_extra_taps(float2 *sm, int S, int lu, int lv, uint2 c,
                                                const float (&wu)[W2], const float (&wv)[W2],
                                                float edge, float2 x)
{
    const float eu = (c.x & kExtraTapBit) ? edge : 0.f;
    const float ev = (c.y & kExtraTapBit) ? edge : 0.f;
    float2 *q = sm + lu * S + lv;
    if (eu != 0.f) {
        const float2 t = make_float2(eu * x.x, eu * x.y);
        for (int j = 0; j < W2; ++j) {
            atomicAdd(&q[j + 1].x, wv[j] * t.x);
            atomicAdd(&q[j + 1].y, wv[j] * t.y);
        }
        atomicAdd(&q[0].x, ev * t.x);
        atomicAdd(&q[0].y, ev * t.y);
    }
    if (ev != 0.f) {
        for (int i = 0; i < W2; ++i) {
            atomicAdd(&q[(i + 1) * S].x, wu[i] * ev * x.x);
            atomicAdd(&q[(i + 1) * S].y, wu[i] * ev * x.y);
        }
    }
}

template <int W2>
__device__ __forceinline__ void grid_flush_extended(const float2 *sm, float2 *__restrict__ grid,
                                                    const WorkItem &it, const GridGeom &g)
{
    constexpr int w = W2 / 2;
    const int a0 = it.tu * g.T - g.Hu - w;
    const int b0 = it.tv * g.T - g.Hv - w;
    const int E = g.E, S = g.stride;
    for (int e = threadIdx.x; e < E * E; e += blockDim.x) {
        const int ea = e / E, eb = e - ea * E;
        float2 val = sm[ea * S + eb];
        if (val.x == 0.f && val.y == 0.f) continue;
        int au = wrap_index(a0 + ea, g.nu);
        int bv = wrap_index(b0 + eb, g.nv);
        if (bv >= g.half_nv) {
            au = (g.nu - au) % g.nu;
            bv = g.nv - bv;
            val.y = -val.y;
        } else if (bv == 0) {
            val.x *= 2.f;
            val.y *= 2.f;
        }
        atomicAdd(&grid[(long long)au * g.half_nv + bv], val);
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
template <int W2>
__global__ void __launch_bounds__(kGridBatch)
    grid_kernel(const float2 *__restrict__ vis, const uint2 *__restrict__ coords,
                float2 *__restrict__ grid, const WorkItem *__restrict__ items,
                const __grid_constant__ KBPoly kb, const GridGeom g)
{
    using LT = LaneTaps<W2>;
    constexpr int PER = LT::PER, STR = LT::STR;
    extern __shared__ float4 smem4[];
    const WorkItem it = items[blockIdx.x];
    const int E = g.E, S = g.stride;
    float2 *sm = reinterpret_cast<float2 *>(smem4);        // E x S extended tile
    float4 *sxk = smem4 + (E * S + 1) / 2;                  // per vis: (x.re, x.im, key, -)
    float *swt = reinterpret_cast<float *>(sxk + kGridBatch);  // per vis: wu[W2] | wv[W2]
    for (int e = threadIdx.x; e < E * S; e += blockDim.x) sm[e] = make_float2(0.f, 0.f);

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
            float wu[W2], wv[W2];
            kb_weights<W2>(kb, c.x, wu);
            kb_weights<W2>(kb, c.y, wv);
            float2 x = vis[it.begin + base + k];
            const float h = tap_parity(it, g, lu, lv) ? -0.5f : 0.5f;
            x = make_float2(h * x.x, h * x.y);
            float *wrow = swt + k * STR;
#pragma unroll
            for (int i = 0; i < W2; ++i) wrow[i] = wu[i];
#pragma unroll
            for (int j = 0; j < W2; ++j) wrow[W2 + j] = wv[j];
            sxk[k] = make_float4(x.x, x.y, __int_as_float((lu << 6) | lv), 0.f);
            if ((c.x | c.y) & kExtraTapBit) grid_extra_taps<W2>(sm, S, lu, lv, c, wu, wv, kb.edge, x);
        }
        __syncthreads();
        const int k0 = warp * 32, k1 = min(n, k0 + 32);
        float2 acc[PER];
#pragma unroll
        for (int r = 0; r < PER; ++r) acc[r] = make_float2(0.f, 0.f);
        int cur = -1;
        for (int k = k0; k < k1; ++k) {
            const float4 xk = sxk[k];
            const int key = __float_as_int(xk.z);
            if (key != cur) {
                if (cur >= 0 && active) {
                    float2 *p = sm + ((cur >> 6) + 1 + ti) * S + (cur & 63) + 1 + tj;
#pragma unroll
                    for (int r = 0; r < PER; ++r) {
                        atomicAdd(&p[r].x, acc[r].x);
                        atomicAdd(&p[r].y, acc[r].y);
                        acc[r] = make_float2(0.f, 0.f);
                    }
                }
                cur = key;
            }
            const float *wrow = swt + k * STR;
            const float wui = wrow[ti];
            const float2 t = make_float2(wui * xk.x, wui * xk.y);
#pragma unroll
            for (int r = 0; r < PER; ++r) acc[r] = __ffma2_rn(f2(wrow[W2 + tj + r]), t, acc[r]);
        }
        if (cur >= 0 && active) {
            float2 *p = sm + ((cur >> 6) + 1 + ti) * S + (cur & 63) + 1 + tj;
#pragma unroll
            for (int r = 0; r < PER; ++r) {
                atomicAdd(&p[r].x, acc[r].x);
                atomicAdd(&p[r].y, acc[r].y);
            }
        }
    }
    __syncthreads();
    grid_flush_extended<W2>(sm, grid, it, g);
}

template <typename K>
static int set_smem(K kernel, size_t smem)
{
    if (smem > 48 * 1024)
        LENTILS_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
    return LENTILS_OK;
}

template <int W2>
static int launch_degrid_t(const lentils_plan *p, const float2 *grid, float2 *vis,
                           cudaStream_t s)
{
    const GridGeom &g = p->geom;
    const size_t smem = sizeof(float2) * (size_t)g.E * g.stride;
    if (int st = set_smem(degrid_kernel<W2>, smem)) return st;
    degrid_kernel<W2><<<p->nitems, 256, smem, s>>>(grid, p->coords, vis, p->items, p->kb, g);
    LENTILS_CHECK_LAUNCH("degrid_kernel");
    return LENTILS_OK;
}

template <int W2>
static int launch_grid_t(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s)
{
    const GridGeom &g = p->geom;
    const size_t tile_bytes = sizeof(float4) * (size_t)((g.E * g.stride + 1) / 2);
    const size_t smem = tile_bytes + sizeof(float4) * kGridBatch +
                        sizeof(float) * (size_t)kGridBatch * LaneTaps<W2>::STR;
    if (int st = set_smem(grid_kernel<W2>, smem)) return st;
    grid_kernel<W2><<<p->nitems, kGridBatch, smem, s>>>(vis, p->coords, grid, p->items, p->kb, g);
    LENTILS_CHECK_LAUNCH("grid_kernel");
    return LENTILS_OK;
}

int launch_degrid(const lentils_plan *p, const float2 *grid, float2 *vis, cudaStream_t s)
{
    if (p->nitems == 0) return LENTILS_OK;
    switch (p->geom.w) {
    case 1: return launch_degrid_t<2>(p, grid, vis, s);
    case 2: return launch_degrid_t<4>(p, grid, vis, s);
    case 3: return launch_degrid_t<6>(p, grid, vis, s);
    case 4: return launch_degrid_t<8>(p, grid, vis, s);
    case 5: return launch_degrid_t<10>(p, grid, vis, s);
    case 6: return launch_degrid_t<12>(p, grid, vis, s);
    case 7: return launch_degrid_t<14>(p, grid, vis, s);
    case 8: return launch_degrid_t<16>(p, grid, vis, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "degrid: w=%d", p->geom.w);
}

int launch_grid(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s)
{
    if (p->nitems == 0) return LENTILS_OK;
    switch (p->geom.w) {
    case 1: return launch_grid_t<2>(p, vis, grid, s);
    case 2: return launch_grid_t<4>(p, vis, grid, s);
    case 3: return launch_grid_t<6>(p, vis, grid, s);
    case 4: return launch_grid_t<8>(p, vis, grid, s);
    case 5: return launch_grid_t<10>(p, vis, grid, s);
    case 6: return launch_grid_t<12>(p, vis, grid, s);
    case 7: return launch_grid_t<14>(p, vis, grid, s);
    case 8: return launch_grid_t<16>(p, vis, grid, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "grid: w=%d", p->geom.w);
}

}  // namespace lentils
