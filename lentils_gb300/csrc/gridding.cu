// Kaiser-Bessel degridding ("K1") and gridding ("K2") on plan-ordered visibilities.
//
// One CTA per work item (a tile of T x T uv cells and up to `chunk` of its visibilities,
// sorted by cell). The CTA stages the tile plus a w-cell halo ("extended tile", E x E cells,
// E = T + 2w) in shared memory:
//   degrid: gathered from the stored r2c half-plane grid with the reference's wrap and
//           Hermitian fold applied on the way in (lentils/backend/nufft.c:83-93), so the
//           inner loop reads a plain full-plane patch;
//   grid:   zeroed, accumulated by all threads with shared-memory atomics, and flushed once
//           through the fold (conjugate on folded cells, x2 on column 0, nufft.c:107-111)
//           with one 8-byte global atomic per touched cell.
// Each thread owns whole visibilities: it evaluates the 2w separable weights per axis as
// degree-9 polynomials of the fixed-point fraction (packed FP32x2 FMAs), then runs the
// 2w x 2w taps.
//
// Tap set. The reference visits round(g)-w .. round(g)+w per axis (nufft.c:65-68) and its
// weight is zero beyond |g - i| > w (nufft.c:12-13). For f = g - floor(g) in (0, 1) the
// non-zero taps are exactly floor(g)-w+1 .. floor(g)+w (2w taps); for f == 0 one more tap,
// floor(g)-w at argument exactly +w, is non-zero (weight I0(0)/(2w)) and is added on a
// separate, rarely taken path. The checkerboard sign (-1)^(i_u+i_v) (nufft.c:78) is folded
// into the polynomial table per tap and a per-visibility parity; the factors 2*0.5 (degrid)
// and 0.5 (grid) of nufft.c:79-80,102-104 are applied here.
#include "common.cuh"

namespace lentils {

__device__ __forceinline__ int wrap_index(int a, int n)
{
    int r = a % n;
    return r < 0 ? r + n : r;
}

template <int W2>
__device__ __forceinline__ void kb_weights(const KBPoly &kb, float f, float (&wt)[W2])
{
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
}

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }

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
        const int lu = (int)(c.x >> kFracBits), lv = (int)(c.y >> kFracBits);
        const uint32_t fui = c.x & kFracMask, fvi = c.y & kFracMask;
        float wu[W2], wv[W2];
        kb_weights<W2>(kb, (float)fui * (1.0f / (float)(1u << kFracBits)), wu);
        kb_weights<W2>(kb, (float)fvi * (1.0f / (float)(1u << kFracBits)), wv);
        const float2 *p = sm + (lu + 1) * S + (lv + 1);
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < W2; ++i) {
            float2 r = make_float2(0.f, 0.f);
#pragma unroll
            for (int j = 0; j < W2; ++j) r = __ffma2_rn(f2(wv[j]), p[i * S + j], r);
            acc = __ffma2_rn(f2(wu[i]), r, acc);
        }
        if (fui == 0 || fvi == 0) {
            // edge taps at argument exactly +w (row lu / column lv of the extended tile)
            const float eu = (fui == 0) ? kb.edge : 0.f;
            const float ev = (fvi == 0) ? kb.edge : 0.f;
            const float2 *q = sm + lu * S + lv;  // extended (lu, lv) = tap (-1, -1)
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

template <int W2>
__global__ void __launch_bounds__(256)
    grid_kernel(const float2 *__restrict__ vis, const uint2 *__restrict__ coords,
                float2 *__restrict__ grid, const WorkItem *__restrict__ items,
                const __grid_constant__ KBPoly kb, const GridGeom g)
{
    extern __shared__ float2 sm[];
    const WorkItem it = items[blockIdx.x];
    constexpr int w = W2 / 2;
    const int a0 = it.tu * g.T - g.Hu - w;
    const int b0 = it.tv * g.T - g.Hv - w;
    const int E = g.E, S = g.stride;
    for (int e = threadIdx.x; e < E * S; e += blockDim.x) sm[e] = make_float2(0.f, 0.f);
    __syncthreads();

    for (int k = threadIdx.x; k < it.count; k += blockDim.x) {
        const uint2 c = coords[it.begin + k];
        const int lu = (int)(c.x >> kFracBits), lv = (int)(c.y >> kFracBits);
        const uint32_t fui = c.x & kFracMask, fvi = c.y & kFracMask;
        float wu[W2], wv[W2];
        kb_weights<W2>(kb, (float)fui * (1.0f / (float)(1u << kFracBits)), wu);
        kb_weights<W2>(kb, (float)fvi * (1.0f / (float)(1u << kFracBits)), wv);
        float2 x = vis[it.begin + k];
        const float h = tap_parity(it, g, lu, lv) ? -0.5f : 0.5f;
        x = make_float2(h * x.x, h * x.y);
        float2 *p = sm + (lu + 1) * S + (lv + 1);
#pragma unroll
        for (int i = 0; i < W2; ++i) {
            const float2 t = make_float2(wu[i] * x.x, wu[i] * x.y);
#pragma unroll
            for (int j = 0; j < W2; ++j) {
                atomicAdd(&p[i * S + j].x, wv[j] * t.x);
                atomicAdd(&p[i * S + j].y, wv[j] * t.y);
            }
        }
        if (fui == 0 || fvi == 0) {
            const float eu = (fui == 0) ? kb.edge : 0.f;
            const float ev = (fvi == 0) ? kb.edge : 0.f;
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
    }
    __syncthreads();

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

template <int W2>
static int launch_degrid_t(const lentils_plan *p, const float2 *grid, float2 *vis,
                           cudaStream_t s)
{
    const GridGeom &g = p->geom;
    const size_t smem = sizeof(float2) * (size_t)g.E * g.stride;
    if (smem > 48 * 1024)
        LENTILS_CUDA_TRY(cudaFuncSetAttribute(degrid_kernel<W2>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
    degrid_kernel<W2><<<p->nitems, 256, smem, s>>>(grid, p->coords, vis, p->items, p->kb, g);
    LENTILS_CHECK_LAUNCH("degrid_kernel");
    return LENTILS_OK;
}

template <int W2>
static int launch_grid_t(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s)
{
    const GridGeom &g = p->geom;
    const size_t smem = sizeof(float2) * (size_t)g.E * g.stride;
    if (smem > 48 * 1024)
        LENTILS_CUDA_TRY(cudaFuncSetAttribute(grid_kernel<W2>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)smem));
    grid_kernel<W2><<<p->nitems, 256, smem, s>>>(vis, p->coords, grid, p->items, p->kb, g);
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
