// Kaiser-Bessel degridding and gridding on plan-ordered visibilities.
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
#include <algorithm>
#include <type_traits>

#include "common.cuh"
#include "gridding_items.cuh"

namespace lentils {

template <int W2, typename R>
__global__ void __launch_bounds__(256)
    degrid_kernel(const typename Prec<R>::C *__restrict__ grid, const uint2 *__restrict__ coords,
                  typename Prec<R>::C *__restrict__ out, const WorkItem *__restrict__ items,
                  const __grid_constant__ typename Prec<R>::Table kb, const GridGeom g,
                  const float2 *__restrict__ cres, const R *__restrict__ vscale)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    degrid_item<W2, R>(grid, coords, out, items[blockIdx.x], kb, g, cres, smraw, vscale);
}


// Layout of one visibility's row in the gridding batch, in units of R:
//   [0, W2)        v-axis weights wv
//   [W2, 2W2)      u-axis weights wu
//   2W2, 2W2+1     weighted value x (re, im)
//   2W2+2          cell key (bit pattern of an int)
// and the split of a warp into V sub-groups of 32/V lanes, each working on its own visibility;
// every active lane owns PER adjacent taps of one row of the 2w x 2w window.
template <int W2, int V, typename R>
struct GridShape {
    static constexpr int STR = 2 * W2 + 4;
    static constexpr int LPV = 32 / V;  // lanes per visibility
    static constexpr int per()
    {
        for (int d = 1; d <= W2; ++d)
            if (W2 % d == 0 && LPV * d >= W2 * W2) return d;
        return W2;
    }
    static constexpr int PER = per();
};

template <typename R>
__device__ __forceinline__ R key_as(int k);
template <>
__device__ __forceinline__ float key_as<float>(int k) { return __int_as_float(k); }
template <>
__device__ __forceinline__ double key_as<double>(int k) { return __longlong_as_double((long long)k); }
template <typename R>
__device__ __forceinline__ int key_of(R v);
template <>
__device__ __forceinline__ int key_of<float>(float v) { return __float_as_int(v); }
template <>
__device__ __forceinline__ int key_of<double>(double v) { return (int)__double_as_longlong(v); }

// Gridding. Per batch of 256 sorted visibilities, each thread evaluates one visibility's
// weights into a shared row. Each warp then walks its 32 visibilities as V sub-groups of 32/V
// lanes (sub-group h takes a contiguous 32/V of them); a lane owns PER adjacent taps of one
// window row and accumulates them in registers while its sub-group's visibilities stay in one
// cell (weights and value are broadcast reads of the shared row). A change of cell, or the
// end of the sub-group's share, flushes the lane's taps into the extended tile.
//
// PRIV (V == 1 only): every warp has its own copy of the extended tile, flushed with plain
// load-add-store -- with V == 1 the whole warp works on one visibility, so the flush branch is
// warp-uniform, the lanes own distinct taps and no other warp writes the copy -- and the copies
// are summed once per work item before the global flush. Otherwise (V == 2, whose half-warps
// flush independently, or when the copies do not fit in shared memory) all warps share one
// tile and flush with shared-memory atomics.
template <int W2, int V, bool PRIV, typename R>
__global__ void __launch_bounds__(kGridBatch)
    grid_kernel(const typename Prec<R>::C *__restrict__ vis, const uint2 *__restrict__ coords,
                typename Prec<R>::C *__restrict__ grid, const WorkItem *__restrict__ items,
                const __grid_constant__ typename Prec<R>::Table kb, const GridGeom g,
                const float2 *__restrict__ cres)
{
    using P = Prec<R>;
    using C = typename P::C;
    using GS = GridShape<W2, V, R>;
    constexpr int STR = GS::STR, LPV = GS::LPV, PER = GS::PER;
    constexpr int NW = kGridBatch / 32;
    static_assert(!PRIV || V == 1, "private warp tiles need a warp-uniform flush (V == 1)");
    extern __shared__ __align__(16) unsigned char smraw[];
    const WorkItem it = items[blockIdx.x];
    if (it.count == 0) return;  // padding item (block-uniform): nothing to clear or flush
    const int E = g.E, S = g.stride;
    const int ntile = PRIV ? NW : 1;
    C *tiles = reinterpret_cast<C *>(smraw);  // ntile x (E x S) extended tiles
    const size_t tile_bytes = ((sizeof(C) * (size_t)ntile * E * S) + 15) & ~size_t(15);
    R *rows = reinterpret_cast<R *>(smraw + tile_bytes);  // kGridBatch x STR
    for (int e = threadIdx.x; e < ntile * E * S; e += blockDim.x) tiles[e] = P::zero();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    C *mytile = tiles + (PRIV ? warp * E * S : 0);
    const int sub = lane / LPV, sl = lane - sub * LPV;
    const int t0 = sl * PER;
    const bool active = t0 < W2 * W2;
    const int ti = active ? t0 / W2 : 0;
    const int tj = active ? t0 - ti * W2 : 0;

    for (int base = 0; base < it.count; base += kGridBatch) {
        const int n = min(kGridBatch, it.count - base);
        __syncthreads();  // tiles zeroed / previous batch consumed
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
            R *row = rows + k * STR;
#pragma unroll
            for (int j = 0; j < W2; ++j) row[j] = wv[j];
#pragma unroll
            for (int i = 0; i < W2; ++i) row[W2 + i] = wu[i];
            row[2 * W2] = x.x;
            row[2 * W2 + 1] = x.y;
            row[2 * W2 + 2] = key_as<R>((lu << 6) | lv);
            if ((c.x | c.y) & kExtraTapBit)  // rare: straight into this warp's tile, atomically
                grid_extra_taps<W2, R>(mytile, S, lu, lv, c, wu, wv, (R)kb.edge, x);
        }
        __syncthreads();
        constexpr int share = 32 / V;
        const int k0 = warp * 32 + sub * share;
        const int k1 = min(n, k0 + share);
        C acc[PER];
#pragma unroll
        for (int r = 0; r < PER; ++r) acc[r] = P::zero();
        int cur = -1;
        auto flush = [&](int key) {
            C *p = mytile + ((key >> 6) + 1 + ti) * S + (key & 63) + 1 + tj;
#pragma unroll
            for (int r = 0; r < PER; ++r) {
                if (PRIV) {
                    C v = p[r];
                    v.x += acc[r].x;
                    v.y += acc[r].y;
                    p[r] = v;
                } else {
                    atomicAdd(&p[r].x, acc[r].x);
                    atomicAdd(&p[r].y, acc[r].y);
                }
                acc[r] = P::zero();
            }
        };
        for (int k = k0; k < k1; ++k) {
            const R *row = rows + k * STR;
            const int key = key_of<R>(row[2 * W2 + 2]);
            if (key != cur) {
                if (cur >= 0 && active) flush(cur);
                cur = key;
            }
            C x;
            x.x = row[2 * W2];
            x.y = row[2 * W2 + 1];
            const C t = P::scale(row[W2 + ti], x);
#pragma unroll
            for (int r = 0; r < PER; ++r) acc[r] = P::fma(row[tj + r], t, acc[r]);
        }
        if (cur >= 0 && active) flush(cur);
    }
    __syncthreads();
    if (PRIV) {  // sum the warps' copies into copy 0
        for (int e = threadIdx.x; e < E * S; e += blockDim.x) {
            C a = tiles[e];
#pragma unroll
            for (int q = 1; q < NW; ++q) {
                const C b = tiles[q * E * S + e];
                a.x += b.x;
                a.y += b.y;
            }
            tiles[e] = a;
        }
        __syncthreads();
    }
    grid_flush_extended<W2, R>(tiles, grid, it, g);
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

template <int W2>
__global__ void degrid_pair_kernel(const float2 *__restrict__ grid,
                                   const uint2 *__restrict__ coords, float2 *__restrict__ out,
                                   const WorkItem *__restrict__ items,
                                   const __grid_constant__ KBPoly kb, const GridGeom g,
                                   const float *__restrict__ vscale);

constexpr int kChunkThreads = 128;

template <int W2, int K>
__global__ void __launch_bounds__(kChunkThreads, 4)
    degrid_chunk_kernel(const float2 *__restrict__ grid, const uint2 *__restrict__ coords,
                        float2 *__restrict__ out, const WorkItem *__restrict__ items,
                        const int2 *__restrict__ item_chunks, const int *__restrict__ chunk_begin,
                        const __grid_constant__ KBPoly kb, const GridGeom g,
                        const float *__restrict__ vscale)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    degrid_item_chunks<W2, K>(grid, coords, out, items[blockIdx.x], item_chunks[blockIdx.x],
                              chunk_begin, kb, g, smraw, vscale);
}

template <int W2, typename R>
static int launch_degrid_t(const lentils_plan *p, const typename Prec<R>::C *grid,
                           typename Prec<R>::C *vis, cudaStream_t s, const R *vscale)
{
    const GridGeom &g = p->geom;
    if constexpr (std::is_same<R, float>::value && W2 <= 8) {
        if (p->degrid_variant == 0 && p->chunk_begin && p->chunk_k == 4) {  // the default
            const size_t smem = sizeof(float2) * (size_t)g.E * g.stride;
            if (int st = set_smem(degrid_chunk_kernel<W2, 4>, smem)) return st;
            degrid_chunk_kernel<W2, 4><<<p->nitems, kChunkThreads, smem, s>>>(
                grid, p->coords, vis, p->items, p->item_chunks, p->chunk_begin, p->kb, g,
                vscale);
            LENTILS_CHECK_LAUNCH("degrid_chunk_kernel");
            return LENTILS_OK;
        }
    }
    if constexpr (std::is_same<R, float>::value && (W2 % 2) == 0) {
        if (p->degrid_variant == 1) {
            const size_t smem = degrid_pair_smem_bytes(g);
            if (int st = set_smem(degrid_pair_kernel<W2>, smem)) return st;
            degrid_pair_kernel<W2><<<p->nitems, 256, smem, s>>>(grid, p->coords, vis, p->items,
                                                                p->kb, g, vscale);
            LENTILS_CHECK_LAUNCH("degrid_pair_kernel");
            return LENTILS_OK;
        }
    }
    const size_t smem = sizeof(typename Prec<R>::C) * (size_t)g.E * g.stride;
    if (int st = set_smem(degrid_kernel<W2, R>, smem)) return st;
    const float2 *cres = std::is_same<R, double>::value ? p->coords_res : nullptr;
    degrid_kernel<W2, R><<<p->nitems, 256, smem, s>>>(grid, p->coords, vis, p->items,
                                                     table_of<R>(p), g, cres, vscale);
    LENTILS_CHECK_LAUNCH("degrid_kernel");
    return LENTILS_OK;
}

template <int W2, bool SHARED, bool MASKED = false, bool ATOMIC = false, bool KAHAN = false>
__global__ void __launch_bounds__(kGridBatch)
    grid_rows_kernel(const float2 *__restrict__ vis, const uint2 *__restrict__ coords,
                     float2 *__restrict__ grid, const WorkItem *__restrict__ items,
                     const __grid_constant__ KBPoly kb, const GridGeom g)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    grid_rows_item<W2, SHARED, MASKED, ATOMIC, KAHAN>(vis, coords, grid, items[blockIdx.x], kb,
                                                      g, smraw);
}

template <int W2>
__global__ void __launch_bounds__(kGridBatch)
    grid_ballot_kernel(const float2 *__restrict__ vis, const uint2 *__restrict__ coords,
                       float2 *__restrict__ grid, const WorkItem *__restrict__ items,
                       const __grid_constant__ KBPoly kb, const GridGeom g)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    grid_rows_item_ballot<W2>(vis, coords, grid, items[blockIdx.x], kb, g, smraw);
}

constexpr size_t kMaxGridSmem = 200 * 1024;

template <int W2, int NW>
__global__ void __launch_bounds__(NW * 32)
    grid_local_kernel(const float2 *__restrict__ vis, const uint2 *__restrict__ coords,
                      float2 *__restrict__ grid, const WorkItem *__restrict__ items,
                      const __grid_constant__ KBPoly kb, const GridGeom g)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    grid_rows_item_local<W2, NW>(vis, coords, grid, items[blockIdx.x], kb, g, smraw);
}

template <int W2, int NW, bool NARROW>
__global__ void __launch_bounds__(NW * 32)
    grid_pairs_kernel(const float2 *__restrict__ vis, const uint2 *__restrict__ coords,
                      float2 *__restrict__ grid, const WorkItem *__restrict__ items,
                      const __grid_constant__ KBPoly kb, const GridGeom g)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    grid_rows_item_pairs<W2, NW, NARROW>(vis, coords, grid, items[blockIdx.x], kb, g, smraw);
}

template <int W2, int NW, bool NARROW = false>
static int launch_grid_pairs(const lentils_plan *p, const float2 *vis, float2 *grid,
                             cudaStream_t s, bool *done)
{
    *done = false;
    const size_t smem = grid_pairs_smem_bytes<W2, NW>(p->geom);
    if (smem > kMaxGridSmem) return LENTILS_OK;
    if (int st = set_smem(grid_pairs_kernel<W2, NW, NARROW>, smem)) return st;
    grid_pairs_kernel<W2, NW, NARROW><<<p->nitems, NW * 32, smem, s>>>(
        vis, p->coords, grid, p->items, p->kb, p->geom);
    LENTILS_CHECK_LAUNCH("grid_pairs_kernel");
    *done = true;
    return LENTILS_OK;
}

template <int W2, int NW>
static int launch_grid_local(const lentils_plan *p, const float2 *vis, float2 *grid,
                             cudaStream_t s, bool *done)
{
    *done = false;
    const size_t smem = grid_local_smem_bytes<W2, NW>(p->geom);
    if (smem > kMaxGridSmem) return LENTILS_OK;
    if (int st = set_smem(grid_local_kernel<W2, NW>, smem)) return st;
    grid_local_kernel<W2, NW><<<p->nitems, NW * 32, smem, s>>>(vis, p->coords, grid, p->items,
                                                              p->kb, p->geom);
    LENTILS_CHECK_LAUNCH("grid_local_kernel");
    *done = true;
    return LENTILS_OK;
}

template <int W2>
__global__ void __launch_bounds__(256)
    degrid_pair_kernel(const float2 *__restrict__ grid, const uint2 *__restrict__ coords,
                       float2 *__restrict__ out, const WorkItem *__restrict__ items,
                       const __grid_constant__ KBPoly kb, const GridGeom g,
                       const float *__restrict__ vscale)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    degrid_item_pair<W2>(grid, coords, out, items[blockIdx.x], kb, g, smraw, vscale);
}


template <int W2, int V, bool PRIV, typename R>
static size_t grid_smem_bytes(const GridGeom &g)
{
    using C = typename Prec<R>::C;
    const size_t ntile = PRIV ? kGridBatch / 32 : 1;
    const size_t tile_bytes = ((sizeof(C) * ntile * g.E * g.stride) + 15) & ~size_t(15);
    return tile_bytes + sizeof(R) * (size_t)kGridBatch * GridShape<W2, V, R>::STR;
}

template <int W2, int V, typename R>
static int launch_grid_tv(const lentils_plan *p, const typename Prec<R>::C *vis,
                          typename Prec<R>::C *grid, cudaStream_t s)
{
    const GridGeom &g = p->geom;
    const float2 *cres = std::is_same<R, double>::value ? p->coords_res : nullptr;
    constexpr bool kPriv = (V == 1);
    const size_t smem_priv = grid_smem_bytes<W2, V, kPriv, R>(g);
    if (kPriv && smem_priv <= kMaxGridSmem) {
        if (int st = set_smem(grid_kernel<W2, V, kPriv, R>, smem_priv)) return st;
        grid_kernel<W2, V, kPriv, R><<<p->nitems, kGridBatch, smem_priv, s>>>(
            vis, p->coords, grid, p->items, table_of<R>(p), g, cres);
    } else {
        const size_t smem = grid_smem_bytes<W2, V, false, R>(g);
        if (int st = set_smem(grid_kernel<W2, V, false, R>, smem)) return st;
        grid_kernel<W2, V, false, R><<<p->nitems, kGridBatch, smem, s>>>(
            vis, p->coords, grid, p->items, table_of<R>(p), g, cres);
    }
    LENTILS_CHECK_LAUNCH("grid_kernel");
    return LENTILS_OK;
}

template <int W2, typename R>
static int launch_grid_t(const lentils_plan *p, const typename Prec<R>::C *vis,
                         typename Prec<R>::C *grid, cudaStream_t s)
{
    if constexpr (std::is_same<R, float>::value && (W2 % 2) == 0) {
        if (p->grid_variant == 0 || p->grid_variant == 11) {
            // the default: column-pair register windows, warp-local batches, 4 warps per CTA
            // (tiles too large for the warp-private copies fall through)
            bool done = false;
            const int st = p->grid_variant == 0
                               ? launch_grid_pairs<W2, 4>(p, vis, grid, s, &done)
                               : launch_grid_pairs<W2, 8>(p, vis, grid, s, &done);
            if (st || done) return st;
        }
        if (p->grid_variant == 10) {
            bool done = false;
            const int st = launch_grid_local<W2, 4>(p, vis, grid, s, &done);
            if (st || done) return st;
        }
        if (p->grid_variant == 12) {
            bool done = false;
            const int st = launch_grid_pairs<W2, 4, true>(p, vis, grid, s, &done);
            if (st || done) return st;
        }
        if (p->grid_variant == 9) {  // flush steps from the producers' ballot, CTA barriers
            const size_t smem = grid_ballot_smem_bytes<W2>(p->geom);
            if (smem <= kMaxGridSmem) {
                if (int st = set_smem(grid_ballot_kernel<W2>, smem)) return st;
                grid_ballot_kernel<W2><<<p->nitems, kGridBatch, smem, s>>>(
                    vis, p->coords, grid, p->items, p->kb, p->geom);
                LENTILS_CHECK_LAUNCH("grid_ballot_kernel");
                return LENTILS_OK;
            }
        }
        if (p->grid_variant == 7) {  // compensated register sums
            const GridGeom &g = p->geom;
            const size_t smem = grid_rows_smem_bytes<W2, false>(g);
            if (smem > kMaxGridSmem) return launch_grid_tv<W2, 1, R>(p, vis, grid, s);
            if (int st = set_smem(grid_rows_kernel<W2, false, true, false, true>, smem)) return st;
            grid_rows_kernel<W2, false, true, false, true><<<p->nitems, kGridBatch, smem, s>>>(
                vis, p->coords, grid, p->items, p->kb, g);
            LENTILS_CHECK_LAUNCH("grid_rows_kernel");
            return LENTILS_OK;
        }
        if (p->grid_variant == 5 || p->grid_variant == 6) {  // atomic flushes
            const GridGeom &g = p->geom;
            if (p->grid_variant == 6) {
                const size_t smem = grid_rows_smem_bytes<W2, true>(g);
                if (int st = set_smem(grid_rows_kernel<W2, true, true, true>, smem)) return st;
                grid_rows_kernel<W2, true, true, true><<<p->nitems, kGridBatch, smem, s>>>(
                    vis, p->coords, grid, p->items, p->kb, g);
            } else {
                const size_t smem = grid_rows_smem_bytes<W2, false>(g);
                if (smem > kMaxGridSmem) return launch_grid_tv<W2, 1, R>(p, vis, grid, s);
                if (int st = set_smem(grid_rows_kernel<W2, false, true, true>, smem)) return st;
                grid_rows_kernel<W2, false, true, true><<<p->nitems, kGridBatch, smem, s>>>(
                    vis, p->coords, grid, p->items, p->kb, g);
            }
            LENTILS_CHECK_LAUNCH("grid_rows_kernel");
            return LENTILS_OK;
        }
        if (p->grid_variant == 0 || p->grid_variant == 3 || p->grid_variant == 4 ||
            p->grid_variant == 8) {
            const GridGeom &g = p->geom;
            if (p->grid_variant == 3) {
                const size_t smem = grid_rows_smem_bytes<W2, true>(g);
                if (int st = set_smem(grid_rows_kernel<W2, true>, smem)) return st;
                grid_rows_kernel<W2, true><<<p->nitems, kGridBatch, smem, s>>>(
                    vis, p->coords, grid, p->items, p->kb, g);
                LENTILS_CHECK_LAUNCH("grid_rows_kernel");
                return LENTILS_OK;
            }
            const size_t smem = grid_rows_smem_bytes<W2, false>(g);
            if (smem <= kMaxGridSmem && (p->grid_variant == 0 || p->grid_variant == 8)) {
                if (int st = set_smem(grid_rows_kernel<W2, false, true>, smem)) return st;
                grid_rows_kernel<W2, false, true><<<p->nitems, kGridBatch, smem, s>>>(
                    vis, p->coords, grid, p->items, p->kb, g);
                LENTILS_CHECK_LAUNCH("grid_rows_kernel");
                return LENTILS_OK;
            }
            if (smem <= kMaxGridSmem) {
                if (int st = set_smem(grid_rows_kernel<W2, false>, smem)) return st;
                grid_rows_kernel<W2, false><<<p->nitems, kGridBatch, smem, s>>>(
                    vis, p->coords, grid, p->items, p->kb, g);
                LENTILS_CHECK_LAUNCH("grid_rows_kernel");
                return LENTILS_OK;
            }
        }
    }
    if (p->grid_variant == 2) return launch_grid_tv<W2, 2, R>(p, vis, grid, s);
    return launch_grid_tv<W2, 1, R>(p, vis, grid, s);
}

template <typename R>
static int launch_degrid_r(const lentils_plan *p, const typename Prec<R>::C *grid,
                           typename Prec<R>::C *vis, cudaStream_t s, const R *vscale)
{
    if (p->nitems == 0) return LENTILS_OK;
    switch (p->geom.w) {
    case 1: return launch_degrid_t<2, R>(p, grid, vis, s, vscale);
    case 2: return launch_degrid_t<4, R>(p, grid, vis, s, vscale);
    case 3: return launch_degrid_t<6, R>(p, grid, vis, s, vscale);
    case 4: return launch_degrid_t<8, R>(p, grid, vis, s, vscale);
    case 5: return launch_degrid_t<10, R>(p, grid, vis, s, vscale);
    case 6: return launch_degrid_t<12, R>(p, grid, vis, s, vscale);
    case 7: return launch_degrid_t<14, R>(p, grid, vis, s, vscale);
    case 8: return launch_degrid_t<16, R>(p, grid, vis, s, vscale);
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

int launch_degrid(const lentils_plan *p, const float2 *grid, float2 *vis, cudaStream_t s,
                  const float *vscale)
{
    return launch_degrid_r<float>(p, grid, vis, s, vscale);
}

int launch_grid(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s)
{
    return launch_grid_r<float>(p, vis, grid, s);
}

int launch_degrid64(const lentils_plan *p, const double2 *grid, double2 *vis, cudaStream_t s,
                    const double *vscale)
{
    return launch_degrid_r<double>(p, grid, vis, s, vscale);
}

int launch_grid64(const lentils_plan *p, const double2 *vis, double2 *grid, cudaStream_t s)
{
    return launch_grid_r<double>(p, vis, grid, s);
}

}  // namespace lentils
