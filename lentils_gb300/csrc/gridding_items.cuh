// Per-work-item Kaiser-Bessel degridding and gridding device functions, shared by the
// one-item-per-CTA kernels (gridding.cu) and the persistent batched sweep (sweep.cu).
// Conventions (tap set, fixed-point cells, fold, factors) are documented in gridding.cu.
#pragma once

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
    constexpr int w = W2 / 2;
    const float f = (float)(word & kFracMask) * (1.0f / (float)(1u << kFracBits));
    const float t = fmaf(2.0f, f, -1.0f);
    const float2 tt = make_float2(t, t);
    const float2 uu = make_float2(t * t, t * t);
#pragma unroll
    for (int p = 0; p < (w + 1) / 2; ++p) {
        float2 e = kb.ce[0][p], o = kb.co[0][p];
#pragma unroll
        for (int k = 1; k < kHalfCoef; ++k) {
            e = __ffma2_rn(e, uu, kb.ce[k][p]);
            o = __ffma2_rn(o, uu, kb.co[k][p]);
        }
        const float2 lo = __ffma2_rn(tt, o, e);                               // P_i(t)
        const float2 hi = __ffma2_rn(tt, o, make_float2(-e.x, -e.y));         // -P_i(-t)
        wt[2 * p] = lo.x;
        wt[W2 - 1 - 2 * p] = hi.x;
        if (2 * p + 1 < w) {
            wt[2 * p + 1] = lo.y;
            wt[W2 - 2 - 2 * p] = hi.y;
        }
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
    const double t = 2.0 * f - 1.0, u = t * t;
    // taps i and 2w-1-i from the even and odd parts of P_i (half the FMAs of one Horner per tap)
#pragma unroll
    for (int i = 0; i < W2 / 2; ++i) {
        double e = kb.ce[0][i], o = kb.co[0][i];
#pragma unroll
        for (int k = 1; k < kHalfCoef; ++k) {
            e = ::fma(e, u, kb.ce[k][i]);
            o = ::fma(o, u, kb.co[k][i]);
        }
        wt[i] = ::fma(t, o, e);
        wt[W2 - 1 - i] = ::fma(t, o, -e);
    }
    if (word & kTopOffBit) wt[W2 - 1] = 0.0;
}

// Parity of the first regular tap (canonical cell index) of a visibility in the item's tile.
__device__ __forceinline__ int tap_parity(const WorkItem &it, const GridGeom &g, int lu, int lv)
{
    return (it.tu * g.T - g.Hu + lu - g.w + 1 + it.tv * g.T - g.Hv + lv - g.w + 1) & 1;
}

// The work item's extended tile (T + 2w cells square, row stride g.stride) gathered from the
// stored half-plane grid by the whole CTA, with the wrap and the Hermitian fold applied
// (folded cells conjugated), so that the degridding loops read a plain full-plane patch.
template <int W2, typename R>
__device__ __forceinline__ void stage_extended_tile(const typename Prec<R>::C *__restrict__ grid,
                                                    const WorkItem &it, const GridGeom &g,
                                                    typename Prec<R>::C *sm)
{
    using C = typename Prec<R>::C;
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
}

// Degridding of one work item by the whole CTA (any block size); smraw: E x stride cells.
// vscale (optional, plan order): each output is multiplied by its factor (the data weights of
// a normal operator, applied here instead of in a separate pass).
template <int W2, typename R>
__device__ __forceinline__ void degrid_item(const typename Prec<R>::C *__restrict__ grid,
                                            const uint2 *__restrict__ coords,
                                            typename Prec<R>::C *__restrict__ out,
                                            const WorkItem &it,
                                            const typename Prec<R>::Table &kb, const GridGeom &g,
                                            const float2 *__restrict__ cres,
                                            unsigned char *smraw,
                                            const R *__restrict__ vscale = nullptr)
{
    using P = Prec<R>;
    using C = typename P::C;
    C *sm = reinterpret_cast<C *>(smraw);
    const int S = g.stride;
    stage_extended_tile<W2, R>(grid, it, g, sm);
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
        if (vscale) {
            const R sc = vscale[it.begin + k];
            acc.x *= sc;
            acc.y *= sc;
        }
        out[it.begin + k] = acc;
    }
}

// Degridding with the extended tile staged as overlapping column pairs: element (a, b) of
// the shared array holds (G[a][b], G[a][b+1]) as one float4, so a visibility's 2w taps along v
// are w 16-byte loads instead of 2w 8-byte loads. Threads of a warp take consecutive sorted
// visibilities, which mostly share a cell or sit in neighbouring ones; their loads are then
// broadcasts or adjacent 16-byte words, so halving the load instructions also halves the
// shared-memory wavefronts that bound this kernel. Same arithmetic, in the same order, as
// degrid_item<W2, float>. smraw: degrid_pair_smem_bytes(g).
template <int W2>
__device__ __forceinline__ void degrid_item_pair(const float2 *__restrict__ grid,
                                                 const uint2 *__restrict__ coords,
                                                 float2 *__restrict__ out, const WorkItem &it,
                                                 const KBPoly &kb, const GridGeom &g,
                                                 unsigned char *smraw,
                                                 const float *__restrict__ vscale = nullptr)
{
    static_assert((W2 % 2) == 0, "pairs of taps");
    float4 *sm = reinterpret_cast<float4 *>(smraw);
    constexpr int w = W2 / 2;
    const int a0 = it.tu * g.T - g.Hu - w;
    const int b0 = it.tv * g.T - g.Hv - w;
    const int E = g.E, S = g.stride;  // S odd: rows 4 words apart modulo 32 banks
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
        float2 *row = reinterpret_cast<float2 *>(sm + ea * S);
        row[2 * eb] = val;                       // (a, b).xy
        if (eb > 0) row[2 * eb - 1] = val;       // (a, b-1).zw
        if (eb == E - 1) row[2 * eb + 1] = make_float2(0.f, 0.f);
    }
    __syncthreads();

    for (int k = threadIdx.x; k < it.count; k += blockDim.x) {
        const uint2 c = coords[it.begin + k];
        const int lu = cell_of(c.x), lv = cell_of(c.y);
        float wu[W2], wv[W2];
        kb_weights<W2>(kb, c.x, wu);
        kb_weights<W2>(kb, c.y, wv);
        const float4 *p = sm + (lu + 1) * S + (lv + 1);
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < W2; ++i) {
            float2 r = make_float2(0.f, 0.f);
#pragma unroll
            for (int m = 0; m < W2 / 2; ++m) {
                const float4 q = p[i * S + 2 * m];
                r = __ffma2_rn(f2(wv[2 * m]), make_float2(q.x, q.y), r);
                r = __ffma2_rn(f2(wv[2 * m + 1]), make_float2(q.z, q.w), r);
            }
            acc = __ffma2_rn(f2(wu[i]), r, acc);
        }
        if ((c.x | c.y) & kExtraTapBit) {
            const float eu = (c.x & kExtraTapBit) ? kb.edge : 0.f;
            const float ev = (c.y & kExtraTapBit) ? kb.edge : 0.f;
            const float4 *q = sm + lu * S + lv;
            float2 r = make_float2(0.f, 0.f);
            for (int j = 0; j < W2; ++j) {
                const float4 t = q[j + 1];
                r = __ffma2_rn(f2(wv[j]), make_float2(t.x, t.y), r);
            }
            r = __ffma2_rn(f2(ev), make_float2(q[0].x, q[0].y), r);
            acc = __ffma2_rn(f2(eu), r, acc);
            float2 cs = make_float2(0.f, 0.f);
            for (int i = 0; i < W2; ++i) {
                const float4 t = q[(i + 1) * S];
                cs = __ffma2_rn(f2(wu[i]), make_float2(t.x, t.y), cs);
            }
            acc = __ffma2_rn(f2(ev), cs, acc);
        }
        if (tap_parity(it, g, lu, lv)) {
            acc.x = -acc.x;
            acc.y = -acc.y;
        }
        if (vscale) {
            const float sc = vscale[it.begin + k];
            acc.x *= sc;
            acc.y *= sc;
        }
        out[it.begin + k] = acc;
    }
}

template <int W2, int K>
__device__ __forceinline__ void degrid_chunks_from_tile(const uint2 *__restrict__ coords,
                                                        float2 *__restrict__ out,
                                                        const WorkItem &it, int2 crange,
                                                        const int *__restrict__ chunk_begin,
                                                        const KBPoly &kb, const GridGeom &g,
                                                        const float2 *sm,
                                                        const float *__restrict__ vscale);

// Degridding by same-cell chunks (the default for float, 2w <= 8). A thread takes one chunk:
// up to K consecutive sorted visibilities of one cell (the plan's chunk_begin). It evaluates
// the K visibilities' weights, then reads each of the 2w rows of the cell's window from the
// staged tile once, into registers, and applies it to all K visibilities. So a tap is read
// from shared memory once per chunk instead of once per visibility: (2w)^2 / K loads per
// visibility slot, where the per-visibility kernel's shared-memory reads bound its time.
// Slots past the chunk's end repeat its last visibility and are not stored. Per visibility the
// arithmetic, and its order, is that of degrid_item<W2, float>: the results are identical.
template <int W2, int K>
__device__ __forceinline__ void degrid_item_chunks(const float2 *__restrict__ grid,
                                                   const uint2 *__restrict__ coords,
                                                   float2 *__restrict__ out, const WorkItem &it,
                                                   int2 crange,
                                                   const int *__restrict__ chunk_begin,
                                                   const KBPoly &kb, const GridGeom &g,
                                                   unsigned char *smraw,
                                                   const float *__restrict__ vscale = nullptr)
{
    float2 *sm = reinterpret_cast<float2 *>(smraw);
    stage_extended_tile<W2, float>(grid, it, g, sm);
    __syncthreads();
    degrid_chunks_from_tile<W2, K>(coords, out, it, crange, chunk_begin, kb, g, sm, vscale);
}

// The same-cell chunks of one work item from its extended tile, already staged in sm. The
// coordinates of a thread's next chunk and the bounds of the one after are loaded while this
// one is evaluated.
template <int W2, int K>
__device__ __forceinline__ void degrid_chunks_from_tile(const uint2 *__restrict__ coords,
                                                        float2 *__restrict__ out,
                                                        const WorkItem &it, int2 crange,
                                                        const int *__restrict__ chunk_begin,
                                                        const KBPoly &kb, const GridGeom &g,
                                                        const float2 *sm,
                                                        const float *__restrict__ vscale)
{
    const int S = g.stride;
    const int B = blockDim.x;
    // chunk c + B's bounds were loaded one iteration ago and its coordinates are loaded now;
    // chunk c + 2B's bounds are loaded now: no load waits on another within an iteration
    int nb0 = 0, nb1 = 1, fb0 = 0, fb1 = 1;
    uint2 ncs[K];
    auto load_coords = [&](int cc) {
        if (cc < crange.y) {
#pragma unroll
            for (int q = 0; q < K; ++q) ncs[q] = coords[nb0 + min(q, nb1 - nb0 - 1)];
        }
    };
    auto load_bounds = [&](int cc) {
        if (cc < crange.y) {
            fb0 = chunk_begin[cc];
            fb1 = chunk_begin[cc + 1];
        }
    };
    const int c0 = crange.x + (int)threadIdx.x;
    load_bounds(c0);
    nb0 = fb0;
    nb1 = fb1;
    load_coords(c0);
    load_bounds(c0 + B);
    for (int c = c0; c < crange.y; c += B) {
        const int b0 = nb0;
        const int n = nb1 - nb0;
        uint2 cs[K];
#pragma unroll
        for (int q = 0; q < K; ++q) cs[q] = ncs[q];
        nb0 = fb0;
        nb1 = fb1;
        load_coords(c + B);
        load_bounds(c + 2 * B);
        const int lu = cell_of(cs[0].x), lv = cell_of(cs[0].y);
        float wu[K][W2], wv[K][W2];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            kb_weights<W2>(kb, cs[q].x, wu[q]);
            kb_weights<W2>(kb, cs[q].y, wv[q]);
        }
        const float2 *p = sm + (lu + 1) * S + (lv + 1);
        float2 acc[K];
#pragma unroll
        for (int q = 0; q < K; ++q) acc[q] = make_float2(0.f, 0.f);
#pragma unroll
        for (int i = 0; i < W2; ++i) {
            float2 row[W2];
#pragma unroll
            for (int j = 0; j < W2; ++j) row[j] = p[i * S + j];
#pragma unroll
            for (int q = 0; q < K; ++q) {
                float2 r = make_float2(0.f, 0.f);
#pragma unroll
                for (int j = 0; j < W2; ++j) r = __ffma2_rn(f2(wv[q][j]), row[j], r);
                acc[q] = __ffma2_rn(f2(wu[q][i]), r, acc[q]);
            }
        }
        const bool neg = tap_parity(it, g, lu, lv);
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (q >= n) break;
            const uint2 cq = cs[q];
            float2 a = acc[q];
            if ((cq.x | cq.y) & kExtraTapBit) {
                const float eu = (cq.x & kExtraTapBit) ? kb.edge : 0.f;
                const float ev = (cq.y & kExtraTapBit) ? kb.edge : 0.f;
                const float2 *e = sm + lu * S + lv;
                float2 r = make_float2(0.f, 0.f);
                for (int j = 0; j < W2; ++j) r = __ffma2_rn(f2(wv[q][j]), e[j + 1], r);
                r = __ffma2_rn(f2(ev), e[0], r);
                a = __ffma2_rn(f2(eu), r, a);
                float2 cs2 = make_float2(0.f, 0.f);
                for (int i = 0; i < W2; ++i) cs2 = __ffma2_rn(f2(wu[q][i]), e[(i + 1) * S], cs2);
                a = __ffma2_rn(f2(ev), cs2, a);
            }
            if (neg) {
                a.x = -a.x;
                a.y = -a.y;
            }
            if (vscale) {
                const float sc = vscale[b0 + q];
                a.x *= sc;
                a.y *= sc;
            }
            out[b0 + q] = a;
        }
    }
}

__host__ __device__ inline size_t degrid_pair_smem_bytes(const GridGeom &g)
{
    return sizeof(float4) * (size_t)g.E * g.stride;
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

constexpr int kGridBatch = 256;  // visibilities per weight batch (= threads per CTA)
constexpr int kRowSkew = 8;      // floats between consecutive groups' weight rows
template <int W2>
constexpr int kBallotRowStride = 2 * W2 + 8;  // floats per row of the ballot gridder
// Floats between consecutive groups' rows in the ballot gridder: the groups of a warp read
// their rows in the same instruction, so group g's rows start 8g (4g when more than four
// groups share a warp) banks later, modulo 32.
template <int W2>
constexpr int ballot_group_skew()
{
    const int want = (32 / W2 <= 4) ? 8 : 4;
    return ((want - (W2 * kBallotRowStride<W2>) % 32) % 32 + 32) % 32;
}

// Row-owner gridding (the default for float). The work item's sorted visibilities are split
// into NG = 8 warps x G contiguous ranges, one per group of 2w lanes (G = 32/(2w) groups per
// warp). Each batch gathers the next SHARE visibilities of every range (SHARE * NG <= 256, one
// per thread), evaluates their weights into 80-byte shared rows [wv | wu | x, key], and the
// groups consume them: lane i of a group owns row i of the 2w x 2w window and accumulates its
// 2w taps in registers -- across batches -- while its range stays in one cell. So a dense
// cell costs one flush per range, not one per batch. Every warp flushes into its own copy of
// the extended tile with plain load-add-store, its groups taking turns (warp vote, then one
// group at a time between __syncwarp), so no two lanes update a cell at once; the copies are
// summed once per work item before the global flush.
// SHARED = true: one extended tile for the whole CTA, flushed by every group at once with
// shared-memory float atomics (collisions only where two groups' windows overlap), which
// removes the turn-taking and the final summation of copies and needs an eighth of the tile
// memory.
// MASKED = true (warp-private tiles): each group reads its SHARE keys once per batch and marks
// the steps where its cell changes in a bit mask; one warp OR of the masks gives the steps at
// which any group flushes, so the fully unrolled step loop is plain loads and FMAs except at
// those steps, and a flush takes turns only among the groups that need one (ballot), not all
// G groups.
// One work item by a CTA of kGridBatch threads; smraw: grid_rows_smem_bytes<W2, SHARED>(g).
// ATOMIC = true (with MASKED): a group that needs a flush adds its rows with shared-memory
// float atomics at once, without waiting for its turn, into the warp's copy (or the CTA's one
// tile when SHARED).
// KAHAN = true (with MASKED): the register sums of a run are compensated (Kahan): each tap
// keeps the rounding error of its running sum and the flush adds the corrected sum.
template <int W2, bool SHARED = false, bool MASKED = false, bool ATOMIC = false,
          bool KAHAN = false>
__device__ __forceinline__ void grid_rows_item(const float2 *__restrict__ vis,
                                               const uint2 *__restrict__ coords,
                                               float2 *__restrict__ grid, const WorkItem &it,
                                               const KBPoly &kb, const GridGeom &g,
                                               unsigned char *smraw)
{
    constexpr int STR = 2 * W2 + 4;                  // floats per row (16-byte multiple)
    constexpr int G = 32 / W2;                        // visibility groups per warp
    constexpr int NW = kGridBatch / 32;
    constexpr int NG = NW * G;                        // groups per CTA
    constexpr int SHARE = kGridBatch / NG;            // visibilities per group and batch
    static_assert((STR % 4) == 0, "rows must stay 16-byte aligned");
    constexpr int NT = SHARED ? 1 : NW;               // tile copies
    const int E = g.E, S = g.stride;
    float2 *tiles = reinterpret_cast<float2 *>(smraw);  // NT x (E x S)
    const size_t tile_bytes = ((sizeof(float2) * (size_t)NT * E * S) + 15) & ~size_t(15);
    // NG*SHARE rows of STR floats; group g's SHARE rows start kRowSkew*g floats later, so the
    // G groups of a warp, which read their rows in the same instruction, hit different banks
    // (SHARE*STR is a multiple of 32 words for W2 = 6 and 8)
    float *rows = reinterpret_cast<float *>(smraw + tile_bytes);
    for (int e = threadIdx.x; e < NT * E * S; e += blockDim.x) tiles[e] = make_float2(0.f, 0.f);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2 *mytile = tiles + (SHARED ? 0 : warp) * E * S;
    const int grp = lane / W2, ri = lane - grp * W2;
    const bool lane_on = grp < G;
    const int gid = warp * G + (lane_on ? grp : 0);   // this lane's range
    const int L = (it.count + NG - 1) / NG;           // range length
    const int rbeg = min(it.count, gid * L), rend = min(it.count, rbeg + L);
    // producer role: thread t fills row t for range t / SHARE
    const int pg = threadIdx.x / SHARE, pj = threadIdx.x - pg * SHARE;
    const int pbeg = min(it.count, pg * L), pend = min(it.count, pbeg + L);

    float2 acc[W2];
    float2 cmp[KAHAN ? W2 : 1];  // Kahan: rounding error of each running sum (acc - cmp is exact)
#pragma unroll
    for (int j = 0; j < W2; ++j) acc[j] = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < (KAHAN ? W2 : 1); ++j) cmp[j] = make_float2(0.f, 0.f);
    int cur = -1;
    const int nbatch = (L + SHARE - 1) / SHARE;
    // add the accumulated taps of cell `cur` to this lane's window row of the warp's tile
    auto flush_rows = [&]() {
        float2 *p = mytile + ((cur >> 6) + 1 + ri) * S + (cur & 63) + 1;
#pragma unroll
        for (int j = 0; j < W2; ++j) {
            if constexpr (KAHAN) {
                p[j] = __fadd2_rn(p[j], __fadd2_rn(acc[j], make_float2(-cmp[j].x, -cmp[j].y)));
                cmp[j] = make_float2(0.f, 0.f);
            } else {
                p[j] = __fadd2_rn(p[j], acc[j]);
            }
            acc[j] = make_float2(0.f, 0.f);
        }
    };
    auto flush_rows_atomic = [&]() {
        float2 *p = mytile + ((cur >> 6) + 1 + ri) * S + (cur & 63) + 1;
#pragma unroll
        for (int j = 0; j < W2; ++j) {
            atomicAdd(&p[j].x, acc[j].x);
            atomicAdd(&p[j].y, acc[j].y);
            acc[j] = make_float2(0.f, 0.f);
        }
    };
    // accumulate one visibility row [wv | wu | x, key] into this lane's window row
    auto consume = [&](const float *row) {
        const float4 xk = reinterpret_cast<const float4 *>(row + 2 * W2)[0];
        const float wui = row[W2 + ri];
        const float2 t = make_float2(wui * xk.x, wui * xk.y);
        float wv[W2];
#pragma unroll
        for (int q = 0; q < W2 / 4; ++q) {
            const float4 v4 = reinterpret_cast<const float4 *>(row)[q];
            wv[4 * q] = v4.x;
            wv[4 * q + 1] = v4.y;
            wv[4 * q + 2] = v4.z;
            wv[4 * q + 3] = v4.w;
        }
#pragma unroll
        for (int j = (W2 / 4) * 4; j < W2; ++j) wv[j] = row[j];
        if constexpr (KAHAN) {
#pragma unroll
            for (int j = 0; j < W2; ++j) {
                const float2 y = __ffma2_rn(f2(wv[j]), t, make_float2(-cmp[j].x, -cmp[j].y));
                const float2 sum = __fadd2_rn(acc[j], y);
                cmp[j] = __fadd2_rn(__fadd2_rn(sum, make_float2(-acc[j].x, -acc[j].y)),
                                    make_float2(-y.x, -y.y));
                acc[j] = sum;
            }
        } else {
#pragma unroll
            for (int j = 0; j < W2; ++j) acc[j] = __ffma2_rn(f2(wv[j]), t, acc[j]);
        }
    };
    // the producer's inputs for batch b + 1 are loaded while batch b is evaluated and consumed
    uint2 cpre = make_uint2(0u, 0u);
    float2 xpre = make_float2(0.f, 0.f);
    auto prefetch = [&](int bb) {
        const int kv = pbeg + bb * SHARE + pj;
        if (bb < nbatch && pg < NG && kv < pend) {
            cpre = coords[it.begin + kv];
            xpre = vis[it.begin + kv];
        }
    };
    prefetch(0);
    for (int b = 0; b <= nbatch; ++b) {
        __syncthreads();  // tiles zeroed / previous batch consumed
        if (b < nbatch && pg < NG) {
            const int kv = pbeg + b * SHARE + pj;
            if (kv < pend) {
                const uint2 c = cpre;
                float2 x = xpre;
                prefetch(b + 1);
                const int lu = cell_of(c.x), lv = cell_of(c.y);
                float wu[W2], wv[W2];
                kb_weights<W2>(kb, c.x, wu);
                kb_weights<W2>(kb, c.y, wv);
                const float h = tap_parity(it, g, lu, lv) ? -0.5f : 0.5f;
                x = make_float2(h * x.x, h * x.y);
                float *row = rows + threadIdx.x * STR + pg * kRowSkew;
                float4 *row4 = reinterpret_cast<float4 *>(row);
#pragma unroll
                for (int q = 0; q < W2 / 4; ++q)
                    row4[q] = make_float4(wv[4 * q], wv[4 * q + 1], wv[4 * q + 2], wv[4 * q + 3]);
#pragma unroll
                for (int j = (W2 / 4) * 4; j < W2; ++j) row[j] = wv[j];
#pragma unroll
                for (int i = 0; i < W2; ++i) row[W2 + i] = wu[i];
                reinterpret_cast<float4 *>(row + 2 * W2)[0] =
                    make_float4(x.x, x.y, __int_as_float((lu << 6) | lv), 0.f);
                if ((c.x | c.y) & kExtraTapBit)  // rare: straight into a tile, atomically
                    grid_extra_taps<W2, float>(tiles + (SHARED ? 0 : warp) * E * S, S, lu, lv,
                                               c, wu, wv, kb.edge, x);
            }
        }
        __syncthreads();
        // consume this batch's rows of my range; after the last batch flush what is left
        const int kfirst = rbeg + b * SHARE;
        if constexpr (MASKED && (ATOMIC || !SHARED)) {
            const int nval = (lane_on && b < nbatch) ? max(0, min(SHARE, rend - kfirst)) : 0;
            const float *rowg = rows + gid * (SHARE * STR + kRowSkew);
            int keys[SHARE];
            unsigned bm = 0;  // bit s: flush `cur` before consuming step s
            int prev = cur;
#pragma unroll
            for (int st = 0; st < SHARE; ++st) {
                keys[st] = (st < nval) ? __float_as_int(rowg[st * STR + 2 * W2 + 2]) : prev;
                if (st < nval && prev >= 0 && keys[st] != prev) bm |= 1u << st;
                prev = keys[st];
            }
            if (b == nbatch && lane_on && cur >= 0) bm = 1u;  // what is left after the last batch
            const unsigned wm = __reduce_or_sync(0xffffffffu, bm);
#pragma unroll
            for (int st = 0; st < SHARE; ++st) {
                if constexpr (ATOMIC) {
                    if ((bm >> st) & 1u) flush_rows_atomic();
                } else if (wm & (1u << st)) {  // warp-uniform
                    const bool need = (bm >> st) & 1u;
                    unsigned gm = __ballot_sync(0xffffffffu, need);
                    while (gm) {  // groups that flush here, one at a time
                        const int g0 = (__ffs(gm) - 1) / W2;
                        if (need && grp == g0) flush_rows();
                        __syncwarp();
                        gm &= ~(((1u << W2) - 1u) << (g0 * W2));
                    }
                }
                if (st < nval) {
                    cur = keys[st];
                    consume(rowg + st * STR);
                }
            }
        } else {
        for (int step = 0; step < SHARE; ++step) {
            const int k = kfirst + step;
            const bool valid = lane_on && b < nbatch && k < rend;
            float4 xk = make_float4(0.f, 0.f, 0.f, 0.f);
            int key = cur;
            const float *row = rows + (gid * SHARE + step) * STR + gid * kRowSkew;
            if (valid) {
                xk = reinterpret_cast<const float4 *>(row + 2 * W2)[0];
                key = __float_as_int(xk.z);
            }
            const bool need = lane_on && cur >= 0 && (b == nbatch || key != cur);
            if constexpr (SHARED) {
                if (need) {
                    float2 *p = mytile + ((cur >> 6) + 1 + ri) * S + (cur & 63) + 1;
#pragma unroll
                    for (int j = 0; j < W2; ++j) {
                        atomicAdd(&p[j].x, acc[j].x);
                        atomicAdd(&p[j].y, acc[j].y);
                        acc[j] = make_float2(0.f, 0.f);
                    }
                    cur = -1;
                }
            } else if (__any_sync(0xffffffffu, need)) {
                for (int hgrp = 0; hgrp < G; ++hgrp) {
                    if (need && grp == hgrp) flush_rows();
                    __syncwarp();
                }
                if (need) cur = -1;
            }
            if (!valid) continue;
            cur = key;
            consume(row);
        }
        }
    }
    __syncthreads();
    if constexpr (!SHARED) {
        for (int e = threadIdx.x; e < E * S; e += blockDim.x) {  // sum the warps' copies
            float2 a = tiles[e];
#pragma unroll
            for (int q = 1; q < NW; ++q) {
                const float2 bq = tiles[q * E * S + e];
                a.x += bq.x;
                a.y += bq.y;
            }
            tiles[e] = a;
        }
        __syncthreads();
    }
    grid_flush_extended<W2, float>(tiles, grid, it, g);
}

// Row-owner gridding with the flush steps found by the producers (the default). Same data
// flow as grid_rows_item<W2, false, true> -- warp-private tiles, producer rows in shared
// memory, lane i of a group of 2w lanes owning window row i -- but each group's rows are
// produced by the group's own lanes (row st by lane g*2w + st; G = 32/(2w) groups per warp, so
// SHARE = 2w rows per group and batch, and the 32 - G*2w lanes left over idle). Each producer
// compares its row's cell with the row before it (a shuffle; the first row with the group's
// last cell of the previous batch), and one warp ballot hands every consumer lane the steps at
// which its group must flush. Rows past the end of a range carry x = 0 and never flush, so the
// consumers run every step unconditionally and read no keys; the cell to flush is read from
// the row before the flush step. Flushes take turns among the groups that flush at the same
// step, as in grid_rows_item.
// The register sums pair taps rather than real and imaginary parts: accr[q] holds the real
// parts of taps 2q and 2q+1, acci[q] their imaginary parts, so a packed FMA takes the two
// taps' v-weights straight from the row (an aligned pair) and the value's real or imaginary
// part, which the producer stores twice, (re, re, im, im): no operand is duplicated per tap.
// smraw: grid_ballot_smem_bytes<W2>(g).
template <int W2>
__device__ __forceinline__ void grid_rows_item_ballot(const float2 *__restrict__ vis,
                                                      const uint2 *__restrict__ coords,
                                                      float2 *__restrict__ grid,
                                                      const WorkItem &it, const KBPoly &kb,
                                                      const GridGeom &g, unsigned char *smraw)
{
    static_assert((W2 % 2) == 0, "taps in pairs");
    constexpr int STR = kBallotRowStride<W2>;  // [wv | wu | re re im im | key, 3 pad]
    constexpr int G = 32 / W2;              // groups per warp
    constexpr int NW = kGridBatch / 32;
    constexpr int NG = NW * G;
    constexpr int SHARE = W2;               // rows per group and batch, one per lane
    static_assert(NG * SHARE <= kGridBatch, "rows fit the batch");
    const int E = g.E, S = g.stride;
    float2 *tiles = reinterpret_cast<float2 *>(smraw);
    const size_t tile_bytes = ((sizeof(float2) * (size_t)NW * E * S) + 15) & ~size_t(15);
    float *rows = reinterpret_cast<float *>(smraw + tile_bytes);
    for (int e = threadIdx.x; e < NW * E * S; e += blockDim.x) tiles[e] = make_float2(0.f, 0.f);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool lane_on = lane < G * W2;
    float2 *mytile = tiles + warp * E * S;
    const int grp = lane_on ? lane / W2 : G - 1;      // consumer: group, window row
    const int ri = lane_on ? lane - grp * W2 : 0;
    const int gid = warp * G + grp;                    // this lane's range (also as producer)
    const int L = (it.count + NG - 1) / NG;
    const int rbeg = min(it.count, gid * L), rend = lane_on ? min(it.count, rbeg + L) : rbeg;
    const int nbatch = (L + SHARE - 1) / SHARE;
    const unsigned gmask = ((1u << W2) - 1u) << (grp * W2);
    constexpr int GSTR = SHARE * STR + ballot_group_skew<W2>();  // floats per group of rows
    const float *rowg = rows + gid * GSTR;  // row st at rowg + st * STR
    float *myrow = rows + gid * GSTR + ri * STR;  // produced by this lane

    float2 accr[W2 / 2], acci[W2 / 2];
#pragma unroll
    for (int q = 0; q < W2 / 2; ++q) {
        accr[q] = make_float2(0.f, 0.f);
        acci[q] = make_float2(0.f, 0.f);
    }
    int plast = -1;  // cell of the group's last valid row so far (-1: none)
    auto flush_to = [&](int cell) {
        float2 *p = mytile + ((cell >> 6) + 1 + ri) * S + (cell & 63) + 1;
#pragma unroll
        for (int q = 0; q < W2 / 2; ++q) {
            float2 a = p[2 * q], b = p[2 * q + 1];
            a.x += accr[q].x;
            a.y += acci[q].x;
            b.x += accr[q].y;
            b.y += acci[q].y;
            p[2 * q] = a;
            p[2 * q + 1] = b;
            accr[q] = make_float2(0.f, 0.f);
            acci[q] = make_float2(0.f, 0.f);
        }
    };
    auto consume = [&](const float *row) {
        const float4 xx = reinterpret_cast<const float4 *>(row + 2 * W2)[0];  // re re im im
        const float wui = row[W2 + ri];
        const float2 w2 = make_float2(wui, wui);
        const float2 tr = __fmul2_rn(w2, make_float2(xx.x, xx.y));
        const float2 ti = __fmul2_rn(w2, make_float2(xx.z, xx.w));
#pragma unroll
        for (int q = 0; q < W2 / 4; ++q) {
            const float4 v4 = reinterpret_cast<const float4 *>(row)[q];
            accr[2 * q] = __ffma2_rn(make_float2(v4.x, v4.y), tr, accr[2 * q]);
            acci[2 * q] = __ffma2_rn(make_float2(v4.x, v4.y), ti, acci[2 * q]);
            accr[2 * q + 1] = __ffma2_rn(make_float2(v4.z, v4.w), tr, accr[2 * q + 1]);
            acci[2 * q + 1] = __ffma2_rn(make_float2(v4.z, v4.w), ti, acci[2 * q + 1]);
        }
        if constexpr ((W2 % 4) != 0) {  // the last pair of taps
            const float2 v2 = reinterpret_cast<const float2 *>(row)[W2 / 2 - 1];
            accr[W2 / 2 - 1] = __ffma2_rn(v2, tr, accr[W2 / 2 - 1]);
            acci[W2 / 2 - 1] = __ffma2_rn(v2, ti, acci[W2 / 2 - 1]);
        }
    };
    uint2 cpre = make_uint2(0u, 0u);
    float2 xpre = make_float2(0.f, 0.f);
    auto prefetch = [&](int bb) {
        const int kv = rbeg + bb * SHARE + ri;
        if (bb < nbatch && kv < rend) {
            cpre = coords[it.begin + kv];
            xpre = vis[it.begin + kv];
        }
    };
    prefetch(0);
    for (int b = 0; b < nbatch; ++b) {
        __syncthreads();  // tiles zeroed / previous batch consumed
        // produce row ri of this group: weights, value, cell; x = 0 past the range's end
        const int kv = rbeg + b * SHARE + ri;
        const bool valid = kv < rend;
        int key = -1;
        {
            const uint2 c = cpre;
            float2 x = xpre;
            prefetch(b + 1);
            const int lu = cell_of(c.x), lv = cell_of(c.y);
            float wu[W2], wv[W2];
            kb_weights<W2>(kb, c.x, wu);
            kb_weights<W2>(kb, c.y, wv);
            const float h = valid ? (tap_parity(it, g, lu, lv) ? -0.5f : 0.5f) : 0.f;
            x = make_float2(h * x.x, h * x.y);
            if (lane_on) {
                float4 *row4 = reinterpret_cast<float4 *>(myrow);
#pragma unroll
                for (int q = 0; q < W2 / 4; ++q)
                    row4[q] = make_float4(wv[4 * q], wv[4 * q + 1], wv[4 * q + 2], wv[4 * q + 3]);
#pragma unroll
                for (int j = (W2 / 4) * 4; j < W2; ++j) myrow[j] = wv[j];
#pragma unroll
                for (int i = 0; i < W2; ++i) myrow[W2 + i] = wu[i];
                key = valid ? ((lu << 6) | lv) : -1;
                reinterpret_cast<float4 *>(myrow + 2 * W2)[0] = make_float4(x.x, x.x, x.y, x.y);
                myrow[2 * W2 + 4] = __int_as_float(key);
            }
            if (valid && ((c.x | c.y) & kExtraTapBit))  // rare: straight into the warp's tile
                grid_extra_taps<W2, float>(mytile, S, lu, lv, c, wu, wv, kb.edge, x);
        }
        // flush steps: row st flushes the group's accumulated cell when its cell differs from
        // the cell of the row before it (valid rows are a prefix of each group's rows)
        const int up = __shfl_up_sync(0xffffffffu, key, 1);
        const int cell0 = plast;  // the cell a flush at step 0 leaves
        const int prev = (ri == 0) ? plast : up;
        const unsigned flags = __ballot_sync(0xffffffffu, valid && prev >= 0 && key != prev);
        const unsigned nvalid = __popc(__ballot_sync(0xffffffffu, valid) & gmask);
        const int lastkey = __shfl_sync(0xffffffffu, key, grp * W2 + max((int)nvalid, 1) - 1);
        if (nvalid) plast = lastkey;
        unsigned wm = 0;  // steps at which any group of the warp flushes
#pragma unroll
        for (int q = 0; q < G; ++q) wm |= flags >> (q * W2);
        wm &= (1u << W2) - 1u;
        const unsigned bm = lane_on ? (flags >> (grp * W2)) & ((1u << W2) - 1u) : 0u;
        __syncthreads();
#pragma unroll
        for (int st = 0; st < SHARE; ++st) {
            if (wm & (1u << st)) {  // warp-uniform
                const bool need = (bm >> st) & 1u;
                unsigned gm = __ballot_sync(0xffffffffu, need);
                while (gm) {  // groups that flush here, one at a time
                    const int g0 = (__ffs(gm) - 1) / W2;
                    if (need && grp == g0)  // the cell being left: the row before's
                        flush_to(st > 0 ? __float_as_int(rowg[(st - 1) * STR + 2 * W2 + 4])
                                        : cell0);
                    __syncwarp();
                    gm &= ~(((1u << W2) - 1u) << (g0 * W2));
                }
            }
            if (lane_on) consume(rowg + st * STR);
        }
    }
    // what is left: every group with a non-empty range flushes its last cell, in turn
#pragma unroll
    for (int g0 = 0; g0 < G; ++g0) {
        if (lane_on && grp == g0 && plast >= 0) flush_to(plast);
        __syncwarp();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < E * S; e += blockDim.x) {  // sum the warps' copies
        float2 a = tiles[e];
#pragma unroll
        for (int q = 1; q < NW; ++q) a = __fadd2_rn(a, tiles[q * E * S + e]);
        tiles[e] = a;
    }
    __syncthreads();
    grid_flush_extended<W2, float>(tiles, grid, it, g);
}

// Tile stride of the warp-local gridder, in float2: at least E + 1 (a flush of a window at an
// odd column reads and writes one cell past it) and 2 modulo 4, so that a row's 16-byte
// alignment depends on its column alone and the 8 rows a group flushes at once, 2S = 4 (mod 8)
// words apart, fall in distinct 16-byte bank quads.
__host__ __device__ inline int grid_local_stride(int E)
{
    const int s = E + 1;
    return s + ((2 - (s & 3)) & 3);
}
template <int W2>
constexpr int kLocalRowStride = 2 * W2 + 4;  // [wv | wu | re, im, key, pad]
template <int W2>
constexpr int local_group_skew()
{
    const int want = (32 / W2 <= 4) ? 8 : 4;
    return ((want - (W2 * kLocalRowStride<W2>) % 32) % 32 + 32) % 32;
}

// Row-owner gridding with warp-local synchronisation (the default for float). The data flow
// of grid_rows_item_ballot -- lane i of a group of 2w lanes owns window row i and sums its 2w
// taps in registers while the group's sorted visibilities stay in one cell; the group's rows
// [wv | wu | x, key] are produced by the group's own lanes; the flush steps come from one warp
// ballot per batch -- with these differences:
// * producers and consumers of a row are lanes of one warp, so a batch needs two __syncwarp
//   and no CTA barrier: warps run their batches independently and wait for each other only
//   at the end of the work item, when the warp-private tiles are summed;
// * each tap's sum is one (re, im) register pair, updated by a packed FMA with the scalar
//   v-weight, and added to the tile by packed adds;
// * the tile stride makes a flushed window row 16-byte aligned or one cell off it, so a flush
//   is w (aligned) or w + 1 (odd column) 16-byte read-modify-writes per lane, not 2w 8-byte
//   ones.
// Flushes take turns among the groups of a warp that flush at the same step, as before.
// smraw: grid_local_smem_bytes<W2>(g).
template <int W2, int NW = 8>
__device__ __forceinline__ void grid_rows_item_local(const float2 *__restrict__ vis,
                                                     const uint2 *__restrict__ coords,
                                                     float2 *__restrict__ grid,
                                                     const WorkItem &it, const KBPoly &kb,
                                                     const GridGeom &gin, unsigned char *smraw)
{
    static_assert((W2 % 2) == 0, "taps in pairs");
    constexpr int STR = kLocalRowStride<W2>;
    constexpr int G = 32 / W2;
    constexpr int NG = NW * G;
    constexpr int SHARE = W2;
    static_assert((STR % 4) == 0, "rows stay 16-byte aligned");
    GridGeom g = gin;
    g.stride = grid_local_stride(g.E);
    const int E = g.E, S = g.stride;
    float2 *tiles = reinterpret_cast<float2 *>(smraw);
    const size_t tile_bytes = ((sizeof(float2) * (size_t)NW * E * S) + 15) & ~size_t(15);
    float *rows = reinterpret_cast<float *>(smraw + tile_bytes);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2 *mytile = tiles + warp * E * S;
    {
        float4 *t4 = reinterpret_cast<float4 *>(mytile);  // E*S even, base 16-byte aligned
        for (int e = lane; e < (E * S) / 2; e += 32) t4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const bool lane_on = lane < G * W2;
    const int grp = lane_on ? lane / W2 : G - 1;
    const int ri = lane_on ? lane - grp * W2 : 0;
    const int gid = warp * G + grp;
    const int L = (it.count + NG - 1) / NG;
    const int rbeg = min(it.count, gid * L), rend = lane_on ? min(it.count, rbeg + L) : rbeg;
    const int nbatch = (L + SHARE - 1) / SHARE;
    const unsigned gmask = ((1u << W2) - 1u) << (grp * W2);
    constexpr int GSTR = SHARE * STR + local_group_skew<W2>();
    const float *rowg = rows + gid * GSTR;
    float *myrow = rows + gid * GSTR + ri * STR;

    float2 acc[W2];
#pragma unroll
    for (int j = 0; j < W2; ++j) acc[j] = make_float2(0.f, 0.f);
    int plast = -1;
    auto flush_to = [&](int cell) {
        const int lv = cell & 63;
        float2 *p = mytile + ((cell >> 6) + 1 + ri) * S + lv + 1;
        if (lv & 1) {  // lv + 1 even: the row segment starts on a 16-byte boundary
            float4 *p4 = reinterpret_cast<float4 *>(p);
#pragma unroll
            for (int q = 0; q < W2 / 2; ++q) {
                float4 f = p4[q];
                const float2 a = __fadd2_rn(make_float2(f.x, f.y), acc[2 * q]);
                const float2 b = __fadd2_rn(make_float2(f.z, f.w), acc[2 * q + 1]);
                p4[q] = make_float4(a.x, a.y, b.x, b.y);
            }
        } else {  // one cell off: w + 1 pairs starting at the cell before
            float4 *p4 = reinterpret_cast<float4 *>(p - 1);
            {
                const float4 f = p4[0];
                const float2 b = __fadd2_rn(make_float2(f.z, f.w), acc[0]);
                p4[0] = make_float4(f.x, f.y, b.x, b.y);
            }
#pragma unroll
            for (int q = 1; q < W2 / 2; ++q) {
                const float4 f = p4[q];
                const float2 a = __fadd2_rn(make_float2(f.x, f.y), acc[2 * q - 1]);
                const float2 b = __fadd2_rn(make_float2(f.z, f.w), acc[2 * q]);
                p4[q] = make_float4(a.x, a.y, b.x, b.y);
            }
            {
                const float4 f = p4[W2 / 2];
                const float2 a = __fadd2_rn(make_float2(f.x, f.y), acc[W2 - 1]);
                p4[W2 / 2] = make_float4(a.x, a.y, f.z, f.w);
            }
        }
#pragma unroll
        for (int j = 0; j < W2; ++j) acc[j] = make_float2(0.f, 0.f);
    };
    // one row's values: value (re, im) and cell, this lane's u-weight, the v-weights
    struct RowVals {
        float4 xk;
        float wui;
        float wv[W2];
    };
    auto load_row = [&](const float *row, RowVals &r) {
        r.xk = reinterpret_cast<const float4 *>(row + 2 * W2)[0];  // re im key pad
        r.wui = row[W2 + ri];
#pragma unroll
        for (int q = 0; q < W2 / 4; ++q) {
            const float4 v4 = reinterpret_cast<const float4 *>(row)[q];
            r.wv[4 * q] = v4.x;
            r.wv[4 * q + 1] = v4.y;
            r.wv[4 * q + 2] = v4.z;
            r.wv[4 * q + 3] = v4.w;
        }
        if constexpr ((W2 % 4) != 0) {
            const float2 v2 = reinterpret_cast<const float2 *>(row)[W2 / 2 - 1];
            r.wv[W2 - 2] = v2.x;
            r.wv[W2 - 1] = v2.y;
        }
    };
    auto consume = [&](const RowVals &r) {
        const float2 t = __fmul2_rn(make_float2(r.wui, r.wui), make_float2(r.xk.x, r.xk.y));
#pragma unroll
        for (int j = 0; j < W2; ++j) acc[j] = __ffma2_rn(f2(r.wv[j]), t, acc[j]);
    };
    uint2 cpre = make_uint2(0u, 0u);
    float2 xpre = make_float2(0.f, 0.f);
    auto prefetch = [&](int bb) {
        const int kv = rbeg + bb * SHARE + ri;
        if (bb < nbatch && kv < rend) {
            cpre = coords[it.begin + kv];
            xpre = vis[it.begin + kv];
        }
    };
    prefetch(0);
    for (int b = 0; b < nbatch; ++b) {
        __syncwarp();  // tile zeroed / the warp's previous batch consumed
        const int kv = rbeg + b * SHARE + ri;
        const bool valid = kv < rend;
        int key = -1;
        {
            const uint2 c = cpre;
            float2 x = xpre;
            prefetch(b + 1);
            const int lu = cell_of(c.x), lv = cell_of(c.y);
            float wt[2 * W2];  // [wv | wu], stored as 16-byte pieces
            float wu[W2], wv[W2];
            kb_weights<W2>(kb, c.x, wu);
            kb_weights<W2>(kb, c.y, wv);
#pragma unroll
            for (int j = 0; j < W2; ++j) {
                wt[j] = wv[j];
                wt[W2 + j] = wu[j];
            }
            const float h = valid ? (tap_parity(it, g, lu, lv) ? -0.5f : 0.5f) : 0.f;
            x = make_float2(h * x.x, h * x.y);
            if (lane_on) {
                float4 *row4 = reinterpret_cast<float4 *>(myrow);
#pragma unroll
                for (int q = 0; q < W2 / 2; ++q)
                    row4[q] = make_float4(wt[4 * q], wt[4 * q + 1], wt[4 * q + 2], wt[4 * q + 3]);
                key = valid ? ((lu << 6) | lv) : -1;
                row4[W2 / 2] = make_float4(x.x, x.y, __int_as_float(key), 0.f);
            }
            if (valid && ((c.x | c.y) & kExtraTapBit))
                grid_extra_taps<W2, float>(mytile, S, lu, lv, c, wu, wv, kb.edge, x);
        }
        const int up = __shfl_up_sync(0xffffffffu, key, 1);
        const int cell0 = plast;
        const int prev = (ri == 0) ? plast : up;
        const unsigned flags = __ballot_sync(0xffffffffu, valid && prev >= 0 && key != prev);
        const unsigned nvalid = __popc(__ballot_sync(0xffffffffu, valid) & gmask);
        const int lastkey = __shfl_sync(0xffffffffu, key, grp * W2 + max((int)nvalid, 1) - 1);
        if (nvalid) plast = lastkey;
        unsigned wm = 0;
#pragma unroll
        for (int q = 0; q < G; ++q) wm |= flags >> (q * W2);
        wm &= (1u << W2) - 1u;
        const unsigned bm = lane_on ? (flags >> (grp * W2)) & ((1u << W2) - 1u) : 0u;
        __syncwarp();  // the warp's rows are written
        // rows are read one step ahead of their use (a flush writes only the tile)
        RowVals cur;
        if (lane_on) load_row(rowg, cur);
        int lastcell = cell0;  // the cell of the row consumed last
#pragma unroll
        for (int st = 0; st < SHARE; ++st) {
            RowVals nxt;
            if (st + 1 < SHARE && lane_on) load_row(rowg + (st + 1) * STR, nxt);
            if (wm & (1u << st)) {  // warp-uniform
                const bool need = (bm >> st) & 1u;
                unsigned gm = __ballot_sync(0xffffffffu, need);
                while (gm) {  // groups that flush here, one at a time
                    const int g0 = (__ffs(gm) - 1) / W2;
                    if (need && grp == g0) flush_to(lastcell);
                    __syncwarp();
                    gm &= ~(((1u << W2) - 1u) << (g0 * W2));
                }
            }
            if (lane_on) {
                consume(cur);
                lastcell = __float_as_int(cur.xk.z);
            }
            if (st + 1 < SHARE) cur = nxt;
        }
    }
#pragma unroll
    for (int g0 = 0; g0 < G; ++g0) {
        if (lane_on && grp == g0 && plast >= 0) flush_to(plast);
        __syncwarp();
    }
    __syncthreads();
    {
        float4 *t4 = reinterpret_cast<float4 *>(tiles);
        const int n4 = (E * S) / 2;
        for (int e = threadIdx.x; e < n4; e += blockDim.x) {  // sum the warps' copies
            float4 a = t4[e];
#pragma unroll
            for (int q = 1; q < NW; ++q) {
                const float4 bq = t4[q * n4 + e];
                a.x += bq.x;
                a.y += bq.y;
                a.z += bq.z;
                a.w += bq.w;
            }
            t4[e] = a;
        }
    }
    __syncthreads();
    grid_flush_extended<W2, float>(tiles, grid, it, g);
}

// Column-pair windows for the warp-local row-owner gridder. The register window of a group
// spans 2w + 1 columns: the cells (lu, 2m) and (lu, 2m + 1) share it, a visibility in the odd
// cell adding its 2w taps one column further right. The producer writes the v-weights into the
// window's 2w + 1 slots at that offset (zero in the other slot), so the consumers run one more
// packed FMA per visibility and flush only when the pair of cells changes: on the 1e7-
// visibility workload 0.050 instead of 0.087 flushes per visibility.
template <int W2>
constexpr int kPairWinPad = ((W2 + 1) + 3) & ~3;  // window slots, padded to 16 bytes
// Floats per row [window | re im key pad | wu], a multiple of 4 with an odd number of 16-byte
// words, so that the 8 rows a group's producers write in one 16-byte store fall in distinct
// bank quads.
template <int W2>
constexpr int pair_row_stride()
{
    const int s = (kPairWinPad<W2> + 4 + W2 + 3) & ~3;
    return ((s / 4) % 2) ? s : s + 4;
}
template <int W2>
constexpr int kPairRowStride = pair_row_stride<W2>();
template <int W2>
constexpr int pair_group_skew()
{
    const int want = (32 / W2 <= 4) ? 8 : 4;
    return ((want - (W2 * kPairRowStride<W2>) % 32) % 32 + 32) % 32;
}

// As grid_rows_item_local, with column-pair windows. smraw: grid_pairs_smem_bytes<W2, NW>(g).
// NARROW: the consumers read a row with 8-byte loads (and the flushed cell from the producers'
// registers) instead of 16-byte loads.
template <int W2, int NW = 8, bool NARROW = false>
__device__ __forceinline__ void grid_rows_item_pairs(const float2 *__restrict__ vis,
                                                     const uint2 *__restrict__ coords,
                                                     float2 *__restrict__ grid,
                                                     const WorkItem &it, const KBPoly &kb,
                                                     const GridGeom &gin, unsigned char *smraw)
{
    static_assert((W2 % 2) == 0, "even kernel width");
    constexpr int WC = W2 + 1;              // window columns
    constexpr int WCP = kPairWinPad<W2>;
    constexpr int STR = kPairRowStride<W2>;
    constexpr int G = 32 / W2;
    constexpr int NG = NW * G;
    constexpr int SHARE = W2;
    GridGeom g = gin;
    g.stride = grid_local_stride(g.E);
    const int E = g.E, S = g.stride;
    float2 *tiles = reinterpret_cast<float2 *>(smraw);
    const size_t tile_bytes = ((sizeof(float2) * (size_t)NW * E * S) + 15) & ~size_t(15);
    float *rows = reinterpret_cast<float *>(smraw + tile_bytes);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float2 *mytile = tiles + warp * E * S;
    {
        float4 *t4 = reinterpret_cast<float4 *>(mytile);
        for (int e = lane; e < (E * S) / 2; e += 32) t4[e] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const bool lane_on = lane < G * W2;
    const int grp = lane_on ? lane / W2 : G - 1;
    const int ri = lane_on ? lane - grp * W2 : 0;
    const int gid = warp * G + grp;
    const int L = (it.count + NG - 1) / NG;
    const int rbeg = min(it.count, gid * L), rend = lane_on ? min(it.count, rbeg + L) : rbeg;
    const int nbatch = (L + SHARE - 1) / SHARE;
    const unsigned gmask = ((1u << W2) - 1u) << (grp * W2);
    constexpr int GSTR = SHARE * STR + pair_group_skew<W2>();
    const float *rowg = rows + gid * GSTR;
    float *myrow = rows + gid * GSTR + ri * STR;

    float2 acc[WC];
#pragma unroll
    for (int j = 0; j < WC; ++j) acc[j] = make_float2(0.f, 0.f);
    int plast = -1;
    // window of key `cell` (row lu, even base column): columns base+1 .. base+WC of the tile
    // row, one float2 past a 16-byte boundary (S even, base + 1 odd)
    auto flush_to = [&](int cell) {
        float4 *p4 = reinterpret_cast<float4 *>(mytile + ((cell >> 6) + 1 + ri) * S + (cell & 63));
        {
            const float4 f = p4[0];
            const float2 b = __fadd2_rn(make_float2(f.z, f.w), acc[0]);
            p4[0] = make_float4(f.x, f.y, b.x, b.y);
        }
#pragma unroll
        for (int q = 1; q <= W2 / 2; ++q) {
            const float4 f = p4[q];
            const float2 a = __fadd2_rn(make_float2(f.x, f.y), acc[2 * q - 1]);
            const float2 b = __fadd2_rn(make_float2(f.z, f.w), acc[2 * q]);
            p4[q] = make_float4(a.x, a.y, b.x, b.y);
        }
#pragma unroll
        for (int j = 0; j < WC; ++j) acc[j] = make_float2(0.f, 0.f);
    };
    struct RowVals {
        float4 xk;
        float wui;
        float wv[WC];
    };
    auto load_row = [&](const float *row, RowVals &r) {
        r.wui = row[WCP + 4 + ri];
        if constexpr (NARROW) {
            const float2 x2 = reinterpret_cast<const float2 *>(row + WCP)[0];  // re im
            r.xk = make_float4(x2.x, x2.y, 0.f, 0.f);
#pragma unroll
            for (int q = 0; q < WC / 2; ++q) {
                const float2 v2 = reinterpret_cast<const float2 *>(row)[q];
                r.wv[2 * q] = v2.x;
                r.wv[2 * q + 1] = v2.y;
            }
            if constexpr ((WC % 2) != 0) r.wv[WC - 1] = row[WC - 1];
        } else {
            r.xk = reinterpret_cast<const float4 *>(row + WCP)[0];  // re im key pad
#pragma unroll
            for (int q = 0; q < WCP / 4; ++q) {
                const float4 v4 = reinterpret_cast<const float4 *>(row)[q];
                if (4 * q < WC) r.wv[4 * q] = v4.x;
                if (4 * q + 1 < WC) r.wv[4 * q + 1] = v4.y;
                if (4 * q + 2 < WC) r.wv[4 * q + 2] = v4.z;
                if (4 * q + 3 < WC) r.wv[4 * q + 3] = v4.w;
            }
        }
    };
    auto consume = [&](const RowVals &r) {
        const float2 t = __fmul2_rn(make_float2(r.wui, r.wui), make_float2(r.xk.x, r.xk.y));
#pragma unroll
        for (int j = 0; j < WC; ++j) acc[j] = __ffma2_rn(f2(r.wv[j]), t, acc[j]);
    };
    uint2 cpre = make_uint2(0u, 0u);
    float2 xpre = make_float2(0.f, 0.f);
    auto prefetch = [&](int bb) {
        const int kv = rbeg + bb * SHARE + ri;
        if (bb < nbatch && kv < rend) {
            cpre = coords[it.begin + kv];
            xpre = vis[it.begin + kv];
        }
    };
    prefetch(0);
    for (int b = 0; b < nbatch; ++b) {
        __syncwarp();
        const int kv = rbeg + b * SHARE + ri;
        const bool valid = kv < rend;
        int key = -1;
        {
            const uint2 c = cpre;
            float2 x = xpre;
            prefetch(b + 1);
            const int lu = cell_of(c.x), lv = cell_of(c.y);
            float wu[W2], wv[W2];
            kb_weights<W2>(kb, c.x, wu);
            kb_weights<W2>(kb, c.y, wv);
            const float h = valid ? (tap_parity(it, g, lu, lv) ? -0.5f : 0.5f) : 0.f;
            x = make_float2(h * x.x, h * x.y);
            if (lane_on) {
                const bool odd = lv & 1;
                float win[WCP];  // the v-weights at the cell's offset in its pair window
#pragma unroll
                for (int m = 0; m < WCP; ++m) {
                    const float e0 = (m < W2) ? wv[m] : 0.f;
                    const float e1 = (m >= 1 && m <= W2) ? wv[m - 1] : 0.f;
                    win[m] = odd ? e1 : e0;
                }
                float4 *row4 = reinterpret_cast<float4 *>(myrow);
#pragma unroll
                for (int q = 0; q < WCP / 4; ++q)
                    row4[q] = make_float4(win[4 * q], win[4 * q + 1], win[4 * q + 2], win[4 * q + 3]);
                key = valid ? ((lu << 6) | (lv & ~1)) : -1;
                row4[WCP / 4] = make_float4(x.x, x.y, __int_as_float(key), 0.f);
                float *wrow = myrow + WCP + 4;  // 16-byte aligned
#pragma unroll
                for (int q = 0; q < W2 / 4; ++q)
                    reinterpret_cast<float4 *>(wrow)[q] =
                        make_float4(wu[4 * q], wu[4 * q + 1], wu[4 * q + 2], wu[4 * q + 3]);
                if constexpr ((W2 % 4) != 0)
                    reinterpret_cast<float2 *>(wrow)[W2 / 2 - 1] = make_float2(wu[W2 - 2], wu[W2 - 1]);
            }
            if (valid && ((c.x | c.y) & kExtraTapBit))
                grid_extra_taps<W2, float>(mytile, S, lu, lv, c, wu, wv, kb.edge, x);
        }
        const int up = __shfl_up_sync(0xffffffffu, key, 1);
        const int cell0 = plast;
        const int prev = (ri == 0) ? plast : up;
        const unsigned flags = __ballot_sync(0xffffffffu, valid && prev >= 0 && key != prev);
        const unsigned nvalid = __popc(__ballot_sync(0xffffffffu, valid) & gmask);
        const int lastkey = __shfl_sync(0xffffffffu, key, grp * W2 + max((int)nvalid, 1) - 1);
        if (nvalid) plast = lastkey;
        unsigned wm = 0;
#pragma unroll
        for (int q = 0; q < G; ++q) wm |= flags >> (q * W2);
        wm &= (1u << W2) - 1u;
        const unsigned bm = lane_on ? (flags >> (grp * W2)) & ((1u << W2) - 1u) : 0u;
        __syncwarp();
        RowVals cur;
        if (lane_on) load_row(rowg, cur);
        int lastcell = cell0;
#pragma unroll
        for (int st = 0; st < SHARE; ++st) {
            RowVals nxt;
            if (st + 1 < SHARE && lane_on) load_row(rowg + (st + 1) * STR, nxt);
            if (wm & (1u << st)) {
                const bool need = (bm >> st) & 1u;
                int fcell = lastcell;  // the cell of the group's row before this step
                if constexpr (NARROW)
                    fcell = (st > 0) ? __shfl_sync(0xffffffffu, key, grp * W2 + st - 1) : cell0;
                unsigned gm = __ballot_sync(0xffffffffu, need);
                while (gm) {
                    const int g0 = (__ffs(gm) - 1) / W2;
                    if (need && grp == g0) flush_to(fcell);
                    __syncwarp();
                    gm &= ~(((1u << W2) - 1u) << (g0 * W2));
                }
            }
            if (lane_on) {
                consume(cur);
                if constexpr (!NARROW) lastcell = __float_as_int(cur.xk.z);
            }
            if (st + 1 < SHARE) cur = nxt;
        }
    }
#pragma unroll
    for (int g0 = 0; g0 < G; ++g0) {
        if (lane_on && grp == g0 && plast >= 0) flush_to(plast);
        __syncwarp();
    }
    __syncthreads();
    {
        float4 *t4 = reinterpret_cast<float4 *>(tiles);
        const int n4 = (E * S) / 2;
        for (int e = threadIdx.x; e < n4; e += blockDim.x) {
            float4 a = t4[e];
#pragma unroll
            for (int q = 1; q < NW; ++q) {
                const float4 bq = t4[q * n4 + e];
                a.x += bq.x;
                a.y += bq.y;
                a.z += bq.z;
                a.w += bq.w;
            }
            t4[e] = a;
        }
    }
    __syncthreads();
    grid_flush_extended<W2, float>(tiles, grid, it, g);
}

template <int W2, int NW = 8>
__host__ __device__ inline size_t grid_pairs_smem_bytes(const GridGeom &g)
{
    const size_t tile_bytes =
        ((sizeof(float2) * NW * g.E * grid_local_stride(g.E)) + 15) & ~size_t(15);
    const size_t ngroups = (size_t)NW * (32 / W2);
    return tile_bytes +
           sizeof(float) * (ngroups * ((size_t)W2 * kPairRowStride<W2> + pair_group_skew<W2>()));
}

template <int W2, int NW = 8>
__host__ __device__ inline size_t grid_local_smem_bytes(const GridGeom &g)
{
    const size_t tile_bytes =
        ((sizeof(float2) * NW * g.E * grid_local_stride(g.E)) + 15) & ~size_t(15);
    const size_t ngroups = (size_t)NW * (32 / W2);
    return tile_bytes +
           sizeof(float) * (ngroups * ((size_t)W2 * kLocalRowStride<W2> + local_group_skew<W2>()));
}

template <int W2>
__host__ __device__ inline size_t grid_ballot_smem_bytes(const GridGeom &g)
{
    const size_t tile_bytes =
        ((sizeof(float2) * (kGridBatch / 32) * g.E * g.stride) + 15) & ~size_t(15);
    const size_t ngroups = (kGridBatch / 32) * (32 / W2);
    return tile_bytes +
           sizeof(float) * (ngroups * ((size_t)W2 * kBallotRowStride<W2> + ballot_group_skew<W2>()));
}

template <int W2, bool SHARED = false>
__host__ __device__ inline size_t grid_rows_smem_bytes(const GridGeom &g)
{
    const size_t ntile = SHARED ? 1 : kGridBatch / 32;
    const size_t tile_bytes = ((sizeof(float2) * ntile * g.E * g.stride) + 15) & ~size_t(15);
    const size_t ngroups = (kGridBatch / 32) * (32 / W2);
    return tile_bytes + sizeof(float) * ((size_t)kGridBatch * (2 * W2 + 4) + ngroups * kRowSkew);
}

template <typename R>
__host__ __device__ inline size_t degrid_smem_bytes(const GridGeom &g)
{
    return sizeof(typename Prec<R>::C) * (size_t)g.E * g.stride;
}

}  // namespace lentils
