// Shared definitions of the lentils_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <utility>

#include "lentils_gb300.h"

namespace lentils {

// Constants as the reference defines them (lentils/backend/common.h:8-11); the phase uses
// the truncated 2*pi so that phases match the reference's to the last bit of FP64.
constexpr double kArcsecToRad = 4.8481368111e-6;
constexpr double kTwoPiTrunc = 6.28318530718;

// Kaiser-Bessel weights are evaluated as per-tap polynomials in t = 2*frac - 1.
constexpr int kMaxW = 8;            // largest supported half-width
constexpr int kMaxTaps = 2 * kMaxW;  // 2w taps per axis (plus a rare edge tap)
constexpr int kPolyCoef = 10;        // degree-9 polynomials (FP32 round-off for 1 <= w <= 8)
// Plan coordinate word, per axis:
//   bits  0..23  fraction of the cell (fixed point, 2^-24 cells)
//   bits 24..29  cell within the tile (tiles up to 64 cells)
//   bit  30      the reference includes the extra tap floor - w (argument +w)
//   bit  31      the reference excludes the top tap floor + w (argument below -w)
// The two flags are decided in FP64 exactly as kb_g tests |arg| <= w (nufft.c:12), so the tap
// set matches the reference even when the fixed-point rounding lands on a cell boundary.
constexpr int kFracBits = 24;
constexpr uint32_t kFracMask = (1u << kFracBits) - 1u;
constexpr uint32_t kCellMask = 63u;
constexpr uint32_t kExtraTapBit = 1u << 30;
constexpr uint32_t kTopOffBit = 1u << 31;

// ---------------------------------------------------------------------------------------
// Error state (per host thread)
// ---------------------------------------------------------------------------------------
int set_error(int code, const char *fmt, ...);
int clear_error();
int cuda_status(cudaError_t e, const char *what);

#define LENTILS_CUDA_TRY(expr)                                                    \
    do {                                                                          \
        cudaError_t _e = (expr);                                                  \
        if (_e != cudaSuccess) return ::lentils::cuda_status(_e, #expr);          \
    } while (0)

#define LENTILS_CHECK_LAUNCH(what)                                                \
    do {                                                                          \
        cudaError_t _e = cudaGetLastError();                                      \
        if (_e != cudaSuccess) return ::lentils::cuda_status(_e, what);           \
    } while (0)

// ---------------------------------------------------------------------------------------
// Kaiser-Bessel polynomial table, passed to kernels by value.
// cp[k][p] = (c_{2p,k}, c_{2p+1,k}): coefficient k of taps 2p and 2p+1, highest degree
// first, with the tap's checkerboard sign (-1)^i and the per-axis 1/(2w) normalisation
// folded in. Tap i (0 <= i < 2w) of a visibility with fractional offset f in [0,1) sits at
// kernel argument f + w - 1 - i.
// ---------------------------------------------------------------------------------------
//
// Symmetry: the profile is even, so tap 2w-1-i is the reflection of tap i,
// P_{2w-1-i}(t) = -P_i(-t). The FP32 table keeps only taps i < w, split into even and odd
// parts in t^2 (P_i(t) = E_i(t^2) + t O_i(t^2)), so one evaluation of E_i and O_i gives both
// taps i and 2w-1-i. ce/co[k][p] pair taps (2p, 2p+1), highest power of t^2 first.
constexpr int kHalfCoef = kPolyCoef / 2;  // 5 even + 5 odd coefficients (degree 9)
struct KBPoly {
    float2 ce[kHalfCoef][kMaxW / 2];
    float2 co[kHalfCoef][kMaxW / 2];
    float edge;  // weight of the extra tap at argument +w (only when f == 0): -1/(2w)
};

// The same table in FP64 (for the double-precision operator used by the refinement residual),
// in the even/odd form of the FP32 table: for tap i < w, P_i(t) = E_i(t^2) + t O_i(t^2) with
// ce[k][i] / co[k][i] the coefficients of E_i / O_i (highest power of t^2 first); tap
// 2w-1-i is -P_i(-t) = t O_i(t^2) - E_i(t^2).
struct KBPoly64 {
    double ce[kHalfCoef][kMaxW];
    double co[kHalfCoef][kMaxW];
    double edge;
};

// Host: fit the table for (w, beta). Returns max abs fit error relative to the peak
// (evaluated in FP64) through *fit_err when non-null. `out64` may be null.
void kb_poly_build(int w, double beta, KBPoly *out, double *fit_err, KBPoly64 *out64 = nullptr);
double host_bessel_i0(double x);

// ---------------------------------------------------------------------------------------
// Canonical grid geometry used by the kernels. The full uv plane is tiled with T x T tiles;
// canonical cell indices a in [-Hu, nu-Hu), b in [-Hv, nv-Hv); tile (tu, tv) covers
// a in [tu*T - Hu, (tu+1)*T - Hu).
// ---------------------------------------------------------------------------------------
struct GridGeom {
    int nu, nv, half_nv;
    int w;       // kernel half-width
    int T;       // tile edge
    int logT;
    int E;       // extended tile edge T + 2w
    int stride;  // shared-memory row stride (float2 units, odd)
    int Hu, Hv;  // nu/2, nv/2
    int ntu, ntv;
};

// Parameters of the binning kernel (plan construction).
struct CanonParams {
    int nu, nv, T, logT, Hu, Hv, ntu, ntv, w;
    int nrows, nch;
    int guard;
    double du, dv, gcx, gcy;
};

struct WorkItem {
    int tu, tv;   // tile coordinates
    int begin;    // first visibility (plan order)
    int count;    // number of visibilities
};

// -- programmatic dependent launch ----------------------------------------------------------
// A kernel launched by pdl_launch may start while the kernel before it in the stream is still
// running. It must call pdl_entry() before it reads anything an earlier kernel writes or writes
// anything an earlier kernel reads: griddepcontrol.wait blocks until the previous kernel has
// completed and its memory is visible (a no-op without the launch attribute), and
// launch_dependents lets the next such kernel start once every CTA of this grid has reached it.
__device__ __forceinline__ void pdl_entry()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class... KArgs, class... Args>
inline cudaError_t pdl_launch(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                              cudaStream_t s, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace lentils

// The opaque plan (device-resident arrays + geometry).
struct lentils_plan {
    lentils_grid_desc desc;
    lentils::GridGeom geom;
    lentils::KBPoly kb;
    lentils::KBPoly64 kb64;
    int device;
    long long nvis;
    int nrows, nchannels;
    int nitems;
    int max_item;
    int heaviest_tile;
    int has_phase;
    int grid_variant;     // work split of the gridding kernel (lentils_plan_set_grid_variant)
    int degrid_variant;   // shared-memory layout of the degridding kernel (0 single, 1 pairs)
    // plan-order arrays
    uint2 *coords;        // fixed-point tile-relative (u, v)
    float2 *coords_res;   // g - q*2^-24 per axis (exact in FP64, stored FP32): FP64 kernels only
    int *perm;            // plan index -> user index (channel*nrows + row)
    int *iperm;           // user index -> plan index (host-buffer forms)
    float2 *phase;        // s * e^{-i phi} per visibility (plan order)
    lentils::WorkItem *items;
    // same-cell chunks (degridding): runs of visibilities in one cell, cut into pieces of at
    // most chunk_k; chunk c covers plan indices [chunk_begin[c], chunk_begin[c + 1]), and work
    // item i covers chunks [item_chunks[i].x, item_chunks[i].y). Null when not built.
    int *chunk_begin;
    int2 *item_chunks;
    int chunk_k;
    long long nchunks;
    long long device_bytes;
    // staging for the host-buffer forms (allocated on first use)
    void *stage_vis64;    // nvis c128
    void *stage_grid64;   // grid c128
    float2 *stage_vis32;  // nvis c64
    float2 *stage_grid32; // grid c64
};
