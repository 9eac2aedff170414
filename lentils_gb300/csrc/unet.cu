// Learned preconditioner for the CG source inversion: a 4-level convolutional U-Net on the
// source grid, trained and evaluated on the GPU with hand-written BF16 tensor-core kernels
// (tcgen05, FP32 accumulation in tensor memory) -- no reference counterpart.
//
// Network (NHWC BF16 activations, channel counts padded to multiples of 8):
//   x0  = [residual, diagonal, 0 x 6]                         H   x W   x 8
//   e1  = relu(conv3x3(x0, 8->32))                            H   x W   x 32
//   e2  = relu(conv3x3(pool2(e1), 32->64))                    H/2 x W/2 x 64
//   e3  = relu(conv3x3(pool2(e2), 64->128))                   H/4 x W/4 x 128
//   b   = relu(conv3x3(pool2(e3), 128->128))                  H/8 x W/8 x 128
//   c3  = relu(conv1x1(up2(b) + e3, 128->64))                 H/4 x W/4 x 64
//   c2  = relu(conv3x3(up2(c3) + e2, 64->32))                 H/2 x W/2 x 32
//   c1  = relu(conv3x3(up2(c2) + e1, 32->32))                 H   x W   x 32
//   out = conv1x1(c1, 32->1)                                  H   x W   (FP32)
// (276k parameters; pool2 = 2x2 average, up2 = nearest-neighbour.)
//
// Every convolution is an implicit GEMM on the generic tcgen05 kernel (tc_gemm.cuh):
//   forward        D[pixel][co] = sum_{tap,ci} X[pixel + off(tap)][ci] * W[co][tap][ci]
//   data gradient  dX[pixel][ci] = sum_{tap,co} dY'[pixel - off(tap)][co] * W[co][tap][ci]
//   weight grad.   dW[co][tap][ci] = sum_pixel dY'[pixel][co] * X[pixel + off(tap)][ci]
// with dY' the output gradient masked by the ReLU (Y > 0); im2col is gathered by the operand
// loaders while staging shared memory. Weight gradients split the pixel reduction over CTAs and
// accumulate in FP32. Adam keeps FP32 master weights and refreshes the BF16 copies.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"
#include "tc_gemm.cuh"
#include "tma.cuh"
#include "unet.cuh"

namespace lentils {

using bf16 = __nv_bfloat16;

struct ConvSpec {
    int cin, cout;        // real channels
    int cin_p, cout_p;    // padded channels (multiples of 8; cout_p >= 32)
    int ks;               // kernel size (3 or 1)
    int relu;
    int level;            // resolution level: 0 = H x W, 1 = H/2, ...
};

constexpr int kNumLayers = 8;
static const ConvSpec kLayers[kNumLayers] = {
    {2, 32, 8, 32, 3, 1, 0},       // e1
    {32, 64, 32, 64, 3, 1, 1},     // e2
    {64, 128, 64, 128, 3, 1, 2},   // e3
    {128, 128, 128, 128, 3, 1, 3}, // b
    {128, 64, 128, 64, 1, 1, 2},   // c3
    {64, 32, 64, 32, 3, 1, 1},     // c2
    {32, 32, 32, 32, 3, 1, 0},     // c1
    {32, 1, 32, 32, 1, 0, 0},      // out
};

__device__ __forceinline__ float bf(bf16 v) { return __bfloat162float(v); }

// -- operand loaders ---------------------------------------------------------------------------
// im2col of an NHWC tensor: row = pixel (n, h, w), piece = 8 channels of one tap
struct ConvFwdA {
    const bf16 *x;
    int npix, H, W, C, ks;
    __device__ __forceinline__ uint4 operator()(int p, int kp) const
    {
        const int k = kp * 8;
        const int t = k / C, c = k - t * C;
        if (p >= npix || t >= ks * ks) return make_uint4(0, 0, 0, 0);
        const int hw = H * W;
        const int n = p / hw, r = p - n * hw, h = r / W, w = r - h * W;
        const int hh = h + t / ks - ks / 2, ww = w + t % ks - ks / 2;
        if (hh < 0 || hh >= H || ww < 0 || ww >= W) return make_uint4(0, 0, 0, 0);
        return *reinterpret_cast<const uint4 *>(x + ((size_t)(n * H + hh) * W + ww) * C + c);
    }
    // the same piece's address (null: a zero piece), for the cp.async pipeline
    __device__ __forceinline__ const void *ptr(int p, int kp) const
    {
        const int k = kp * 8;
        const int t = k / C, c = k - t * C;
        if (p >= npix || t >= ks * ks) return nullptr;
        const int hw = H * W;
        const int n = p / hw, r = p - n * hw, h = r / W, w = r - h * W;
        const int hh = h + t / ks - ks / 2, ww = w + t % ks - ks / 2;
        if (hh < 0 || hh >= H || ww < 0 || ww >= W) return nullptr;
        return x + ((size_t)(n * H + hh) * W + ww) * C + c;
    }
    __device__ __forceinline__ const void *base() const { return x; }
};

__device__ __forceinline__ uint4 relu_mask(uint4 g, uint4 y)
{
    const bf16 *gv = reinterpret_cast<const bf16 *>(&g);
    const bf16 *yv = reinterpret_cast<const bf16 *>(&y);
    uint4 out;
    bf16 *ov = reinterpret_cast<bf16 *>(&out);
#pragma unroll
    for (int i = 0; i < 8; ++i) ov[i] = (bf(yv[i]) > 0.f) ? gv[i] : __float2bfloat16(0.f);
    return out;
}

// data gradient: row = pixel, piece = 8 output channels of one tap, taken at pixel - off(tap)
struct ConvBwdDataA {
    const bf16 *dy, *y;  // y = layer output for the ReLU mask (null: no ReLU)
    int npix, H, W, C, ks;
    __device__ __forceinline__ uint4 operator()(int p, int kp) const
    {
        const int k = kp * 8;
        const int t = k / C, c = k - t * C;
        if (p >= npix || t >= ks * ks) return make_uint4(0, 0, 0, 0);
        const int hw = H * W;
        const int n = p / hw, r = p - n * hw, h = r / W, w = r - h * W;
        const int hh = h - (t / ks - ks / 2), ww = w - (t % ks - ks / 2);
        if (hh < 0 || hh >= H || ww < 0 || ww >= W) return make_uint4(0, 0, 0, 0);
        const size_t off = ((size_t)(n * H + hh) * W + ww) * C + c;
        const uint4 g = *reinterpret_cast<const uint4 *>(dy + off);
        if (!y) return g;
        return relu_mask(g, *reinterpret_cast<const uint4 *>(y + off));
    }
    // address of the unmasked piece (y must be null: the pipeline copies bytes as they are)
    __device__ __forceinline__ const void *ptr(int p, int kp) const
    {
        const int k = kp * 8;
        const int t = k / C, c = k - t * C;
        if (p >= npix || t >= ks * ks) return nullptr;
        const int hw = H * W;
        const int n = p / hw, r = p - n * hw, h = r / W, w = r - h * W;
        const int hh = h - (t / ks - ks / 2), ww = w - (t % ks - ks / 2);
        if (hh < 0 || hh >= H || ww < 0 || ww >= W) return nullptr;
        return dy + ((size_t)(n * H + hh) * W + ww) * C + c;
    }
    __device__ __forceinline__ const void *base() const { return dy; }
};

// weight gradient, A side: row = output channel, piece = 8 pixels of the masked gradient
struct ConvBwdWA {
    const bf16 *dy, *y;
    int npix, C;
    __device__ __forceinline__ uint4 operator()(int co, int kp) const
    {
        uint4 out = make_uint4(0, 0, 0, 0);
        if (co >= C) return out;
        bf16 *ov = reinterpret_cast<bf16 *>(&out);
        const int p0 = kp * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int p = p0 + j;
            if (p < npix) {
                const size_t o = (size_t)p * C + co;
                const bf16 g = dy[o];
                ov[j] = (!y || bf(y[o]) > 0.f) ? g : __float2bfloat16(0.f);
            }
        }
        return out;
    }
};

// weight gradient, B side: row = (tap, input channel), piece = 8 pixels of the shifted input
struct ConvBwdWB {
    const bf16 *x;
    int npix, H, W, C, ks;
    __device__ __forceinline__ uint4 operator()(int kk, int kp) const
    {
        uint4 out = make_uint4(0, 0, 0, 0);
        const int t = kk / C, c = kk - t * C;
        if (t >= ks * ks) return out;
        bf16 *ov = reinterpret_cast<bf16 *>(&out);
        const int dh = t / ks - ks / 2, dw = t % ks - ks / 2;
        const int hw = H * W;
        const int p0 = kp * 8;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int p = p0 + j;
            if (p < npix) {
                const int n = p / hw, r = p - n * hw, h = r / W, w = r - h * W;
                const int hh = h + dh, ww = w + dw;
                if (hh >= 0 && hh < H && ww >= 0 && ww < W)
                    ov[j] = x[((size_t)(n * H + hh) * W + ww) * C + c];
            }
        }
        return out;
    }
};

// Weight gradient on transposed operands (the pipelined forms): the GEMM rows are the (tap,
// input channel) pairs and the columns the output channels, K runs over pixels, and both
// operands are read as pieces of consecutive pixels from channel-major copies made per layer:
// xT[s][c][q] = x[p + s - 1][c] within the image row (zero across its ends), for the three
// column shifts s of a 3 x 3 tap (one copy, s = 1, for 1 x 1), in a row-padded layout with a
// zero row above and below each image (shift_transpose_kernel), and dyT[co][p] = the
// ReLU-masked output gradient. A tap's row shift is then a whole-row offset, and a 16-byte
// piece of 8 pixels is one aligned load.
struct ConvWgXT {
    const bf16 *xT;  // [3 or 1][C][qtot]
    int npix, H, W, C, ks;
    long long qtot;
    __device__ __forceinline__ const void *ptr(int kk, int kp) const
    {
        const int t = kk / C, c = kk - t * C;
        const int p0 = kp * 8;
        if (t >= ks * ks || p0 >= npix) return nullptr;
        const int dh = t / ks - ks / 2, dw = t % ks - ks / 2;
        const int hw = H * W, n = p0 / hw, r = p0 - n * hw, h = r / W, w = r - h * W;
        const long long q = ((long long)n * (H + 2) + h + 1 + dh) * W + w;
        return xT + ((size_t)(dw + ks / 2) * C + c) * qtot + q;
    }
    __device__ __forceinline__ const void *base() const { return xT; }
};

struct ConvWgDyT {
    const bf16 *dyT;  // [C][npix]
    int npix, C;
    __device__ __forceinline__ const void *ptr(int co, int kp) const
    {
        const int p0 = kp * 8;
        if (co >= C || p0 >= npix) return nullptr;
        return dyT + (size_t)co * npix + p0;
    }
    __device__ __forceinline__ const void *base() const { return dyT; }
};

// The same operands loaded by TMA (tc::gemm_tma_kernel): xT in the row-padded layout of
// shift_transpose_kernel as a 2-D tensor (padded pixel position innermost, (shift, channel)
// rows), one box of 64 positions x C rows per tap of the row tile (a tap past the kernel's
// reads rows past the tensor: zeros); dyT as a 2-D tensor (pixel innermost, output-channel
// rows). A K chunk is 64 pixels of one image (H W is a multiple of 64), contiguous in both.
struct ConvWgXTTma {
    static constexpr int kChunk = 64, kSwz = 128;
    static constexpr uint32_t kBytes = 128 * 128;
    CUtensorMap map;
    int C, ks, H, W, rows;  // rows = (number of shifts) * C
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int m0, int kp0) const
    {
        const int p0 = kp0 * 8, hw = H * W;
        const int n = p0 / hw, r = p0 - n * hw, h = r / W, w = r - h * W;
        const int q0 = (n * (H + 2) + h + 1) * W + w;
        const int t0 = m0 / C;
        for (int j = 0; j < 128 / C; ++j) {
            const int t = t0 + j;
            unsigned char *d = static_cast<unsigned char *>(dst) + j * C * 128;
            if (t < ks * ks) {
                const int dh = t / ks - ks / 2, dw = t % ks - ks / 2;
                tc::tma_load_2d(d, &map, q0 + dh * W, (dw + ks / 2) * C, bar);
            } else {
                tc::tma_load_2d(d, &map, q0, rows, bar);  // past the last row: zeros
            }
        }
    }
};

template <int N>
struct ConvWgDyTTma {
    static constexpr int kChunk = 64, kSwz = 128;
    static constexpr uint32_t kBytes = N * 128;
    CUtensorMap map;
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int n0, int kp0) const
    {
        tc::tma_load_2d(dst, &map, kp0 * 8, n0, bar);
    }
};

// The same operands in the blocked layouts (W a multiple of 64): a tap's rows for a 64-pixel
// chunk are one contiguous run of C x 128 bytes, loaded as a 3-D box (64, C, 1).
struct ConvWgXTTmaBlk {
    static constexpr int kChunk = 64, kSwz = 128;
    static constexpr uint32_t kBytes = 128 * 128;
    CUtensorMap map;  // (64, C, nshift * qtot / 64)
    int C, ks, H, W, nblk;  // nblk = qtot / 64
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int m0, int kp0) const
    {
        const int p0 = kp0 * 8, hw = H * W;
        const int n = p0 / hw, r = p0 - n * hw, h = r / W, w = r - h * W;
        const int q0 = (n * (H + 2) + h + 1) * W + w;  // a multiple of 64
        const int t0 = m0 / C;
        for (int j = 0; j < 128 / C; ++j) {
            const int t = t0 + j;
            unsigned char *d = static_cast<unsigned char *>(dst) + j * C * 128;
            if (t < ks * ks) {
                const int dh = t / ks - ks / 2, dw = t % ks - ks / 2;
                tc::tma_load_3d(d, &map, 0, 0, (dw + ks / 2) * nblk + (q0 + dh * W) / 64, bar);
            } else {
                tc::tma_load_3d(d, &map, 0, 0, (ks == 3 ? 3 : 1) * nblk, bar);  // zeros
            }
        }
    }
};

template <int N>
struct ConvWgDyTTmaBlk {
    static constexpr int kChunk = 64, kSwz = 128;
    static constexpr uint32_t kBytes = N * 128;
    CUtensorMap map;  // (64, N, npix / 64)
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int n0, int kp0) const
    {
        tc::tma_load_3d(dst, &map, 0, n0, kp0 / 8, bar);
    }
};

// A operand of a convolution over NHWC activations (forward: the input, taps as they are; data
// gradient: the masked output gradient, taps flipped) through a 4-D tensor map (C, W, H, B)
// with box (CB, WB, HB, 1): a row tile is 128 consecutive pixels of one image (WB HB = 128),
// a K chunk is CB channels of one tap (K = tap C + c). The box is placed at the tap's pixel
// offset, and the tensor map reads zeros where it leaves the image: the zero padding of the
// convolution. CB = 64 (128-byte rows, 128-byte swizzle) or 32 (64-byte).
template <int CB>
struct ConvTmaA {
    static constexpr int kChunk = CB, kSwz = 2 * CB;
    static constexpr uint32_t kBytes = 128 * CB * 2;
    CUtensorMap map;
    int C, ks, H, W, flip;
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int m0, int kp0) const
    {
        const int k = kp0 * 8, t = k / C, c0 = k - t * C;
        const int hw = H * W, n = m0 / hw, r = m0 - n * hw, h = r / W, w = r - h * W;
        if (t >= ks * ks) {  // past the last tap: a box past the channels reads zeros
            tc::tma_load_4d(dst, &map, C, w, h, n, bar);
            return;
        }
        int dh = t / ks - ks / 2, dw = t % ks - ks / 2;
        if (flip) {
            dh = -dh;
            dw = -dw;
        }
        tc::tma_load_4d(dst, &map, c0, w + dw, h + dh, n, bar);
    }
    // The persistent GEMM walks the chunks of a tile with a cursor: the tile's pixel is split
    // once, and each chunk steps the channel offset and the tap with adds and compares (the
    // single producer thread otherwise spends most of a chunk's time in integer divisions).
    // K = ks^2 C exactly (C a multiple of CB).
    struct Cursor {
        int c0, ky, kx, w, h, n;
    };
    __device__ __forceinline__ Cursor begin(int m0) const
    {
        const int hw = H * W, n = m0 / hw, r = m0 - n * hw, h = r / W;
        return Cursor{0, 0, 0, r - h * W, h, n};
    }
    __device__ __forceinline__ void next(void *dst, uint64_t *bar, Cursor &c) const
    {
        int dh = c.ky - ks / 2, dw = c.kx - ks / 2;
        if (flip) {
            dh = -dh;
            dw = -dw;
        }
        tc::tma_load_4d(dst, &map, c.c0, c.w + dw, c.h + dh, c.n, bar);
        c.c0 += CB;
        if (c.c0 == C) {
            c.c0 = 0;
            if (++c.kx == ks) {
                c.kx = 0;
                ++c.ky;
            }
        }
    }
};

// B operand: row-major [N][K] BF16 weights through a 2-D tensor map, box (CB, N).
template <int CB, int N>
struct ConvTmaB {
    static constexpr int kChunk = CB, kSwz = 2 * CB;
    static constexpr uint32_t kBytes = N * CB * 2;
    CUtensorMap map;
    __device__ __forceinline__ void load(void *dst, uint64_t *bar, int n0, int kp0) const
    {
        tc::tma_load_2d(dst, &map, kp0 * 8, n0, bar);
    }
    struct Cursor {
        int k, n0;
    };
    __device__ __forceinline__ Cursor begin(int n0) const { return Cursor{0, n0}; }
    __device__ __forceinline__ void next(void *dst, uint64_t *bar, Cursor &c) const
    {
        tc::tma_load_2d(dst, &map, c.k, c.n0, bar);
        c.k += CB;
    }
};

// -- epilogues -------------------------------------------------------------------------------------
struct EpiAct {  // y[pixel][co] = bf16(relu?(v + bias))
    bf16 *y;
    const float *bias;
    int npix, C, relu;
    __device__ __forceinline__ void operator()(int p, int co, float v) const
    {
        if (p >= npix || co >= C) return;
        v += bias[co];
        if (relu) v = fmaxf(v, 0.f);
        y[(size_t)p * C + co] = __float2bfloat16(v);
    }
};

struct EpiOut {  // out[pixel] = v + bias (channel 0 only), FP32
    static constexpr bool kRowPerLane = true;
    float *out;
    const float *bias;
    int npix;
    __device__ __forceinline__ void operator()(int p, int co, float v) const
    {
        if (co == 0 && p < npix) out[p] = v + bias[0];
    }
};

struct EpiStoreBf16 {  // dx[pixel][ci] = bf16(v)
    bf16 *dx;
    int npix, C;
    __device__ __forceinline__ void operator()(int p, int c, float v) const
    {
        if (p < npix && c < C) dx[(size_t)p * C + c] = __float2bfloat16(v);
    }
};

struct EpiAtomicF32 {  // g[row][col] += v
    float *g;
    int rows, cols;
    __device__ __forceinline__ void operator()(int r, int c, float v) const
    {
        if (r < rows && c < cols && v != 0.f) atomicAdd(&g[(size_t)r * cols + c], v);
    }
};

struct EpiAtomicF32T {  // g[col][row] += v (the weight gradient from its transposed GEMM)
    float *g;
    int rows, cols;  // rows = taps * cin_p (GEMM rows), cols = cout_p
    __device__ __forceinline__ void operator()(int r, int c, float v) const
    {
        if (r < rows && c < cols && v != 0.f) atomicAdd(&g[(size_t)c * rows + r], v);
    }
};

struct EpiPartialF32 {  // slab blockIdx.z of g: g[z][row][col] = v (split-K partial sums)
    float *g;
    int rows, cols;
    __device__ __forceinline__ void operator()(int r, int c, float v) const
    {
        if (r < rows && c < cols) g[((size_t)blockIdx.z * rows + r) * cols + c] = v;
    }
};

// Row epilogues of the persistent GEMM (tc::gemm_tma_persist_kernel): one thread per output
// pixel, 32 channels per call, BF16 rows written 16 bytes at a time. prepare() copies the
// per-channel constants into the kernel's shared scratch `sh` (the 128 epilogue threads, tid
// 0..127) once per CTA; row() reads them from there.
__device__ __forceinline__ void act32_bf16(const float (&v)[32], const float *sb, int relu,
                                           uint4 (&u)[4])
{
    bf16 *b = reinterpret_cast<bf16 *>(u);
#pragma unroll
    for (int i = 0; i < 32; ++i) {
        float t = v[i] + sb[i];
        if (relu) t = fmaxf(t, 0.f);
        b[i] = __float2bfloat16(t);
    }
}

struct RowAct {  // y[pixel][n0 + i] = bf16(relu?(v + bias)), C channels per pixel
    bf16 *y;
    const float *bias;
    int npix, C, relu;
    __device__ __forceinline__ void prepare(float *sh, int tid) const
    {
        for (int i = tid; i < C; i += 128) sh[i] = bias[i];
    }
    __device__ __forceinline__ void row(int m, int n0, const float (&v)[32], float &,
                                        const float *sh) const
    {
        if (m >= npix) return;
        uint4 u[4];
        act32_bf16(v, sh + n0, relu, u);
        uint4 *dst = reinterpret_cast<uint4 *>(y + (size_t)m * C + n0);
#pragma unroll
        for (int i = 0; i < 4; ++i) dst[i] = u[i];
    }
    __device__ __forceinline__ void row_end(int, float, const float *) const {}
};

struct RowStore {  // dx[pixel][n0 + i] = bf16(v), C channels per pixel (a data gradient)
    bf16 *y;
    int npix, C;
    __device__ __forceinline__ void prepare(float *, int) const {}
    __device__ __forceinline__ void row(int m, int n0, const float (&v)[32], float &,
                                        const float *) const
    {
        if (m >= npix) return;
        uint4 u[4];
        bf16 *b = reinterpret_cast<bf16 *>(u);
#pragma unroll
        for (int i = 0; i < 32; ++i) b[i] = __float2bfloat16(v[i]);
        uint4 *dst = reinterpret_cast<uint4 *>(y + (size_t)m * C + n0);
#pragma unroll
        for (int i = 0; i < 4; ++i) dst[i] = u[i];
    }
    __device__ __forceinline__ void row_end(int, float, const float *) const {}
};

// The last hidden layer (32 channels, ReLU) fused with the 1 x 1 output layer: y as RowAct (not
// stored when y is null), then out = sum_c wo[c] * y[c] + bo over the BF16 values of y in
// channel order. With z set, the preconditioner's combination z = s * out + gamma * dinv * r
// is written instead of out.
struct RowActOut {
    bf16 *y;
    const float *bias;
    int npix;
    const bf16 *wo;   // output-layer weights, 32 values
    const float *bo;  // output-layer bias
    float *out;
    float *z;
    const float *r, *dinv, *scale;
    float gamma;
    // sh: [0, 32) bias, [32, 64) output weights, 64 output bias, 65 s
    __device__ __forceinline__ void prepare(float *sh, int tid) const
    {
        if (tid < 32) {
            sh[tid] = bias[tid];
            sh[32 + tid] = bf(wo[tid]);
        } else if (tid == 32) {
            sh[64] = bo[0];
            sh[65] = z ? scale[0] : 0.f;
        }
    }
    __device__ __forceinline__ void row(int m, int n0, const float (&v)[32], float &acc,
                                        const float *sh) const
    {
        if (m >= npix) return;
        uint4 u[4];
        act32_bf16(v, sh + n0, 1, u);
        const bf16 *b = reinterpret_cast<const bf16 *>(u);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc = fmaf(bf(b[i]), sh[32 + n0 + i], acc);
        if (y) {
            uint4 *dst = reinterpret_cast<uint4 *>(y + (size_t)m * 32 + n0);
#pragma unroll
            for (int i = 0; i < 4; ++i) dst[i] = u[i];
        }
    }
    __device__ __forceinline__ void row_end(int m, float acc, const float *sh) const
    {
        if (m >= npix) return;
        const float o = acc + sh[64];
        if (z) z[m] = fmaf(sh[65], o, gamma * dinv[m] * r[m]);
        else out[m] = o;
    }
};

// A forward layer whose output has fewer than kSplitMaxPix pixels (fewer than 64 row tiles of
// 128) splits its K reduction over CTAs: each split writes an FP32 partial slab, and a second
// kernel sums the slabs in a fixed order and applies bias / ReLU / BF16, so the result does not
// depend on CTA timing. At batch 1 this turns the deep layers' long serial chunk chains (9-18
// chunks on 2-8 CTAs) into a few chunks on many CTAs. The number of splits is at most
// max(2, 128 / row tiles), so the slabs hold at most kSplitSlabPix pixels x 128 channels.
constexpr int kSplitMaxPix = 64 * 128;
// at most this many splits: each adds an FP32 slab that the finalize kernel reads
constexpr int kSplitMax = 8;
constexpr int kSplitSlabPix = 2 * kSplitMaxPix;

// -- elementwise kernels ----------------------------------------------------------------------------
static int blocks_n(long long n)
{
    long long b = (n + 255) / 256;
    return (int)std::max(1LL, std::min(b, 152LL * 16));
}

// blocks of 64 threads for n work items (the small batch-1 kernels: more SMs, fewer threads each)
static int blocks_small(long long n)
{
    long long b = (n + 63) / 64;
    return (int)std::max(1LL, std::min(b, 152LL * 32));
}

#define LENTILS_GRID_STRIDE(i, n)                                                              \
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < (n);             \
         i += (long long)gridDim.x * blockDim.x)

__global__ void make_input_kernel(const float *__restrict__ r, const float *__restrict__ d,
                                  bf16 *__restrict__ x0, long long npix)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(p, npix)
    {
        bf16 v[8];
        v[0] = __float2bfloat16(r[p]);
        v[1] = __float2bfloat16(d[p]);
        for (int i = 2; i < 8; ++i) v[i] = __float2bfloat16(0.f);
        *reinterpret_cast<uint4 *>(x0 + p * 8) = *reinterpret_cast<uint4 *>(v);
    }
}

// y[pixel][c] = bf16(relu?(sum_z part[z][pixel][c] + bias)), slabs summed in order z = 0, 1, ...
__global__ void finalize_act_kernel(const float *__restrict__ part, int nz,
                                    const float *__restrict__ bias, bf16 *__restrict__ y,
                                    long long n, int C, int relu)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(e, n)
    {
        float acc = part[e];
        for (int z = 1; z < nz; ++z) acc += part[(size_t)z * n + e];
        float v = acc + bias[e % C];
        if (relu) v = fmaxf(v, 0.f);
        y[e] = __float2bfloat16(v);
    }
}

// The pooling / upsampling kernels below work on 8 channels (16 bytes) per thread; C is a
// multiple of 8. Per element the arithmetic (FP32 sums of BF16 values, one rounding) is that
// of a one-element-per-thread form.
__device__ __forceinline__ void bf8_load(const bf16 *p, float (&v)[8])
{
    const uint4 u = *reinterpret_cast<const uint4 *>(p);
    const bf16 *b = reinterpret_cast<const bf16 *>(&u);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = bf(b[i]);
}
__device__ __forceinline__ void bf8_store(bf16 *p, const float (&v)[8])
{
    uint4 u;
    bf16 *b = reinterpret_cast<bf16 *>(&u);
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = __float2bfloat16(v[i]);
    *reinterpret_cast<uint4 *>(p) = u;
}

// First layer (2 -> 32 channels, 3 x 3, ReLU) on the CUDA cores, fused with the input packing
// and the 2 x 2 pooling that follows it: a GEMM over K = 9 taps x 2 channels would leave the
// tensor core and its operand staging mostly idle. One thread computes a 2 x 2 block of
// output pixels, 8 channels at a time, from the 4 x 4 input patch around it:
//   channel 0 = bf16(a * a2 * inv) (a2, inv optional: a2 = dinv and inv = 1 / scale for the
//   preconditioner), channel 1 = bf16(b); x0 (optional) = the packed 8-channel input,
//   y = bf16(relu(conv + bias)), yp = the 2 x 2 mean of y with pool2_kernel's arithmetic.
// The products are exact in FP32; their sum is taken in tap order (the GEMM's order is the
// tensor core's), so y can differ from the GEMM form by the BF16 rounding of an FP32 ulp.
__global__ void __launch_bounds__(128, 5)
    e1_direct_kernel(const float *__restrict__ a, const float *__restrict__ a2,
                     const float *__restrict__ scale, const float *__restrict__ b,
                     const bf16 *__restrict__ wf, const float *__restrict__ bias,
                     bf16 *__restrict__ x0, bf16 *__restrict__ y, bf16 *__restrict__ yp, int Bn,
                     int H, int W, int nh)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ __align__(16) float ws[18][32];  // [tap * 2 + ci][co]
    __shared__ float bs[32];
    for (int i = threadIdx.x; i < 18 * 32; i += blockDim.x) {
        const int co = i / 18, r = i - co * 18, t = r >> 1, ci = r & 1;
        ws[r][co] = bf(wf[co * 72 + t * 8 + ci]);
    }
    if (threadIdx.x < 32) bs[threadIdx.x] = bias[threadIdx.x];
    __syncthreads();
    const float inv = scale ? 1.f / scale[0] : 1.f;
    const int h2 = H / 2, w2 = W / 2;
    const long long nblk = (long long)Bn * h2 * w2;
    // nh = 2: two threads per block of pixels, one for each half of the channels
    LENTILS_GRID_STRIDE(item, nblk * nh)
    {
        const long long q = item / nh;
        const int half0 = nh == 2 ? (int)(item & 1) : 0, half1 = nh == 2 ? half0 + 1 : 2;
        const int ww = (int)(q % w2);
        const long long rq = q / w2;
        const int hh = (int)(rq % h2);
        const int n = (int)(rq / h2);
        const int h0 = 2 * hh, w0 = 2 * ww;
        const size_t img = (size_t)n * H * W;
        float in0[4][4], in1[4][4];
#pragma unroll
        for (int dy = 0; dy < 4; ++dy) {
#pragma unroll
            for (int dx = 0; dx < 4; ++dx) {
                const int h = h0 - 1 + dy, w = w0 - 1 + dx;
                float v0 = 0.f, v1 = 0.f;
                if (h >= 0 && h < H && w >= 0 && w < W) {
                    const size_t p = img + (size_t)h * W + w;
                    float x = a[p];
                    if (a2) x = a2[p] * x;
                    if (scale) x = x * inv;
                    v0 = bf(__float2bfloat16(x));
                    v1 = bf(__float2bfloat16(b[p]));
                }
                in0[dy][dx] = v0;
                in1[dy][dx] = v1;
            }
        }
        if (x0 && half0 == 0) {
#pragma unroll
            for (int py = 0; py < 2; ++py)
#pragma unroll
                for (int px = 0; px < 2; ++px) {
                    bf16 v[8];
                    v[0] = __float2bfloat16(in0[py + 1][px + 1]);
                    v[1] = __float2bfloat16(in1[py + 1][px + 1]);
#pragma unroll
                    for (int i = 2; i < 8; ++i) v[i] = __float2bfloat16(0.f);
                    const size_t p = img + (size_t)(h0 + py) * W + w0 + px;
                    *reinterpret_cast<uint4 *>(x0 + p * 8) = *reinterpret_cast<const uint4 *>(v);
                }
        }
#pragma unroll 1
        for (int g = 2 * half0; g < 2 * half1; ++g) {  // 8 channels at a time: 8 g .. 8 g + 7
            float acc[4][8];
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
                for (int c = 0; c < 8; ++c) acc[k][c] = 0.f;
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int ky = t / 3, kx = t % 3;
#pragma unroll
                for (int ci = 0; ci < 2; ++ci) {
#pragma unroll
                    for (int c4 = 0; c4 < 2; ++c4) {
                        const float4 wv =
                            *reinterpret_cast<const float4 *>(&ws[t * 2 + ci][g * 8 + c4 * 4]);
#pragma unroll
                        for (int py = 0; py < 2; ++py)
#pragma unroll
                            for (int px = 0; px < 2; ++px) {
                                const float xv =
                                    ci ? in1[py + ky][px + kx] : in0[py + ky][px + kx];
                                float *ac = &acc[py * 2 + px][c4 * 4];
                                ac[0] = fmaf(xv, wv.x, ac[0]);
                                ac[1] = fmaf(xv, wv.y, ac[1]);
                                ac[2] = fmaf(xv, wv.z, ac[2]);
                                ac[3] = fmaf(xv, wv.w, ac[3]);
                            }
                    }
                }
            }
            float ps[8];  // the pooling sum, in pool2_kernel's order ((y0 + y1) + y2) + y3
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int py = k >> 1, px = k & 1;
                uint4 u;
                bf16 *ub = reinterpret_cast<bf16 *>(&u);
#pragma unroll
                for (int c = 0; c < 8; ++c) {
                    const bf16 r = __float2bfloat16(fmaxf(acc[k][c] + bs[g * 8 + c], 0.f));
                    ub[c] = r;
                    ps[c] = k == 0 ? bf(r) : ps[c] + bf(r);
                }
                const size_t p = img + (size_t)(h0 + py) * W + w0 + px;
                *reinterpret_cast<uint4 *>(y + p * 32 + g * 8) = u;
            }
            uint4 u;
            bf16 *ub = reinterpret_cast<bf16 *>(&u);
#pragma unroll
            for (int c = 0; c < 8; ++c) ub[c] = __float2bfloat16(0.25f * ps[c]);
            *reinterpret_cast<uint4 *>(yp + ((size_t)n * h2 * w2 + (size_t)hh * w2 + ww) * 32 + g * 8) = u;
        }
    }
}

// Sum of the split-K slabs part[z][o .. o + 7], z = 0, 1, ... in order, plus bias, ReLU
__device__ __forceinline__ void finalize8(const float *__restrict__ part, int nz, long long slab,
                                          size_t o, const float *__restrict__ bias, int relu,
                                          float (&v)[8])
{
    const float4 *p = reinterpret_cast<const float4 *>(part + o);
    float4 a = __ldg(p), b = __ldg(p + 1);
    v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
#pragma unroll 4
    for (int z = 1; z < nz; ++z) {
        const float4 *q = reinterpret_cast<const float4 *>(part + (size_t)z * slab + o);
        a = __ldg(q);
        b = __ldg(q + 1);
        v[0] += a.x, v[1] += a.y, v[2] += a.z, v[3] += a.w;
        v[4] += b.x, v[5] += b.y, v[6] += b.z, v[7] += b.w;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float t = v[i] + bias[i];
        if (relu) t = fmaxf(t, 0.f);
        v[i] = t;
    }
}

// finalize_act_kernel fused with the 2 x 2 pooling of its output: one thread per pixel and 8
// channels, the four pixels of a pooling block in four consecutive lanes (the pooled value is
// gathered by shuffles into the first); y (Bn, H, W, C) and yp (Bn, H/2, W/2, C) are both
// written, with the arithmetic of finalize_act_kernel and pool2_kernel. The thread count
// Bn H W C / 8 is a multiple of 32 (H and W are multiples of 8), so whole warps run each
// iteration.
__global__ void finalize_pool_kernel(const float *__restrict__ part, int nz,
                                     const float *__restrict__ bias, bf16 *__restrict__ y,
                                     bf16 *__restrict__ yp, int Bn, int H, int W, int C, int relu)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    const int h2 = H / 2, w2 = W / 2, cv = C / 8;
    const long long n = (long long)Bn * H * W * cv;
    const long long slab = (long long)Bn * H * W * C;
    LENTILS_GRID_STRIDE(e, n)
    {
        const int k = (int)(e & 3);
        const long long rest = e >> 2;
        const int c = (int)(rest % cv) * 8;
        const long long q = rest / cv;  // pooled pixel
        const int w = (int)(q % w2);
        const long long r = q / w2;
        const int h = (int)(r % h2);
        const int b = (int)(r / h2);
        const size_t p = (size_t)(b * H + 2 * h + (k >> 1)) * W + 2 * w + (k & 1);
        const size_t o = p * C + c;
        float v[8];
        finalize8(part, nz, slab, o, bias + c, relu, v);
        bf8_store(y + o, v);
        float s[8];
        const int lane = threadIdx.x & 31, src = lane & ~3;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const float yv = bf(__float2bfloat16(v[i]));  // the stored value, as pool2 reads it
            const float y1 = __shfl_sync(0xffffffffu, yv, src + 1);
            const float y2 = __shfl_sync(0xffffffffu, yv, src + 2);
            const float y3 = __shfl_sync(0xffffffffu, yv, src + 3);
            s[i] = 0.25f * (((yv + y1) + y2) + y3);
        }
        if (k == 0) bf8_store(yp + q * C + c, s);
    }
}

// finalize_act_kernel fused with up2add_kernel: y (Bn, H, W, C) is the layer output at low
// resolution; u (Bn, 2H, 2W, C) = up2(y) + skip. One thread per low-resolution pixel and 8
// channels.
__global__ void finalize_up_kernel(const float *__restrict__ part, int nz,
                                   const float *__restrict__ bias, bf16 *__restrict__ y,
                                   const bf16 *__restrict__ skip, bf16 *__restrict__ u, int Bn,
                                   int H, int W, int C, int relu)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    const int cv = C / 8;
    const long long n = (long long)Bn * H * W * cv;
    const long long slab = (long long)Bn * H * W * C;
    LENTILS_GRID_STRIDE(e, n)
    {
        const int c = (int)(e % cv) * 8;
        const long long q = e / cv;
        const int w = (int)(q % W);
        const long long r = q / W;
        const int h = (int)(r % H);
        const int b = (int)(r / H);
        const size_t o = q * C + c;
        float t[4][8];
        size_t ph[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {  // the skip values, loaded ahead of the slab sums
            ph[k] = ((size_t)(b * 2 * H + 2 * h + (k >> 1)) * (2 * W) + 2 * w + (k & 1)) * C + c;
            bf8_load(skip + ph[k], t[k]);
        }
        float v[8];
        finalize8(part, nz, slab, o, bias + c, relu, v);
        bf8_store(y + o, v);
        float lo[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) lo[i] = bf(__float2bfloat16(v[i]));
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            float s[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) s[i] = lo[i] + t[k][i];
            bf8_store(u + ph[k], s);
        }
    }
}

// out (n, H/2, W/2, C) = mean of the 2 x 2 block
__global__ void pool2_kernel(const bf16 *__restrict__ x, bf16 *__restrict__ y, int Bn, int H,
                             int W, int C)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    const int h2 = H / 2, w2 = W / 2, cv = C / 8;
    const long long n = (long long)Bn * h2 * w2 * cv;
    LENTILS_GRID_STRIDE(e, n)
    {
        const int c = (int)(e % cv) * 8;
        const long long q = e / cv;  // output pixel
        const int w = (int)(q % w2);
        const long long r = q / w2;
        const int h = (int)(r % h2);
        const int b = (int)(r / h2);
        const size_t base = ((size_t)(b * H + 2 * h) * W + 2 * w) * C + c;
        float a[8], t[8];
        bf8_load(x + base, a);
        bf8_load(x + base + C, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] += t[i];
        bf8_load(x + base + (size_t)W * C, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] += t[i];
        bf8_load(x + base + (size_t)W * C + C, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = 0.25f * (a[i] + t[i]);
        bf8_store(y + q * C + c, a);
    }
}

// out (n, H, W, C) = up2(low) + skip
__global__ void up2add_kernel(const bf16 *__restrict__ low, const bf16 *__restrict__ skip,
                              bf16 *__restrict__ y, int Bn, int H, int W, int C)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    const int cv = C / 8;
    const long long n = (long long)Bn * H * W * cv;
    LENTILS_GRID_STRIDE(e, n)
    {
        const int c = (int)(e % cv) * 8;
        const long long q = e / cv;
        const int w = (int)(q % W);
        const long long r = q / W;
        const int h = (int)(r % H);
        const int b = (int)(r / H);
        float a[8], t[8];
        bf8_load(low + ((size_t)(b * (H / 2) + h / 2) * (W / 2) + w / 2) * C + c, a);
        bf8_load(skip + q * C + c, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] += t[i];
        bf8_store(y + q * C + c, a);
    }
}

// dlow (n, H/2, W/2, C) = sum of the 2 x 2 children of dy (gradient of up2)
// With y set, the result is also masked by y > 0 (the ReLU of the layer whose output gradient
// it is: grad_prep_kernel's dym) and db[c] += its sum over pixels (that layer's bias gradient).
// The grid-stride step is a multiple of C / 8, so a thread keeps its 8 channels.
__device__ __forceinline__ void mask8(float (&v)[8], const bf16 *y)
{
    float t[8];
    bf8_load(y, t);
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = t[i] > 0.f ? bf(__float2bfloat16(v[i])) : 0.f;
}

__device__ __forceinline__ void db_flush(const float (&acc)[8], int c, int C, float *sdb,
                                         float *__restrict__ db)
{
#pragma unroll
    for (int i = 0; i < 8; ++i) atomicAdd(&sdb[c + i], acc[i]);
    __syncthreads();
    for (int i = threadIdx.x; i < C; i += blockDim.x) atomicAdd(&db[i], sdb[i]);
}

__global__ void sum4_kernel(const bf16 *__restrict__ dy, bf16 *__restrict__ dlow, int Bn, int H,
                            int W, int C, const bf16 *__restrict__ y, float *__restrict__ db)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ float sdb[128];
    const int h2 = H / 2, w2 = W / 2, cv = C / 8;
    const long long n = (long long)Bn * h2 * w2 * cv;
    if (db) {
        for (int i = threadIdx.x; i < C; i += blockDim.x) sdb[i] = 0.f;
        __syncthreads();
    }
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int cthr = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) % cv) * 8;
    LENTILS_GRID_STRIDE(e, n)
    {
        const int c = (int)(e % cv) * 8;
        const long long q = e / cv;
        const int w = (int)(q % w2);
        const long long r = q / w2;
        const int h = (int)(r % h2);
        const int b = (int)(r / h2);
        const size_t base = ((size_t)(b * H + 2 * h) * W + 2 * w) * C + c;
        float a[8], t[8];
        bf8_load(dy + base, a);
        bf8_load(dy + base + C, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] += t[i];
        bf8_load(dy + base + (size_t)W * C, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] += t[i];
        bf8_load(dy + base + (size_t)W * C + C, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] += t[i];
        if (y) {
            mask8(a, y + q * C + c);
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i] += a[i];
        }
        bf8_store(dlow + q * C + c, a);
    }
    if (db) db_flush(acc, cthr, C, sdb, db);
}

// d (n, H, W, C) = a + 0.25 * up2(dp) (gradient through pool2 added to another gradient)
// (y, db: masked, with the bias gradient, as sum4_kernel)
__global__ void add_pool_grad_kernel(const bf16 *__restrict__ a, const bf16 *__restrict__ dp,
                                     bf16 *__restrict__ d, int Bn, int H, int W, int C,
                                     const bf16 *__restrict__ y, float *__restrict__ db)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ float sdb[128];
    const int cv = C / 8;
    const long long n = (long long)Bn * H * W * cv;
    if (db) {
        for (int i = threadIdx.x; i < C; i += blockDim.x) sdb[i] = 0.f;
        __syncthreads();
    }
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const int cthr = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) % cv) * 8;
    LENTILS_GRID_STRIDE(e, n)
    {
        const int c = (int)(e % cv) * 8;
        const long long q = e / cv;
        const int w = (int)(q % W);
        const long long r = q / W;
        const int h = (int)(r % H);
        const int b = (int)(r / H);
        float v[8], t[8];
        bf8_load(a + q * C + c, v);
        bf8_load(dp + ((size_t)(b * (H / 2) + h / 2) * (W / 2) + w / 2) * C + c, t);
#pragma unroll
        for (int i = 0; i < 8; ++i) v[i] += 0.25f * t[i];
        if (y) {
            mask8(v, y + q * C + c);
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[i] += v[i];
        }
        bf8_store(d + q * C + c, v);
    }
    if (db) db_flush(acc, cthr, C, sdb, db);
}

// loss = mean((out - tgt)^2); dy[pixel][0..31] = (2/npix (out - tgt), 0, ...)
// compact: dy[pixel] = the gradient alone (the output layer's fused backward pass reads only
// channel 0), else the 32-channel row the GEMM forms read
__device__ __forceinline__ void store_out_grad(bf16 *dy, long long p, float g, int compact)
{
    if (compact) {
        dy[p] = __float2bfloat16(g);
        return;
    }
    bf16 v[8];
    v[0] = __float2bfloat16(g);
    for (int i = 1; i < 8; ++i) v[i] = __float2bfloat16(0.f);
    uint4 *dst = reinterpret_cast<uint4 *>(dy + p * 32);
    dst[0] = *reinterpret_cast<uint4 *>(v);
    dst[1] = dst[2] = dst[3] = make_uint4(0, 0, 0, 0);
}

__global__ void mse_kernel(const float *__restrict__ out, const float *__restrict__ tgt,
                           bf16 *__restrict__ dy, long long npix, float *__restrict__ loss,
                           int compact)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ float sh[256];
    float acc = 0.f;
    const float scale = 2.f / (float)npix;
    LENTILS_GRID_STRIDE(p, npix)
    {
        const float e = out[p] - tgt[p];
        acc += e * e;
        store_out_grad(dy, p, scale * e, compact);
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, sh[0] / (float)npix);
}

// dy[pixel][0..31] = (dout[pixel], 0, ...), or dy[pixel] = dout[pixel] (compact): an external
// gradient of the output
__global__ void pack_dout_kernel(const float *__restrict__ dout, bf16 *__restrict__ dy,
                                 long long npix, int compact)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(p, npix) store_out_grad(dy, p, dout[p], compact);
}

// db[co] += sum_pixel dy'[pixel][co]
__global__ void bias_grad_kernel(const bf16 *__restrict__ dy, const bf16 *__restrict__ y,
                                 float *__restrict__ db, long long npix, int C, int creal)
{
    // blockDim.x == C (padded channels, <= 128); each block sums a slice of pixels
    const int c = threadIdx.x;
    float acc = 0.f;
    for (long long p = blockIdx.x; p < npix; p += gridDim.x) {
        const size_t o = (size_t)p * C + c;
        if (!y || bf(y[o]) > 0.f) acc += bf(dy[o]);
    }
    if (c < creal) atomicAdd(&db[c], acc);
}

// Operands of the pipelined backward pass of a layer, from its output gradient dy and output y
// (ReLU mask; null: none), C channels (a multiple of 8, <= 128), 64 pixels per block of 256
// threads: dym[p][c] = the masked gradient (pixel-major, for the data gradient), dyT[c][p]
// (channel-major, for the weight gradient), and the bias gradient db[c] += sum over the
// block's pixels (c < creal). 16-byte loads and stores; the transpose goes through shared
// memory with rows padded to C + 8 values.
// blocked: dyT in 64-pixel blocks, dyT[(p / 64) C + c][p % 64], so that a block's C rows are
// one contiguous 128 C-byte run. dyT null: no transposed copy (the MN-major weight gradient).
__global__ void __launch_bounds__(256)
    grad_prep_kernel(const bf16 *__restrict__ dy, const bf16 *__restrict__ y,
                     bf16 *__restrict__ dym, bf16 *__restrict__ dyT, float *__restrict__ db,
                     int npix, int C, int creal, int blocked)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ __align__(16) bf16 tile[64][136];
    const int p0 = blockIdx.x * 64;
    const int cv = C / 8;
    for (int e = threadIdx.x; e < 64 * cv; e += blockDim.x) {
        const int i = e / cv, c8 = (e - i * cv) * 8, p = p0 + i;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (p < npix) {
            const size_t o = (size_t)p * C + c8;
            v = *reinterpret_cast<const uint4 *>(dy + o);
            if (y) v = relu_mask(v, *reinterpret_cast<const uint4 *>(y + o));
            *reinterpret_cast<uint4 *>(dym + o) = v;
        }
        *reinterpret_cast<uint4 *>(&tile[i][c8]) = v;
    }
    __syncthreads();
    if (threadIdx.x < creal) {
        float acc = 0.f;
        for (int i = 0; i < 64; ++i) acc += bf(tile[i][threadIdx.x]);
        atomicAdd(&db[threadIdx.x], acc);
    }
    for (int e = threadIdx.x; dyT && e < 8 * C; e += blockDim.x) {  // 8 runs of 8 pixels per channel
        const int c = e / 8, j = (e - c * 8) * 8;
        if (p0 + j >= npix) continue;  // npix is a multiple of 8
        bf16 r[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = tile[j + k][c];
        const size_t o = blocked ? ((size_t)blockIdx.x * C + c) * 64 + j : (size_t)c * npix + p0 + j;
        *reinterpret_cast<uint4 *>(dyT + o) = *reinterpret_cast<uint4 *>(r);
    }
}

// The output layer's backward pass fused with grad_prep_kernel of the layer below it (c1, 32
// channels, ReLU). The output layer is 1 x 1 from 32 channels to 1, so its data gradient is
// the outer product dx[p][c] = bf16(g[p] wo[c]) of the output gradient g (channel 0 of dyo)
// and its weights (exact in FP32, as the GEMM form gives it), and its weight and bias gradients
// are gw_out[c] += sum_p g[p] x[p][c], gb_out += sum_p g[p], with x = y = c1, the layer's input.
// dyo is the compact output gradient (one value per pixel).
// dx is masked by c1's ReLU and written as grad_prep_kernel writes it (dym, dyT unless null,
// db of c1).
// 64 pixels per block of 256 threads.
__global__ void __launch_bounds__(256)
    out_grad_prep_kernel(const bf16 *__restrict__ dyo, const bf16 *__restrict__ wo,
                         const bf16 *__restrict__ y, bf16 *__restrict__ dym,
                         bf16 *__restrict__ dyT, float *__restrict__ db,
                         float *__restrict__ gw_out, float *__restrict__ gb_out, int npix,
                         int blocked)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    constexpr int C = 32;
    __shared__ __align__(16) bf16 tile[64][C + 8];
    __shared__ __align__(16) bf16 ytile[64][C + 8];
    __shared__ float g[64];
    const int p0 = blockIdx.x * 64;
    if (threadIdx.x < 64) {
        const int p = p0 + threadIdx.x;
        g[threadIdx.x] = p < npix ? bf(dyo[p]) : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * (C / 8); e += blockDim.x) {
        const int i = e / (C / 8), c8 = (e % (C / 8)) * 8, p = p0 + i;
        uint4 v = make_uint4(0, 0, 0, 0), yv = make_uint4(0, 0, 0, 0);
        if (p < npix) {
            const size_t o = (size_t)p * C + c8;
            yv = *reinterpret_cast<const uint4 *>(y + o);
            uint4 d;
            bf16 *dv = reinterpret_cast<bf16 *>(&d);
#pragma unroll
            for (int k = 0; k < 8; ++k) dv[k] = __float2bfloat16(g[i] * bf(wo[c8 + k]));
            v = relu_mask(d, yv);
            *reinterpret_cast<uint4 *>(dym + o) = v;
        }
        *reinterpret_cast<uint4 *>(&tile[i][c8]) = v;
        *reinterpret_cast<uint4 *>(&ytile[i][c8]) = yv;
    }
    __syncthreads();
    if (threadIdx.x < C) {
        float acc = 0.f, accw = 0.f;
        for (int i = 0; i < 64; ++i) {
            acc += bf(tile[i][threadIdx.x]);
            accw = fmaf(g[i], bf(ytile[i][threadIdx.x]), accw);
        }
        atomicAdd(&db[threadIdx.x], acc);
        atomicAdd(&gw_out[threadIdx.x], accw);
    } else if (threadIdx.x == C) {
        float acc = 0.f;
        for (int i = 0; i < 64; ++i) acc += g[i];
        atomicAdd(gb_out, acc);
    }
    for (int e = threadIdx.x; dyT && e < 8 * C; e += blockDim.x) {  // 8 runs of 8 pixels per channel
        const int c = e / 8, j = (e - c * 8) * 8;
        if (p0 + j >= npix) continue;  // npix is a multiple of 8
        bf16 r[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) r[k] = tile[j + k][c];
        const size_t o = blocked ? ((size_t)blockIdx.x * C + c) * 64 + j : (size_t)c * npix + p0 + j;
        *reinterpret_cast<uint4 *>(dyT + o) = *reinterpret_cast<uint4 *>(r);
    }
}

// Weight and bias gradients of the first layer (2 -> 32 channels, 3 x 3, ReLU) on the CUDA
// cores: gw[co][t][ci] += sum_p m[p][co] x0[p + off(t)][ci] and gb[co] += sum_p m[p][co], with
// m = dy masked by y > 0 (dy, y: (Bn, H, W, 32) BF16), x0 the packed 8-channel input (channels
// 0 and 1), gw in the padded [co][tap][8] layout, taps t = (dh + 1) 3 + dw + 1. A GEMM over
// K = pixels would leave the tensor core idle behind transposed copies of dy and x0. A thread
// owns four output channels (72 products per pixel from one 8-byte gradient load and three new
// input pairs) and walks runs of kE1Run pixels along a row with the 3 x 3 x 2 input window in
// registers; the four threads of a warp that share a channel quad are summed by shuffles, the
// warps in shared memory, and each block adds to gw / gb atomically. W is a multiple of kE1Run.
constexpr int kE1Run = 16;
__global__ void __launch_bounds__(256, 2)
    e1_wgrad_kernel(const bf16 *__restrict__ dy, const bf16 *__restrict__ y,
                    const bf16 *__restrict__ x0, float *__restrict__ gw, float *__restrict__ gb,
                    int Bn, int H, int W)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ float red[8][8][76];  // [warp][channel quad][4 x 18 taps, 4 biases]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int cq = lane & 7;                      // channels 4 cq .. 4 cq + 3
    const int slot = warp * 4 + (lane >> 3);      // 32 runs per block iteration
    float acc[4][18], accb[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int k = 0; k < 18; ++k) acc[q][k] = 0.f;
    const int wr = W / kE1Run;
    const long long nruns = (long long)Bn * H * wr;
    for (long long run = (long long)blockIdx.x * 32 + slot; run < nruns; run += (long long)gridDim.x * 32) {
        const int w0 = (int)(run % wr) * kE1Run;
        const long long rh = run / wr;
        const int h = (int)(rh % H), n = (int)(rh / H);
        // loads at clamped addresses, zeroed outside the image, so that they do not depend on
        // branches and the unrolled loop can issue them early
        auto ld = [&](int hh, int ww, float (&v)[2]) {
            const bool ok = hh >= 0 && hh < H && ww >= 0 && ww < W;
            const size_t idx = ok ? ((size_t)(n * H + hh) * W + ww) * 8 : 0;
            const __nv_bfloat162 t = *reinterpret_cast<const __nv_bfloat162 *>(x0 + idx);
            v[0] = ok ? __low2float(t) : 0.f;
            v[1] = ok ? __high2float(t) : 0.f;
        };
        float xw[3][3][2];  // rows h - 1 .. h + 1, columns w - 1 .. w + 1, 2 channels
#pragma unroll
        for (int dh = 0; dh < 3; ++dh) {
            ld(h - 1 + dh, w0 - 1, xw[dh][0]);
            ld(h - 1 + dh, w0, xw[dh][1]);
        }
        const size_t o0 = ((size_t)(n * H + h) * W + w0) * 32 + 4 * cq;
#pragma unroll 2
        for (int k = 0; k < kE1Run; ++k) {
            const int w = w0 + k;
#pragma unroll
            for (int dh = 0; dh < 3; ++dh) ld(h - 1 + dh, w + 1, xw[dh][2]);
            const uint2 dd = *reinterpret_cast<const uint2 *>(dy + o0 + k * 32);
            const uint2 yy = *reinterpret_cast<const uint2 *>(y + o0 + k * 32);
            const bf16 *dv = reinterpret_cast<const bf16 *>(&dd);
            const bf16 *yv = reinterpret_cast<const bf16 *>(&yy);
            float m[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                m[q] = bf(yv[q]) > 0.f ? bf(dv[q]) : 0.f;
                accb[q] += m[q];
            }
#pragma unroll
            for (int dh = 0; dh < 3; ++dh)
#pragma unroll
                for (int dx = 0; dx < 3; ++dx)
#pragma unroll
                    for (int ci = 0; ci < 2; ++ci) {
                        const int t = (dh * 3 + dx) * 2 + ci;
#pragma unroll
                        for (int q = 0; q < 4; ++q) acc[q][t] = fmaf(m[q], xw[dh][dx][ci], acc[q][t]);
                    }
#pragma unroll
            for (int dh = 0; dh < 3; ++dh) {
#pragma unroll
                for (int ci = 0; ci < 2; ++ci) {
                    xw[dh][0][ci] = xw[dh][1][ci];
                    xw[dh][1][ci] = xw[dh][2][ci];
                }
            }
        }
    }
    // lanes cq, cq + 8, cq + 16, cq + 24 hold the same channels
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int k = 0; k < 18; ++k) {
            float v = acc[q][k];
            v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            if (lane < 8) red[warp][cq][q * 18 + k] = v;
        }
        float b = accb[q];
        b += __shfl_xor_sync(0xffffffffu, b, 8);
        b += __shfl_xor_sync(0xffffffffu, b, 16);
        if (lane < 8) red[warp][cq][72 + q] = b;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 8 * 76; e += blockDim.x) {
        const int c = e / 76, k = e - c * 76;
        float t = 0.f;
#pragma unroll
        for (int wv = 0; wv < 8; ++wv) t += red[wv][c][k];
        if (k < 72) {
            const int co = 4 * c + k / 18, tk = k % 18, tap = tk / 2, ci = tk % 2;
            atomicAdd(&gw[co * 72 + tap * 8 + ci], t);
        } else {
            atomicAdd(&gb[4 * c + (k - 72)], t);
        }
    }
}

// xT[s][c][q] = x[p + s - nshift / 2][c] when that pixel is in p's image row, else 0, for the
// nshift column shifts s (3 for a 3 x 3 kernel: -1, 0, +1; 1 for 1 x 1: 0). q is p's position
// in the row-padded layout, q = (n (H + 2) + h + 1) W + w, with a zero row above and below each
// image (written here too), so that a tap's row shift is a whole-row offset that reads zeros at
// the image's edges. qtot = B (H + 2) W. C a multiple of 8, <= 128; 64 pixels per block.
// blocked (W a multiple of 64): xT in 64-position blocks of the padded layout,
// xT[(s qtot / 64 + q / 64) C + c][q % 64].
__global__ void __launch_bounds__(256)
    shift_transpose_kernel(const bf16 *__restrict__ x, bf16 *__restrict__ xT, int npix, int H,
                           int W, int C, int nshift, long long qtot, int blocked)
{
    __shared__ __align__(16) bf16 tile[66][136];  // pixels p0 - 1 .. p0 + 64
    const int p0 = blockIdx.x * 64;
    const int cv = C / 8;
    for (int e = threadIdx.x; e < 66 * cv; e += blockDim.x) {
        const int i = e / cv, c8 = (e - i * cv) * 8, p = p0 - 1 + i;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (p >= 0 && p < npix) v = *reinterpret_cast<const uint4 *>(x + (size_t)p * C + c8);
        *reinterpret_cast<uint4 *>(&tile[i][c8]) = v;
    }
    __syncthreads();
    const int half = nshift / 2, hw = H * W;
    for (int e = threadIdx.x; e < nshift * 8 * C; e += blockDim.x) {
        const int sc = e / 8, j = (e - sc * 8) * 8;  // sc = shift * C + c
        const int sh = sc / C, c = sc - sh * C, p = p0 + j;
        if (p >= npix) continue;  // npix is a multiple of 8 and W of 8: a run stays in one row
        const int dw = sh - half;
        const int n = p / hw, r = p - n * hw, h = r / W, w0 = r - h * W;
        bf16 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int w = w0 + k;
            v[k] = (w + dw >= 0 && w + dw < W) ? tile[j + k + 1 + dw][c] : __float2bfloat16(0.f);
        }
        const long long q = ((long long)n * (H + 2) + h + 1) * W + w0;
        auto at = [&](long long qq) {
            return blocked ? xT + (((size_t)sh * (qtot / 64) + qq / 64) * C + c) * 64 + qq % 64
                           : xT + (size_t)sc * qtot + qq;
        };
        *reinterpret_cast<uint4 *>(at(q)) = *reinterpret_cast<uint4 *>(v);
        if (h == 0) *reinterpret_cast<uint4 *>(at(q - W)) = make_uint4(0, 0, 0, 0);
        if (h == H - 1) *reinterpret_cast<uint4 *>(at(q + W)) = make_uint4(0, 0, 0, 0);
    }
}

// Adam step on a flat parameter vector; bias correction folded into the step size
__global__ void adam_kernel(float *__restrict__ w, const float *__restrict__ g,
                            float *__restrict__ m, float *__restrict__ v, long long n, float lr,
                            float b1, float b2, float eps, float c1, float c2)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(i, n)
    {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// Zeroes up to 16 FP32 buffers in one launch (the gradient accumulators of a backward pass)
struct ZeroList {
    float *p[16];
    long long off[17];
    int count;
};
__global__ void zero_kernel(const ZeroList L)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(e, L.off[L.count])
    {
        int b = 0;
        while (b < L.count - 1 && e >= L.off[b + 1]) ++b;
        L.p[b][e - L.off[b]] = 0.f;
    }
}

// Every layer's weight refresh (after an Adam step) or gradient gather in one launch: the
// layers' index spaces are concatenated (off[l] .. off[l + 1]).
struct AllLayers {
    const float *src[kNumLayers];
    float *dst32[kNumLayers];
    bf16 *fwd[kNumLayers], *bwd[kNumLayers];
    int cin[kNumLayers], cout[kNumLayers], cin_p[kNumLayers], cout_p[kNumLayers], taps[kNumLayers];
    long long off[kNumLayers + 1];
};

__device__ __forceinline__ int layer_of(const AllLayers &P, long long e)
{
    int l = 0;
    while (l < kNumLayers - 1 && e >= P.off[l + 1]) ++l;
    return l;
}

// BF16 copies of the FP32 weights src: fwd[co][tap cin_p + ci], bwd[ci][tap cout_p + co] (zero in
// the padding); index space cout_p taps cin_p
__global__ void refresh_all_kernel(const AllLayers P)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(e, P.off[kNumLayers])
    {
        const int l = layer_of(P, e);
        const long long k = e - P.off[l];
        const int cin_p = P.cin_p[l], taps = P.taps[l];
        const int ci = (int)(k % cin_p);
        const long long r = k / cin_p;
        const int t = (int)(r % taps), co = (int)(r / taps);
        float v = 0.f;
        if (co < P.cout[l] && ci < P.cin[l]) v = P.src[l][((size_t)co * taps + t) * P.cin[l] + ci];
        const bf16 b = __float2bfloat16(v);
        P.fwd[l][((size_t)co * taps + t) * cin_p + ci] = b;
        P.bwd[l][((size_t)ci * taps + t) * P.cout_p[l] + co] = b;
    }
}

// the padded FP32 weight gradients src [cout_p][taps cin_p] gathered into the flat parameter
// layout dst32 [cout][taps][cin]; index space cout taps cin
__global__ void gather_all_kernel(const AllLayers P)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    LENTILS_GRID_STRIDE(e, P.off[kNumLayers])
    {
        const int l = layer_of(P, e);
        const long long k = e - P.off[l];
        const int cin = P.cin[l], taps = P.taps[l];
        const int ci = (int)(k % cin);
        const long long r = k / cin;
        const int t = (int)(r % taps), co = (int)(r / taps);
        P.dst32[l][k] = P.src[l][(size_t)co * taps * P.cin_p[l] + (size_t)t * P.cin_p[l] + ci];
    }
}


// Preconditioner pieces (one sample of n = H * W values):
//   u = dinv * r, s = rms(u) (1 where u = 0), x0 = (u / s, feat, 0...),
//   z = gamma * u + s * out
__global__ void __launch_bounds__(1024)
    precond_scale_kernel(const float *__restrict__ r, const float *__restrict__ dinv, int n,
                         float *__restrict__ scale)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    __shared__ double sh[32];
    __shared__ float shm[32];
    // FP64 arithmetic is slow on this part: the sum of squares is taken in FP32 on values scaled
    // by the largest |u| (no overflow or underflow of the squares that matter), FP64 across
    // threads
    // 16-byte loads, four per array in flight per thread at 128^2, where the pointers allow
    const bool vec = ((reinterpret_cast<uintptr_t>(r) | reinterpret_cast<uintptr_t>(dinv)) & 15) == 0 &&
                     (n & 3) == 0;
    const float4 *r4 = reinterpret_cast<const float4 *>(r);
    const float4 *d4 = reinterpret_cast<const float4 *>(dinv);
    float m = 0.f;
    if (vec) {
#pragma unroll 4
        for (int i = threadIdx.x; i < n / 4; i += blockDim.x) {
            const float4 a = r4[i], b = d4[i];
            m = fmaxf(fmaxf(m, fabsf(b.x * a.x)), fmaxf(fabsf(b.y * a.y), fmaxf(fabsf(b.z * a.z), fabsf(b.w * a.w))));
        }
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, fabsf(dinv[i] * r[i]));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = m;
    __syncthreads();
    m = 0.f;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) m = fmaxf(m, shm[i]);
    if (!(m > 0.f) || !(m < INFINITY)) {  // zero, NaN or infinite
        if (threadIdx.x == 0) scale[0] = 1.f;
        return;
    }
    const float inv = 1.f / m;
    float part = 0.f;
    if (vec) {
#pragma unroll 4
        for (int i = threadIdx.x; i < n / 4; i += blockDim.x) {
            const float4 a = r4[i], b = d4[i];
            const float u0 = b.x * a.x * inv, u1 = b.y * a.y * inv, u2 = b.z * a.z * inv,
                        u3 = b.w * a.w * inv;
            part = fmaf(u0, u0, part);
            part = fmaf(u1, u1, part);
            part = fmaf(u2, u2, part);
            part = fmaf(u3, u3, part);
        }
    } else {
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const float u = dinv[i] * r[i] * inv;
            part = fmaf(u, u, part);
        }
    }
    double acc = part;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) scale[0] = (float)((double)m * sqrt(t / (double)n));
    }
}

__global__ void precond_input_kernel(const float *__restrict__ r, const float *__restrict__ dinv,
                                     const float *__restrict__ feat,
                                     const float *__restrict__ scale, bf16 *__restrict__ x0, int n)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    const float inv = 1.f / scale[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bf16 v[8];
        v[0] = __float2bfloat16(dinv[i] * r[i] * inv);
        v[1] = __float2bfloat16(feat[i]);
        for (int k = 2; k < 8; ++k) v[k] = __float2bfloat16(0.f);
        *reinterpret_cast<uint4 *>(x0 + (size_t)i * 8) = *reinterpret_cast<uint4 *>(v);
    }
}

__global__ void precond_combine_kernel(const float *__restrict__ r, const float *__restrict__ dinv,
                                       const float *__restrict__ out,
                                       const float *__restrict__ scale, float gamma,
                                       float *__restrict__ z, int n)
{
    tc::pdl_wait();
    tc::pdl_trigger();
    const float s = scale[0];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        z[i] = fmaf(s, out[i], gamma * dinv[i] * r[i]);
}

// feat = log(dinv) - mean(log(dinv)), one block
__global__ void __launch_bounds__(1024)
    features_kernel(const float *__restrict__ dinv, float *__restrict__ feat, int n)
{
    __shared__ double sh[32];
    __shared__ double mean;
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += log((double)dinv[i]);
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) mean = t / (double)n;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) feat[i] = (float)(log((double)dinv[i]) - mean);
}

}  // namespace lentils

// ------------------------------------------------------------------------------------------------
// Network object
// ------------------------------------------------------------------------------------------------
struct lentils_unet {
    int H, W, maxB;
    int gemm_form;        // 0: persistent TMA convolutions with fused first / last layers,
                          // 1: synchronous staging, 2: per-tile TMA / cp.async-ring GEMMs
    int wgrad_ctas;       // CTAs of a weight-gradient GEMM (its pixel reduction is split to fill them)
    float jacobi_weight;  // gamma of the preconditioner form
    long long nparams;
    // per layer
    float *w32[lentils::kNumLayers], *b32[lentils::kNumLayers];  // views into params
    lentils::bf16 *wf[lentils::kNumLayers], *wb[lentils::kNumLayers];
    float *gw_pad[lentils::kNumLayers];  // FP32 weight gradients, padded layout
    float *gw[lentils::kNumLayers], *gb[lentils::kNumLayers];  // views into grads
    float *params, *grads, *adam_m, *adam_v;
    long long step;
    // activations (max batch)
    lentils::bf16 *x0, *e1, *p1, *e2, *p2, *e3, *p3, *b, *u3, *c3, *u2, *c2, *u1, *c1;
    float *out;
    float *pscale;  // preconditioner scale (device)
    float *splitk;  // FP32 partial slabs of split-K forward layers (kSplitSlabPix x 128)
    // gradients
    lentils::bf16 *dy_out, *d_c1, *d_u1, *d_c2, *d_u2, *d_c3, *d_u3, *d_b, *d_p3, *d_e3, *d_p2,
        *d_e2, *d_p1, *d_e1;
    // operands of the pipelined backward pass (sized for the largest layer)
    lentils::bf16 *dym, *dyT, *xT;
    float *loss;
    int *err;
    void *block;  // single allocation backing everything above
};

namespace lentils {

static long long layer_wcount(int l)
{
    const ConvSpec &s = kLayers[l];
    return (long long)s.cout * s.ks * s.ks * s.cin;
}

// raises the dynamic shared-memory limit of one kernel instantiation (once per process)
template <int N, class LA, class LB, class EP>
static cudaError_t gemm_smem_attr()
{
    static const cudaError_t e = cudaFuncSetAttribute(
        tc::gemm_kernel<N, LA, LB, EP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)tc::GemmSmem<N>::kBytes);
    return e;
}

// stages of the pipelined convolution GEMM (tc::gemm_pipe_kernel)
constexpr int kConvStages = 3;
// forward layers with fewer row tiles than this run the pipelined GEMM (measured at batch 32
// on 128^2: faster for 64 and 256 tiles, slower for 1024 and 4096)
constexpr int kPipeMaxTiles = 512;

template <int N, class LA, class LB, class EP>
static cudaError_t gemm_pipe_smem_attr()
{
    static const cudaError_t e = cudaFuncSetAttribute(
        tc::gemm_pipe_kernel<N, kConvStages, LA, LB, EP>,
        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::PipeSmem<N, kConvStages>::kBytes);
    return e;
}

// One convolution GEMM over grid (mtiles, 1, nz) with kp_per_split pieces per split; pipe
// selects tc::gemm_pipe_kernel (operands copied by cp.async; the loader must give addresses).
template <int N, class LA, class EP>
static int conv_gemm_launch(const LA &la, const tc::RowMajorLoader &lb, const EP &ep,
                            int mtiles, int kp, int per, int nz, bool pipe, int *err,
                            cudaStream_t s)
{
    if (pipe) {
        auto kern = tc::gemm_pipe_kernel<N, kConvStages, LA, tc::RowMajorLoader, EP>;
        LENTILS_CUDA_TRY((gemm_pipe_smem_attr<N, LA, tc::RowMajorLoader, EP>()));
        kern<<<dim3(mtiles, 1, nz), tc::kPipeThreads, tc::PipeSmem<N, kConvStages>::kBytes, s>>>(
            la, lb, ep, kp, per, err);
    } else {
        auto kern = tc::gemm_kernel<N, LA, tc::RowMajorLoader, EP>;
        LENTILS_CUDA_TRY((gemm_smem_attr<N, LA, tc::RowMajorLoader, EP>()));
        kern<<<dim3(mtiles, 1, nz), 128, tc::GemmSmem<N>::kBytes, s>>>(la, lb, ep, kp, per, err);
    }
    LENTILS_CHECK_LAUNCH("conv gemm");
    return LENTILS_OK;
}

template <int N, class LA, class EP>
static int conv_gemm(const LA &la, const tc::RowMajorLoader &lb, const EP &ep, int M, int K,
                     bool pipe, int *err, cudaStream_t s)
{
    const int kp = (K + 7) / 8;
    return conv_gemm_launch<N>(la, lb, ep, (M + 127) / 128, kp, kp, 1, pipe, err, s);
}

template <int N>
static int conv_gemm_split(const ConvFwdA &la, const tc::RowMajorLoader &lb,
                           const EpiPartialF32 &ep, int mtiles, int kp, int per, int nz, bool pipe,
                           int *err, cudaStream_t s)
{
    return conv_gemm_launch<N>(la, lb, ep, mtiles, kp, per, nz, pipe, err, s);
}

template <class LA, class EP>
static int conv_gemm_n(int N, const LA &la, const tc::RowMajorLoader &lb, const EP &ep, int M,
                       int K, bool pipe, int *err, cudaStream_t s)
{
    switch (N) {
    case 32: return conv_gemm<32>(la, lb, ep, M, K, pipe, err, s);
    case 64: return conv_gemm<64>(la, lb, ep, M, K, pipe, err, s);
    case 128: return conv_gemm<128>(la, lb, ep, M, K, pipe, err, s);
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "conv gemm N=%d", N);
}

// Weight gradient of a convolution layer as a GEMM whose operands are both MN-major, read
// straight from the pixel-major (NHWC) activations and gradients, with no transposed copies:
//   D[(t, ci)][co] = sum_p x[p + off(t)][ci] dym[p][co],   rows (t, ci) = t C + ci,
// K = pixels in chunks of 64 (consecutive in raster order, inside one image), one 128-row tile
// per blockIdx.x, the chunks split over blockIdx.y. An A tile is four boxes of 32 channels x 64
// pixels of x, each at its tap's pixel offset (the tensor map reads zeros outside the image,
// the convolution's padding); a B tile is N / 32 such boxes of dym at the chunk itself. With
// 64-byte rows and the 64-byte swizzle, a box is one 32-wide MN atom column: K groups of 8
// pixels 512 bytes apart (SBO), boxes 4096 bytes apart (LBO). Row tiles past the last tap
// leave their boxes unloaded; those rows of D are not written. The epilogue adds each row's N
// values to g[co][rows] with atomics (the per-split partial sums). Warps: 0-3 epilogue, lane 0
// of 4 the TMA producer, 5 TMEM and the MMA issuer. Waits are bounded (*err on a timeout).
constexpr int kWgMnThreads = 192;
constexpr int kWgMnStages = 4;

template <int N>
struct WgMnSmem {
    static constexpr int kA = 4 * 4096, kB = N / 32 * 4096, kStage = kA + kB;
    static constexpr int kBytes = kWgMnStages * kStage + 1024;
};

template <int N>
__global__ void __launch_bounds__(kWgMnThreads, 1)
    wgrad_mn_kernel(const __grid_constant__ CUtensorMap mx, const __grid_constant__ CUtensorMap mdy,
                    float *__restrict__ g, int C, int ks, int H, int W, int rows, int nchunks,
                    int per_cta, int *err)
{
    constexpr int S = kWgMnStages;
    constexpr int kA = WgMnSmem<N>::kA, kStage = WgMnSmem<N>::kStage;
    constexpr uint32_t ncols = N < 32 ? 32 : N;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t full[S], empty[S], done;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    unsigned char *smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = blockIdx.x;
    const int c0 = blockIdx.y * per_cta, c1 = min(nchunks, c0 + per_cta);
    const int nch = c1 > c0 ? c1 - c0 : 0;
    if (warp == 5) {
        tc::tmem_alloc(&tmem_base, ncols);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            tc::mbar_init(&full[i], 1);
            tc::mbar_init(&empty[i], 1);
        }
        tc::mbar_init(&done, 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    if (threadIdx.x == 128) {
        tc::prefetch_tensormap(&mx);
        tc::prefetch_tensormap(&mdy);
    }
    tc::pdl_wait();
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    tc::pdl_trigger();
    const uint32_t tmem = tmem_base;

    if (warp == 4) {
        if (lane == 0) {  // the TMA producer
            // the tile's four boxes: tap offset and first channel (fixed for the CTA)
            int bdh[4], bdw[4], bci[4], nvalid = 0;
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int r0 = mt * 128 + 32 * b, t = r0 / C;
                bci[b] = r0 - t * C;
                bdh[b] = t / ks - ks / 2;
                bdw[b] = t % ks - ks / 2;
                if (r0 < rows) nvalid = b + 1;
            }
            const uint32_t bytes = (uint32_t)nvalid * 4096u + (uint32_t)N / 32u * 4096u;
            // the first chunk's pixel, then 64 pixels per chunk
            const int hw = H * W;
            const long long p0 = (long long)c0 * 64;
            int n = (int)(p0 / hw), r = (int)(p0 - (long long)n * hw), h = r / W, w0 = r - h * W;
            const int hstep = W >= 64 ? 0 : 64 / W;
            int it = 0;
            for (; it < nch; ++it) {
                const int st = it % S;
                if (it >= S && !tc::mbar_wait(&empty[st], ((it / S) - 1) & 1)) {
                    atomicExch(&abort_flag, 1);
                    break;
                }
                unsigned char *sa = smem + st * kStage;
                tc::mbar_arrive_expect_tx(&full[st], bytes);
#pragma unroll
                for (int b = 0; b < 4; ++b)
                    if (b < nvalid)
                        tc::tma_load_4d(sa + 4096 * b, &mx, bci[b], w0 + bdw[b], h + bdh[b], n, &full[st]);
#pragma unroll
                for (int b = 0; b < N / 32; ++b)
                    tc::tma_load_4d(sa + kA + 4096 * b, &mdy, 32 * b, w0, h, n, &full[st]);
                if (hstep == 0) {
                    w0 += 64;
                    if (w0 == W) {
                        w0 = 0;
                        if (++h == H) {
                            h = 0;
                            ++n;
                        }
                    }
                } else {
                    h += hstep;
                    if (h >= H) {
                        h -= H;
                        ++n;
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < S; ++i) {
                if (i >= it) continue;
                const int last = i + ((it - 1 - i) / S) * S;
                if (!tc::mbar_wait(&full[i], (last / S) & 1)) atomicExch(&abort_flag, 1);
            }
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {  // the MMA issuer
            constexpr uint32_t idesc = tc::idesc_bf16_f32_mn(128, N);
            for (int it = 0; it < nch; ++it) {
                const int st = it % S;
                if (!tc::mbar_wait(&full[st], (it / S) & 1)) {
                    atomicExch(&abort_flag, 1);
                    break;
                }
                tc::tc_fence_after();
                const uint32_t sa = tc::smem_u32(smem + st * kStage), sb = sa + kA;
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    tc::mma_bf16(tmem, tc::smem_desc_mn_sw64(sa + 1024 * k, 4096, 512),
                                 tc::smem_desc_mn_sw64(sb + 1024 * k, 4096, 512), idesc,
                                 (it > 0 || k > 0) ? 1u : 0u);
                tc::mma_commit(&empty[st]);
            }
            tc::mma_commit(&done);
        }
        __syncwarp();
    }
    const bool fin = tc::mbar_wait(&done, 0);
    tc::tc_fence_after();
    __syncthreads();
    const bool bad = !fin || *(volatile int *)&abort_flag;
    if (threadIdx.x == 0 && bad) atomicExch(err, 1);
    if (!bad && nch > 0 && warp < 4) {
        const int r = mt * 128 + warp * 32 + lane;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
        for (int n0 = 0; n0 < N; n0 += 32) {
            uint32_t v[32];
            tc::tmem_ld32(taddr + n0, v);
            tc::tmem_wait_ld();
            if (r < rows) {
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float f = __uint_as_float(v[i]);
                    if (f != 0.f) atomicAdd(&g[(size_t)(n0 + i) * rows + r], f);
                }
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 5) tc::tmem_dealloc(tmem, ncols);
}

// Launches wgrad_mn_kernel for layer input x (C channels) and masked output gradient dym
// (N = cout_p channels), Bn images of H x W, accumulating into g (padded [co][t][ci] layout).
template <int N>
static int wgrad_mn_launch(const bf16 *x, const bf16 *dym, float *g, int C, int ks, int Bn, int H,
                           int W, int ctas_want, int *err, cudaStream_t s)
{
    const int WB = std::min(W, 64), HB = 64 / WB;
    CUtensorMap mx, mdy;
    const uint64_t dx[4] = {(uint64_t)C, (uint64_t)W, (uint64_t)H, (uint64_t)Bn};
    const uint64_t sx[3] = {(uint64_t)C * 2, (uint64_t)W * C * 2, (uint64_t)H * W * C * 2};
    const uint32_t bx[4] = {32, (uint32_t)WB, (uint32_t)HB, 1};
    if (int st = tma_map_bf16(&mx, x, 4, dx, sx, bx, 64)) return st;
    const uint64_t dd[4] = {(uint64_t)N, (uint64_t)W, (uint64_t)H, (uint64_t)Bn};
    const uint64_t sd[3] = {(uint64_t)N * 2, (uint64_t)W * N * 2, (uint64_t)H * W * N * 2};
    if (int st = tma_map_bf16(&mdy, dym, 4, dd, sd, bx, 64)) return st;
    const int rows = ks * ks * C, mtiles = (rows + 127) / 128;
    const int nchunks = Bn * H * W / 64;
    const int want = std::max(1, ctas_want / mtiles);
    const int per = std::max(8, (nchunks + want - 1) / want);
    const int nsplit = (nchunks + per - 1) / per;
    auto kern = wgrad_mn_kernel<N>;
    static const cudaError_t attr = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, WgMnSmem<N>::kBytes);
    LENTILS_CUDA_TRY(attr);
    LENTILS_CUDA_TRY(pdl_launch(kern, dim3(mtiles, nsplit), dim3(kWgMnThreads),
                                (size_t)WgMnSmem<N>::kBytes, s, mx, mdy, g, C, ks, H, W, rows,
                                nchunks, per, err));
    LENTILS_CHECK_LAUNCH("weight gradient gemm (MN-major operands)");
    return LENTILS_OK;
}

// whether wgrad_mn_kernel takes a layer: 32-channel boxes, 64-pixel chunks inside an image
static bool wgrad_mn_ok(int C, int N, int H, int W)
{
    return C % 32 == 0 && C <= 128 && (N == 32 || N == 64 || N == 128) && (H * W) % 64 == 0 &&
           (W >= 64 ? W % 64 == 0 : (64 % W == 0 && H % (64 / W) == 0));
}

// the weight-gradient GEMM splits its pixel reduction so that about kWgradCtas CTAs run, each
// over at least kWgradMinPieces pieces of 8 pixels
constexpr int kWgradCtas = 1024;
constexpr int kWgradMinPieces = 64;
constexpr int kTmaStages = 4;

template <int N>
static int wgrad_tma_launch(const ConvWgXTTma &la, const bf16 *dyT, const uint64_t *db,
                            const uint64_t *sb, const uint32_t *bb, const EpiAtomicF32T &ep,
                            int mtiles, int kpieces, int per, int nz, int *err, cudaStream_t s)
{
    ConvWgDyTTma<N> lb;
    if (int st = tma_map_bf16(&lb.map, dyT, 2, db, sb, bb)) return st;
    auto kern = tc::gemm_tma_kernel<N, kTmaStages, ConvWgXTTma, ConvWgDyTTma<N>, EpiAtomicF32T>;
    static const cudaError_t attr = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::TmaSmem<N, kTmaStages>::kBytes);
    LENTILS_CUDA_TRY(attr);
    kern<<<dim3(mtiles, 1, nz), tc::kPipeThreads, tc::TmaSmem<N, kTmaStages>::kBytes, s>>>(
        la, lb, ep, kpieces, per, err);
    LENTILS_CHECK_LAUNCH("weight gradient gemm (TMA)");
    return LENTILS_OK;
}

template <int N>
static int wgrad_launch(const ConvWgXT &la, const ConvWgDyT &lb, const EpiAtomicF32T &ep,
                        int mtiles, int kpieces, int per, int nz, int *err, cudaStream_t s)
{
    auto kern = tc::gemm_pipe_kernel<N, kConvStages, ConvWgXT, ConvWgDyT, EpiAtomicF32T>;
    LENTILS_CUDA_TRY((gemm_pipe_smem_attr<N, ConvWgXT, ConvWgDyT, EpiAtomicF32T>()));
    kern<<<dim3(mtiles, 1, nz), tc::kPipeThreads, tc::PipeSmem<N, kConvStages>::kBytes, s>>>(
        la, lb, ep, kpieces, per, err);
    LENTILS_CHECK_LAUNCH("weight gradient gemm (pipelined)");
    return LENTILS_OK;
}

// A convolution GEMM with TMA operands: activations act (NHWC, C channels, Bn images of
// H x W; flip: data gradient), weights wt (row-major [N][K], K = ks^2 C), rows = pixels,
// split over nz CTAs of kp_per_split pieces along K.
template <int CB, int N, class EP>
static int conv_tma_launch(const bf16 *act, int C, int ks, int Bn, int H, int W, int flip,
                           const bf16 *wt, int K, const EP &ep, int nz, int kp_per_split,
                           int *err, cudaStream_t s)
{
    constexpr int kStages = (CB == 64 && N == 128) ? 3 : 4;
    ConvTmaA<CB> la;
    la.C = C;
    la.ks = ks;
    la.H = H;
    la.W = W;
    la.flip = flip;
    const int WB = std::min(W, 128), HB = 128 / WB;
    const uint64_t da[4] = {(uint64_t)C, (uint64_t)W, (uint64_t)H, (uint64_t)Bn};
    const uint64_t sa[3] = {(uint64_t)C * 2, (uint64_t)W * C * 2, (uint64_t)H * W * C * 2};
    const uint32_t ba[4] = {(uint32_t)CB, (uint32_t)WB, (uint32_t)HB, 1};
    if (int st = tma_map_bf16(&la.map, act, 4, da, sa, ba, 2 * CB)) return st;
    ConvTmaB<CB, N> lb;
    const uint64_t db[2] = {(uint64_t)K, (uint64_t)N};
    const uint64_t sb[1] = {(uint64_t)K * 2};
    const uint32_t bb[2] = {(uint32_t)CB, (uint32_t)N};
    if (int st = tma_map_bf16(&lb.map, wt, 2, db, sb, bb, 2 * CB)) return st;
    auto kern = tc::gemm_tma_kernel<N, kStages, ConvTmaA<CB>, ConvTmaB<CB, N>, EP>;
    constexpr int smem = tc::TmaSmem<N, kStages, CB>::kBytes;
    static const cudaError_t attr =
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    LENTILS_CUDA_TRY(attr);
    const int mtiles = Bn * H * W / 128;
    LENTILS_CUDA_TRY(pdl_launch(kern, dim3(mtiles, 1, nz), dim3(tc::kPipeThreads), smem, s, la, lb, ep,
                                K / 8, kp_per_split, err));
    LENTILS_CHECK_LAUNCH("convolution gemm (TMA)");
    return LENTILS_OK;
}

static int num_sms()
{
    static const int n = [] {
        int dev = 0, v = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return 0;
        return v;
    }();
    return n;
}

// CTAs per SM of a persistent GEMM instantiation: as many as the SM's shared memory, registers
// and threads hold, and at most as many as fit their tensor memory (2 N columns each, 512 per
// SM). Counted from the kernel's attributes (the occupancy query reported one CTA per SM for
// these kernels where the hardware holds two or three).
struct PersistShape {
    cudaError_t err;
    int per_sm;
};
template <class Kern>
static PersistShape persist_shape(Kern kern, int smem, int tmem_cols)
{
    PersistShape r{cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem), 1};
    if (r.err == cudaSuccess)
        r.err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared);
    cudaFuncAttributes fa;
    int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0;
    if (r.err == cudaSuccess) r.err = cudaFuncGetAttributes(&fa, kern);
    if (r.err == cudaSuccess) r.err = cudaGetDevice(&dev);
    if (r.err == cudaSuccess)
        r.err = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (r.err == cudaSuccess)
        r.err = cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (r.err == cudaSuccess)
        r.err = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    if (r.err != cudaSuccess) return r;
    const int by_smem = smem_sm / (smem + (int)fa.sharedSizeBytes + reserved);
    // registers are allocated per warp in units of 256
    const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256;
    const int by_regs = regs_sm / (warp_regs * (tc::kPersistThreads / 32));
    const int by_threads = 2048 / tc::kPersistThreads;
    r.per_sm = std::max(1, std::min(std::min(by_smem, by_regs), std::min(by_threads, 512 / tmem_cols)));
    return r;
}

template <int CB>
constexpr int persist_stages(int N)
{
    return CB == 32 ? 6 : (N == 128 ? 3 : 4);
}

// shared-memory limit and CTAs per SM of one persistent convolution instantiation (set up once
// per process)
template <int CB, int N, class EP>
static const PersistShape &conv_persist_shape()
{
    constexpr int kStages = persist_stages<CB>(N);
    static const PersistShape shape = persist_shape(
        tc::gemm_tma_persist_kernel<N, kStages, ConvTmaA<CB>, ConvTmaB<CB, N>, EP>,
        tc::TmaSmem<N, kStages, CB>::kBytes, 2 * N <= 64 ? 64 : 2 * N);
    return shape;
}

// The convolution GEMM with TMA operands as a persistent kernel (whole K per tile, row
// epilogue), one wave of CTAs over all row tiles.
template <int CB, int N, class EP>
static int conv_persist_launch(const bf16 *act, int C, int ks, int Bn, int H, int W, int flip,
                               const bf16 *wt, int K, const EP &ep, int *err, cudaStream_t s)
{
    constexpr int kStages = persist_stages<CB>(N);
    ConvTmaA<CB> la;
    la.C = C;
    la.ks = ks;
    la.H = H;
    la.W = W;
    la.flip = flip;
    const int WB = std::min(W, 128), HB = 128 / WB;
    const uint64_t da[4] = {(uint64_t)C, (uint64_t)W, (uint64_t)H, (uint64_t)Bn};
    const uint64_t sa[3] = {(uint64_t)C * 2, (uint64_t)W * C * 2, (uint64_t)H * W * C * 2};
    const uint32_t ba[4] = {(uint32_t)CB, (uint32_t)WB, (uint32_t)HB, 1};
    if (int st = tma_map_bf16(&la.map, act, 4, da, sa, ba, 2 * CB)) return st;
    ConvTmaB<CB, N> lb;
    const uint64_t db[2] = {(uint64_t)K, (uint64_t)N};
    const uint64_t sb[1] = {(uint64_t)K * 2};
    const uint32_t bb[2] = {(uint32_t)CB, (uint32_t)N};
    if (int st = tma_map_bf16(&lb.map, wt, 2, db, sb, bb, 2 * CB)) return st;
    auto kern = tc::gemm_tma_persist_kernel<N, kStages, ConvTmaA<CB>, ConvTmaB<CB, N>, EP>;
    constexpr int smem = tc::TmaSmem<N, kStages, CB>::kBytes;
    const PersistShape &shape = conv_persist_shape<CB, N, EP>();
    LENTILS_CUDA_TRY(shape.err);
    const int mtiles = Bn * H * W / 128;
    const int grid = std::min(mtiles, std::max(1, num_sms() * shape.per_sm));
    LENTILS_CUDA_TRY(pdl_launch(kern, dim3(grid), dim3(tc::kPersistThreads), smem, s, la, lb, ep,
                                mtiles, K / 8, err));
    LENTILS_CHECK_LAUNCH("convolution gemm (TMA, persistent)");
    return LENTILS_OK;
}

// flip: the data gradient (taps mirrored; act = the masked output gradient)
template <class EP>
static int conv_persist(const bf16 *act, int C, int ks, int Bn, int H, int W, int flip,
                        const bf16 *wt, int N, const EP &ep, int *err, cudaStream_t s)
{
    const int K = ks * ks * C;
    if (C == 32) {
        switch (N) {
        case 32: return conv_persist_launch<32, 32>(act, C, ks, Bn, H, W, flip, wt, K, ep, err, s);
        case 64: return conv_persist_launch<32, 64>(act, C, ks, Bn, H, W, flip, wt, K, ep, err, s);
        case 128: return conv_persist_launch<32, 128>(act, C, ks, Bn, H, W, flip, wt, K, ep, err, s);
        }
    } else {
        switch (N) {
        case 32: return conv_persist_launch<64, 32>(act, C, ks, Bn, H, W, flip, wt, K, ep, err, s);
        case 64: return conv_persist_launch<64, 64>(act, C, ks, Bn, H, W, flip, wt, K, ep, err, s);
        case 128: return conv_persist_launch<64, 128>(act, C, ks, Bn, H, W, flip, wt, K, ep, err, s);
        }
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "conv_persist: C=%d N=%d", C, N);
}

// 3 x 3 convolution from 32 to 32 channels on a grid 128 pixels wide (c1's forward and data
// gradient) with input-row reuse. A row tile is one image row; the implicit GEMM of the
// persistent kernel loads each input row nine times (three taps in each of three output rows,
// 64-byte box rows), and that L2 -> SM traffic bounds it. Here a CTA takes bands of kRowBand
// consecutive output rows of one image; each input row of the band (kRowBand + 2 of them) is
// loaded once, as three boxes shifted by -1, 0, +1 columns (the zero fill at the image edge is
// the padding), into a ring of kRowSlots slots; the output tile of row h reads its nine A
// operands from the slots of rows h - 1, h, h + 1, and the slot of row h - 1 is released (MMA
// commit) after it. The 9 x 32 x 32 weights stay in shared memory. Accumulators double
// buffered in TMEM and the row epilogues as in tc::gemm_tma_persist_kernel. flip: taps mirrored
// (data gradient). Warps: 0-3 epilogue, lane 0 of 4 TMA, 5 TMEM + MMA.
constexpr int kRowBand = 4;
constexpr int kRowSlots = 6;
struct RowsSmem {
    static constexpr int kB = 9 * 2048, kVar = 8192, kSlot = 3 * kVar;
    static constexpr int kBytes = kB + kRowSlots * kSlot + 1024;
};

template <class EP>
__global__ void __launch_bounds__(tc::kPersistThreads, 1)
    conv3_rows_kernel(const __grid_constant__ CUtensorMap ma, const __grid_constant__ CUtensorMap mb,
                      const EP ep, int Bn, int H, int flip, int *err)
{
    constexpr int S = kRowSlots, R = kRowBand;
    constexpr int kB = RowsSmem::kB, kVar = RowsSmem::kVar, kSlot = RowsSmem::kSlot;
    constexpr uint32_t ncols = 64;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t bfull, sfull[S], sempty[S], tfull[2], tempty[2], mdone;
    __shared__ uint32_t tmem_base;
    __shared__ int abort_flag;
    __shared__ float scratch[256];
    unsigned char *smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
    unsigned char *bres = smem, *slots = smem + kB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bpi = (H + R - 1) / R, nbands = Bn * bpi;

    if (warp == 5) {
        tc::tmem_alloc(&tmem_base, ncols);
        tc::tmem_relinquish();
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(&bfull, 1);
        for (int i = 0; i < S; ++i) {
            tc::mbar_init(&sfull[i], 1);
            tc::mbar_init(&sempty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            tc::mbar_init(&tfull[i], 1);
            tc::mbar_init(&tempty[i], 4);
        }
        tc::mbar_init(&mdone, 1);
        abort_flag = 0;
        tc::fence_mbar_init();
    }
    if (threadIdx.x == 128) {
        tc::prefetch_tensormap(&ma);
        tc::prefetch_tensormap(&mb);
    }
    tc::pdl_wait();
    if (warp < 4) ep.prepare(scratch, threadIdx.x);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    tc::pdl_trigger();
    const uint32_t tmem = tmem_base;

    if (warp == 4) {
        if (lane == 0) {  // the TMA producer: the weights once, then each band's input rows
            tc::mbar_arrive_expect_tx(&bfull, 9 * 2048);
            for (int t = 0; t < 9; ++t) tc::tma_load_2d(bres + t * 2048, &mb, t * 32, 0, &bfull);
            int L = 0;
            bool ok = true;
            for (int b = blockIdx.x; b < nbands && ok; b += gridDim.x) {
                const int n = b / bpi, h0 = (b - n * bpi) * R, h1 = min(H, h0 + R);
                for (int r = h0 - 1; r <= h1; ++r, ++L) {
                    const int sl = L % S;
                    if (L >= S && !tc::mbar_wait(&sempty[sl], ((L / S) - 1) & 1)) {
                        atomicExch(&abort_flag, 1);
                        ok = false;
                        break;
                    }
                    unsigned char *dst = slots + sl * kSlot;
                    tc::mbar_arrive_expect_tx(&sfull[sl], 3 * kVar);
#pragma unroll
                    for (int v = 0; v < 3; ++v) tc::tma_load_4d(dst + v * kVar, &ma, 0, v - 1, r, n, &sfull[sl]);
                }
            }
            if (!tc::mbar_wait(&bfull, 0)) atomicExch(&abort_flag, 1);
#pragma unroll 1
            for (int i = 0; i < S; ++i) {
                if (i >= L) continue;
                const int last = i + ((L - 1 - i) / S) * S;
                if (!tc::mbar_wait(&sfull[i], (last / S) & 1)) atomicExch(&abort_flag, 1);
            }
        }
        __syncwarp();
    } else if (warp == 5) {
        if (lane == 0) {  // the MMA issuer
            constexpr uint32_t idesc = tc::idesc_bf16_f32(128, 32);
            bool ok = tc::mbar_wait(&bfull, 0);
            tc::tc_fence_after();
            int L = 0, j = 0;
            for (int b = blockIdx.x; b < nbands && ok; b += gridDim.x) {
                const int n = b / bpi, h0 = (b - n * bpi) * R, h1 = min(H, h0 + R);
                (void)n;
                const int nrows = h1 - h0 + 2;
                int ready = 0;  // loads of this band known to have landed
                for (int h = h0; h < h1 && ok; ++h, ++j) {
                    const int buf = j & 1;
                    if (j >= 2 && !tc::mbar_wait(&tempty[buf], ((j >> 1) - 1) & 1)) {
                        ok = false;
                        break;
                    }
                    while (ok && ready <= h - h0 + 2) {
                        const int Lr = L + ready;
                        ok = tc::mbar_wait(&sfull[Lr % S], (Lr / S) & 1);
                        ++ready;
                    }
                    if (!ok) break;
                    tc::tc_fence_after();
                    const uint32_t acc = tmem + (uint32_t)(buf * 32);
#pragma unroll
                    for (int t = 0; t < 9; ++t) {
                        int dh = t / 3 - 1, dw = t % 3 - 1;
                        if (flip) {
                            dh = -dh;
                            dw = -dw;
                        }
                        const int Lr = L + (h + dh) - (h0 - 1);
                        const uint32_t a = tc::smem_u32(slots + (Lr % S) * kSlot + (dw + 1) * kVar);
                        const uint32_t bb = tc::smem_u32(bres + t * 2048);
#pragma unroll
                        for (int k = 0; k < 2; ++k)
                            tc::mma_bf16(acc, tc::smem_desc_sw64(a + 32 * k), tc::smem_desc_sw64(bb + 32 * k),
                                         idesc, (t > 0 || k > 0) ? 1u : 0u);
                    }
                    tc::mma_commit(&tfull[buf]);
                    tc::mma_commit(&sempty[(L + h - h0) % S]);  // row h - 1: no later tile reads it
                }
                if (!ok) break;
                tc::mma_commit(&sempty[(L + nrows - 2) % S]);
                tc::mma_commit(&sempty[(L + nrows - 1) % S]);
                L += nrows;
            }
            if (!ok) atomicExch(&abort_flag, 1);
            tc::mma_commit(&mdone);
            if (!tc::mbar_wait(&mdone, 0)) atomicExch(&abort_flag, 1);
        }
        __syncwarp();
    } else {  // the epilogue warps
        const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
        int j = 0;
        bool go_on = true;
        for (int b = blockIdx.x; b < nbands && go_on; b += gridDim.x) {
            const int n = b / bpi, h0 = (b - n * bpi) * R, h1 = min(H, h0 + R);
            for (int h = h0; h < h1; ++h, ++j) {
                const int buf = j & 1;
                int go = 0;
                if (lane == 0)
                    go = tc::mbar_wait(&tfull[buf], (j >> 1) & 1) && !*(volatile int *)&abort_flag;
                go = __shfl_sync(0xffffffffu, go, 0);
                if (!go) {
                    if (lane == 0) atomicExch(&abort_flag, 1);
                    go_on = false;
                    break;
                }
                tc::tc_fence_after();
                const int m = ((n * H + h) << 7) + warp * 32 + lane;
                uint32_t r[32];
                tc::tmem_ld32(tmem + lane_base + (uint32_t)(buf * 32), r);
                tc::tmem_wait_ld();
                tc::tc_fence_before();
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&tempty[buf]);
                float v[32], acc = 0.f;
#pragma unroll
                for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
                ep.row(m, 0, v, acc, scratch);
                ep.row_end(m, acc, scratch);
            }
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (threadIdx.x == 0 && *(volatile int *)&abort_flag) atomicExch(err, 1);
    if (warp == 5) tc::tmem_dealloc(tmem, ncols);
}

template <class EP>
static const PersistShape &conv3_rows_shape()
{
    static const PersistShape shape = persist_shape(conv3_rows_kernel<EP>, RowsSmem::kBytes, 64);
    return shape;
}

// c1's convolution (32 -> 32 channels, 3 x 3, W = 128) on conv3_rows_kernel: act NHWC BF16,
// wt [32][288] BF16 (K = tap 32 + channel)
template <class EP>
static int conv3_rows_launch(const bf16 *act, int Bn, int H, int flip, const bf16 *wt, const EP &ep,
                             int *err, cudaStream_t s)
{
    constexpr int W = 128, C = 32;
    CUtensorMap ma, mb;
    const uint64_t da[4] = {(uint64_t)C, (uint64_t)W, (uint64_t)H, (uint64_t)Bn};
    const uint64_t sa[3] = {(uint64_t)C * 2, (uint64_t)W * C * 2, (uint64_t)H * W * C * 2};
    const uint32_t ba[4] = {32, 128, 1, 1};
    if (int st = tma_map_bf16(&ma, act, 4, da, sa, ba, 64)) return st;
    const uint64_t db[2] = {288, 32};
    const uint64_t sb[1] = {288 * 2};
    const uint32_t bb[2] = {32, 32};
    if (int st = tma_map_bf16(&mb, wt, 2, db, sb, bb, 64)) return st;
    const PersistShape &shape = conv3_rows_shape<EP>();
    LENTILS_CUDA_TRY(shape.err);
    const int nbands = Bn * ((H + kRowBand - 1) / kRowBand);
    const int grid = std::min(nbands, std::max(1, num_sms() * shape.per_sm));
    LENTILS_CUDA_TRY(pdl_launch(conv3_rows_kernel<EP>, dim3(grid), dim3(tc::kPersistThreads),
                                (size_t)RowsSmem::kBytes, s, ma, mb, ep, Bn, H, flip, err));
    LENTILS_CHECK_LAUNCH("conv3_rows_kernel");
    return LENTILS_OK;
}

// the band kernel for a convolution of Bn images of H x W: the shape it takes, and enough bands
// (kRowBand rows each) to give every SM one; with fewer (batch 1) the persistent GEMM's
// row tiles spread wider
static bool conv3_rows_ok(int C, int N, int ks, int W, int Bn, int H)
{
    return C == 32 && N == 32 && ks == 3 && W == 128 &&
           (long long)Bn * ((H + kRowBand - 1) / kRowBand) >= num_sms();
}

// whether a layer's convolution can take the TMA operands: row tiles of 128 pixels inside one
// image, CB-channel chunks, N in {32, 64, 128}
static bool conv_tma_ok(int C, int N, int H, int W)
{
    return (C == 32 || C == 64 || C == 128) && (N == 32 || N == 64 || N == 128) &&
           (H * W) % 128 == 0 && (W >= 128 ? W % 128 == 0 : 128 % W == 0);
}

template <class EP>
static int conv_tma(const bf16 *act, int C, int ks, int Bn, int H, int W, int flip,
                    const bf16 *wt, int N, const EP &ep, int nz, int kp_per_split, int *err,
                    cudaStream_t s)
{
    const int K = ks * ks * C;
    if (C == 32) {
        switch (N) {
        case 32: return conv_tma_launch<32, 32>(act, C, ks, Bn, H, W, flip, wt, K, ep, nz, kp_per_split, err, s);
        case 64: return conv_tma_launch<32, 64>(act, C, ks, Bn, H, W, flip, wt, K, ep, nz, kp_per_split, err, s);
        case 128: return conv_tma_launch<32, 128>(act, C, ks, Bn, H, W, flip, wt, K, ep, nz, kp_per_split, err, s);
        }
    } else {
        switch (N) {
        case 32: return conv_tma_launch<64, 32>(act, C, ks, Bn, H, W, flip, wt, K, ep, nz, kp_per_split, err, s);
        case 64: return conv_tma_launch<64, 64>(act, C, ks, Bn, H, W, flip, wt, K, ep, nz, kp_per_split, err, s);
        case 128: return conv_tma_launch<64, 128>(act, C, ks, Bn, H, W, flip, wt, K, ep, nz, kp_per_split, err, s);
        }
    }
    return set_error(LENTILS_ERR_UNSUPPORTED, "conv_tma: C=%d N=%d", C, N);
}

template <int N>
static int wgrad_tma_blk(const ConvWgXTTmaBlk &la, const bf16 *dyT, const uint64_t *db,
                         const uint64_t *sb, const uint32_t *bb, const EpiAtomicF32T &ep,
                         int mtiles, int kpieces, int per, int nz, int *err, cudaStream_t s)
{
    ConvWgDyTTmaBlk<N> lb;
    if (int st = tma_map_bf16(&lb.map, dyT, 3, db, sb, bb)) return st;
    auto kern = tc::gemm_tma_kernel<N, kTmaStages, ConvWgXTTmaBlk, ConvWgDyTTmaBlk<N>, EpiAtomicF32T>;
    static const cudaError_t attr = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc::TmaSmem<N, kTmaStages>::kBytes);
    LENTILS_CUDA_TRY(attr);
    kern<<<dim3(mtiles, 1, nz), tc::kPipeThreads, tc::TmaSmem<N, kTmaStages>::kBytes, s>>>(
        la, lb, ep, kpieces, per, err);
    LENTILS_CHECK_LAUNCH("weight gradient gemm (TMA, blocked)");
    return LENTILS_OK;
}

static int level_dims(const lentils_unet *net, int level, int &H, int &W)
{
    H = net->H >> level;
    W = net->W >> level;
    return LENTILS_OK;
}

// What follows a hidden layer in the forward pass: a 2 x 2 pooling of its output into pool, or
// an upsampling of it added to skip into up (the next level's input), or nothing.
struct FwdPost {
    bf16 *pool = nullptr;
    const bf16 *skip = nullptr;
    bf16 *up = nullptr;
};

static int run_post(lentils_unet *net, const ConvSpec &c, const bf16 *y, const FwdPost &post,
                    int Bn, int H, int W, cudaStream_t s)
{
    const long long npix = (long long)Bn * H * W;
    if (post.pool)
        LENTILS_CUDA_TRY(pdl_launch(pool2_kernel, dim3(blocks_n(npix / 4 * c.cout_p / 8)), dim3(256), 0, s,
                                    y, post.pool, Bn, H, W, c.cout_p));
    else if (post.up)
        LENTILS_CUDA_TRY(pdl_launch(up2add_kernel, dim3(blocks_n(npix * 4 * c.cout_p / 8)), dim3(256), 0, s,
                                    y, post.skip, post.up, Bn, 2 * H, 2 * W, c.cout_p));
    LENTILS_CHECK_LAUNCH("pool2 / up2add");
    return LENTILS_OK;
}

// forward of layer l: y = act(conv(x)), then the post step
static int layer_forward(lentils_unet *net, int l, const bf16 *x, void *y, int Bn, cudaStream_t s,
                         const FwdPost &post = FwdPost())
{
    const ConvSpec &c = kLayers[l];
    int H, W;
    level_dims(net, c.level, H, W);
    const int npix = Bn * H * W;
    const int K = c.ks * c.ks * c.cin_p;
    ConvFwdA la{x, npix, H, W, c.cin_p, c.ks};
    tc::RowMajorLoader lb{net->wf[l], c.cout_p, K, K};
    // the pipelined GEMM wins where a layer has few row tiles (the deep layers); with many
    // CTAs the staged GEMM keeps more of them resident and hides its loads by occupancy
    const int mt = (npix + 127) / 128;
    const bool fast = net->gemm_form != 1;
    const bool pipe = fast && mt < kPipeMaxTiles;
    const bool tma = fast && conv_tma_ok(c.cin_p, c.cout_p, H, W);
    const bool persist = net->gemm_form == 0 && tma;
    if (l == kNumLayers - 1) {
        EpiOut ep{(float *)y, net->b32[l], npix};
        if (tma) return conv_tma(x, c.cin_p, c.ks, Bn, H, W, 0, net->wf[l], c.cout_p, ep, 1, K / 8, net->err, s);
        return conv_gemm_n(c.cout_p, la, lb, ep, npix, K, fast, net->err, s);
    }
    const int mtiles = (npix + 127) / 128;
    const int kp = (K + 7) / 8, nchunks = (kp + 7) / 8;
    const int split = std::min(nchunks, std::max(2, std::min(kSplitMax, 128 / mtiles)));
    const int per = ((nchunks + split - 1) / split) * 8;  // pieces per split (whole chunks)
    const int nz = (kp + per - 1) / per;
    const long long n = (long long)npix * c.cout_p;
    if (npix < kSplitMaxPix && nz > 1 && nz * n <= (long long)kSplitSlabPix * 128) {
        EpiPartialF32 ep{net->splitk, npix, c.cout_p};
        int st = LENTILS_OK;
        if (tma) st = conv_tma(x, c.cin_p, c.ks, Bn, H, W, 0, net->wf[l], c.cout_p, ep, nz, per, net->err, s);
        else switch (c.cout_p) {
        case 32: st = conv_gemm_split<32>(la, lb, ep, mtiles, kp, per, nz, pipe, net->err, s); break;
        case 64: st = conv_gemm_split<64>(la, lb, ep, mtiles, kp, per, nz, pipe, net->err, s); break;
        case 128: st = conv_gemm_split<128>(la, lb, ep, mtiles, kp, per, nz, pipe, net->err, s); break;
        default: return set_error(LENTILS_ERR_UNSUPPORTED, "split-K N=%d", c.cout_p);
        }
        if (st) return st;
        // the slabs are summed together with the post step
        const float *part = net->splitk;
        if (post.pool)
            LENTILS_CUDA_TRY(pdl_launch(finalize_pool_kernel, dim3(blocks_small(n / 8)), dim3(64), 0, s, part,
                                        nz, net->b32[l], (bf16 *)y, post.pool, Bn, H, W, c.cout_p, c.relu));
        else if (post.up)
            LENTILS_CUDA_TRY(pdl_launch(finalize_up_kernel, dim3(blocks_small(n / 8)), dim3(64), 0, s, part,
                                        nz, net->b32[l], (bf16 *)y, post.skip, post.up, Bn, H, W, c.cout_p,
                                        c.relu));
        else
            LENTILS_CUDA_TRY(pdl_launch(finalize_act_kernel, dim3(blocks_n(n)), dim3(256), 0, s, part, nz,
                                        net->b32[l], (bf16 *)y, n, c.cout_p, c.relu));
        LENTILS_CHECK_LAUNCH("finalize kernel");
        return LENTILS_OK;
    }
    int st;
    if (persist) {
        RowAct ep{(bf16 *)y, net->b32[l], npix, c.cout_p, c.relu};
        st = conv3_rows_ok(c.cin_p, c.cout_p, c.ks, W, Bn, H)
                 ? conv3_rows_launch(x, Bn, H, 0, net->wf[l], ep, net->err, s)
                 : conv_persist(x, c.cin_p, c.ks, Bn, H, W, 0, net->wf[l], c.cout_p, ep, net->err, s);
    } else {
        EpiAct ep{(bf16 *)y, net->b32[l], npix, c.cout_p, c.relu};
        st = tma ? conv_tma(x, c.cin_p, c.ks, Bn, H, W, 0, net->wf[l], c.cout_p, ep, 1, K / 8, net->err, s)
                 : conv_gemm_n(c.cout_p, la, lb, ep, npix, K, pipe, net->err, s);
    }
    if (st) return st;
    return run_post(net, c, (const bf16 *)y, post, Bn, H, W, s);
}

// The last hidden layer (c1) fused with the output layer on the persistent GEMM, when c1 takes
// that path; returns 1 (nothing run) otherwise. y (c1's output) may be null; with z set the
// preconditioner's combination is written instead of out.
static int fused_c1_out(lentils_unet *net, const bf16 *x, bf16 *y, float *out, float *z,
                        const float *r, const float *dinv, int Bn, cudaStream_t s)
{
    const int l = kNumLayers - 2;
    const ConvSpec &c = kLayers[l];
    int H, W;
    level_dims(net, c.level, H, W);
    const int npix = Bn * H * W;
    if (net->gemm_form != 0 || !conv_tma_ok(c.cin_p, c.cout_p, H, W) || c.cout_p != 32 ||
        c.cin_p != 32 || npix < kSplitMaxPix)
        return 1;
    RowActOut ep{y, net->b32[l], npix, net->wf[l + 1], net->b32[l + 1], out, z, r, dinv,
                 net->pscale, net->jacobi_weight};
    if (conv3_rows_ok(c.cin_p, c.cout_p, c.ks, W, Bn, H))
        return conv3_rows_launch(x, Bn, H, 0, net->wf[l], ep, net->err, s);
    return conv_persist_launch<32, 32>(x, c.cin_p, c.ks, Bn, H, W, 0, net->wf[l],
                                       c.ks * c.ks * c.cin_p, ep, net->err, s);
}

// whether layer l's weight gradient runs on wgrad_mn_kernel (form 0, shapes it takes)
static bool wgrad_mn_uses(const lentils_unet *net, int l)
{
    const ConvSpec &c = kLayers[l];
    return net->gemm_form == 0 && wgrad_mn_ok(c.cin_p, c.cout_p, net->H >> c.level, net->W >> c.level);
}

// backward of layer l: dy (gradient of its output, before the ReLU mask), y (its output, for
// the mask; null for the output layer), x (its input); accumulates gw/gb, writes dx (optional).
// prepared: the masked gradient operands (dym, dyT) and the bias gradient have been written
// already (out_grad_prep_kernel); dy is then unused.
static int layer_backward(lentils_unet *net, int l, const bf16 *dy, const bf16 *y, const bf16 *x,
                          bf16 *dx, int Bn, cudaStream_t s, bool prepared = false)
{
    const ConvSpec &c = kLayers[l];
    int H, W;
    level_dims(net, c.level, H, W);
    const int npix = Bn * H * W;
    const int taps = c.ks * c.ks;
    const bf16 *mask = c.relu ? y : nullptr;
    // the transposed weight-gradient operands take 8 pixels of one image row per piece
    const bool pipe = net->gemm_form != 1 && c.cout_p <= 128 && c.cin_p <= 128 && (W % 8) == 0;
    if (prepared && !pipe) return set_error(LENTILS_ERR_UNSUPPORTED, "prepared backward, layer %d", l);
    if (!pipe) {  // bias gradient (the pipelined form sums it in grad_prep_kernel)
        bias_grad_kernel<<<std::min(npix, 1024), c.cout_p, 0, s>>>(dy, mask, net->gb[l], npix,
                                                                   c.cout_p, c.cout);
        LENTILS_CHECK_LAUNCH("bias_grad_kernel");
    }
    if (pipe) {
        // masked gradient (pixel-major and transposed) and the shifted transposed input
        const int blocks = (npix + 63) / 64;
        // 64-pixel blocks (W a multiple of 64) keep a TMA box in one contiguous run
        const bool blocked = (W % 64) == 0;
        // form 0: the weight gradient reads x and dym as they are (MN-major operands)
        const bool mn = wgrad_mn_uses(net, l);
        if (!prepared) {
            grad_prep_kernel<<<blocks, 256, 0, s>>>(dy, mask, net->dym, mn ? nullptr : net->dyT,
                                                    net->gb[l], npix, c.cout_p, c.cout,
                                                    blocked ? 1 : 0);
            LENTILS_CHECK_LAUNCH("grad_prep_kernel");
        }
        int st = LENTILS_OK;
        if (mn) {
            const int ctas = net->wgrad_ctas > 0 ? net->wgrad_ctas : kWgradCtas;
            switch (c.cout_p) {
            case 32: st = wgrad_mn_launch<32>(x, net->dym, net->gw_pad[l], c.cin_p, c.ks, Bn, H, W, ctas, net->err, s); break;
            case 64: st = wgrad_mn_launch<64>(x, net->dym, net->gw_pad[l], c.cin_p, c.ks, Bn, H, W, ctas, net->err, s); break;
            case 128: st = wgrad_mn_launch<128>(x, net->dym, net->gw_pad[l], c.cin_p, c.ks, Bn, H, W, ctas, net->err, s); break;
            default: return set_error(LENTILS_ERR_UNSUPPORTED, "weight gradient N=%d", c.cout_p);
            }
            if (st) return st;
        }
        const int nshift = c.ks == 3 ? 3 : 1;
        const long long qtot = (long long)(npix / (H * W)) * (H + 2) * W;
        if (!mn) {
            shift_transpose_kernel<<<blocks, 256, 0, s>>>(x, net->xT, npix, H, W, c.cin_p, nshift,
                                                          qtot, blocked ? 1 : 0);
            LENTILS_CHECK_LAUNCH("shift_transpose_kernel");
        }
        // weight gradient: rows = taps * cin_p, columns = cout_p, K = pixels split over CTAs,
        // about kWgradCtas CTAs in all
        const int Kw = taps * c.cin_p;
        EpiAtomicF32T ep{net->gw_pad[l], Kw, c.cout_p};
        const int kpieces = npix / 8;  // npix is a multiple of 8 (W is)
        const int mtiles = (Kw + 127) / 128;
        const int want = std::max(1, (net->wgrad_ctas > 0 ? net->wgrad_ctas : kWgradCtas) / mtiles);
        int per = (kpieces + want - 1) / want;
        per = std::max(kWgradMinPieces, (per + 7) / 8 * 8);  // whole chunks
        const int nz = (kpieces + per - 1) / per;
        if (mn) {
            // done above
        } else if (blocked) {
            ConvWgXTTmaBlk la;
            la.C = c.cin_p;
            la.ks = c.ks;
            la.H = H;
            la.W = W;
            la.nblk = (int)(qtot / 64);
            const uint64_t da[3] = {64, (uint64_t)c.cin_p, (uint64_t)nshift * la.nblk};
            const uint64_t sa[2] = {128, (uint64_t)c.cin_p * 128};
            const uint32_t ba[3] = {64, (uint32_t)c.cin_p, 1};
            if ((st = tma_map_bf16(&la.map, net->xT, 3, da, sa, ba))) return st;
            const uint64_t db[3] = {64, (uint64_t)c.cout_p, (uint64_t)npix / 64};
            const uint64_t sb[2] = {128, (uint64_t)c.cout_p * 128};
            const uint32_t bb[3] = {64, (uint32_t)c.cout_p, 1};
            switch (c.cout_p) {
            case 32: st = wgrad_tma_blk<32>(la, net->dyT, db, sb, bb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            case 64: st = wgrad_tma_blk<64>(la, net->dyT, db, sb, bb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            case 128: st = wgrad_tma_blk<128>(la, net->dyT, db, sb, bb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            default: return set_error(LENTILS_ERR_UNSUPPORTED, "weight gradient N=%d", c.cout_p);
            }
        } else if ((H * W) % 64 == 0) {
            ConvWgXTTma la;
            la.C = c.cin_p;
            la.ks = c.ks;
            la.H = H;
            la.W = W;
            la.rows = nshift * c.cin_p;
            const uint64_t da[2] = {(uint64_t)qtot, (uint64_t)la.rows};
            const uint64_t sa[1] = {(uint64_t)qtot * 2};
            const uint32_t ba[2] = {64, (uint32_t)c.cin_p};
            if ((st = tma_map_bf16(&la.map, net->xT, 2, da, sa, ba))) return st;
            const uint64_t db[2] = {(uint64_t)npix, (uint64_t)c.cout_p};
            const uint64_t sb[1] = {(uint64_t)npix * 2};
            const uint32_t bb[2] = {64, (uint32_t)c.cout_p};
            switch (c.cout_p) {
            case 32: st = wgrad_tma_launch<32>(la, net->dyT, db, sb, bb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            case 64: st = wgrad_tma_launch<64>(la, net->dyT, db, sb, bb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            case 128: st = wgrad_tma_launch<128>(la, net->dyT, db, sb, bb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            default: return set_error(LENTILS_ERR_UNSUPPORTED, "weight gradient N=%d", c.cout_p);
            }
        } else {
            ConvWgXT la{net->xT, npix, H, W, c.cin_p, c.ks, qtot};
            ConvWgDyT lb{net->dyT, npix, c.cout_p};
            switch (c.cout_p) {
            case 32: st = wgrad_launch<32>(la, lb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            case 64: st = wgrad_launch<64>(la, lb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            case 128: st = wgrad_launch<128>(la, lb, ep, mtiles, kpieces, per, nz, net->err, s); break;
            default: return set_error(LENTILS_ERR_UNSUPPORTED, "weight gradient N=%d", c.cout_p);
            }
        }
        if (st) return st;
        if (dx && conv_tma_ok(c.cout_p, c.cin_p, H, W)) {  // data gradient, TMA operands
            int st2;
            if (net->gemm_form == 0 && conv3_rows_ok(c.cout_p, c.cin_p, c.ks, W, Bn, H)) {
                st2 = conv3_rows_launch(net->dym, Bn, H, 1, net->wb[l], RowStore{dx, npix, c.cin_p},
                                        net->err, s);
            } else if (net->gemm_form == 0) {
                st2 = conv_persist(net->dym, c.cout_p, c.ks, Bn, H, W, 1, net->wb[l], c.cin_p,
                                   RowStore{dx, npix, c.cin_p}, net->err, s);
            } else {
                EpiStoreBf16 epd{dx, npix, c.cin_p};
                const int K = taps * c.cout_p;
                st2 = conv_tma(net->dym, c.cout_p, c.ks, Bn, H, W, 1, net->wb[l], c.cin_p, epd, 1,
                               K / 8, net->err, s);
            }
            if (st2) return st2;
        } else if (dx) {  // data gradient from the masked copy: plain gathers, pipelined
            const int K = taps * c.cout_p;
            ConvBwdDataA lad{net->dym, nullptr, npix, H, W, c.cout_p, c.ks};
            tc::RowMajorLoader lbd{net->wb[l], c.cin_p, K, K};
            EpiStoreBf16 epd{dx, npix, c.cin_p};
            if (int st2 = conv_gemm_n(std::max(32, c.cin_p), lad, lbd, epd, npix, K, true,
                                      net->err, s))
                return st2;
        }
        return LENTILS_OK;
    }
    // weight gradient: M = cout_p (one tile), N = taps * cin_p in tiles of <= 256, K = pixels
    {
        const int Kw = taps * c.cin_p;
        ConvBwdWA la{dy, mask, npix, c.cout_p};
        ConvBwdWB lb{x, npix, H, W, c.cin_p, c.ks};
        EpiAtomicF32 ep{net->gw_pad[l], c.cout_p, Kw};
        const int kpieces = (npix + 7) / 8;
        const int split = 128;  // pieces (1024 pixels) per CTA along K
        const int nz = (kpieces + split - 1) / split;
        if (Kw <= 32) {
            auto kern = tc::gemm_kernel<32, ConvBwdWA, ConvBwdWB, EpiAtomicF32>;
            const size_t smem = tc::GemmSmem<32>::kBytes;
            LENTILS_CUDA_TRY((gemm_smem_attr<32, ConvBwdWA, ConvBwdWB, EpiAtomicF32>()));
            kern<<<dim3(1, 1, nz), 128, smem, s>>>(la, lb, ep, kpieces, split, net->err);
        } else if (Kw <= 128) {
            auto kern = tc::gemm_kernel<128, ConvBwdWA, ConvBwdWB, EpiAtomicF32>;
            const size_t smem = tc::GemmSmem<128>::kBytes;
            LENTILS_CUDA_TRY((gemm_smem_attr<128, ConvBwdWA, ConvBwdWB, EpiAtomicF32>()));
            kern<<<dim3(1, 1, nz), 128, smem, s>>>(la, lb, ep, kpieces, split, net->err);
        } else {
            auto kern = tc::gemm_kernel<256, ConvBwdWA, ConvBwdWB, EpiAtomicF32>;
            const size_t smem = tc::GemmSmem<256>::kBytes;
            LENTILS_CUDA_TRY((gemm_smem_attr<256, ConvBwdWA, ConvBwdWB, EpiAtomicF32>()));
            kern<<<dim3(1, (Kw + 255) / 256, nz), 128, smem, s>>>(la, lb, ep, kpieces, split, net->err);
        }
        LENTILS_CHECK_LAUNCH("weight gradient gemm");
    }
    // data gradient
    if (dx) {
        const int K = taps * c.cout_p;
        ConvBwdDataA la{dy, mask, npix, H, W, c.cout_p, c.ks};
        tc::RowMajorLoader lb{net->wb[l], c.cin_p, K, K};
        EpiStoreBf16 ep{dx, npix, c.cin_p};
        if (int st = conv_gemm_n(std::max(32, c.cin_p), la, lb, ep, npix, K,
                                 net->gemm_form != 1 && !mask, net->err, s))
            return st;
    }
    return LENTILS_OK;
}

// all layers, from the packed input x0 to out
// Input of a forward pass: channel 0 = a (times a2 and 1 / scale where those are given),
// channel 1 = b. With z set (the preconditioner: a = r, a2 = dinv, b = feat) the result is the
// combination z = s * out + gamma * dinv * r, and the activations that only a backward pass
// reads (the packed input, c1) are not written where the fused kernels can skip them.
struct FwdIn {
    const float *a, *a2, *scale, *b;
    float *z;
};

static int net_forward_in(lentils_unet *net, const FwdIn &in, int Bn, cudaStream_t s)
{
    const int H = net->H, W = net->W;
    const long long np0 = (long long)Bn * H * W;
    const bool pre = in.z != nullptr;
    int st;
    if (net->gemm_form == 0) {
        // below about two waves of blocks, each thread takes half the channels
        const long long nblk = np0 / 4;
        const int nh = nblk < 152LL * 256 ? 2 : 1;
        const int blocks = (int)std::max(1LL, std::min((nblk * nh + 127) / 128, 152LL * 16));
        LENTILS_CUDA_TRY(pdl_launch(e1_direct_kernel, dim3(blocks), dim3(128), 0, s, in.a, in.a2, in.scale,
                                    in.b, (const bf16 *)net->wf[0], (const float *)net->b32[0],
                                    pre ? nullptr : net->x0, net->e1, net->p1, Bn, H, W, nh));
        LENTILS_CHECK_LAUNCH("e1_direct_kernel");
    } else {
        if (pre)
            LENTILS_CUDA_TRY(pdl_launch(precond_input_kernel, dim3(blocks_n(np0)), dim3(256), 0, s, in.a,
                                        in.a2, in.b, in.scale, net->x0, (int)np0));
        else
            LENTILS_CUDA_TRY(pdl_launch(make_input_kernel, dim3(blocks_n(np0)), dim3(256), 0, s, in.a, in.b,
                                        net->x0, np0));
        FwdPost p0;
        p0.pool = net->p1;
        if ((st = layer_forward(net, 0, net->x0, net->e1, Bn, s, p0))) return st;
    }
    FwdPost p1, p2, p3, p4, p5;
    p1.pool = net->p2;
    p2.pool = net->p3;
    p3.skip = net->e3;
    p3.up = net->u3;
    p4.skip = net->e2;
    p4.up = net->u2;
    p5.skip = net->e1;
    p5.up = net->u1;
    if ((st = layer_forward(net, 1, net->p1, net->e2, Bn, s, p1))) return st;
    if ((st = layer_forward(net, 2, net->p2, net->e3, Bn, s, p2))) return st;
    if ((st = layer_forward(net, 3, net->p3, net->b, Bn, s, p3))) return st;
    if ((st = layer_forward(net, 4, net->u3, net->c3, Bn, s, p4))) return st;
    if ((st = layer_forward(net, 5, net->u2, net->c2, Bn, s, p5))) return st;
    st = fused_c1_out(net, net->u1, pre ? nullptr : net->c1, net->out, in.z, in.a, in.a2, Bn, s);
    if (st == 1) {
        if ((st = layer_forward(net, 6, net->u1, net->c1, Bn, s))) return st;
        if ((st = layer_forward(net, 7, net->c1, net->out, Bn, s))) return st;
        if (pre) {
            LENTILS_CUDA_TRY(pdl_launch(precond_combine_kernel, dim3(blocks_n(np0)), dim3(256), 0, s, in.a,
                                        in.a2, (const float *)net->out, (const float *)net->pscale,
                                        net->jacobi_weight, in.z, (int)np0));
            LENTILS_CHECK_LAUNCH("precond_combine_kernel");
        }
    } else if (st) {
        return st;
    }
    LENTILS_CHECK_LAUNCH("unet forward");
    return LENTILS_OK;
}

static int net_forward(lentils_unet *net, const float *r, const float *d, int Bn, cudaStream_t s)
{
    return net_forward_in(net, FwdIn{r, nullptr, nullptr, d, nullptr}, Bn, s);
}

// the per-layer shapes and BF16 weight copies of all layers (src, dst32 and off left to the caller)
static AllLayers all_layers(const lentils_unet *net)
{
    AllLayers P{};
    for (int l = 0; l < kNumLayers; ++l) {
        const ConvSpec &c = kLayers[l];
        P.fwd[l] = net->wf[l];
        P.bwd[l] = net->wb[l];
        P.cin[l] = c.cin;
        P.cout[l] = c.cout;
        P.cin_p[l] = c.cin_p;
        P.cout_p[l] = c.cout_p;
        P.taps[l] = c.ks * c.ks;
    }
    return P;
}

// parameter gradients (forward must have run for this batch): of the mean squared error
// against tgt, or, with dout, for the given gradient of the output
static int net_backward(lentils_unet *net, const float *tgt, const float *dout, int Bn,
                        cudaStream_t s)
{
    const int H = net->H, W = net->W;
    const long long np0 = (long long)Bn * H * W;
    {
        ZeroList Z{};
        auto add = [&](float *p, long long n) {
            Z.p[Z.count] = p;
            Z.off[Z.count + 1] = Z.off[Z.count] + n;
            ++Z.count;
        };
        add(net->grads, net->nparams);
        for (int l = 0; l < kNumLayers; ++l) {
            const ConvSpec &c = kLayers[l];
            add(net->gw_pad[l], (long long)c.cout_p * c.ks * c.ks * c.cin_p);
        }
        add(net->loss, 1);
        LENTILS_CUDA_TRY(pdl_launch(zero_kernel, dim3(blocks_n(Z.off[Z.count])), dim3(256), 0, s, Z));
    }
    // the fused output-layer backward pass (form 0) reads a compact gradient
    const bool fuse_out = net->gemm_form == 0 && kLayers[6].cout_p == 32 && (W % 8) == 0;
    if (dout)
        LENTILS_CUDA_TRY(pdl_launch(pack_dout_kernel, dim3(blocks_n(np0)), dim3(256), 0, s, dout,
                                    net->dy_out, np0, fuse_out ? 1 : 0));
    else
        LENTILS_CUDA_TRY(pdl_launch(mse_kernel, dim3(blocks_n(np0)), dim3(256), 0, s,
                                    (const float *)net->out, tgt, net->dy_out, np0, net->loss,
                                    fuse_out ? 1 : 0));
    int st;
    if (fuse_out) {
        // the output layer's whole backward pass in c1's gradient preparation
        LENTILS_CUDA_TRY(pdl_launch(
            out_grad_prep_kernel, dim3((int)((np0 + 63) / 64)), dim3(256), 0, s,
            (const bf16 *)net->dy_out, (const bf16 *)net->wf[7], (const bf16 *)net->c1, net->dym,
            wgrad_mn_uses(net, 6) ? nullptr : net->dyT, net->gb[6], net->gw_pad[7], net->gb[7],
            (int)np0, (W % 64) == 0 ? 1 : 0));
        LENTILS_CHECK_LAUNCH("out_grad_prep_kernel");
        if ((st = layer_backward(net, 6, nullptr, net->c1, net->u1, net->d_u1, Bn, s, true))) return st;
    } else {
        if ((st = layer_backward(net, 7, net->dy_out, nullptr, net->c1, net->d_c1, Bn, s))) return st;
        if ((st = layer_backward(net, 6, net->d_c1, net->c1, net->u1, net->d_u1, Bn, s))) return st;
    }
    // The gradient of each hidden layer's output comes from the adjoint of the upsampling (sum4)
    // or of the pooling plus the skip (add_pool_grad); where the layer's weight gradient takes
    // the MN-major form, that kernel also applies the layer's ReLU mask and sums its bias
    // gradient, writing the operand (dym) that layer_backward then uses as prepared.
    auto adj_sum4 = [&](int l, const bf16 *dhi, bf16 *dlow, const bf16 *y, int h, int w, int C) -> int {
        const bool mn = wgrad_mn_uses(net, l);
        const cudaError_t e = pdl_launch(sum4_kernel, dim3(blocks_n((long long)Bn * h / 2 * (w / 2) * C / 8)),
                                         dim3(256), 0, s, dhi, mn ? net->dym : dlow, Bn, h, w, C,
                                         mn ? y : nullptr, mn ? net->gb[l] : nullptr);
        return e == cudaSuccess ? (mn ? 1 : 0) : -1;
    };
    auto adj_pool = [&](int l, const bf16 *a, const bf16 *dp, bf16 *d, const bf16 *y, int h, int w,
                        int C) -> int {
        const bool mn = wgrad_mn_uses(net, l);
        const cudaError_t e = pdl_launch(add_pool_grad_kernel, dim3(blocks_n((long long)Bn * h * w * C / 8)),
                                         dim3(256), 0, s, a, dp, mn ? net->dym : d, Bn, h, w, C,
                                         mn ? y : nullptr, mn ? net->gb[l] : nullptr);
        return e == cudaSuccess ? (mn ? 1 : 0) : -1;
    };
    int prep;  // 1: dym prepared, 0: not, -1: the launch failed
    // u1 = up2(c2) + e1
    prep = adj_sum4(5, net->d_u1, net->d_c2, net->c2, H, W, 32);
    if (prep < 0) return set_error(LENTILS_ERR_CUDA, "gradient adjoint launch");
    if ((st = layer_backward(net, 5, net->d_c2, net->c2, net->u2, net->d_u2, Bn, s, prep == 1))) return st;
    prep = adj_sum4(4, net->d_u2, net->d_c3, net->c3, H / 2, W / 2, 64);
    if (prep < 0) return set_error(LENTILS_ERR_CUDA, "gradient adjoint launch");
    if ((st = layer_backward(net, 4, net->d_c3, net->c3, net->u3, net->d_u3, Bn, s, prep == 1))) return st;
    prep = adj_sum4(3, net->d_u3, net->d_b, net->b, H / 4, W / 4, 128);
    if (prep < 0) return set_error(LENTILS_ERR_CUDA, "gradient adjoint launch");
    if ((st = layer_backward(net, 3, net->d_b, net->b, net->p3, net->d_p3, Bn, s, prep == 1))) return st;
    // e3 feeds u3 (skip) and p3 (pool)
    prep = adj_pool(2, net->d_u3, net->d_p3, net->d_e3, net->e3, H / 4, W / 4, 128);
    if (prep < 0) return set_error(LENTILS_ERR_CUDA, "gradient adjoint launch");
    if ((st = layer_backward(net, 2, net->d_e3, net->e3, net->p2, net->d_p2, Bn, s, prep == 1))) return st;
    prep = adj_pool(1, net->d_u2, net->d_p2, net->d_e2, net->e2, H / 2, W / 2, 64);
    if (prep < 0) return set_error(LENTILS_ERR_CUDA, "gradient adjoint launch");
    if ((st = layer_backward(net, 1, net->d_e2, net->e2, net->p1, net->d_p1, Bn, s, prep == 1))) return st;
    LENTILS_CUDA_TRY(pdl_launch(add_pool_grad_kernel, dim3(blocks_n(np0 * 4)), dim3(256), 0, s,
                                (const bf16 *)net->d_u1, (const bf16 *)net->d_p1, net->d_e1, Bn, H, W,
                                32, (const bf16 *)nullptr, (float *)nullptr));
    if (net->gemm_form == 0 && W % kE1Run == 0) {
        const long long items = np0 / kE1Run / 32;  // block iterations of 32 runs
        const int blocks = (int)std::max(1LL, std::min(items, 152LL * 2));
        LENTILS_CUDA_TRY(pdl_launch(e1_wgrad_kernel, dim3(blocks), dim3(256), 0, s,
                                    (const bf16 *)net->d_e1, (const bf16 *)net->e1,
                                    (const bf16 *)net->x0, net->gw_pad[0], net->gb[0], Bn, H, W));
        LENTILS_CHECK_LAUNCH("e1_wgrad_kernel");
    } else if ((st = layer_backward(net, 0, net->d_e1, net->e1, net->x0, nullptr, Bn, s))) {
        return st;
    }
    {
        AllLayers P = all_layers(net);
        P.off[0] = 0;
        for (int l = 0; l < kNumLayers; ++l) {
            P.src[l] = net->gw_pad[l];
            P.dst32[l] = net->gw[l];
            P.off[l + 1] = P.off[l] + layer_wcount(l);
        }
        LENTILS_CUDA_TRY(pdl_launch(gather_all_kernel, dim3(blocks_n(P.off[kNumLayers])), dim3(256), 0,
                                    s, P));
    }
    LENTILS_CHECK_LAUNCH("unet backward");
    return LENTILS_OK;
}

static int refresh_all(lentils_unet *net, cudaStream_t s)
{
    AllLayers P = all_layers(net);
    P.off[0] = 0;
    for (int l = 0; l < kNumLayers; ++l) {
        const ConvSpec &c = kLayers[l];
        P.src[l] = net->w32[l];
        P.off[l + 1] = P.off[l] + (long long)c.cout_p * c.ks * c.ks * c.cin_p;
    }
    LENTILS_CUDA_TRY(pdl_launch(refresh_all_kernel, dim3(blocks_n(P.off[kNumLayers])), dim3(256), 0, s, P));
    LENTILS_CHECK_LAUNCH("refresh_all_kernel");
    return LENTILS_OK;
}

// Sets the shared-memory limits of every GEMM instantiation the forward pass uses, so that a
// forward pass can be captured into a CUDA graph without first-use set-up inside the capture.
static int prepare_forward()
{
    LENTILS_CUDA_TRY((gemm_smem_attr<32, ConvFwdA, tc::RowMajorLoader, EpiAct>()));
    LENTILS_CUDA_TRY((gemm_smem_attr<64, ConvFwdA, tc::RowMajorLoader, EpiAct>()));
    LENTILS_CUDA_TRY((gemm_smem_attr<128, ConvFwdA, tc::RowMajorLoader, EpiAct>()));
    LENTILS_CUDA_TRY((gemm_smem_attr<32, ConvFwdA, tc::RowMajorLoader, EpiOut>()));
    LENTILS_CUDA_TRY((gemm_smem_attr<32, ConvFwdA, tc::RowMajorLoader, EpiPartialF32>()));
    LENTILS_CUDA_TRY((gemm_smem_attr<64, ConvFwdA, tc::RowMajorLoader, EpiPartialF32>()));
    LENTILS_CUDA_TRY((gemm_smem_attr<128, ConvFwdA, tc::RowMajorLoader, EpiPartialF32>()));
    LENTILS_CUDA_TRY((conv_persist_shape<32, 32, RowAct>().err));
    LENTILS_CUDA_TRY((conv_persist_shape<32, 64, RowAct>().err));
    LENTILS_CUDA_TRY((conv_persist_shape<32, 128, RowAct>().err));
    LENTILS_CUDA_TRY((conv_persist_shape<64, 32, RowAct>().err));
    LENTILS_CUDA_TRY((conv_persist_shape<64, 64, RowAct>().err));
    LENTILS_CUDA_TRY((conv_persist_shape<64, 128, RowAct>().err));
    LENTILS_CUDA_TRY((conv_persist_shape<32, 32, RowActOut>().err));
    LENTILS_CUDA_TRY((conv3_rows_shape<RowAct>().err));
    LENTILS_CUDA_TRY((conv3_rows_shape<RowActOut>().err));
    return num_sms() > 0 ? LENTILS_OK : set_error(LENTILS_ERR_CUDA, "SM count");
}

int unet_precondition(lentils_unet *net, const float *r, const float *dinv, const float *feat,
                      float *z, cudaStream_t s)
{
    const int n = net->H * net->W;
    LENTILS_CUDA_TRY(pdl_launch(precond_scale_kernel, dim3(1), dim3(1024), 0, s, r, dinv, n, net->pscale));
    LENTILS_CHECK_LAUNCH("precond_scale_kernel");
    return net_forward_in(net, FwdIn{r, dinv, net->pscale, feat, z}, 1, s);
}

int unet_prepare(lentils_unet *net) { return net ? prepare_forward() : LENTILS_OK; }

int unet_size(const lentils_unet *net) { return net ? net->H * net->W : 0; }

int unet_error_flag_device(lentils_unet *net, int *flag)
{
    LENTILS_CUDA_TRY(cudaMemcpy(flag, net->err, sizeof(int), cudaMemcpyDeviceToHost));
    return LENTILS_OK;
}

static int adam_update(lentils_unet *net, float lr, cudaStream_t s)
{
    net->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - powf(b1, (float)net->step), c2 = 1.f - powf(b2, (float)net->step);
    LENTILS_CUDA_TRY(pdl_launch(adam_kernel, dim3(blocks_n(net->nparams)), dim3(256), 0, s, net->params,
                                (const float *)net->grads, net->adam_m, net->adam_v, net->nparams,
                                lr, b1, b2, 1e-8f, c1, c2));
    LENTILS_CHECK_LAUNCH("adam_kernel");
    return refresh_all(net, s);
}

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_unet_features(const float *dinv, float *feat, int n, void *stream)
{
    clear_error();
    if (!dinv || !feat || n < 1) return set_error(LENTILS_ERR_INVALID, "unet_features: bad arguments");
    features_kernel<<<1, 1024, 0, (cudaStream_t)stream>>>(dinv, feat, n);
    LENTILS_CHECK_LAUNCH("features_kernel");
    return LENTILS_OK;
}

int lentils_unet_precondition(lentils_unet *net, const float *r, const float *dinv,
                              const float *feat, float *z, void *stream)
{
    clear_error();
    if (!net || !r || !dinv || !feat || !z)
        return set_error(LENTILS_ERR_INVALID, "unet_precondition: null");
    return unet_precondition(net, r, dinv, feat, z, (cudaStream_t)stream);
}


long long lentils_unet_param_count(void)
{
    long long n = 0;
    for (int l = 0; l < kNumLayers; ++l) n += layer_wcount(l) + kLayers[l].cout;
    return n;
}

// Parameters are one flat FP32 vector: for each layer in order, the weights [cout][ks*ks][cin]
// then the biases [cout].
int lentils_unet_create(lentils_unet **out, int H, int W, int max_batch, const float *init_params,
                        void *stream)
{
    clear_error();
    if (!out || !init_params || H < 16 || W < 16 || (H % 8) || (W % 8) || max_batch < 1)
        return set_error(LENTILS_ERR_INVALID, "unet_create: H, W multiples of 8 (>= 16)");
    *out = nullptr;
    lentils_unet *net = new (std::nothrow) lentils_unet();
    if (!net) return set_error(LENTILS_ERR_ALLOC, "unet_create: host allocation");
    memset(net, 0, sizeof(*net));
    net->H = H;
    net->W = W;
    net->maxB = max_batch;
    net->nparams = lentils_unet_param_count();
    const long long np0 = (long long)max_batch * H * W;
    // carve one allocation
    std::vector<std::pair<void **, size_t>> parts;
    auto add = [&](void **p, size_t bytes) { parts.push_back({p, (bytes + 255) & ~size_t(255)}); };
    add((void **)&net->params, sizeof(float) * net->nparams);
    add((void **)&net->grads, sizeof(float) * net->nparams);
    add((void **)&net->adam_m, sizeof(float) * net->nparams);
    add((void **)&net->adam_v, sizeof(float) * net->nparams);
    for (int l = 0; l < kNumLayers; ++l) {
        const ConvSpec &c = kLayers[l];
        const size_t n = (size_t)c.cout_p * c.ks * c.ks * c.cin_p;
        add((void **)&net->wf[l], sizeof(bf16) * n);
        add((void **)&net->wb[l], sizeof(bf16) * n);
        add((void **)&net->gw_pad[l], sizeof(float) * n);
    }
    const size_t b2 = sizeof(bf16);
    add((void **)&net->x0, b2 * np0 * 8);
    add((void **)&net->e1, b2 * np0 * 32);
    add((void **)&net->p1, b2 * np0 / 4 * 32);
    add((void **)&net->e2, b2 * np0 / 4 * 64);
    add((void **)&net->p2, b2 * np0 / 16 * 64);
    add((void **)&net->e3, b2 * np0 / 16 * 128);
    add((void **)&net->p3, b2 * np0 / 64 * 128);
    add((void **)&net->b, b2 * np0 / 64 * 128);
    add((void **)&net->u3, b2 * np0 / 16 * 128);
    add((void **)&net->c3, b2 * np0 / 16 * 64);
    add((void **)&net->u2, b2 * np0 / 4 * 64);
    add((void **)&net->c2, b2 * np0 / 4 * 32);
    add((void **)&net->u1, b2 * np0 * 32);
    add((void **)&net->c1, b2 * np0 * 32);
    add((void **)&net->out, sizeof(float) * np0);
    add((void **)&net->dy_out, b2 * np0 * 32);
    add((void **)&net->d_c1, b2 * np0 * 32);
    add((void **)&net->d_u1, b2 * np0 * 32);
    add((void **)&net->d_c2, b2 * np0 / 4 * 32);
    add((void **)&net->d_u2, b2 * np0 / 4 * 64);
    add((void **)&net->d_c3, b2 * np0 / 16 * 64);
    add((void **)&net->d_u3, b2 * np0 / 16 * 128);
    add((void **)&net->d_b, b2 * np0 / 64 * 128);
    add((void **)&net->d_p3, b2 * np0 / 64 * 128);
    add((void **)&net->d_e3, b2 * np0 / 16 * 128);
    add((void **)&net->d_p2, b2 * np0 / 16 * 64);
    add((void **)&net->d_e2, b2 * np0 / 4 * 64);
    add((void **)&net->d_p1, b2 * np0 / 4 * 32);
    add((void **)&net->d_e1, b2 * np0 * 32);
    {
        size_t dmax = 0, xmax = 0;  // largest npix * cout_p and 3 * npix * cin_p over the layers
        for (int l = 0; l < kNumLayers; ++l) {
            const ConvSpec &c = kLayers[l];
            const size_t np = (size_t)np0 >> (2 * c.level);
            const size_t Hl = (size_t)(H >> c.level);
            dmax = std::max(dmax, np * c.cout_p);
            // row-padded: (H + 2) rows per image
            xmax = std::max(xmax, np / std::max<size_t>(Hl, 1) * (Hl + 2) * c.cin_p *
                                      (c.ks == 3 ? 3 : 1));
        }
        add((void **)&net->dym, b2 * dmax);
        add((void **)&net->dyT, b2 * dmax);
        add((void **)&net->xT, b2 * xmax);
    }
    add((void **)&net->loss, sizeof(float));
    add((void **)&net->pscale, sizeof(float));
    add((void **)&net->splitk, sizeof(float) * kSplitSlabPix * 128);
    add((void **)&net->err, sizeof(int));
    size_t total = 0;
    for (auto &p : parts) total += p.second;
    cudaError_t e = cudaMalloc(&net->block, total);
    if (e != cudaSuccess) {
        delete net;
        return cuda_status(e, "unet_create alloc");
    }
    size_t off = 0;
    for (auto &p : parts) {
        *p.first = (unsigned char *)net->block + off;
        off += p.second;
    }
    // parameter views
    long long po = 0;
    for (int l = 0; l < kNumLayers; ++l) {
        net->w32[l] = net->params + po;
        net->gw[l] = net->grads + po;
        po += layer_wcount(l);
        net->b32[l] = net->params + po;
        net->gb[l] = net->grads + po;
        po += kLayers[l].cout;
    }
    cudaStream_t s = (cudaStream_t)stream;
    e = cudaMemcpyAsync(net->params, init_params, sizeof(float) * net->nparams, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->adam_m, 0, sizeof(float) * net->nparams, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->adam_v, 0, sizeof(float) * net->nparams, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(net->err, 0, sizeof(int), s);
    int st = (e == cudaSuccess) ? refresh_all(net, s) : cuda_status(e, "unet_create init");
    if (!st) {
        e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) st = cuda_status(e, "unet_create sync");
    }
    if (st) {
        cudaFree(net->block);
        delete net;
        return st;
    }
    *out = net;
    return LENTILS_OK;
}

int lentils_unet_destroy(lentils_unet *net)
{
    clear_error();
    if (!net) return LENTILS_OK;
    cudaFree(net->block);
    delete net;
    return LENTILS_OK;
}

int lentils_unet_get_params(lentils_unet *net, float *host_out)
{
    clear_error();
    if (!net || !host_out) return set_error(LENTILS_ERR_INVALID, "unet_get_params: null");
    // training steps may still be running on the caller's stream, whatever its flags
    LENTILS_CUDA_TRY(cudaDeviceSynchronize());
    LENTILS_CUDA_TRY(cudaMemcpy(host_out, net->params, sizeof(float) * net->nparams, cudaMemcpyDeviceToHost));
    return LENTILS_OK;
}

int lentils_unet_set_params(lentils_unet *net, const float *host_in, void *stream)
{
    clear_error();
    if (!net || !host_in) return set_error(LENTILS_ERR_INVALID, "unet_set_params: null");
    cudaStream_t s = (cudaStream_t)stream;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(net->params, host_in, sizeof(float) * net->nparams, cudaMemcpyHostToDevice, s));
    return refresh_all(net, s);
}

// out = net(r, d) for Bn samples of H x W (device FP32 arrays)
int lentils_unet_forward(lentils_unet *net, const float *r, const float *d, float *out, int Bn,
                         void *stream)
{
    clear_error();
    if (!net || !r || !d || !out || Bn < 1 || Bn > net->maxB)
        return set_error(LENTILS_ERR_INVALID, "unet_forward: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    if (int st = net_forward(net, r, d, Bn, s)) return st;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(out, net->out, sizeof(float) * Bn * net->H * net->W,
                                     cudaMemcpyDeviceToDevice, s));
    return LENTILS_OK;
}

// forward + backward without updating: flat gradient (host) and loss (host)
int lentils_unet_gradients(lentils_unet *net, const float *r, const float *d, const float *tgt,
                           int Bn, float *grad_host, float *loss_host, void *stream)
{
    clear_error();
    if (!net || !r || !d || !tgt || Bn < 1 || Bn > net->maxB)
        return set_error(LENTILS_ERR_INVALID, "unet_gradients: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if ((st = net_forward(net, r, d, Bn, s))) return st;
    if ((st = net_backward(net, tgt, nullptr, Bn, s))) return st;
    if (grad_host)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(grad_host, net->grads, sizeof(float) * net->nparams, cudaMemcpyDeviceToHost, s));
    if (loss_host)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(loss_host, net->loss, sizeof(float), cudaMemcpyDeviceToHost, s));
    int herr = 0;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&herr, net->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr) return set_error(LENTILS_ERR_TIMEOUT, "unet: a tensor-core wait gave up");
    return LENTILS_OK;
}

// one Adam step on the mean squared error; loss_dev (device float) receives the batch loss
int lentils_unet_train_step(lentils_unet *net, const float *r, const float *d, const float *tgt,
                            int Bn, float lr, float *loss_dev, void *stream)
{
    clear_error();
    if (!net || !r || !d || !tgt || Bn < 1 || Bn > net->maxB)
        return set_error(LENTILS_ERR_INVALID, "unet_train_step: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if ((st = net_forward(net, r, d, Bn, s))) return st;
    if ((st = net_backward(net, tgt, nullptr, Bn, s))) return st;
    if ((st = adam_update(net, lr, s))) return st;
    if (loss_dev)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(loss_dev, net->loss, sizeof(float), cudaMemcpyDeviceToDevice, s));
    return LENTILS_OK;
}

// backward from the most recent forward pass (same batch size) for an external gradient of
// the output; optional Adam step (lr > 0) and copy of the flat gradient to host memory
int lentils_unet_backward(lentils_unet *net, const float *dout, int Bn, float lr,
                          float *grad_host, void *stream)
{
    clear_error();
    if (!net || !dout || Bn < 1 || Bn > net->maxB)
        return set_error(LENTILS_ERR_INVALID, "unet_backward: bad arguments");
    cudaStream_t s = (cudaStream_t)stream;
    int st;
    if ((st = net_backward(net, nullptr, dout, Bn, s))) return st;
    if (grad_host) {
        LENTILS_CUDA_TRY(cudaMemcpyAsync(grad_host, net->grads, sizeof(float) * net->nparams,
                                         cudaMemcpyDeviceToHost, s));
        LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (lr > 0.f && (st = adam_update(net, lr, s))) return st;
    return LENTILS_OK;
}

int lentils_unet_set_wgrad_ctas(lentils_unet *net, int ctas)
{
    clear_error();
    if (!net || ctas < 0 || ctas > 1 << 16) return set_error(LENTILS_ERR_INVALID, "unet_set_wgrad_ctas");
    net->wgrad_ctas = ctas;
    return LENTILS_OK;
}

int lentils_unet_set_gemm_form(lentils_unet *net, int form)
{
    clear_error();
    if (!net || form < 0 || form > 2) return set_error(LENTILS_ERR_INVALID, "unet_set_gemm_form");
    net->gemm_form = form;
    return LENTILS_OK;
}

int lentils_unet_set_jacobi_weight(lentils_unet *net, float gamma)
{
    clear_error();
    if (!net || !(gamma >= 0.f)) return set_error(LENTILS_ERR_INVALID, "unet_set_jacobi_weight");
    net->jacobi_weight = gamma;
    return LENTILS_OK;
}

// status of the bounded tensor-core waits since creation (1 = a wait gave up)
int lentils_unet_error_flag(lentils_unet *net, int *flag)
{
    clear_error();
    if (!net || !flag) return set_error(LENTILS_ERR_INVALID, "unet_error_flag: null");
    LENTILS_CUDA_TRY(cudaDeviceSynchronize());  // after every launch already issued
    LENTILS_CUDA_TRY(cudaMemcpy(flag, net->err, sizeof(int), cudaMemcpyDeviceToHost));
    return LENTILS_OK;
}

}  // extern "C"
