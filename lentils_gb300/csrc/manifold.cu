// The reference's ManifoldLensOperator matrix on the GPU (manifold_lens_matrix_csr,
// lentils/backend/raster.c:272-395, with rasterize_triangle :120-268, split_edge :57-114 and
// reduce_triangle :32-54), built in FP64 with one thread per image pixel.
//
// Per unmasked image pixel: the 4 corners, 4 edge midpoints and the centre are deflected
// (FP64, the reference's formulas), the 8 triangles fanned around the centre are split
// recursively along source-pixel boundaries (longest index range first, at its middle grid
// line) until each piece lies in one source pixel, and each piece contributes
// -0.25 * (cross product of its barycentric corners) to that pixel. The reference then sorts
// the pixel's fragments by source pixel and reduces runs with two quirks kept here:
//   - the first fragment of every run after the first is not added (the loop starts a new run
//     without adding the fragment that starts it);
//   - a pixel without fragments still emits one entry of value 0, whose column is the first
//     column of the last earlier pixel that had fragments (the sorted buffer's first element),
//     or 0.
// The fragments are produced in the reference's order (depth-first stack), sorted stably, and
// reduced in that order. This file is compiled without floating-point contraction, so its
// FP64 arithmetic rounds like the reference's plain C.
//
// Two launches of the same per-pixel routine: the first counts fragments, the second writes
// them at the scanned offsets; a stable radix sort on (pixel, source pixel) keeps generation
// order within equal keys; a per-pixel reduction counts and then writes the CSR entries.
#include <cub/cub.cuh>

#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"

namespace lentils {

constexpr int kRasterStack = 64;  // STACK_SIZE of raster.c
constexpr long long kFragLimit = 128000;  // FRAGBUF_SIZE of raster.c (per image pixel)
enum { kRasterStackOverflow = 1, kRasterFragOverflow = 2 };

struct RTri {
    double verts[3][2];
    double barys[3][2];
    int idxmin[2], idxmax[2];
};

struct RGrid {
    int nx, ny;
    double xmin, ymin, dx, dy;
};

// ---- FP64 deflection, the reference's formulas (deflect.c) ----------------------------------
struct zc {
    double x, y;
};
__device__ __forceinline__ zc zmul(zc a, zc b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ __forceinline__ zc zdiv(zc a, zc b)
{
    const double d = b.x * b.x + b.y * b.y;
    return {(a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d};
}
__device__ __forceinline__ zc zsqrt(zc z)
{
    const double r = hypot(z.x, z.y);
    if (r == 0.0) return {0.0, 0.0};
    double re = sqrt(0.5 * (r + fabs(z.x)));
    double im = z.y / (2.0 * re);
    if (z.x < 0.0) {
        const double t = fabs(im);
        im = copysign(re, z.y);
        re = t;
    }
    return {re, im};
}

__device__ void alpha_pemd64(const double *p, double px, double py, double &ax, double &ay)
{
    const double t = 2.0 * p[7], q = p[2];
    const double b = pow(0.5 * p[6] * pow(q, t - 0.5) * (3.0 - t) / (2.0 - t), 1.0 / t);
    const zc crot = {p[5], -p[4]};
    const zc z = zmul({px - p[0], py - p[1]}, crot);
    const double x = z.x, y = z.y;
    const double rs2 = q * q * x * x + y * y;
    const double rs = sqrt(rs2);
    const zc qz = {q * z.x, q * z.y};
    zc A = zdiv({b * b, 0.0}, qz);
    const double pw = pow(b / rs, t - 2.0);
    A = {A.x * pw, A.y * pw};
    // hyp2f1_series (deflect.c:179-239) without derivatives
    const double r2 = q * q * x * x + y * y;
    const double qq = (1.0 - q * q) / (q * q);
    const zc w2 = zdiv({qq * r2, 0.0}, zmul(z, z));
    const zc s = zsqrt({1.0 - w2.x, -w2.y});
    const zc u = {0.5 * (1.0 - s.x), 0.5 * (0.0 - s.y)};
    zc f = {0.0, 0.0}, un = {1.0, 0.0};
    double an = 1.0;
    for (int n = 0; n < 20; ++n) {
        f = {f.x + an * un.x, f.y + an * un.y};
        const double ntf = 2 * n + 4 - t;
        un = zmul(un, u);
        an *= (ntf - t) / ntf;
    }
    const zc a = zmul(zmul(A, f), crot);
    ax += a.x;
    ay += -a.y;
}

__device__ void alpha_shear64(const double *p, double px, double py, double &ax, double &ay)
{
    const double sx = px - p[0], sy = py - p[1];
    const double cs2 = -p[5] * p[5] + p[4] * p[4];
    const double sn2 = -2 * p[4] * p[5];
    ax += p[2] * (cs2 * sx + sn2 * sy);
    ay += p[2] * (sn2 * sx - cs2 * sy);
    double sxr = sx * p[9] + sy * p[8];
    double syr = -sx * p[8] + sy * p[9];
    double dx = -0.25 * p[6] * (3 * sxr * sxr + syr * syr);
    double dy = -0.5 * p[6] * sxr * syr;
    ax += dx * p[9] - dy * p[8];
    ay += dx * p[8] + dy * p[9];
    sxr = sx * p[13] + sy * p[12];
    syr = -sx * p[12] + sy * p[13];
    dx = -0.5 * p[10] * (sxr * sxr - syr * syr);
    dy = 1.0 * p[10] * sxr * syr;
    ax += dx * p[13] - dy * p[12];
    ay += dx * p[12] + dy * p[13];
}

__device__ void alpha_multipoles64(const double *p, int order, double px, double py, double &ax,
                                   double &ay)
{
    const double sx = px - p[0], sy = py - p[1];
    const double r = sqrt(sx * sx + sy * sy);
    const double th = atan2(sy, sx);
    const double cn = sx / r, sn = sy / r;
    for (int m = 3; m <= order; ++m) {
        const double am = p[3 + 2 * (m - 3)], bm = p[3 + 2 * (m - 3) + 1];
        const double alpha = 2.0 * p[2];
        const double norm = 2.0 * pow(1.0, alpha) / (m * m - (alpha - 2) * (alpha - 2));
        const double cm = cos(m * th), sm = sin(m * th);
        const double dr = -norm * (2.0 - alpha) * pow(r, 1.0 - alpha) * (bm * sm + am * cm);
        const double dt = norm * m * pow(r, 1.0 - alpha) * (-bm * cm + am * sm);
        ax += cn * dr - sn * dt;
        ay += sn * dr + cn * dt;
    }
}

__device__ void deflect64(const lentils_mass_model *__restrict__ lenses, int nl, double px,
                          double py, double &bx, double &by)
{
    bx = px;
    by = py;
    for (int l = 0; l < nl; ++l) {
        double ax = 0.0, ay = 0.0;
        const lentils_mass_model &m = lenses[l];
        if (m.type == 0) alpha_pemd64(m.fpars, px, py, ax, ay);
        else if (m.type == 1) alpha_shear64(m.fpars, px, py, ax, ay);
        else if (m.type == 2) alpha_multipoles64(m.fpars, m.ipars[0], px, py, ax, ay);
        bx -= ax;
        by -= ay;
    }
}

// ---- rasterisation (raster.c), fragments to a sink ----------------------------------------------
__constant__ int c_num_new_verts[8] = {0, 2, 2, 2, 2, 2, 2, 0};
__constant__ int c_edge_inds[8][2][2] = {{{0, 0}, {0, 0}}, {{0, 1}, {0, 2}}, {{0, 1}, {1, 2}},
                                         {{0, 2}, {1, 2}}, {{0, 2}, {1, 2}}, {{0, 1}, {1, 2}},
                                         {{0, 1}, {0, 2}}, {{0, 0}, {0, 0}}};
__constant__ int c_num_new_tris[8] = {1, 3, 3, 3, 3, 3, 3, 1};
__constant__ int c_new_tri_inds[8][3][3] = {
    {{0, 1, 2}, {0, 0, 0}, {0, 0, 0}}, {{1, 2, 4}, {1, 4, 3}, {0, 3, 4}},
    {{0, 3, 4}, {0, 4, 2}, {1, 4, 3}}, {{2, 3, 4}, {0, 4, 3}, {0, 1, 4}},
    {{0, 1, 4}, {0, 4, 3}, {2, 3, 4}}, {{1, 4, 3}, {0, 3, 4}, {0, 4, 2}},
    {{0, 3, 4}, {1, 2, 4}, {1, 4, 3}}, {{0, 1, 2}, {0, 0, 0}, {0, 0, 0}}};
__constant__ int c_new_tri_sides[8][3] = {{0, 0, 0}, {0, 0, 1}, {0, 0, 1}, {0, 1, 1},
                                          {0, 0, 1}, {0, 1, 1}, {0, 1, 1}, {1, 0, 0}};

struct FragSink {
    double *area;   // null: count only
    int *col;
    long long base, n;
    int flags;
    __device__ void put(double a, int c)
    {
        if (n >= kFragLimit) {
            flags |= kRasterFragOverflow;
            return;
        }
        if (area) {
            area[base + n] = a;
            col[base + n] = c;
        }
        ++n;
    }
};

__device__ void rasterize_triangle_dev(const double (&vin)[3][2], const RGrid &g, FragSink &sink)
{
    RTri stack[kRasterStack];
    const double dd[2] = {g.dx, g.dy};
    const double bmin[2] = {g.xmin, g.ymin};
    RTri tri;
    tri.idxmin[0] = g.nx;
    tri.idxmin[1] = g.ny;
    tri.idxmax[0] = 0;
    tri.idxmax[1] = 0;
    tri.barys[0][0] = 0.0;
    tri.barys[0][1] = 0.0;
    tri.barys[1][0] = 0.0;
    tri.barys[1][1] = 1.0;
    tri.barys[2][0] = 1.0;
    tri.barys[2][1] = 0.0;
    for (int v = 0; v < 3; ++v) {
        tri.verts[v][0] = vin[v][0];
        tri.verts[v][1] = vin[v][1];
        const int i = (int)floor((tri.verts[v][0] - g.xmin) / g.dx);
        const int j = (int)floor((tri.verts[v][1] - g.ymin) / g.dy);
        if (i < tri.idxmin[0]) tri.idxmin[0] = i;
        if (j < tri.idxmin[1]) tri.idxmin[1] = j;
        if (i + 1 > tri.idxmax[0]) tri.idxmax[0] = i + 1;
        if (j + 1 > tri.idxmax[1]) tri.idxmax[1] = j + 1;
    }
    int nstack = 0;
    stack[nstack++] = tri;
    while (nstack > 0) {
        tri = stack[--nstack];
        int dmax = 0, spax = 0;
        for (int i = 0; i < 2; ++i) {
            const int siz = tri.idxmax[i] - tri.idxmin[i];
            if (siz > dmax) {
                dmax = siz;
                spax = i;
            }
        }
        const int spind = tri.idxmin[spax] + dmax / 2;
        const double spcoord = spind * dd[spax] + bmin[spax];
        if (dmax == 1) {
            const int i = tri.idxmin[0], j = tri.idxmin[1];
            if (i < 0 || i >= g.nx) continue;
            if (j < 0 || j >= g.ny) continue;
            const double x1 = tri.barys[0][0], y1 = tri.barys[0][1];
            const double x2 = tri.barys[1][0], y2 = tri.barys[1][1];
            const double x3 = tri.barys[2][0], y3 = tri.barys[2][1];
            sink.put(-0.25 * (x1 * (y2 - y3) + x2 * (y3 - y1) + x3 * (y1 - y2)), g.ny * i + j);
            if (sink.n >= kFragLimit) return;  // the reference stops this triangle
            continue;
        }
        double vb[5][2], bb[5][2], vdists[3];
        for (int v = 0; v < 3; ++v) {
            vb[v][0] = tri.verts[v][0];
            vb[v][1] = tri.verts[v][1];
            bb[v][0] = tri.barys[v][0];
            bb[v][1] = tri.barys[v][1];
        }
        vb[3][0] = vb[3][1] = vb[4][0] = vb[4][1] = 0.0;
        bb[3][0] = bb[3][1] = bb[4][0] = bb[4][1] = 0.0;
        int vbits = 0;
        for (int v = 0; v < 3; ++v) {
            vdists[v] = vb[v][spax] - spcoord;
            vbits |= ((vdists[v] > 0.) << v);
        }
        const int inds[3] = {tri.idxmin[spax], spind, tri.idxmax[spax]};
        for (int v = 0; v < c_num_new_verts[vbits]; ++v) {
            const int v0 = c_edge_inds[vbits][v][0], v1 = c_edge_inds[vbits][v][1];
            const double w0 = vdists[v1], w1 = -vdists[v0];
            const double wnorm = 1.0 / (w0 + w1);
            const double a = w0 * wnorm, b = w1 * wnorm;
            vb[3 + v][0] = a * vb[v0][0] + b * vb[v1][0];
            vb[3 + v][1] = a * vb[v0][1] + b * vb[v1][1];
            bb[3 + v][0] = a * bb[v0][0] + b * bb[v1][0];
            bb[3 + v][1] = a * bb[v0][1] + b * bb[v1][1];
        }
        for (int t = 0; t < c_num_new_tris[vbits]; ++t) {
            const int s = c_new_tri_sides[vbits][t];
            tri.idxmin[spax] = inds[s];
            tri.idxmax[spax] = inds[s + 1];
            if (tri.idxmax[0] <= 0 || tri.idxmin[0] >= g.nx) continue;
            if (tri.idxmax[1] <= 0 || tri.idxmin[1] >= g.ny) continue;
            for (int v = 0; v < 3; ++v) {
                const int k = c_new_tri_inds[vbits][t][v];
                tri.verts[v][0] = vb[k][0];
                tri.verts[v][1] = vb[k][1];
                tri.barys[v][0] = bb[k][0];
                tri.barys[v][1] = bb[k][1];
            }
            stack[nstack++] = tri;
            if (nstack >= kRasterStack) {
                sink.flags |= kRasterStackOverflow;
                return;
            }
        }
    }
}

// the fragments of image pixel (iim, jim) in the reference's order
__device__ void pixel_fragments(int iim, int jim, const RGrid &img, const RGrid &src,
                                const lentils_mass_model *__restrict__ lenses, int nl,
                                FragSink &sink)
{
    const double pxmin = img.xmin + iim * img.dx, pxmax = img.xmin + (iim + 1) * img.dx;
    const double pymin = img.ymin + jim * img.dy, pymax = img.ymin + (jim + 1) * img.dy;
    const double mx = 0.5 * (pxmin + pxmax), my = 0.5 * (pymin + pymax);
    const double im[9][2] = {{pxmin, pymin}, {mx, pymin}, {pxmax, pymin}, {pxmax, my},
                             {pxmax, pymax}, {mx, pymax}, {pxmin, pymax}, {pxmin, my}, {mx, my}};
    double sp[9][2];
    for (int k = 0; k < 9; ++k) deflect64(lenses, nl, im[k][0], im[k][1], sp[k][0], sp[k][1]);
    for (int t = 0; t < 8; ++t) {
        double tp[3][2];
        tp[1][0] = sp[t][0];
        tp[1][1] = sp[t][1];
        tp[0][0] = sp[(t + 1) % 8][0];
        tp[0][1] = sp[(t + 1) % 8][1];
        tp[2][0] = sp[8][0];
        tp[2][1] = sp[8][1];
        rasterize_triangle_dev(tp, src, sink);
    }
}

__global__ void __launch_bounds__(128)
    frag_kernel(RGrid img, RGrid src, const unsigned char *__restrict__ mask,
                const lentils_mass_model *__restrict__ lenses, int nl,
                long long *__restrict__ counts, const long long *__restrict__ offsets,
                double *__restrict__ area, int *__restrict__ col, int *__restrict__ flags)
{
    const long long n = (long long)img.nx * img.ny;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x) {
        FragSink sink{nullptr, nullptr, 0, 0, 0};
        if (mask[p]) {
            if (offsets) {
                sink.area = area;
                sink.col = col;
                sink.base = offsets[p];
            }
            pixel_fragments((int)(p / img.ny), (int)(p % img.ny), img, src, lenses, nl, sink);
        }
        if (counts) counts[p] = sink.n;
        if (sink.flags) atomicOr(flags, sink.flags);
    }
}

// sort keys: (pixel << 32) | column; generation index as the value
__global__ void frag_keys_kernel(const long long *__restrict__ offsets, const int *__restrict__ col,
                                 unsigned long long *__restrict__ keys, long long npix,
                                 long long nfrag)
{
    // one thread per pixel writes its fragments' keys
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        const long long b = offsets[p], e = (p + 1 < npix) ? offsets[p + 1] : nfrag;
        for (long long f = b; f < e; ++f)
            keys[f] = ((unsigned long long)p << 32) | (unsigned int)col[f];
    }
}

// per pixel: first column of its sorted fragments (-1: none)
__global__ void first_col_kernel(const long long *__restrict__ offsets,
                                 const unsigned long long *__restrict__ skeys,
                                 int *__restrict__ first, long long npix, long long nfrag)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        const long long b = offsets[p], e = (p + 1 < npix) ? offsets[p + 1] : nfrag;
        first[p] = (e > b) ? (int)(skeys[b] & 0xffffffffu) : -1;
    }
}

struct LastValid {
    __device__ int operator()(int a, int b) const { return b >= 0 ? b : a; }
};

// per pixel: the reference's reduction of its sorted fragments; count (rows == null) or write
__global__ void reduce_kernel(const long long *__restrict__ offsets,
                              const unsigned long long *__restrict__ skeys,
                              const double *__restrict__ sarea, const unsigned char *__restrict__ mask,
                              const int *__restrict__ stale, int *__restrict__ counts,
                              const int *__restrict__ rows, int *__restrict__ cols,
                              double *__restrict__ vals, long long npix, long long nfrag)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < npix;
         p += (long long)gridDim.x * blockDim.x) {
        if (!mask[p]) {
            if (counts) counts[p] = 0;
            continue;
        }
        const long long b = offsets[p], e = (p + 1 < npix) ? offsets[p + 1] : nfrag;
        int k = 0;
        const int base = rows ? rows[p] : 0;
        if (e == b) {  // no fragments: one zero entry with the stale column
            if (rows) {
                cols[base] = (p > 0 && stale[p - 1] >= 0) ? stale[p - 1] : 0;
                vals[base] = 0.0;
            }
            k = 1;
        } else {
            double val = 0.0;
            int c = (int)(skeys[b] & 0xffffffffu);
            for (long long f = b; f < e; ++f) {
                const int cf = (int)(skeys[f] & 0xffffffffu);
                if (cf != c) {
                    if (rows) {
                        cols[base + k] = c;
                        vals[base + k] = val;
                    }
                    ++k;
                    val = 0.0;
                    c = cf;
                } else {
                    val += sarea[f];
                }
            }
            if (rows) {
                cols[base + k] = c;
                vals[base + k] = val;
            }
            ++k;
        }
        if (counts) counts[p] = k;
    }
}

__global__ void gather_area_kernel(const int *__restrict__ order, const double *__restrict__ area,
                                   double *__restrict__ sarea, long long n)
{
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n;
         f += (long long)gridDim.x * blockDim.x)
        sarea[f] = area[order[f]];
}

__global__ void iota_kernel(int *__restrict__ v, long long n)
{
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < n;
         f += (long long)gridDim.x * blockDim.x)
        v[f] = (int)f;
}

static int nblocks(long long n, int bs)
{
    return (int)std::max(1LL, std::min((n + bs - 1) / bs, 152LL * 64));
}

struct DevScratch {
    std::vector<void *> ptrs;
    ~DevScratch()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    template <typename T>
    int alloc(T **p, size_t n)
    {
        cudaError_t e = cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(1, n));
        if (e != cudaSuccess) return cuda_status(e, "manifold scratch");
        ptrs.push_back(*p);
        return LENTILS_OK;
    }
};

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_manifold_lens_matrix(const lentils_image_space *im, const lentils_image_space *src,
                                 const lentils_mass_model *lenses, int nlenses,
                                 const unsigned char *mask_dev, int **row_inds, int **cols,
                                 double **vals, long long *nnz_out, void *stream)
{
    clear_error();
    if (!im || !src || (nlenses > 0 && !lenses) || nlenses < 0 || !mask_dev || !row_inds ||
        !cols || !vals || !nnz_out || im->nx < 1 || im->ny < 1 || src->nx < 1 || src->ny < 1)
        return set_error(LENTILS_ERR_INVALID, "manifold_lens_matrix: bad arguments");
    *row_inds = nullptr;
    *cols = nullptr;
    *vals = nullptr;
    *nnz_out = 0;
    cudaStream_t s = (cudaStream_t)stream;
    const long long npix = (long long)im->nx * im->ny;
    RGrid gi{im->nx, im->ny, im->xmin, im->ymin, im->dx, im->dy};
    RGrid gs{src->nx, src->ny, src->xmin, src->ymin, src->dx, src->dy};
    DevScratch tmp;
    lentils_mass_model *dl;
    long long *fcount, *foff;
    int *flags;
    int st;
    if ((st = tmp.alloc(&dl, nlenses))) return st;
    if ((st = tmp.alloc(&fcount, npix))) return st;
    if ((st = tmp.alloc(&foff, npix))) return st;
    if ((st = tmp.alloc(&flags, 1))) return st;
    if (nlenses > 0)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(dl, lenses, sizeof(lentils_mass_model) * nlenses,
                                         cudaMemcpyHostToDevice, s));
    LENTILS_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int), s));
    frag_kernel<<<nblocks(npix, 128), 128, 0, s>>>(gi, gs, mask_dev, dl, nlenses, fcount,
                                                   nullptr, nullptr, nullptr, flags);
    LENTILS_CHECK_LAUNCH("frag_kernel (count)");
    // offsets and total
    size_t tb = 0;
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, fcount, foff, npix, s));
    unsigned char *scan_tmp;
    if ((st = tmp.alloc(&scan_tmp, tb))) return st;
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(scan_tmp, tb, fcount, foff, npix, s));
    long long last_off = 0, last_cnt = 0;
    int hflags = 0;
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&last_off, foff + npix - 1, sizeof(long long), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&last_cnt, fcount + npix - 1, sizeof(long long), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaMemcpyAsync(&hflags, flags, sizeof(int), cudaMemcpyDeviceToHost, s));
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    if (hflags)
        return set_error(LENTILS_ERR_UNSUPPORTED,
                         "manifold_lens_matrix: rasterisation %s overflow (the reference stops "
                         "there too)", (hflags & kRasterStackOverflow) ? "stack" : "fragment");
    const long long nfrag = last_off + last_cnt;
    if (nfrag > 0x7fffffffLL)
        return set_error(LENTILS_ERR_UNSUPPORTED, "manifold_lens_matrix: %lld fragments", nfrag);
    double *area, *sarea;
    int *fcol, *order, *sorder, *first, *stale, *ecount;
    unsigned long long *keys, *skeys;
    if ((st = tmp.alloc(&area, nfrag))) return st;
    if ((st = tmp.alloc(&sarea, nfrag))) return st;
    if ((st = tmp.alloc(&fcol, nfrag))) return st;
    if ((st = tmp.alloc(&order, nfrag))) return st;
    if ((st = tmp.alloc(&sorder, nfrag))) return st;
    if ((st = tmp.alloc(&keys, nfrag))) return st;
    if ((st = tmp.alloc(&skeys, nfrag))) return st;
    if ((st = tmp.alloc(&first, npix))) return st;
    if ((st = tmp.alloc(&stale, npix))) return st;
    if ((st = tmp.alloc(&ecount, npix + 1))) return st;
    frag_kernel<<<nblocks(npix, 128), 128, 0, s>>>(gi, gs, mask_dev, dl, nlenses, nullptr, foff,
                                                   area, fcol, flags);
    LENTILS_CHECK_LAUNCH("frag_kernel (write)");
    frag_keys_kernel<<<nblocks(npix, 256), 256, 0, s>>>(foff, fcol, keys, npix, nfrag);
    iota_kernel<<<nblocks(nfrag, 256), 256, 0, s>>>(order, nfrag);
    LENTILS_CHECK_LAUNCH("frag_keys_kernel");
    int bits = 32;
    while (bits < 64 && (1LL << (bits - 32)) < npix) ++bits;
    tb = 0;
    LENTILS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, skeys, order, sorder,
                                                     (int64_t)nfrag, 0, bits, s));
    unsigned char *sort_tmp;
    if ((st = tmp.alloc(&sort_tmp, tb))) return st;
    LENTILS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(sort_tmp, tb, keys, skeys, order, sorder,
                                                     (int64_t)nfrag, 0, bits, s));
    gather_area_kernel<<<nblocks(nfrag, 256), 256, 0, s>>>(sorder, area, sarea, nfrag);
    first_col_kernel<<<nblocks(npix, 256), 256, 0, s>>>(foff, skeys, first, npix, nfrag);
    LENTILS_CHECK_LAUNCH("first_col_kernel");
    // stale[p] = first column of the last pixel <= p with fragments (-1 if none)
    tb = 0;
    LENTILS_CUDA_TRY(cub::DeviceScan::InclusiveScan(nullptr, tb, first, stale, LastValid(), npix, s));
    unsigned char *scan2;
    if ((st = tmp.alloc(&scan2, tb))) return st;
    LENTILS_CUDA_TRY(cub::DeviceScan::InclusiveScan(scan2, tb, first, stale, LastValid(), npix, s));
    reduce_kernel<<<nblocks(npix, 256), 256, 0, s>>>(foff, skeys, sarea, mask_dev, stale, ecount,
                                                     nullptr, nullptr, nullptr, npix, nfrag);
    LENTILS_CHECK_LAUNCH("reduce_kernel (count)");
    LENTILS_CUDA_TRY(cudaMemsetAsync(ecount + npix, 0, sizeof(int), s));
    int *rows_out;
    LENTILS_CUDA_TRY(cudaMalloc(&rows_out, sizeof(int) * (npix + 1)));
    tb = 0;
    cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, tb, ecount, rows_out, npix + 1, s);
    unsigned char *scan3 = nullptr;
    if (e == cudaSuccess && (st = tmp.alloc(&scan3, tb))) {
        cudaFree(rows_out);
        return st;
    }
    if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(scan3, tb, ecount, rows_out, npix + 1, s);
    int nnz = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nnz, rows_out + npix, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(rows_out);
        return cuda_status(e, "manifold_lens_matrix rows");
    }
    int *cols_out = nullptr;
    double *vals_out = nullptr;
    e = cudaMalloc(&cols_out, sizeof(int) * std::max(1, nnz));
    if (e == cudaSuccess) e = cudaMalloc(&vals_out, sizeof(double) * std::max(1, nnz));
    if (e == cudaSuccess) {
        reduce_kernel<<<nblocks(npix, 256), 256, 0, s>>>(foff, skeys, sarea, mask_dev, stale,
                                                         nullptr, rows_out, cols_out, vals_out,
                                                         npix, nfrag);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(rows_out);
        cudaFree(cols_out);
        cudaFree(vals_out);
        return cuda_status(e, "manifold_lens_matrix reduce");
    }
    *row_inds = rows_out;
    *cols = cols_out;
    *vals = vals_out;
    *nnz_out = nnz;
    return LENTILS_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// FP64 deflection with the reference's formulas, and the Delaunay lens matrix
// (delaunay_lens_matrix_csr, lentils/backend/triangles.c:105-140, with the barycentric weights
// of triangle_geometry :7-30).
// ------------------------------------------------------------------------------------------------
namespace lentils {

__global__ void deflect64_kernel(const lentils_mass_model *__restrict__ lenses, int nl,
                                 const double2 *__restrict__ pin, double2 *__restrict__ pout,
                                 long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double2 p = pin[i];
        double bx, by;
        deflect64(lenses, nl, p.x, p.y, bx, by);
        pout[i] = make_double2(bx, by);
    }
}

// per pixel: 1 if unmasked and casted / uncasted (for the running indices of the reference)
__global__ void delaunay_flags_kernel(const unsigned char *__restrict__ mask, int nx, int ny,
                                      int ncast, int *__restrict__ cflag, int *__restrict__ uflag)
{
    const long long n = (long long)nx * ny;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p / ny), j = (int)(p - (long long)i * ny);
        const bool on = mask[p] != 0;
        const bool cast = (i % ncast == 0) && (j % ncast == 0);
        cflag[p] = (on && cast) ? 1 : 0;
        uflag[p] = (on && !cast) ? 1 : 0;
    }
}

// entries per pixel (counts) or the entries themselves (rows != null)
__global__ void delaunay_entries_kernel(const unsigned char *__restrict__ mask, int nx, int ny,
                                        int ncast, const int *__restrict__ cidx,
                                        const int *__restrict__ uidx,
                                        const double2 *__restrict__ upts,
                                        const int *__restrict__ tind, const int *__restrict__ tris,
                                        const double2 *__restrict__ tpts, int *__restrict__ counts,
                                        const int *__restrict__ rows, int *__restrict__ cols,
                                        double *__restrict__ vals)
{
    const long long n = (long long)nx * ny;
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n;
         p += (long long)gridDim.x * blockDim.x) {
        int k = 0;
        if (mask[p]) {
            const int i = (int)(p / ny), j = (int)(p - (long long)i * ny);
            if ((i % ncast) || (j % ncast)) {
                const int u = uidx[p];
                const int t = tind[u];
                if (t >= 0) {
                    k = 3;
                    if (rows) {
                        const double2 s = upts[u];
                        int pv[3];
                        double a[3][2];
                        for (int v = 0; v < 3; ++v) {
                            pv[v] = tris[3 * t + v];
                            a[v][0] = tpts[pv[v]].x - s.x;
                            a[v][1] = tpts[pv[v]].y - s.y;
                        }
                        double w0 = a[1][0] * a[2][1] - a[2][0] * a[1][1];
                        double w1 = a[2][0] * a[0][1] - a[0][0] * a[2][1];
                        double w2 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
                        const double area = w0 + w1 + w2;
                        const double inv = 1.0 / area;
                        w0 *= inv;
                        w1 *= inv;
                        w2 *= inv;
                        const int b = rows[p];
                        vals[b] = w0;
                        cols[b] = pv[0];
                        vals[b + 1] = w1;
                        cols[b + 1] = pv[1];
                        vals[b + 2] = w2;
                        cols[b + 2] = pv[2];
                    }
                }
            } else {
                k = 1;
                if (rows) {
                    vals[rows[p]] = 1.0;
                    cols[rows[p]] = cidx[p];
                }
            }
        }
        if (counts) counts[p] = k;
    }
}

}  // namespace lentils

extern "C" {

int lentils_deflect64(const lentils_mass_model *lenses, int nlenses, const double *points,
                      double *out, long long npoints, void *stream)
{
    clear_error();
    if ((nlenses > 0 && !lenses) || nlenses < 0 || npoints < 0 ||
        (npoints > 0 && (!points || !out)))
        return set_error(LENTILS_ERR_INVALID, "deflect64: bad arguments");
    if (npoints == 0) return LENTILS_OK;
    cudaStream_t s = (cudaStream_t)stream;
    DevScratch tmp;
    lentils_mass_model *dl;
    if (int st = tmp.alloc(&dl, nlenses)) return st;
    if (nlenses > 0)
        LENTILS_CUDA_TRY(cudaMemcpyAsync(dl, lenses, sizeof(lentils_mass_model) * nlenses,
                                         cudaMemcpyHostToDevice, s));
    deflect64_kernel<<<nblocks(npoints, 256), 256, 0, s>>>(dl, nlenses, (const double2 *)points,
                                                           (double2 *)out, npoints);
    LENTILS_CHECK_LAUNCH("deflect64_kernel");
    LENTILS_CUDA_TRY(cudaStreamSynchronize(s));
    return LENTILS_OK;
}

int lentils_delaunay_lens_matrix(const unsigned char *mask_dev, int nx, int ny, int ncast,
                                 const double *uncasted_points, const int *uncasted_tri_inds,
                                 const int *triangles, const double *tri_points, int **row_inds,
                                 int **cols, double **vals, long long *nnz_out, void *stream)
{
    clear_error();
    if (!mask_dev || nx < 1 || ny < 1 || ncast < 1 || !row_inds || !cols || !vals || !nnz_out)
        return set_error(LENTILS_ERR_INVALID, "delaunay_lens_matrix: bad arguments");
    *row_inds = nullptr;
    *cols = nullptr;
    *vals = nullptr;
    *nnz_out = 0;
    cudaStream_t s = (cudaStream_t)stream;
    const long long npix = (long long)nx * ny;
    DevScratch tmp;
    int *cflag, *uflag, *cidx, *uidx, *counts;
    int st;
    if ((st = tmp.alloc(&cflag, npix))) return st;
    if ((st = tmp.alloc(&uflag, npix))) return st;
    if ((st = tmp.alloc(&cidx, npix))) return st;
    if ((st = tmp.alloc(&uidx, npix))) return st;
    if ((st = tmp.alloc(&counts, npix + 1))) return st;
    delaunay_flags_kernel<<<nblocks(npix, 256), 256, 0, s>>>(mask_dev, nx, ny, ncast, cflag, uflag);
    LENTILS_CHECK_LAUNCH("delaunay_flags_kernel");
    size_t tb = 0;
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, cflag, cidx, npix, s));
    unsigned char *t1;
    if ((st = tmp.alloc(&t1, tb))) return st;
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t1, tb, cflag, cidx, npix, s));
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(t1, tb, uflag, uidx, npix, s));
    delaunay_entries_kernel<<<nblocks(npix, 256), 256, 0, s>>>(
        mask_dev, nx, ny, ncast, cidx, uidx, (const double2 *)uncasted_points, uncasted_tri_inds,
        triangles, (const double2 *)tri_points, counts, nullptr, nullptr, nullptr);
    LENTILS_CHECK_LAUNCH("delaunay_entries_kernel (count)");
    LENTILS_CUDA_TRY(cudaMemsetAsync(counts + npix, 0, sizeof(int), s));
    int *rows_out = nullptr, *cols_out = nullptr;
    double *vals_out = nullptr;
    tb = 0;
    LENTILS_CUDA_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tb, counts, counts, npix + 1, s));
    unsigned char *t2;
    if ((st = tmp.alloc(&t2, tb))) return st;
    LENTILS_CUDA_TRY(cudaMalloc(&rows_out, sizeof(int) * (npix + 1)));
    cudaError_t e = cub::DeviceScan::ExclusiveSum(t2, tb, counts, rows_out, npix + 1, s);
    int nnz = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nnz, rows_out + npix, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMalloc(&cols_out, sizeof(int) * std::max(1, nnz));
    if (e == cudaSuccess) e = cudaMalloc(&vals_out, sizeof(double) * std::max(1, nnz));
    if (e == cudaSuccess) {
        delaunay_entries_kernel<<<nblocks(npix, 256), 256, 0, s>>>(
            mask_dev, nx, ny, ncast, cidx, uidx, (const double2 *)uncasted_points,
            uncasted_tri_inds, triangles, (const double2 *)tri_points, nullptr, rows_out,
            cols_out, vals_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        cudaFree(rows_out);
        cudaFree(cols_out);
        cudaFree(vals_out);
        return cuda_status(e, "delaunay_lens_matrix");
    }
    *row_inds = rows_out;
    *cols = cols_out;
    *vals = vals_out;
    *nnz_out = nnz;
    return LENTILS_OK;
}

}  // extern "C"
