// Batched lens-parameter sweep: hundreds of samples with uneven image sizes and visibility
// counts go through deflection, degridding and gridding in ONE persistent launch.
//
// Every sample brings its own plan (binned visibilities; tile, KB width and chunk chosen per
// sample), its lens model and its pixel grid. The host flattens all of the samples' work into
// one queue of items, ordered longest first:
//   grid    -- one plan work item of a sample: row-owner gridding (grid_rows_item) into the
//              sample's half-plane grid;
//   degrid  -- one plan work item of a sample (degrid_item) into plan-order visibilities;
//   deflect -- kDeflectChunk pixels of a sample's grid: beta = theta - sum_l alpha_l(theta).
// A persistent kernel (one CTA per resident slot on every SM) takes items from the queue with
// one atomic counter per CTA and item, so big samples spread over the whole GPU and small ones
// fill the gaps; KB width 6 and 8 items run side by side in the same launch. One run is the
// counter reset, the zeroing of the samples' output grids and the kernel, captured once in a
// CUDA graph and replayed.
#include <algorithm>
#include <new>
#include <vector>

#include "common.cuh"
#include "deflect_device.cuh"
#include "gridding_items.cuh"

namespace lentils {

constexpr int kDeflectChunk = 2048;  // pixels per deflection item
constexpr int kSweepMaxLenses = 8;   // lenses per sample

enum SweepKind { kSweepGrid = 0, kSweepDegrid = 1, kSweepDeflect = 2 };

struct SweepWork {
    int sample, kind, index, pad;
};

struct SweepSampleDev {
    GridGeom g;
    KBPoly kb;
    int w2;
    int nitems;
    const uint2 *coords;
    const WorkItem *items;
    const int *chunk_begin;   // same-cell chunks (null: not built)
    const int2 *item_chunks;
    const float2 *grid_in;
    float2 *vis_out;
    const float2 *vis_in;
    float2 *grid_out;
    int lens0, nlenses;
    int nx, ny;
    double x0, y0, dx, dy;
    float2 *beta_out;
};

__device__ __forceinline__ void deflect_chunk(const SweepSampleDev &s,
                                              const DevLens *__restrict__ lenses, int chunk)
{
    const long long npix = (long long)s.nx * s.ny;
    const long long p0 = (long long)chunk * kDeflectChunk;
    const long long p1 = min(npix, p0 + kDeflectChunk);
    // positions x0 + i dx in FP32 pairs (hi + lo), so the pixel loop stays off the FP64 units:
    // the offset from a lens centre, (x0 - xc) + i dx with x0 - xc a pair made on the host, is
    // formed with an exact product error (fma) and a two-sum, rounded once
    const float dxh = (float)s.dx, dxl = (float)(s.dx - (double)dxh);
    const float dyh = (float)s.dy, dyl = (float)(s.dy - (double)dyh);
    const float xh = (float)s.x0, xl = (float)(s.x0 - (double)xh);
    const float yh = (float)s.y0, yl = (float)(s.y0 - (double)yh);
    auto pair_sum = [](float ch, float cl, float k, float dh, float dl) {  // (ch+cl) + k(dh+dl)
        const float pr = k * dh;
        const float pe = fmaf(k, dh, -pr);
        const float sm = ch + pr;
        const float bp = sm - ch;
        const float e = (ch - (sm - bp)) + (pr - bp);
        return sm + ((e + pe) + fmaf(k, dl, cl));
    };
    for (long long p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const int i = (int)(p / s.ny), j = (int)(p - (long long)i * s.ny);
        float axs = 0.f, ays = 0.f;
        for (int l = 0; l < s.nlenses; ++l) {
            const DevLens &L = lenses[s.lens0 + l];
            float ax, ay;
            lens_alpha(L, pair_sum(L.gxh, L.gxl, (float)i, dxh, dxl),
                       pair_sum(L.gyh, L.gyl, (float)j, dyh, dyl), ax, ay);
            axs += ax;
            ays += ay;
        }
        s.beta_out[p] = make_float2(pair_sum(xh, xl, (float)i, dxh, dxl) - axs,
                                    pair_sum(yh, yl, (float)j, dyh, dyl) - ays);
    }
}

// FORM 0: the ballot gridder and one visibility per degridding thread, three CTAs per SM (80
// registers, a few bytes of spill). FORM 1: the column-pair gridder and same-cell chunk
// degridding, two CTAs per SM (128 registers). FORM 2: the column-pair gridder and one
// visibility per degridding thread, two CTAs per SM.
template <int FORM>
__global__ void __launch_bounds__(kGridBatch, FORM == 0 ? 3 : 2)
    sweep_kernel(const SweepSampleDev *__restrict__ samples, const SweepWork *__restrict__ work,
                 int nwork, const DevLens *__restrict__ lenses, int *__restrict__ counter)
{
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ int next;
    __shared__ KBPoly kb;
    __shared__ GridGeom g;
    for (;;) {
        __syncthreads();  // the previous item is done with shared memory
        if (threadIdx.x == 0) next = atomicAdd(counter, 1);
        __syncthreads();
        const int w = next;
        if (w >= nwork) break;
        const SweepWork d = work[w];
        const SweepSampleDev &s = samples[d.sample];
        if (d.kind == kSweepDeflect) {
            deflect_chunk(s, lenses, d.index);
            continue;
        }
        // the sample's KB table and geometry, staged once per item
        {
            const int *src = reinterpret_cast<const int *>(&s.kb);
            int *dst = reinterpret_cast<int *>(&kb);
            for (int k = threadIdx.x; k < (int)(sizeof(KBPoly) / 4); k += blockDim.x) dst[k] = src[k];
            if (threadIdx.x == 0) g = s.g;
        }
        __syncthreads();
        const WorkItem it = s.items[d.index];
        if constexpr (FORM != 0) {
            if (d.kind == kSweepGrid) {
                if (s.w2 == 8)
                    grid_rows_item_pairs<8, 8>(s.vis_in, s.coords, s.grid_out, it, kb, g, smraw);
                else
                    grid_rows_item_pairs<6, 8>(s.vis_in, s.coords, s.grid_out, it, kb, g, smraw);
            } else if constexpr (FORM == 1) {
                const int2 cr = s.item_chunks[d.index];
                if (s.w2 == 8)
                    degrid_item_chunks<8, 4>(s.grid_in, s.coords, s.vis_out, it, cr,
                                             s.chunk_begin, kb, g, smraw);
                else
                    degrid_item_chunks<6, 4>(s.grid_in, s.coords, s.vis_out, it, cr,
                                             s.chunk_begin, kb, g, smraw);
            } else {
                if (s.w2 == 8) degrid_item<8, float>(s.grid_in, s.coords, s.vis_out, it, kb, g, nullptr, smraw);
                else degrid_item<6, float>(s.grid_in, s.coords, s.vis_out, it, kb, g, nullptr, smraw);
            }
        } else {
            if (d.kind == kSweepGrid) {
                if (s.w2 == 8)
                    grid_rows_item_ballot<8>(s.vis_in, s.coords, s.grid_out, it, kb, g, smraw);
                else
                    grid_rows_item_ballot<6>(s.vis_in, s.coords, s.grid_out, it, kb, g, smraw);
            } else {
                if (s.w2 == 8) degrid_item<8, float>(s.grid_in, s.coords, s.vis_out, it, kb, g, nullptr, smraw);
                else degrid_item<6, float>(s.grid_in, s.coords, s.vis_out, it, kb, g, nullptr, smraw);
            }
        }
    }
}

}  // namespace lentils

struct lentils_sweep {
    int nsamples;
    int nwork;
    int blocks;
    int form;  // sweep_kernel<form>
    size_t smem;
    long long total_vis, total_pixels;
    double algorithmic_bytes;
    lentils::SweepSampleDev *samples;
    lentils::SweepWork *work;
    lentils::DevLens *lenses;
    int *counter;
    std::vector<std::pair<float2 *, size_t>> zero;  // output grids to clear per run
    cudaGraph_t graph;
    cudaGraphExec_t gexec;
};

using namespace lentils;

static void sweep_free(lentils_sweep *sw)
{
    if (sw->gexec) cudaGraphExecDestroy(sw->gexec);
    if (sw->graph) cudaGraphDestroy(sw->graph);
    cudaFree(sw->samples);
    cudaFree(sw->work);
    cudaFree(sw->lenses);
    cudaFree(sw->counter);
}

static cudaError_t sweep_set_smem(int form, int smem)
{
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    if (form == 1) return cudaFuncSetAttribute(sweep_kernel<1>, a, smem);
    if (form == 2) return cudaFuncSetAttribute(sweep_kernel<2>, a, smem);
    return cudaFuncSetAttribute(sweep_kernel<0>, a, smem);
}

static cudaError_t sweep_occupancy(int form, int *per_sm, size_t smem)
{
    if (form == 1)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, sweep_kernel<1>, kGridBatch, smem);
    if (form == 2)
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, sweep_kernel<2>, kGridBatch, smem);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, sweep_kernel<0>, kGridBatch, smem);
}

static int sweep_enqueue(lentils_sweep *sw, cudaStream_t s)
{
    LENTILS_CUDA_TRY(cudaMemsetAsync(sw->counter, 0, sizeof(int), s));
    for (auto &z : sw->zero) LENTILS_CUDA_TRY(cudaMemsetAsync(z.first, 0, z.second, s));
    if (sw->nwork > 0) {
        if (sw->form == 1)
            sweep_kernel<1><<<sw->blocks, kGridBatch, sw->smem, s>>>(
                sw->samples, sw->work, sw->nwork, sw->lenses, sw->counter);
        else if (sw->form == 2)
            sweep_kernel<2><<<sw->blocks, kGridBatch, sw->smem, s>>>(
                sw->samples, sw->work, sw->nwork, sw->lenses, sw->counter);
        else
            sweep_kernel<0><<<sw->blocks, kGridBatch, sw->smem, s>>>(
                sw->samples, sw->work, sw->nwork, sw->lenses, sw->counter);
        LENTILS_CHECK_LAUNCH("sweep_kernel");
    }
    return LENTILS_OK;
}

extern "C" {

int lentils_sweep_create(lentils_sweep **out, const lentils_sweep_sample *in, int n, int flags,
                         void *stream)
{
    clear_error();
    if (!out || (!in && n > 0) || n < 0) return set_error(LENTILS_ERR_INVALID, "sweep_create: bad arguments");
    *out = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<SweepSampleDev> hs(n);
    std::vector<DevLens> hl;
    std::vector<std::pair<double, SweepWork>> items;
    lentils_sweep *sw = new (std::nothrow) lentils_sweep();
    if (!sw) return set_error(LENTILS_ERR_ALLOC, "sweep_create: host allocation");
    sw->form = flags & LENTILS_SWEEP_FORM_MASK;
    if (sw->form > 2) {
        delete sw;
        return set_error(LENTILS_ERR_INVALID, "sweep_create: kernel form %d (0 to 2)", flags & 3);
    }
    size_t smem = 0;
    int st = LENTILS_OK;
    for (int k = 0; k < n && !st; ++k) {
        const lentils_sweep_sample &a = in[k];
        const lentils_plan *p = a.plan;
        SweepSampleDev &d = hs[k];
        memset(&d, 0, sizeof(d));
        d.lens0 = (int)hl.size();
        d.nlenses = a.nlenses;
        d.nx = a.nx;
        d.ny = a.ny;
        d.x0 = a.x0;
        d.y0 = a.y0;
        d.dx = a.dx;
        d.dy = a.dy;
        d.beta_out = reinterpret_cast<float2 *>(a.beta_out);
        if (a.nlenses < 0 || a.nlenses > kSweepMaxLenses || (a.nlenses > 0 && !a.lenses) ||
            a.nx < 0 || a.ny < 0 || ((long long)a.nx * a.ny > 0 && !a.beta_out)) {
            st = set_error(LENTILS_ERR_INVALID, "sweep_create: sample %d: lenses or pixel grid", k);
            break;
        }
        for (int l = 0; l < a.nlenses && !st; ++l) {
            DevLens L;
            st = build_lens(a.lenses[l], L);
            const double gx = a.x0 - L.x0, gy = a.y0 - L.y0;
            L.gxh = (float)gx;
            L.gxl = (float)(gx - (double)L.gxh);
            L.gyh = (float)gy;
            L.gyl = (float)(gy - (double)L.gyh);
            hl.push_back(L);
        }
        if (st) break;
        const long long npix = (long long)a.nx * a.ny;
        sw->total_pixels += npix;
        for (long long c = 0; c * kDeflectChunk < npix; ++c)
            items.push_back({(double)std::min<long long>(kDeflectChunk, npix - c * kDeflectChunk) *
                                 (0.6 + 0.3 * a.nlenses),
                             SweepWork{k, kSweepDeflect, (int)c, 0}});
        if (!p) continue;
        const int w2 = 2 * p->geom.w;
        if (w2 != 6 && w2 != 8) {
            st = set_error(LENTILS_ERR_UNSUPPORTED, "sweep_create: sample %d: KB width %d (6 or 8)", k, w2);
            break;
        }
        if (!a.grid_in || !a.vis_out || !a.vis_in || !a.grid_out) {
            st = set_error(LENTILS_ERR_INVALID, "sweep_create: sample %d: null grid/vis buffer", k);
            break;
        }
        d.g = p->geom;
        d.kb = p->kb;
        d.w2 = w2;
        d.nitems = p->nitems;
        d.coords = p->coords;
        d.items = p->items;
        d.chunk_begin = p->chunk_begin;
        d.item_chunks = p->item_chunks;
        if (sw->form == 1 && p->nitems > 0 && (!p->chunk_begin || p->chunk_k != 4)) {
            st = set_error(LENTILS_ERR_UNSUPPORTED, "sweep_create: sample %d: no chunks", k);
            break;
        }
        d.grid_in = reinterpret_cast<const float2 *>(a.grid_in);
        d.vis_out = reinterpret_cast<float2 *>(a.vis_out);
        d.vis_in = reinterpret_cast<const float2 *>(a.vis_in);
        d.grid_out = reinterpret_cast<float2 *>(a.grid_out);
        const size_t gbytes = sizeof(float2) * (size_t)p->geom.nu * p->geom.half_nv;
        sw->zero.push_back({d.grid_out, gbytes});
        sw->total_vis += p->nvis;
        sw->algorithmic_bytes += 2.0 * (16.0 * (double)p->nvis + (double)gbytes);
        if (sw->form != 0)
            smem = std::max(smem, w2 == 8 ? grid_pairs_smem_bytes<8, 8>(p->geom)
                                          : grid_pairs_smem_bytes<6, 8>(p->geom));
        else
            smem = std::max(smem, w2 == 8 ? grid_ballot_smem_bytes<8>(p->geom)
                                          : grid_ballot_smem_bytes<6>(p->geom));
        smem = std::max(smem, degrid_smem_bytes<float>(p->geom));
        std::vector<WorkItem> hitems(p->nitems);
        if (p->nitems > 0) {
            cudaError_t e = cudaMemcpy(hitems.data(), p->items, sizeof(WorkItem) * p->nitems,
                                       cudaMemcpyDeviceToHost);
            if (e != cudaSuccess) {
                st = cuda_status(e, "sweep_create items");
                break;
            }
        }
        const double tile_cost = (double)p->geom.E * p->geom.E;
        const double taps = (double)w2 * w2;
        for (int i = 0; i < p->nitems; ++i) {
            const double c = (double)hitems[i].count;
            items.push_back({2.0 * tile_cost + c * taps * 0.35, SweepWork{k, kSweepGrid, i, 0}});
            items.push_back({tile_cost + c * taps * 0.2, SweepWork{k, kSweepDegrid, i, 0}});
        }
    }
    sw->algorithmic_bytes += 8.0 * (double)sw->total_pixels;
    if (!st && smem > 200 * 1024)
        st = set_error(LENTILS_ERR_UNSUPPORTED, "sweep_create: %zu bytes of shared memory per item", smem);
    if (st) {
        delete sw;
        return st;
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const std::pair<double, SweepWork> &a, const std::pair<double, SweepWork> &b) {
                         return a.first > b.first;
                     });
    std::vector<SweepWork> hw(items.size());
    for (size_t i = 0; i < items.size(); ++i) hw[i] = items[i].second;
    sw->nsamples = n;
    sw->nwork = (int)hw.size();
    sw->smem = std::max<size_t>(smem, 16);
    cudaError_t e = cudaMalloc(&sw->samples, sizeof(SweepSampleDev) * std::max(1, n));
    if (e == cudaSuccess) e = cudaMalloc(&sw->work, sizeof(SweepWork) * std::max<size_t>(1, hw.size()));
    if (e == cudaSuccess) e = cudaMalloc(&sw->lenses, sizeof(DevLens) * std::max<size_t>(1, hl.size()));
    if (e == cudaSuccess) e = cudaMalloc(&sw->counter, sizeof(int));
    if (e == cudaSuccess && n > 0)
        e = cudaMemcpyAsync(sw->samples, hs.data(), sizeof(SweepSampleDev) * n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !hw.empty())
        e = cudaMemcpyAsync(sw->work, hw.data(), sizeof(SweepWork) * hw.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !hl.empty())
        e = cudaMemcpyAsync(sw->lenses, hl.data(), sizeof(DevLens) * hl.size(), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = sweep_set_smem(sw->form, (int)sw->smem);
    int per_sm = 0, nsm = 0, dev = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = sweep_occupancy(sw->form, &per_sm, sw->smem);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        st = cuda_status(e, "sweep_create");
        sweep_free(sw);
        delete sw;
        return st;
    }
    sw->blocks = std::max(1, std::min(sw->nwork, std::max(1, per_sm) * nsm));
    *out = sw;
    return LENTILS_OK;
}

int lentils_sweep_destroy(lentils_sweep *sw)
{
    clear_error();
    if (!sw) return LENTILS_OK;
    sweep_free(sw);
    delete sw;
    return LENTILS_OK;
}

int lentils_sweep_run(lentils_sweep *sw, int use_graph, void *stream)
{
    clear_error();
    if (!sw) return set_error(LENTILS_ERR_INVALID, "sweep_run: null");
    cudaStream_t s = (cudaStream_t)stream;
    if (!use_graph) return sweep_enqueue(sw, s);
    if (!s) return set_error(LENTILS_ERR_INVALID, "sweep_run: graph capture needs a non-default stream");
    if (!sw->gexec) {
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_status(e, "sweep capture");
        const int q = sweep_enqueue(sw, s);
        e = cudaStreamEndCapture(s, &sw->graph);
        if (q) return q;
        if (e != cudaSuccess) return cuda_status(e, "sweep capture end");
        e = cudaGraphInstantiate(&sw->gexec, sw->graph, 0);
        if (e != cudaSuccess) return cuda_status(e, "sweep graph instantiate");
    }
    LENTILS_CUDA_TRY(cudaGraphLaunch(sw->gexec, s));
    return LENTILS_OK;
}

int lentils_sweep_get_stats(const lentils_sweep *sw, lentils_sweep_stats *st)
{
    clear_error();
    if (!sw || !st) return set_error(LENTILS_ERR_INVALID, "sweep_get_stats: null");
    st->nsamples = sw->nsamples;
    st->nwork = sw->nwork;
    st->blocks = sw->blocks;
    st->smem_bytes = (long long)sw->smem;
    st->total_vis = sw->total_vis;
    st->total_pixels = sw->total_pixels;
    st->algorithmic_bytes = sw->algorithmic_bytes;
    return LENTILS_OK;
}

}  // extern "C"
