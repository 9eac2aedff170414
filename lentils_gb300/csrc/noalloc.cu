// Gridding without any device allocation, for callers that cannot call cudaMalloc.
//
// Who needs this: code that runs where allocating device memory is not allowed or not
// possible -- inside a host callback or a CUDA stream-ordered section that must not
// synchronise, with device memory that another framework's pool has already claimed in full,
// or in a long-running real-time pipeline that forbids allocation after start-up. Such a caller
// owns its inputs and outputs in device memory and needs the visibilities gridded without the
// plan object (lentils_plan_create allocates the plan arrays, its temporaries and the sort's
// storage).
//
// lentils_grid_noalloc runs the same binning and gridding kernels as the plan path
// (lentils_plan_create + lentils_vis_to_plan + lentils_grid), but every temporary array --
// binning keys, permutation, plan-frame coordinates and visibilities, tile counts, work items
// and the radix sort's storage -- lives in one file-scope device array of fixed size, so the call
// allocates nothing. The size bounds the batch: at most kNoAllocMaxVis visibilities
// (nrows * nchannels) and kNoAllocMaxTiles uv tiles per call; larger inputs are rejected with
// LENTILS_ERR_INVALID. Gridding accumulates into the caller's grid, so larger sets are gridded
// by calling once per batch of visibilities.
//
// Sharing: every call on a device uses the same array, which keeps the previous call's
// contents (everything that must start at zero is cleared on the stream by each call). Calls
// whose GPU work overlaps -- on different streams, or from different host threads without
// ordering -- race on the array and corrupt each other's results; order them on one stream.
#include <cuda.h>  // driver types for the context lookup (entry points fetched at run time)
#include <cub/cub.cuh>

#include <algorithm>
#include <mutex>

#include "common.cuh"

namespace lentils {

constexpr int kNoAllocMaxVis = 1 << 16;     // visibilities per call
constexpr int kNoAllocMaxTiles = 1 << 16;   // uv tiles of the grid
constexpr int kNoAllocChunk = 256;          // visibilities per work item
constexpr int kNoAllocMaxItems = kNoAllocMaxVis / kNoAllocChunk + kNoAllocMaxVis;
constexpr size_t kNoAllocSortBytes = 2u << 20;  // radix-sort storage reserved

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of the regions inside the scratch array.
constexpr size_t kOffKeysIn = 0;
constexpr size_t kOffKeysOut = kOffKeysIn + align256(sizeof(unsigned) * kNoAllocMaxVis);
constexpr size_t kOffIdx = kOffKeysOut + align256(sizeof(unsigned) * kNoAllocMaxVis);
constexpr size_t kOffPerm = kOffIdx + align256(sizeof(int) * kNoAllocMaxVis);
constexpr size_t kOffCoordsUser = kOffPerm + align256(sizeof(int) * kNoAllocMaxVis);
constexpr size_t kOffCoordsPlan = kOffCoordsUser + align256(sizeof(uint2) * kNoAllocMaxVis);
constexpr size_t kOffPhaseUser = kOffCoordsPlan + align256(sizeof(uint2) * kNoAllocMaxVis);
constexpr size_t kOffPhasePlan = kOffPhaseUser + align256(sizeof(float2) * kNoAllocMaxVis);
constexpr size_t kOffVisPlan = kOffPhasePlan + align256(sizeof(float2) * kNoAllocMaxVis);
constexpr size_t kOffTileCounts = kOffVisPlan + align256(sizeof(float2) * kNoAllocMaxVis);
constexpr size_t kOffItems = kOffTileCounts + align256(sizeof(int) * kNoAllocMaxTiles);
constexpr size_t kOffFlags = kOffItems + align256(sizeof(WorkItem) * kNoAllocMaxItems);
constexpr size_t kOffSort = kOffFlags + 256;
constexpr size_t kNoAllocScratchBytes = kOffSort + kNoAllocSortBytes;  // about 7.3 MB

// The scratch array. Every GPU that loads this library holds it until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch, looked up with the device current. (In host code the
// symbol names a host-side stand-in, not device memory; only the address returned by
// cudaGetSymbolAddress may be handed to kernels.) The address belongs to the CUDA context the
// module was loaded into: after cudaDeviceReset, or when the primary context is released and
// created again, the module is loaded anew and the array may sit elsewhere. So the cached
// address is kept per device together with the unique ID of the context it was looked up in
// (cuCtxGetId), and looked up again whenever the current context's ID differs.
constexpr int kMaxDevices = 64;
struct ScratchAddr {
    unsigned long long ctx_id;
    void *ptr;
};
static ScratchAddr g_scratch_dev[kMaxDevices] = {};
static std::mutex g_scratch_mu;

using PfnCtxGetCurrent = CUresult (*)(CUcontext *);
using PfnCtxGetId = CUresult (*)(CUcontext, unsigned long long *);

// The current context's unique ID through driver entry points fetched from the runtime (the
// library does not link libcuda); 0 when no context is current yet.
static int current_context_id(unsigned long long *id)
{
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!get_current || !get_id) {
        void *f1 = nullptr, *f2 = nullptr;
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        LENTILS_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                          cudaEnableDefault, &q1));
        LENTILS_CUDA_TRY(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000,
                                                          cudaEnableDefault, &q2));
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return set_error(LENTILS_ERR_CUDA, "grid_noalloc: driver context queries unavailable");
        get_current = (PfnCtxGetCurrent)f1;
        get_id = (PfnCtxGetId)f2;
    }
    CUcontext ctx = nullptr;
    if (get_current(&ctx) != CUDA_SUCCESS)
        return set_error(LENTILS_ERR_CUDA, "grid_noalloc: cuCtxGetCurrent failed");
    *id = 0;
    if (ctx && get_id(ctx, id) != CUDA_SUCCESS)
        return set_error(LENTILS_ERR_CUDA, "grid_noalloc: cuCtxGetId failed");
    return LENTILS_OK;
}

static int scratch_for_current_device(unsigned char **out)
{
    int dev = 0;
    LENTILS_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(LENTILS_ERR_UNSUPPORTED, "grid_noalloc: device ordinal %d", dev);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    unsigned long long id = 0;
    if (int st = current_context_id(&id)) return st;
    ScratchAddr &a = g_scratch_dev[dev];
    if (id == 0 || !a.ptr || a.ctx_id != id) {
        // set-up for this device and context: also makes the device's primary context current
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        if (!ptr) return set_error(LENTILS_ERR_CUDA, "grid_noalloc: null scratch address");
        if (int st = current_context_id(&id)) return st;
        a.ctx_id = id;
        a.ptr = ptr;
    }
    *out = (unsigned char *)a.ptr;
    return LENTILS_OK;
}

// Work items from the per-tile counts, in one block: exclusive scans of the visibility counts
// and of the items per tile, then the items of each tile; the remaining slots up to max_items
// become empty items (count 0), which the gridding kernel skips.
__global__ void __launch_bounds__(1024)
    noalloc_items_kernel(const int *__restrict__ tile_counts, int ntiles, int ntv, int chunk,
                         WorkItem *__restrict__ items, int max_items)
{
    __shared__ int s_vis[1024];
    __shared__ int s_it[1024];
    __shared__ int carry[2];
    const int tid = threadIdx.x;
    if (tid == 0) carry[0] = carry[1] = 0;
    __syncthreads();
    for (int base = 0; base < ntiles; base += 1024) {
        const int t = base + tid;
        const int c = (t < ntiles) ? tile_counts[t] : 0;
        const int ni = (c + chunk - 1) / chunk;
        s_vis[tid] = c;
        s_it[tid] = ni;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan
            const int a = (tid >= off) ? s_vis[tid - off] : 0;
            const int b = (tid >= off) ? s_it[tid - off] : 0;
            __syncthreads();
            s_vis[tid] += a;
            s_it[tid] += b;
            __syncthreads();
        }
        const int vbeg = carry[0] + s_vis[tid] - c;
        const int ibeg = carry[1] + s_it[tid] - ni;
        for (int j = 0; j < ni; ++j) {
            WorkItem it;
            it.tu = t / ntv;
            it.tv = t - it.tu * ntv;
            it.begin = vbeg + j * chunk;
            it.count = min(chunk, c - j * chunk);
            if (ibeg + j < max_items) items[ibeg + j] = it;
        }
        __syncthreads();
        if (tid == 1023) {
            carry[0] += s_vis[1023];
            carry[1] += s_it[1023];
        }
        __syncthreads();
    }
    for (int i = carry[1] + tid; i < max_items; i += blockDim.x) {
        WorkItem it;
        it.tu = it.tv = it.begin = it.count = 0;
        items[i] = it;
    }
}

// binning and gridding kernels of plan.cu / gridding.cu
int launch_canon(const double *uvw, const double *chans, const CanonParams &p, unsigned *keys,
                 int *idx, uint2 *coords, float2 *phase, int *tile_counts, int *flags,
                 long long nvis, cudaStream_t s);
int launch_gather_plan(const int *perm, const uint2 *cin, const float2 *pin, uint2 *cout,
                       float2 *pout, long long n, cudaStream_t s);
int launch_to_plan_c64(const int *perm, const float2 *phase, const float2 *vu, float2 *vp,
                       long long n, cudaStream_t s);
int launch_grid(const lentils_plan *p, const float2 *vis, float2 *grid, cudaStream_t s);

}  // namespace lentils

using namespace lentils;

extern "C" {

int lentils_noalloc_max_vis(void) { return kNoAllocMaxVis; }
long long lentils_noalloc_scratch_bytes(void) { return (long long)kNoAllocScratchBytes; }

int lentils_grid_noalloc(const lentils_grid_desc *gd, const double *uvw, int nrows,
                         const double *channels, int nchannels, const float *vis, float *grid,
                         void *stream)
{
    clear_error();
    if (!gd) return set_error(LENTILS_ERR_INVALID, "grid_noalloc: null descriptor");
    if (nrows < 0 || nchannels < 1)
        return set_error(LENTILS_ERR_INVALID, "grid_noalloc: bad rows/channels");
    const long long nvis = (long long)nrows * nchannels;
    if (nvis > kNoAllocMaxVis)
        return set_error(LENTILS_ERR_INVALID,
                         "grid_noalloc: %lld visibilities exceed the fixed maximum of %d per call",
                         nvis, kNoAllocMaxVis);
    if (nvis > 0 && (!uvw || !channels || !vis || !grid))
        return set_error(LENTILS_ERR_INVALID, "grid_noalloc: null buffer");
    if (gd->nu < 2 || gd->nv < 2 || gd->nu > 65536 || gd->nv > 65536)
        return set_error(LENTILS_ERR_INVALID, "grid_noalloc: grid %dx%d out of range", gd->nu,
                         gd->nv);
    if (gd->wsup < 1 || gd->wsup > kMaxW)
        return set_error(LENTILS_ERR_UNSUPPORTED, "grid_noalloc: wsup=%d (supported 1..%d)",
                         gd->wsup, kMaxW);
    if (!(gd->du > 0) || !(gd->dv > 0) || !isfinite(gd->kb_beta))
        return set_error(LENTILS_ERR_INVALID, "grid_noalloc: bad du/dv/beta");

    unsigned char *scr = nullptr;
    if (int st = scratch_for_current_device(&scr)) return st;
    if (nvis == 0) return LENTILS_OK;

    // geometry (same tiling rule as lentils_plan_create)
    lentils_plan p;
    memset(&p, 0, sizeof(p));
    p.desc = *gd;
    int T = gd->tile;
    if (T == 0) T = 16;
    int logT = 0;
    while ((1 << logT) < T) ++logT;
    if ((1 << logT) != T || logT < 3 || logT > 6)
        return set_error(LENTILS_ERR_INVALID, "grid_noalloc: tile %d (use 8, 16, 32 or 64)", T);
    GridGeom &g = p.geom;
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
    const int ntiles = g.ntu * g.ntv;
    if (ntiles > kNoAllocMaxTiles)
        return set_error(LENTILS_ERR_INVALID,
                         "grid_noalloc: %d uv tiles exceed the fixed maximum of %d (use a larger "
                         "tile)", ntiles, kNoAllocMaxTiles);
    kb_poly_build(g.w, gd->kb_beta, &p.kb, nullptr);

    unsigned *keys_in = (unsigned *)(scr + kOffKeysIn);
    unsigned *keys_out = (unsigned *)(scr + kOffKeysOut);
    int *idx = (int *)(scr + kOffIdx);
    int *perm = (int *)(scr + kOffPerm);
    uint2 *coords_user = (uint2 *)(scr + kOffCoordsUser);
    uint2 *coords_plan = (uint2 *)(scr + kOffCoordsPlan);
    float2 *phase_user = (float2 *)(scr + kOffPhaseUser);
    float2 *phase_plan = (float2 *)(scr + kOffPhasePlan);
    float2 *vis_plan = (float2 *)(scr + kOffVisPlan);
    int *tile_counts = (int *)(scr + kOffTileCounts);
    WorkItem *items = (WorkItem *)(scr + kOffItems);
    int *flags = (int *)(scr + kOffFlags);
    void *sort_tmp = (void *)(scr + kOffSort);

    cudaStream_t s = (cudaStream_t)stream;
    // a non-finite coordinate gets the key 0xffffffff and is counted in no tile; the tile
    // field is sized for ntiles + 1 values so that key sorts after every real tile's cells
    int tile_bits = 1;
    while ((1 << tile_bits) < ntiles + 1) ++tile_bits;
    const int key_bits = std::min(32, 2 * logT + tile_bits);
    size_t sort_bytes = 0;
    LENTILS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, keys_in, keys_out, idx,
                                                     perm, (int64_t)nvis, 0, key_bits, s));
    if (sort_bytes > kNoAllocSortBytes)
        return set_error(LENTILS_ERR_UNSUPPORTED,
                         "grid_noalloc: radix sort needs %zu bytes, %zu reserved", sort_bytes,
                         kNoAllocSortBytes);

    // clear what must start at zero, then bin, sort, reorder, build items, grid
    LENTILS_CUDA_TRY(cudaMemsetAsync(tile_counts, 0, sizeof(int) * ntiles, s));
    LENTILS_CUDA_TRY(cudaMemsetAsync(flags, 0, sizeof(int), s));
    CanonParams cp;
    cp.nu = g.nu; cp.nv = g.nv; cp.T = g.T; cp.logT = g.logT; cp.Hu = g.Hu; cp.Hv = g.Hv;
    cp.ntu = g.ntu; cp.ntv = g.ntv; cp.w = g.w; cp.nrows = nrows; cp.nch = nchannels;
    cp.guard = 0;
    cp.du = gd->du; cp.dv = gd->dv; cp.gcx = gd->gcx; cp.gcy = gd->gcy;
    if (int st = launch_canon(uvw, channels, cp, keys_in, idx, coords_user, phase_user,
                              tile_counts, flags, nvis, s))
        return st;
    LENTILS_CUDA_TRY(cub::DeviceRadixSort::SortPairs(sort_tmp, sort_bytes, keys_in, keys_out,
                                                     idx, perm, (int64_t)nvis, 0, key_bits, s));
    if (int st = launch_gather_plan(perm, coords_user, phase_user, coords_plan, phase_plan, nvis,
                                    s))
        return st;
    if (int st = launch_to_plan_c64(perm, phase_plan, (const float2 *)vis, vis_plan, nvis, s))
        return st;
    const int max_items = (int)std::min<long long>(
        kNoAllocMaxItems, std::min<long long>(ntiles, nvis) + (nvis + kNoAllocChunk - 1) / kNoAllocChunk);
    noalloc_items_kernel<<<1, 1024, 0, s>>>(tile_counts, ntiles, g.ntv, kNoAllocChunk, items,
                                            max_items);
    LENTILS_CHECK_LAUNCH("noalloc_items_kernel");
    p.grid_variant = 1;
    p.coords = coords_plan;
    p.items = items;
    p.nitems = max_items;
    p.nvis = nvis;
    return launch_grid(&p, vis_plan, (float2 *)grid, s);
}

}  // extern "C"
