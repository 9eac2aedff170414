/*
 * lentils_gb300 -- C ABI of the GB300 (sm_103a) lensed visibility-operator library.
 *
 * Two families of entry points:
 *
 *  1. Drop-in replacements with the exact signatures and by-value struct ABI of the
 *     reference's C backend, so the reference's ctypes layer can bind this library in place
 *     of libnufft / libdeflect:
 *        grid_cpu                 <- lentils/backend/nufft.c:42-43   (bound at load_backend.py:95-97)
 *        deflect_points           <- lentils/backend/deflect.c:60    (bound at load_backend.py:59-61)
 *        grad_matrix_findiff_csr  <- lentils/backend/nufft.c:163     (bound at load_backend.py:107-109)
 *     They take HOST pointers, keep the reference's accumulate (+=) semantics and FP64 in/out,
 *     compute in FP32 on the GPU, and return void like the reference. Their status is
 *     available afterwards from lentils_last_error().
 *
 *  2. Device-resident entry points (prefix lentils_): device pointers, an explicit CUDA
 *     stream (cudaStream_t passed as void*; NULL = legacy default stream), an int status
 *     (LENTILS_OK on success), and no hidden host synchronisation unless stated.
 *
 * All arrays of complex numbers are interleaved (re, im). "c64" = two float32 per element,
 * "c128" = two float64 per element. Grids are the r2c half-plane, row-major, shape
 * (nu, nv/2+1), flat index (nv/2+1)*i_u + i_v (reference nufft.c:96).
 */
#ifndef LENTILS_GB300_H
#define LENTILS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------------------------
 * By-value structs. Field order, types and padding are the reference's C ABI, so a ctypes
 * Structure built for the reference passes unchanged.
 * ---------------------------------------------------------------------------------------- */

/* lentils/backend/common.h:13-23 */
typedef struct {
    int nx, ny;
    int nchannels;
    int nstokes;
    double xmin, xmax, ymin, ymax;
    double dx, dy;
    double *channels;
    char *mask;
} lentils_image_space;

/* lentils/backend/common.h:39-49 */
typedef struct {
    int nu, nv;
    int half_nv;
    int nchannels;
    int nstokes;
    double du, dv;
    double gcx, gcy;
    double *channels;
} lentils_fourier_space;

/* lentils/backend/common.h:52-61 */
typedef struct {
    int nrows;
    int nchannels;
    int nstokes;
    double *uv;       /* (nrows, 3) u, v, w in wavelengths */
    double *channels; /* (nchannels) scale factors applied to u and v */
} lentils_visibility_space;

/* lentils/backend/deflect.h:8-17 (320 bytes). Mass-model parameters live in fpars; the
 * per-type packing is documented at lentils_deflect below. */
typedef struct {
    unsigned int type;
    unsigned int _pad;
    double z_l, z_s, d_l, d_s, d_ls, sigma_c, beta;
    double fpars[24];
    int ipars[8];
    unsigned char flags[32];
} lentils_mass_model;

/* lentils/backend/deflect.h:20-26 */
typedef struct {
    int num_lenses;
    int num_zplanes;
    lentils_mass_model *lenses;
} lentils_global_lens_model;

/* ------------------------------------------------------------------------------------------
 * Status codes
 * ---------------------------------------------------------------------------------------- */
enum {
    LENTILS_OK = 0,
    LENTILS_ERR_INVALID = 1,      /* null pointer, negative size, unknown direction/type   */
    LENTILS_ERR_NYQUIST = 2,      /* a visibility lies beyond the grid's Nyquist guard     */
    LENTILS_ERR_ALLOC = 3,        /* device or pinned-host allocation failed               */
    LENTILS_ERR_CUDA = 4,         /* a CUDA runtime / cuFFT call failed                    */
    LENTILS_ERR_UNSUPPORTED = 5,  /* valid request the library does not implement         */
    LENTILS_ERR_TIMEOUT = 6,      /* a bounded device-side wait gave up                    */
    LENTILS_ERR_NONFINITE = 7,    /* NaN/Inf detected where the caller asked for a check   */
    LENTILS_ERR_NO_DEVICE = 8     /* no CUDA device visible                                */
};

/* Status of the most recent call made on this host thread (drop-in functions return void). */
int lentils_last_error(void);
/* Human-readable text of the most recent failure on this host thread ("" if none). */
const char *lentils_last_error_message(void);
/* Library version as major*10000 + minor*100 + patch. */
int lentils_version(void);
/* Copy bytes from a device array to host memory after all device work has finished. */
int lentils_copy_to_host(void *dst, const void *src, long long bytes);
/* Release a device array that an entry point allocated for the caller (cudaFree). */
int lentils_device_free(void *ptr);

/* Host-only (no GPU needed): the per-tap Kaiser-Bessel polynomial table the gridding kernels
 * evaluate, 2w taps x lentils_kb_poly_ncoef() coefficients in t = 2*frac - 1 (highest degree
 * first, checkerboard sign and 1/(2w) folded in), and the FP64 fit error relative to the
 * kernel peak. Tap i of a visibility with fractional cell offset frac sits at kernel argument
 * frac + w - 1 - i; the weight is I0(beta*sqrt(1-(a/w)^2))/(2w) as in kb_g,
 * lentils/backend/nufft.c:11-21. */
int lentils_kb_poly_table(int w, double beta, float *coef, int ncoef_capacity, double *fit_err);
int lentils_kb_poly_ncoef(void);

/* ------------------------------------------------------------------------------------------
 * Drop-in entry points (host pointers, reference semantics)
 * ---------------------------------------------------------------------------------------- */

/* Kaiser-Bessel gridding (direction 1, ADJOINT: visibilities -> half-plane grid) and
 * degridding (direction 0, FORWARD: grid -> visibilities). Replaces grid_cpu,
 * lentils/backend/nufft.c:42-122. vis is (nchannels, 1, nrows) c128, grid is (nu, nv/2+1)
 * c128; the output is ACCUMULATED (+=) like the reference. wsup is the kernel half-width w
 * (the reference loops over 2w+1 taps per axis). */
void grid_cpu(lentils_visibility_space visspace, double *vis, lentils_fourier_space gspace,
              double *grid, int wsup, double kb_beta, int direction);

/* The uv binning of grid_cpu is cached: the reference calls grid_cpu on every operator
 * application with the same visibility space (fourier_operators.py:85-93), so the plan
 * (lentils_plan_create) is kept for up to 4 uv sets, keyed by device, uv address, nrows,
 * channels, grid geometry, wsup, beta and a digest of the uv contents. Mode 1 (default)
 * digests 4096 evenly spaced rows plus the last; mode 2 digests every row (about 30 ms per
 * 1e7 rows); mode 0 bins on every call. A caller that rewrites a uv buffer in place between
 * calls must use mode 2 or call lentils_dropin_cache_clear. No counterpart in the reference
 * (its grid_cpu has no set-up to keep). grid_cpu calls are serialised by one lock. */
int lentils_dropin_cache_mode(int mode);
int lentils_dropin_cache_clear(void);
int lentils_dropin_cache_size(void);

/* Lens equation beta = theta - sum_l alpha_l(theta) for npoints interleaved (x, y) points.
 * Replaces deflect_points, lentils/backend/deflect.c:60-66. With want_deriv != 0 it also does
 * what the reference does with its single deriv pointer: deriv[0..11] += the PEMD parameter
 * derivatives d alpha / d (b, qh, q, x, y, th), (x, y) components, summed over all points and
 * PEMD lenses (deflect.c:330-338; the per-point layout is lentils_deflect_grad). */
void deflect_points(lentils_global_lens_model glm, double *p_in, int npoints, double *p_out,
                    int want_deriv, double *deriv);

/* Forward-difference gradient operator as CSR with 2*nx*ny rows and 2 entries per interior
 * row. Replaces grad_matrix_findiff_csr, lentils/backend/nufft.c:163-194. Arrays are host
 * buffers sized as the reference's PriorCovarianceOperator allocates them
 * (lentils/operators/operator_base.py:226-228). */
void grad_matrix_findiff_csr(lentils_image_space imspace, int *row_inds, int *cols,
                             double *vals);

/* ------------------------------------------------------------------------------------------
 * Gridding plan: visibilities binned by grid tile once per uv set.
 *
 * A plan re-orders the visibilities (plan order = sorted by tile and cell) and stores each as
 * two 32-bit fixed-point tile-relative coordinates. The degrid/grid kernels read and write
 * visibilities in plan order and in the plan frame (phase-centre factor and the sign of a
 * wrap by an odd grid size removed). lentils_vis_to_plan / lentils_vis_from_plan convert to and from the reference's
 * row order and frame. In the normal-equation product F^T C^-1 F the frame factors cancel, so
 * an iterative solver stays in plan order throughout.
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_plan lentils_plan;

typedef struct {
    int nu, nv;          /* full uv grid; the stored half-plane is nu x (nv/2+1)            */
    double du, dv;       /* cell size (wavelengths)                                          */
    double gcx, gcy;     /* phase centre (radians)                                           */
    int wsup;            /* kernel half-width w, 1 <= w <= 8                                 */
    double kb_beta;      /* Kaiser-Bessel shape parameter                                    */
    int tile;            /* tile edge in cells (16, 32 or 64), 0 = choose automatically      */
    int chunk;           /* max visibilities per work item, 0 = choose automatically         */
} lentils_grid_desc;

enum {
    LENTILS_PLAN_UVW_ON_DEVICE = 1, /* uvw/channels pointers are device memory            */
    LENTILS_PLAN_NYQUIST_GUARD = 2  /* reject uv beyond the guard of
                                       lentils/operators/fourier_operators.py:77-80           */
};

typedef struct {
    long long nvis;          /* nrows * nchannels                                           */
    int ntiles_u, ntiles_v;  /* tile grid over the canonical half plane                     */
    int tile;                /* tile edge (cells)                                           */
    int nitems;              /* work items (tile, visibility range)                         */
    int max_item_vis;        /* largest work item                                           */
    int heaviest_tile_vis;   /* visibilities in the most populated tile                     */
    int wsup;
    int has_phase;           /* 1 if the phase centre is off the origin                     */
    long long device_bytes;  /* device memory held by the plan                              */
} lentils_plan_stats;

/* Build a plan from uvw (nrows x 3, f64) and channel scale factors (nchannels, f64).
 * Pointers are host memory unless LENTILS_PLAN_UVW_ON_DEVICE is set. Synchronises stream
 * once at the end (the work-item count must reach the host). */
int lentils_plan_create(lentils_plan **plan, const lentils_grid_desc *grid, const double *uvw,
                        int nrows, const double *channels, int nchannels, int flags,
                        void *stream);
int lentils_plan_destroy(lentils_plan *plan);
int lentils_plan_get_stats(const lentils_plan *plan, lentils_plan_stats *stats);
/* Tuning: the gridding kernel's work split. Every form gives the same result up to FP32
 * summation order.
 *  0 (default): lanes own window rows: 32/(2w) visibilities side by side per warp, each lane
 *     summing its 2w + 1 taps in registers while its group's sorted visibilities stay in one
 *     pair of cells (lu, 2m), (lu, 2m + 1); weights produced by the group's own lanes, warp-
 *     local batches, warp-private tiles, flushes taking turns only among the groups that
 *     flush, 4 warps per CTA;
 *  1: lanes own taps, one visibility per warp; 2: two visibilities per warp;
 *  3: as 8 with one tile per CTA flushed by shared-memory atomics, cell changes checked at
 *     every step; 4: as 8 with cell changes checked at every step and flush turns for every
 *     group; 5: as 8 with flushes by shared-memory atomics; 6: as 5 into one tile per CTA;
 *  7: as 8 with compensated (Kahan) register sums; 8: row owners with a CTA-wide weight batch
 *     and per-group flush masks; 9: as 0 with one-cell windows, CTA barriers per batch and
 *     8 warps per CTA; 10: as 0 with one-cell windows; 11: as 0 with 8 warps per CTA.
 * Tiles too large for the warp-private copies fall back to 8, then to 1. */
int lentils_plan_set_grid_variant(lentils_plan *plan, int variant);
/* Tuning: the degridding kernel's form. 0 (default): a thread takes up to 4 sorted visibilities
 * of one cell and reads each window row from shared memory once for all of them (2w <= 8;
 * wider kernels use 2); 1 (even 2w): one visibility per thread, the staged tile holding
 * overlapping column pairs (16-byte loads, two taps each); 2: one visibility per thread.
 * Identical results. */
int lentils_plan_set_degrid_variant(lentils_plan *plan, int variant);

/* Degrid: half-plane grid (c64, device) -> visibilities (c64, device, plan order, plan frame).
 * vis_plan is OVERWRITTEN. */
int lentils_degrid(const lentils_plan *plan, const float *grid, float *vis_plan, void *stream);

/* Grid: visibilities (c64, device, plan order, plan frame) -> half-plane grid (c64, device).
 * The grid is ACCUMULATED (+=); zero it first for a fresh result. */
int lentils_grid(const lentils_plan *plan, const float *vis_plan, float *grid, void *stream);

/* Reference row order/frame (c128 or c64 by `user_is_c128`) -> plan order/frame (c64). */
int lentils_vis_to_plan(const lentils_plan *plan, const void *vis_user, int user_is_c128,
                        float *vis_plan, void *stream);
/* Plan order/frame (c64) -> reference row order/frame. accumulate != 0 adds into vis_user. */
int lentils_vis_from_plan(const lentils_plan *plan, const float *vis_plan, void *vis_user,
                          int user_is_c128, int accumulate, void *stream);

/* Host-buffer forms: the same operators on HOST c128 buffers in reference row order, with the
 * host<->device copies and precision conversions done inside (staging buffers are owned by
 * the plan and allocated on first use). accumulate != 0 adds into the output like grid_cpu
 * (the output is then also copied host->device); accumulate == 0 overwrites it, which is what
 * the reference's GriddingOperator gets from its fresh zero buffers
 * (lentils/operators/fourier_operators.py:85-93). Pinned host buffers give full-rate copies.
 * Synchronise stream before returning. */
int lentils_degrid_host(lentils_plan *plan, const double *grid_host, double *vis_host,
                        int accumulate, void *stream);
int lentils_grid_host(lentils_plan *plan, const double *vis_host, double *grid_host,
                      int accumulate, void *stream);

/* FP64 forms of the plan operators (the double-precision operator used for refinement
 * residuals): c128 plan-order visibilities and c128 half-plane grids. The phase-centre factor
 * of the plan frame is stored in FP32 (exact for a centred image, 1e-7 otherwise). */
int lentils_degrid64(const lentils_plan *plan, const double *grid, double *vis_plan, void *stream);
int lentils_grid64(const lentils_plan *plan, const double *vis_plan, double *grid, void *stream);
int lentils_vis_to_plan64(const lentils_plan *plan, const double *vis_user, double *vis_plan,
                          void *stream);
int lentils_vis_from_plan64(const lentils_plan *plan, const double *vis_plan, double *vis_user,
                            int accumulate, void *stream);
/* Real per-visibility values (e.g. inverse variances) from row order to plan order. */
int lentils_plan_gather_real(const lentils_plan *plan, const double *user, double *plan_out,
                             void *stream);

/* ------------------------------------------------------------------------------------------
 * NUFFT operator F = Degrid . rFFT2 . ZeroPad . Apod (NUFFTOperator,
 * lentils/operators/fourier_operators.py:96-126) and its transpose, on device buffers.
 * The image is (nx, ny) row-major real; it is zero-padded by (padx, pady) on each side to the
 * plan's (nu, nv) grid; apod_x (nx) and apod_y (ny) are the two separable factors of the
 * apodisation correction (fourier_operators.py:54-68). precisions: bit 0 = build the FP32
 * operator, bit 1 = the FP64 operator. Visibilities are plan-order, plan-frame; the adjoint
 * OVERWRITES the image.
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_nufft lentils_nufft;
int lentils_nufft_create(lentils_nufft **op, const lentils_plan *plan, int nx, int ny, int padx,
                         int pady, const double *apod_x, const double *apod_y, int precisions,
                         void *stream);
int lentils_nufft_destroy(lentils_nufft *op);
int lentils_nufft_forward(lentils_nufft *op, const float *image, float *vis_plan, void *stream);
int lentils_nufft_adjoint(lentils_nufft *op, const float *vis_plan, float *image, void *stream);
int lentils_nufft_forward64(lentils_nufft *op, const double *image, double *vis_plan,
                            void *stream);
int lentils_nufft_adjoint64(lentils_nufft *op, const double *vis_plan, double *image,
                            void *stream);

/* ------------------------------------------------------------------------------------------
 * Bilinear lens operator L: image pixels <- regular source grid (nsx x nsy nodes at
 * (sxmin + j*sdx, symin + k*sdy)). src_points: deflected image-pixel positions (nimg x 2, f64,
 * device), mask: nimg bytes (device, NULL = all pixels). No reference counterpart (the
 * reference interpolates on Delaunay meshes, lentils/backend/triangles.c:105-140); a pixel
 * outside the node lattice or masked has an empty row. apply: img = L src; apply_t:
 * src = L^T img (both overwrite).
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_lensop lentils_lensop;
/* A general lens matrix in CSR form (device arrays, copied): nimg rows (image pixels), nsrc
 * columns, int32 row pointers and columns, FP64 values; L^T by a stable sort on the column. */
int lentils_lensop_create_csr(lentils_lensop **op, const int *row_ptr, const int *cols,
                              const double *vals, int nimg, int nsrc, int nnz, void *stream);
/* The reference's ManifoldLensOperator matrix (manifold_lens_matrix_csr,
 * lentils/backend/raster.c:272-395) built on the GPU in FP64, one image pixel per thread: 9
 * deflected points per unmasked pixel, 8 triangles fanned around the centre, recursively split
 * along source-pixel lines, areas from the barycentric corners, and the reference's per-pixel
 * reduction of the sorted fragments (including its two quirks: the first fragment of every
 * column after the first is not added, and a pixel without fragments gets one zero entry in
 * the previous such column). im, src: image and source spaces (host structs; src.mask unused);
 * lenses: HOST array; mask_dev: nx*ny bytes on the device. Outputs are device arrays allocated
 * here (free with cudaFree): *row_inds (nx*ny + 1), *cols, *vals (*nnz). A stack or fragment
 * overflow (which the reference only prints) returns LENTILS_ERR_UNSUPPORTED. */
int lentils_manifold_lens_matrix(const lentils_image_space *im, const lentils_image_space *src,
                                 const lentils_mass_model *lenses, int nlenses,
                                 const unsigned char *mask_dev, int **row_inds, int **cols,
                                 double **vals, long long *nnz, void *stream);
/* FP64 deflection with the reference's formulas (deflect.c; PEMD, shear, multipoles), device
 * points and output (interleaved x, y); synchronises the stream. */
int lentils_deflect64(const lentils_mass_model *lenses, int nlenses, const double *points,
                      double *out, long long npoints, void *stream);
/* The reference's DelaunayLensOperator matrix (delaunay_lens_matrix_csr,
 * lentils/backend/triangles.c:105-140): unmasked image pixels on the ncast lattice are casted
 * points (one entry 1.0 in their own column, numbered in row-major order); every other
 * unmasked pixel takes the barycentric weights (triangle_geometry, triangles.c:7-30) of its
 * deflected position in its triangle tri_inds[u] (no entries when < 0), u numbering the
 * uncasted pixels in row-major order. The triangulation (triangles, 3 ints each, over
 * tri_points) and the point location come from the caller, as the reference takes them from
 * scipy's Delaunay (lens_operators.py:67-70). Device inputs; outputs as for
 * lentils_manifold_lens_matrix. */
int lentils_delaunay_lens_matrix(const unsigned char *mask_dev, int nx, int ny, int ncast,
                                 const double *uncasted_points, const int *uncasted_tri_inds,
                                 const int *triangles, const double *tri_points, int **row_inds,
                                 int **cols, double **vals, long long *nnz, void *stream);
int lentils_lensop_create(lentils_lensop **op, const double *src_points,
                          const unsigned char *mask, int nimg, int nsx, int nsy, double sxmin,
                          double symin, double sdx, double sdy, void *stream);
int lentils_lensop_destroy(lentils_lensop *op);
int lentils_lensop_nnz(const lentils_lensop *op);
int lentils_lensop_apply(const lentils_lensop *op, const float *src, float *img, void *stream);
int lentils_lensop_apply_t(const lentils_lensop *op, const float *img, float *src, void *stream);
int lentils_lensop_apply64(const lentils_lensop *op, const double *src, double *img,
                           void *stream);
int lentils_lensop_apply_t64(const lentils_lensop *op, const double *img, double *src,
                             void *stream);
int lentils_lensop_diag_ltl(const lentils_lensop *op, double *diag, void *stream);

/* ------------------------------------------------------------------------------------------
 * Normal-equation operator A = L^T F^T C^-1 F L + lambda R^T R of the CG source inversion
 * (the pattern of lentils/tests/solver_tests.py:97-114 with the 'gradient' prior of
 * lentils/operators/operator_base.py:225-242) and its mixed-precision CG solver.
 * weights_plan: C^-1 per visibility in plan order (f64, device); src_dx/src_dy: source pixel
 * size (the R of grad_matrix_findiff_csr uses +-1/dx, +-1/dy). apply overwrites out.
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_normal_op lentils_normal_op;
int lentils_normal_op_create(lentils_normal_op **op, lentils_lensop *L, lentils_nufft *F,
                             const double *weights_plan, long long nvis, int nimg, int nsx,
                             int nsy, double src_dx, double src_dy, double lambda, void *stream);
int lentils_normal_op_destroy(lentils_normal_op *op);
int lentils_normal_op_apply(lentils_normal_op *op, const float *s, float *out, void *stream);
int lentils_normal_op_apply64(lentils_normal_op *op, const double *s, double *out, void *stream);
/* b = L^T F^T C^-1 d in FP64 (d: plan-order, plan-frame c128 visibilities). */
int lentils_normal_op_rhs64(lentils_normal_op *op, const double *d_plan, double *b, void *stream);
/* Inverse Jacobi diagonal 1 / (sum(C^-1) * diag(L^T L) + lambda * diag(R^T R)). */
int lentils_normal_op_jacobi(lentils_normal_op *op, double *inv_diag, float *inv_diag32,
                             void *stream);
double lentils_normal_op_weight_sum(const lentils_normal_op *op);

typedef struct {
    double tol;        /* target true relative residual ||b - A x|| / ||b|| (FP64 operator) */
    double inner_tol;  /* relative residual reduction of each inner FP32 solve              */
    int max_outer;
    int max_inner;
    int check_every;   /* inner iterations between host reads of the residual norm         */
    int use_graph;     /* capture one inner iteration in a CUDA graph and replay it        */
    int window;        /* lentils_fcg_solve: directions kept for A-orthogonalisation (1-8;
                          0 means 1); ignored by lentils_cg_solve                          */
    int net_every;     /* lentils_fcg_solve with a network: it proposes every net_every-th
                          direction (0 or 1: every one), the others are Jacobi directions  */
} lentils_cg_options;

typedef struct {
    int converged;
    int outer;
    int inner_total;
    double rel_residual; /* final true FP64 relative residual */
    double seconds;      /* wall time of the solve            */
    int net_iterations;  /* flexible CG: iterations that took the network's direction */
    int fallback;        /* flexible CG: 1 if it switched to plain Jacobi-CG on stagnation */
} lentils_cg_result;

/* ------------------------------------------------------------------------------------------
 * Direct Fourier sum (DFTOperator, lentils/operators/fourier_operators.py:130-145, matrix of
 * dft_matrix_csr, lentils/backend/nufft.c:128-161), FP64 on the GPU, as a validator of the
 * NUFFT: V_k = sum_p x_p e^{i a_kp} over unmasked pixels, a_kp = -2 pi ARCSEC_TO_RADIANS
 * (u x + v y) with u = uv[0] ch[0], v = -uv[1] ch[0] and x = xmin + i dx, y = ymin + j dy;
 * the adjoint is its real transpose. Device arrays: uvw (nrows x 3), channels (first used),
 * mask (nx*ny bytes), image (nx*ny f64), vis (nrows c128); im is a host struct.
 * ---------------------------------------------------------------------------------------- */
int lentils_dft_forward(const double *uvw, int nrows, const double *channels,
                        const lentils_image_space *im, const unsigned char *mask,
                        const double *image, double *vis, void *stream);
int lentils_dft_adjoint(const double *uvw, int nrows, const double *channels,
                        const lentils_image_space *im, const unsigned char *mask,
                        const double *vis, double *image, void *stream);

/* ------------------------------------------------------------------------------------------
 * Dirty-beam (blurred covariance) form of F^T C^-1 F, the reference's production CG data term
 * (RadioDataset.blurred_covariance_operator, lentils/common/data_base.py:115-129):
 *   B x = crop(pad(x) (*) roll(beam))   (circular convolution on the 2nx x 2ny padded grid)
 * beam: the dirty beam NUFFT_beam^T C^-1 1 on the beam space (2nx x 2ny pixels, bounds
 * +-(nx dx, ny dy), data_base.py:147-172), device FP64, x-major; nx, ny even. Applied with
 * cuFFT in FP32 (lentils_bcb_apply) or FP64 (lentils_bcb_apply64) on (nx, ny) images.
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_bcb lentils_bcb;
int lentils_bcb_create(lentils_bcb **op, const double *beam, int nx, int ny, void *stream);
int lentils_bcb_destroy(lentils_bcb *op);
int lentils_bcb_apply(lentils_bcb *op, const float *x, float *out, void *stream);
int lentils_bcb_apply64(lentils_bcb *op, const double *x, double *out, void *stream);
double lentils_bcb_centre(const lentils_bcb *op);
/* The normal operator with the dirty-beam data term: A = L^T B L + lambda R^T R (nimg = nx*ny
 * of B); its right-hand side from the dirty image F^T C^-1 d by lentils_normal_op_rhs_image64.
 * Works with lentils_cg_solve / lentils_fcg_solve as the visibility form does. */
int lentils_normal_op_create_bcb(lentils_normal_op **out, lentils_lensop *L, lentils_bcb *B,
                                 int nimg, int nsx, int nsy, double src_dx, double src_dy,
                                 double lambda, void *stream);
/* b = L^T d_img (FP64, device) */
int lentils_normal_op_rhs_image64(lentils_normal_op *op, const double *d_img, double *b,
                                  void *stream);

/* Iterative refinement: outer FP64 residuals r = b - A x, inner Jacobi-preconditioned CG with
 * the FP32 operator (inv_diag32 may be NULL for no preconditioner). x (f64, device) holds the
 * initial guess and receives the solution; an all-zero guess starts from r = b without an FP64
 * matvec. */
int lentils_cg_solve(lentils_normal_op *op, const double *b, double *x, const float *inv_diag32,
                     const lentils_cg_options *opt, lentils_cg_result *res, void *stream);
/* lambda R^T R s of the 'gradient' prior (R = forward differences of
 * grad_matrix_findiff_csr, lentils/backend/nufft.c:163-194) on an (nx, ny) x-major grid,
 * matrix-free; overwrites out. */
int lentils_prior_gradient_apply(const float *s, float *out, int nx, int ny, double dx, double dy,
                                 double lambda, void *stream);
int lentils_prior_gradient_apply64(const double *s, double *out, int nx, int ny, double dx,
                                   double dy, double lambda, void *stream);
/* FP64 dot product of two device vectors (synchronises the stream). */
int lentils_dot64(const double *a, const double *b, int n, double *out, void *stream);

/* ------------------------------------------------------------------------------------------
 * BF16 tensor-core GEMM (tcgen05, FP32 accumulation in tensor memory): C = A * B^T with A
 * (M x K) and B (N x K) row-major BF16 and C (M x N) row-major FP32, all device pointers; N in
 * {32, 64, 128, 256}, K a multiple of 8. The core of the learned preconditioner's kernels,
 * exposed for testing. form 0: the threads stage each K chunk and then the tensor core runs it
 * (double-buffered); form 1: the pipelined kernel (operands copied by cp.async into a ring of
 * chunks, the MMAs issued by a thread of a fifth warp); form 2: operands loaded by TMA
 * (tensor maps, 128-byte swizzled shared-memory tiles; A and B 16-byte aligned). *err_dev
 * (device int) is set to 1 if a bounded wait on the tensor core gave up (the result is then
 * invalid).
 * ---------------------------------------------------------------------------------------- */
int lentils_tc_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K,
                         int form, int *err_dev, void *stream);
/* Failure-path self-test of the bounded tensor-core waits: a kernel holding tensor memory
 * waits on an mbarrier that nothing completes, gives up after poll_limit polls (1..2^20), sets
 * *err_dev = 1, frees its tensor memory and returns; the context stays usable. */
int lentils_tc_timeout_selftest(int *err_dev, int poll_limit, void *stream);

/* ------------------------------------------------------------------------------------------
 * Batched lens-parameter sweep (no counterpart in the reference, whose operators run one lens
 * model at a time): per sample, deflection of its pixel grid, degridding of its grid and
 * gridding of its visibilities, for all samples in ONE persistent kernel launch (captured in a
 * CUDA graph by lentils_sweep_run with use_graph = 1).
 *
 * Each sample names its plan (KB width 6 or 8; tile and chunk are the plan's), DEVICE buffers
 * in the plan's order and frame as for lentils_degrid / lentils_grid -- grid_in (half plane
 * c64) -> vis_out (c64), vis_in (c64) -> grid_out (half plane c64, OVERWRITTEN) -- its lens
 * models (HOST array, at most 8, packed as for deflect_points) and its pixel grid: points
 * (x0 + i dx, y0 + j dy), i < nx, j < ny, x-major, deflected to beta = theta - sum alpha into
 * beta_out (device, nx * ny interleaved float (x, y)). plan = NULL or nx * ny = 0 skips that
 * part. Plans and buffers must outlive the sweep.
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_sweep lentils_sweep;
typedef struct {
    lentils_plan *plan;
    const float *grid_in;
    float *vis_out;
    const float *vis_in;
    float *grid_out;
    const lentils_mass_model *lenses;
    int nlenses;
    int nx, ny;
    double x0, y0, dx, dy;
    float *beta_out;
} lentils_sweep_sample;
typedef struct {
    int nsamples;
    int nwork;        /* work items in the queue                       */
    int blocks;       /* persistent CTAs (resident slots on all SMs)    */
    long long smem_bytes;
    long long total_vis;
    long long total_pixels;
    double algorithmic_bytes; /* per run: 2 x (16 B per visibility + grid) + 8 B per pixel */
} lentils_sweep_stats;
/* flags & LENTILS_SWEEP_FORM_MASK: the form of the sweep kernel's items. 0: the ballot gridder
 * and one visibility per degridding thread, three CTAs per SM; 1: the column-pair gridder and
 * same-cell chunk degridding, two CTAs per SM; 2: the column-pair gridder and one visibility
 * per degridding thread, two CTAs per SM. Tuning only: equal results up to FP32 summation
 * order in the grids, identical visibilities. */
#define LENTILS_SWEEP_FORM_MASK 3
int lentils_sweep_create(lentils_sweep **sweep, const lentils_sweep_sample *samples, int n,
                         int flags, void *stream);
int lentils_sweep_destroy(lentils_sweep *sweep);
int lentils_sweep_run(lentils_sweep *sweep, int use_graph, void *stream);
int lentils_sweep_get_stats(const lentils_sweep *sweep, lentils_sweep_stats *stats);

/* ------------------------------------------------------------------------------------------
 * Learned preconditioner (no counterpart in the reference): a 4-level convolutional U-Net on the
 * source grid, BF16 activations and weights on the tensor cores (tcgen05) with FP32
 * accumulation, trained on the GPU by its own forward and backward kernels.
 *
 * Parameters are one flat FP32 vector of lentils_unet_param_count() values: for each of the 8
 * convolutions in order (3x3 2->32, 3x3 32->64, 3x3 64->128, 3x3 128->128, 1x1 128->64,
 * 3x3 64->32, 3x3 32->32, 1x1 32->1) the weights [cout][kh*3+kw or 0][cin] then the biases
 * [cout]. Input channels: (scaled residual, diagonal feature), each an (B, H, W) FP32 device
 * array, H and W multiples of 8; output (B, H, W) FP32.
 *
 * Preconditioner form (lentils_unet_precondition, lentils_fcg_solve):
 *   u = dinv * r,  s = rms(u),  f = log(dinv) - mean(log(dinv))
 *   z = gamma * u + s * net(u / s, f)
 * The network is trained to give the direction of the error e = A^-1 r (target e / rms(e));
 * flexible CG is invariant to the scale of z. gamma (lentils_unet_set_jacobi_weight, default
 * 0) adds a share of the Jacobi direction.
 * ---------------------------------------------------------------------------------------- */
typedef struct lentils_unet lentils_unet;
long long lentils_unet_param_count(void);
/* init_params: the flat parameter vector in HOST memory */
int lentils_unet_create(lentils_unet **out, int H, int W, int max_batch, const float *init_params,
                        void *stream);
int lentils_unet_destroy(lentils_unet *net);
/* FP32 master parameters to host memory (waits for all device work first). */
int lentils_unet_get_params(lentils_unet *net, float *host_out);
int lentils_unet_set_params(lentils_unet *net, const float *host_in, void *stream);
int lentils_unet_forward(lentils_unet *net, const float *r, const float *d, float *out, int B,
                         void *stream);
/* forward + backward of the mean squared error against tgt; flat gradient and loss to HOST
 * memory (either may be NULL); synchronises the stream */
int lentils_unet_gradients(lentils_unet *net, const float *r, const float *d, const float *tgt,
                           int B, float *grad_host, float *loss_host, void *stream);
/* one Adam step (beta1 0.9, beta2 0.999, eps 1e-8) on the mean squared error; loss_dev
 * (device float, may be NULL) receives the batch loss before the step; no synchronisation */
int lentils_unet_train_step(lentils_unet *net, const float *r, const float *d, const float *tgt,
                            int B, float lr, float *loss_dev, void *stream);
/* backward pass from the activations of the most recent lentils_unet_forward (same B) for an
 * external gradient dout (B, H, W) FP32 (device) of the output; then an Adam step if lr > 0,
 * and a copy of the flat parameter gradient to HOST grad_host if non-NULL (synchronising) */
int lentils_unet_backward(lentils_unet *net, const float *dout, int B, float lr,
                          float *grad_host, void *stream);
/* Tuning, the convolution kernels: 0 (default) runs the forward convolutions with TMA operands
 * on the persistent GEMM (one wave of CTAs, accumulators double buffered in tensor memory), the
 * first layer with its input packing and pooling as one CUDA-core kernel, and the last hidden
 * layer with the 1 x 1 output layer (and, for lentils_unet_precondition, the combination) in
 * one GEMM epilogue; 2 runs every layer as its own per-tile TMA or cp.async-ring GEMM; 1 runs
 * the GEMMs whose operands are plain gathers on the staged kernel. The forms agree up to FP32
 * summation order and the BF16 roundings it can flip. */
int lentils_unet_set_gemm_form(lentils_unet *net, int form);
/* Tuning: about how many CTAs a weight-gradient GEMM runs (its pixel reduction is split over
 * them); 0 selects the built-in default. */
int lentils_unet_set_wgrad_ctas(lentils_unet *net, int ctas);
/* gamma of the preconditioner form (default 0) */
int lentils_unet_set_jacobi_weight(lentils_unet *net, float gamma);
/* 1 if a bounded tensor-core wait gave up since creation (results then invalid) */
int lentils_unet_error_flag(lentils_unet *net, int *flag);
/* f = log(dinv) - mean(log(dinv)) over n values (device) */
int lentils_unet_features(const float *dinv, float *feat, int n, void *stream);
/* z = M(r) for one H x W residual (device FP32), the preconditioner form above */
int lentils_unet_precondition(lentils_unet *net, const float *r, const float *dinv,
                              const float *feat, float *z, void *stream);
/* Truncated flexible CG on the normal equations, inside the same FP64 iterative refinement as
 * lentils_cg_solve: each new direction is A-orthogonalised against the last opt->window
 * directions, p = d - sum_j (d . A p_j) / (p_j . A p_j) p_j. With the learned preconditioner,
 * d is the network's direction on every opt->net_every-th iteration and the Jacobi direction
 * otherwise. Where the network's direction is not a descent direction (z . r <= 0), that
 * iteration uses the Jacobi direction instead. If the inner residual has not halved over the
 * last 20 checks (20 * check_every iterations), the solve continues as plain Jacobi-CG
 * (res->fallback = 1). net = NULL runs the same iteration with Jacobi only. */
int lentils_fcg_solve(lentils_normal_op *op, const double *b, double *x, const float *inv_diag32,
                      lentils_unet *net, const lentils_cg_options *opt, lentils_cg_result *res,
                      void *stream);

/* ------------------------------------------------------------------------------------------
 * Gridding without device allocation. No counterpart in the reference: it exists for callers
 * that cannot call cudaMalloc -- code running where allocation is forbidden or impossible
 * (host callbacks and stream-ordered sections that must not synchronise, device memory that
 * another framework's pool has already claimed, real-time pipelines that do not allocate after
 * start-up).
 *
 * Grids up to lentils_noalloc_max_vis() visibilities (nrows * nchannels, 65536) per call from
 * caller-owned DEVICE buffers: uvw (nrows x 3 f64), channels (nchannels f64), vis (row order,
 * c64), grid (half plane c64, ACCUMULATED). Same result as lentils_plan_create +
 * lentils_vis_to_plan + lentils_grid, without the plan: all working memory (binning keys,
 * permutation, plan-frame data, work items, radix-sort storage) is one static device array of
 * lentils_noalloc_scratch_bytes() (about 7.3 MB) that every GPU loading this library holds
 * until the process exits. Larger batches are rejected with LENTILS_ERR_INVALID; grid them in
 * several calls. The first call on a device looks the array's address up (set-up, once per
 * device and CUDA context: again after cudaDeviceReset or a re-created primary context); make
 * that first call before any stream capture. Calls share the array: calls whose
 * GPU work overlaps race and corrupt each other's results, so order them on one stream. The
 * call does not synchronise the stream; the guard of fourier_operators.py:77-80 is not applied
 * (as grid_cpu), and non-finite coordinates are skipped.
 * ---------------------------------------------------------------------------------------- */
int lentils_grid_noalloc(const lentils_grid_desc *grid, const double *uvw, int nrows,
                         const double *channels, int nchannels, const float *vis, float *grid_out,
                         void *stream);
int lentils_noalloc_max_vis(void);
long long lentils_noalloc_scratch_bytes(void);

/* ------------------------------------------------------------------------------------------
 * PEMD + external-shear deflection (device)
 *
 * lenses: HOST array of nlenses mass models packed as the reference packs them
 * (lentils/models/lens_models.py:102-147); types 0 (PEMD, 2F1 series), 1 (external
 * potential) and 2 (internal multipoles) are supported. points/out: device arrays of
 * interleaved (x, y). All lenses deflect the same input position (single plane,
 * lentils/backend/deflect.c:43).
 * ---------------------------------------------------------------------------------------- */
int lentils_deflect_f32(const lentils_mass_model *lenses, int nlenses, const float *points,
                        float *out, long long npoints, void *stream);
int lentils_deflect_f64io(const lentils_mass_model *lenses, int nlenses, const double *points,
                          double *out, long long npoints, void *stream);
/* Parameter derivatives of the deflection at each point, FP64: grads (device, float64) is
 * (8, npoints, 2), OVERWRITTEN, for the parameters (b, qh, q, x, y, th, ss, sa) summed over
 * the lenses -- the per-point layout the reference's GlobalLensModel.deflect(deriv=True)
 * allocates (lens_models.py:71-73). PEMD terms as deflect_PEMD_series computes them
 * (deflect.c:304-338, hyp2f1_series :186-236); external shear (x, y, ss, sa) as the
 * derivative block of deflect_external_potential states it (deflect.c:110-119, compiled out
 * in the reference); multipoles contribute none. At most 8 lenses. The drop-in
 * deflect_points(want_deriv = 1) keeps the reference's own accumulation instead: deriv[0..11]
 * += the PEMD terms summed over all points. */
int lentils_deflect_grad(const lentils_mass_model *lenses, int nlenses, const double *points,
                         double *grads, long long npoints, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* LENTILS_GB300_H */
