/*
 * vissat_gb300.h -- C ABI of the GB300 (sm_103a) geometry path of VisSat satellite stereo.
 *
 * Every entry point:
 *   - is plain C (extern "C"), takes device pointers, sizes and a cudaStream_t passed as
 *     void* (NULL = legacy default stream), and never throws;
 *   - returns an int status (VS_OK = 0) and records a message for vs_last_error();
 *   - is asynchronous on the given stream (results are valid after the stream is
 *     synchronised); device-side per-problem failures are written to a caller buffer;
 *   - allocates no device memory: scratch comes from a caller-provided workspace whose
 *     size the matching *_workspace_size() function reports.
 * Calls on different streams may run concurrently; calls sharing a workspace must be
 * ordered by the caller.
 *
 * Each function names the reference routine it replaces (paths relative to the
 * VisSatSatelliteStereo repository).
 */
#ifndef VISSAT_GB300_H
#define VISSAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------- */
#define VS_OK 0
#define VS_ERR_ARG 1        /* invalid argument: null pointer, negative size, bad enum */
#define VS_ERR_CUDA 2       /* a CUDA runtime call or kernel launch failed */
#define VS_ERR_WORKSPACE 3  /* caller workspace smaller than *_workspace_size() */
#define VS_ERR_FACTORIZE 4  /* per-view: factorisation check failed (the reference asserts) */
#define VS_ERR_DEGENERATE 5 /* per-view: fewer than 6 kept points / singular system */
#define VS_ERR_TIMEOUT 6    /* a kernel gave up a bounded wait; its outputs are incomplete */

/* ---- data types ------------------------------------------------------------------ */

/* One RPC camera (RPC00B): the fields RPCModel.__init__ reads from meta_dict
 * (lib/rpc_model.py:132-158).  Coefficients follow the RPC monomial order with
 * x = normalised latitude, y = longitude, z = altitude (lib/rpc_model.py:40-63). */
typedef struct VsRpcCamera {
    double row_off, row_scale, col_off, col_scale;
    double lat_off, lat_scale, lon_off, lon_scale, alt_off, alt_scale;
    double row_num[20], row_den[20], col_num[20], col_den[20];
    double width, height;
} VsRpcCamera;

/* Projection arithmetic. */
#define VS_PROJ_EXACT 0   /* FP64 in the reference's operation order: bit-identical results */
#define VS_PROJ_FAST 1    /* compensated FP32 (double-float) evaluation, |err| < 1e-4 px   */

/* Layouts of a stack of per-view DSMs. */
#define VS_LAYOUT_HWV 0   /* [H][W][V]: the reference's np.concatenate(all_dsm, axis=2)   */
#define VS_LAYOUT_VHW 1   /* [V][H][W]: one plane per view                                 */

/* Length of the per-view camera parameter vector:
 * [w, h, fx, fy, cx, cy, s, qw, qx, qy, qz, tx, ty, tz] (camera_approx.py:178-182). */
#define VS_CAMERA_PARAMS 14
/* Length of the per-view error vector: mean/median/max reprojection error (px) and
 * mean/median/max inverse-projection error (m) (lib/check_error.py:121). */
#define VS_ERROR_STATS 6

/* ---- library ----------------------------------------------------------------------- */
const char *vs_version(void);
/* Message of the last failing call on this host thread ("" if none). */
const char *vs_last_error(void);

/* ---- (a) RPC projection ------------------------------------------------------------ */

/* Replaces RPCModel.projection (lib/rpc_model.py:160-168), for n_cams cameras at once.
 * cams: device array of n_cams cameras.  lat/lon/alt: device FP64 arrays; camera c reads
 * its n points at lat + c*point_stride (point_stride 0: one point set shared by all).
 * col/row: device FP64 outputs [n_cams][n].  keep (nullable): device uint8 [n_cams][n],
 * the in-image mask of camera_approx.py:170-174.  mode: VS_PROJ_EXACT or VS_PROJ_FAST. */
int vs_rpc_project(const VsRpcCamera *cams, int n_cams, const double *lat, const double *lon,
                   const double *alt, int64_t n, int64_t point_stride, double *col, double *row,
                   uint8_t *keep, int mode, void *stream);

/* Precision form of the same projection for n_cams cameras over ONE point set given in the
 * normalised frame (RPCModel.projection after its normalisation, lib/rpc_model.py:164-168
 * with apply_poly :40-63 and apply_rfm :66-79), evaluated as the contraction
 * [n x 20 monomials] x [20 x 4*n_cams coefficients] with FP32 accumulation.
 * xyz: device float32 [3][n] (x = normalised latitude, y = longitude, z = altitude).
 * colrow: device float32 [n_cams][2][n] (col plane, then row plane, per camera).
 * variant: VS_CUBE_*.  Max. pixel error against the FP64 projection of the same points
 * (cameras with line/sample scale 2048, 16 M points): FP32 and BF16X6 below 1e-3 px,
 * TF32X3 ~1.3e-3 px (two tf32 pieces keep 22 bits), BF16X3 ~0.04 px (two bf16 pieces
 * keep ~17 bits).  No counterpart in the reference, which evaluates per camera in FP64. */
#define VS_CUBE_FP32 0     /* CUDA cores, FP32 FMA                                         */
#define VS_CUBE_BF16X3 1   /* tensor cores, 2 bf16 pieces per factor, 3 products             */
#define VS_CUBE_TF32X3 2   /* tensor cores, 2 tf32 pieces per factor, 3 products             */
#define VS_CUBE_BF16X6 3   /* tensor cores, 3 bf16 pieces per factor, 6 products             */
#define VS_CUBE_BF16X3_TC 4 /* as BF16X3 on tcgen05 (TMEM accumulators), at most 64 cameras   */
#define VS_CUBE_BF16X3_LIN 5 /* BF16X3 for the 16 higher-order terms; constant + linear terms in
                              * FP32 on CUDA cores (the split forms' error sits in the large
                              * linear coefficients): FP32's accuracy, below 1e-3 px, faster
                              * than BF16X6                                                  */
#define VS_CUBE_BF16X3_LIN_TC 6 /* as BF16X3_LIN with the contraction on tcgen05 (TMEM
                                 * accumulators, overlapped epilogue), at most 64 cameras     */
#define VS_CUBE_MAX_CAMERAS 128
size_t vs_rpc_project_cube_workspace_size(int n_cams);
int vs_rpc_project_cube(const VsRpcCamera *cams, int n_cams, const float *xyz, int64_t n, float *colrow,
                        int variant, void *workspace, size_t workspace_bytes, void *stream);
/* Device-side status of the last vs_rpc_project_cube call that used `workspace` (same
 * n_cams and variant): copies its error word back and synchronises `stream`.  VS_OK, or
 * VS_ERR_TIMEOUT when a CTA of a tcgen05 variant gave up its bounded wait for the
 * tensor cores (its tiles of colrow are then unwritten).  The other variants have no
 * device-side waits and always report VS_OK.  No counterpart in the reference. */
int vs_rpc_project_cube_status(const void *workspace, int n_cams, int variant, void *stream);
/* Polls of the tcgen05 variants' completion waits before a CTA gives up (default 2^24,
 * far beyond any real completion time); 0 gives up at once, so tests can drive the
 * timeout path without a faulty device.  Process-wide; not thread-safe. */
void vs_set_tc_wait_limit(unsigned polls);
/* Caps the CTAs per SM of the point-binning launches of vs_proj_to_grid and
 * vs_dsm_from_points* (0, the default: as many as fit).  A cap leaves room on every SM for
 * kernels of other streams (the camera fit running concurrently with the rasterisation);
 * process-wide, read at each launch. */
void vs_set_binning_ctas_per_sm(int ctas);
/* Reserves up to `bytes` of L2 in the current context for persisting accesses
 * (cudaLimitPersistingL2CacheSize, clamped to the device's maximum; the reservation ends
 * with the context) and makes the point-binning launches of vs_proj_to_grid and
 * vs_dsm_from_points* mark their key grid persisting with a per-launch access-policy
 * window, so the streamed points cannot evict the grid the atomics update (in
 * vs_dsm_from_points_overlap also the epilogue's clear of the grid two views ahead, so
 * its zeros stay in L2 until that view's binning).  0 turns it off
 * and releases the reservation.  Results are unchanged.  Process-wide, read at each
 * launch; not thread-safe.  No counterpart in the reference. */
int vs_set_l2_persisting(size_t bytes);

/* Replaces RPCModel.inverse_projection (lib/rpc_model.py:170-249) for n_cams cameras:
 * (lon, lat) of image points (col, row) at altitudes alt, by the reference's iteration
 * (start lon = lat = -1 in the normalised frame, finite-difference steps 2 then 0.1),
 * repeated for all of a camera's points until every one reprojects within sqrt(1e-18)
 * normalised units -- the same global iteration count, so bit-identical results.
 * col/row/alt: device FP64; camera c reads its n points at col + c*point_stride.
 * lon/lat: device FP64 [n_cams][n] (normalised when `normalized` != 0, as
 * return_normalized=True); alt_out (nullable): the input altitudes, or the normalised ones.
 * iterations (nullable, HOST int32 [n_cams]): the iteration counts.  The reference loops
 * without a bound; here a camera exceeding max_iter fails with VS_ERR_DEGENERATE.  The
 * call synchronises `stream` once per iteration (the host runs the global loop). */
size_t vs_rpc_inverse_project_workspace_size(int n_cams, int64_t n);
int vs_rpc_inverse_project(const VsRpcCamera *cams, int n_cams, const double *col, const double *row,
                           const double *alt, int64_t n, int64_t point_stride, int normalized, double *lon,
                           double *lat, double *alt_out, int max_iter, int32_t *iterations, void *workspace,
                           size_t workspace_bytes, void *stream);

/* ---- (b) perspective fit ------------------------------------------------------------ */

/* Replaces solve_perspective (lib/solve_perspective.py:82-126) and its factorize
 * (:38-79) for n_views independent problems.  x/y/z: device FP64 ENU points, view v at
 * x + v*xyz_stride (0: shared).  col/row: device FP64 [n_views][n].  keep (nullable):
 * device uint8 [n_views][n].  Outputs (device, row-major FP64): K [n_views][9],
 * R [n_views][9], t [n_views][3]; status (device int32 [n_views]): VS_OK,
 * VS_ERR_FACTORIZE or VS_ERR_DEGENERATE. */
size_t vs_dlt_fit_workspace_size(int n_views, int64_t n);
int vs_dlt_fit(const double *x, const double *y, const double *z, int64_t xyz_stride,
               const double *col, const double *row, const uint8_t *keep, int n_views, int64_t n,
               double *K, double *R, double *t, int32_t *status, void *workspace,
               size_t workspace_bytes, void *stream);

/* Replaces solve_affine (lib/solve_affine.py:37-72) for n_views independent problems: the
 * least-squares affine camera [col; row] = P [x y z 1]^T over the kept points.  x/y/z:
 * device FP64, view v at x + v*xyz_stride; col/row: device FP64 [n_views][n]; keep
 * (nullable): device uint8 [n_views][n].  P: device FP64 [n_views][2][4] (row-major, the
 * reference's reshape((2, 4))); status (nullable): VS_OK or VS_ERR_DEGENERATE (fewer than
 * 4 kept points or a singular system; P is NaN).  FP64 normal equations in per-axis
 * normalised coordinates: predictions agree with LAPACK's solution to well below 1e-6 px. */
size_t vs_affine_fit_workspace_size(int n_views, int64_t n);
int vs_affine_fit(const double *x, const double *y, const double *z, int64_t xyz_stride, const double *col,
                  const double *row, const uint8_t *keep, int n_views, int64_t n, double *P, int32_t *status,
                  void *workspace, size_t workspace_bytes, void *stream);

/* Replaces the per-view loop of CameraApprox.approx_affine_latlonalt
 * (camera_approx.py:112-137): FP64 projection of the lat/lon/alt grid through each RPC
 * camera (as RPCModel.projection), in-image mask, affine fit with (x, y, z) = (lat, lon,
 * alt).  params: device FP64 [n_views][10] = [width, height, P (8)]. */
size_t vs_camera_approx_affine_workspace_size(int n_views, int64_t n);
int vs_camera_approx_affine(const VsRpcCamera *cams, int n_views, const double *lat, const double *lon,
                            const double *alt, int64_t n, int64_t point_stride, double *params, int32_t *status,
                            void *workspace, size_t workspace_bytes, void *stream);

/* Replaces check_perspective_error (lib/check_error.py:37-121): per view the
 * mean/median/max pixel reprojection error and mean/median/max inverse-projection error
 * of camera K[R|t] over the kept points.  err: device FP64 [n_views][6]. */
size_t vs_perspective_error_workspace_size(int n_views, int64_t n);
int vs_perspective_error(const double *x, const double *y, const double *z, int64_t xyz_stride,
                         const double *col, const double *row, const uint8_t *keep, int n_views,
                         int64_t n, const double *K, const double *R, const double *t, double *err,
                         void *workspace, size_t workspace_bytes, void *stream);

/* Replaces the per-view loop of CameraApprox.approx_perspective_enu
 * (camera_approx.py:166-189): projection of the lat/lon/alt grid through each RPC
 * camera, in-image mask, DLT fit, factorisation, quaternion and error statistics, for
 * all views in one call.  Points of view v at lat + v*point_stride (0: shared grid, as in
 * the reference).  params: device FP64 [n_views][14]; err: device FP64 [n_views][6]
 * (nullable: skip the statistics); status: device int32 [n_views]. */
size_t vs_camera_approx_workspace_size(int n_views, int64_t n);
int vs_camera_approx_perspective(const VsRpcCamera *cams, int n_views, const double *lat,
                                 const double *lon, const double *alt, const double *x,
                                 const double *y, const double *z, int64_t n,
                                 int64_t point_stride, int proj_mode, double *params, double *err,
                                 int32_t *status, void *workspace, size_t workspace_bytes,
                                 void *stream);

/* ---- (c) rasterisation ----------------------------------------------------------------- */

/* Replaces proj_to_grid (lib/proj_to_grid.py:41-81): FP64 binning of (easting, northing,
 * height) points, per-cell nanmax of the heights and the non-propagating 3x3 median hole
 * fill.  points: device FP64 [n][3] row-major.  dsm: device FP64 [ysize][xsize].
 * Bit-identical to the reference (NaN payloads aside). */
size_t vs_proj_to_grid_workspace_size(int64_t xsize, int64_t ysize);
int vs_proj_to_grid(const double *points, int64_t n, double xoff, double yoff, double xresolution,
                    double yresolution, int64_t xsize, int64_t ysize, double *dsm, void *workspace,
                    size_t workspace_bytes, void *stream);

/* 3x3 median blur with replicated borders, the cv2.medianBlur(img, 3) calls of
 * produce_dsm.py:58 and aggregate_2p5d.py:81 (NaN ordered after every number).
 * n_img images of [h][w]; the _f64 variant first rounds FP64 input to float32
 * (dsm.astype(np.float32)). */
int vs_median_blur3x3_f32(const float *in, float *out, int64_t h, int64_t w, int64_t n_img,
                          void *stream);
int vs_median_blur3x3_f64(const double *in, float *out, int64_t h, int64_t w, int64_t n_img,
                          void *stream);

/* Batched form of produce_dsm_from_points (produce_dsm.py:46-58) over n_views point
 * clouds on one DSM grid: proj_to_grid then the float32 3x3 median blur per view.
 * points: device FP64 [total][3]; offsets: device int64 [n_views+1] (view v owns rows
 * offsets[v] .. offsets[v+1]-1).  dsm: device float32 [n_views][ysize][xsize]. */
size_t vs_dsm_from_points_workspace_size(int n_views, int64_t xsize, int64_t ysize);
int vs_dsm_from_points(const double *points, const int64_t *offsets, int n_views, double xoff,
                       double yoff, double xresolution, double yresolution, int64_t xsize,
                       int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                       void *stream);

/* vs_dsm_from_points with each view's decode / hole fill / blur on `epilogue_stream`,
 * overlapped with the binning of the next view on `stream` (three rotating key grids, two
 * alternating "first zero" arrays, ordering events).  `stream` covers all of the work when
 * the call's operations complete.  Same results as vs_dsm_from_points.  bin_events
 * (nullable): 2 * n_views cudaEvent_t created by the caller; events 2v and 2v+1 are
 * recorded on `stream` just before and after view v's binning launch (kernel timing). */
size_t vs_dsm_from_points_overlap_workspace_size(int n_views, int64_t xsize, int64_t ysize);
int vs_dsm_from_points_overlap(const double *points, const int64_t *offsets, int n_views, double xoff,
                               double yoff, double xresolution, double yresolution, int64_t xsize,
                               int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                               void *stream, void *epilogue_stream, void *const *bin_events);

/* vs_dsm_from_points as n_views + 1 launches on one stream, launch v binning view v while
 * its other CTAs run view v-1's decode / hole fill / blur (work items handed out by a
 * device counter), so the HBM-bound binning and the issue-bound epilogue share every SM.
 * Same arguments and results as vs_dsm_from_points (produce_dsm.py:46-58 per view).  Grids
 * outside the fast binning's precondition run the two kernels view by view.  launch_events
 * (nullable): 2 * (n_views + 1) cudaEvent_t created by the caller; on the fast path events
 * 2v and 2v+1 are recorded on `stream` just before and after launch v (kernel timing). */
size_t vs_dsm_from_points_pipelined_workspace_size(int n_views, int64_t xsize, int64_t ysize);
int vs_dsm_from_points_pipelined(const double *points, const int64_t *offsets, int n_views, double xoff,
                                 double yoff, double xresolution, double yresolution, int64_t xsize,
                                 int64_t ysize, float *dsm, void *workspace, size_t workspace_bytes,
                                 void *stream, void *const *launch_events);

/* vs_dsm_from_points with the points in HOST memory (the reference's numpy arrays; pinned
 * memory lets the copies overlap the binning): view v's points are copied into staging
 * buffer v % ring (ring 1..8, device buffers in the workspace) on `copy_stream` while the
 * earlier views are binned on `stream`.  host_offsets: host int64 [n_views + 1].  Same
 * results as vs_dsm_from_points; when the call's work on `stream` completes, so have the
 * copies.  The host buffers must stay unchanged until then. */
size_t vs_dsm_from_points_host_workspace_size(int64_t max_view_points, int ring, int64_t xsize, int64_t ysize);
int vs_dsm_from_points_host(const double *host_points, const int64_t *host_offsets, int n_views, double xoff,
                            double yoff, double xresolution, double yresolution, int64_t xsize, int64_t ysize,
                            float *dsm, int ring, void *workspace, size_t workspace_bytes, void *stream,
                            void *copy_stream);

/* ---- (c') batched form: many AOIs, per-view FP32 height maps ----------------------------
 * The per-view point lists of aggregate_2p5d_util.py:75-98 (pixel -> UTM of a height map)
 * feeding produce_dsm_from_points (produce_dsm.py:46-58) and the per-AOI fusion of
 * aggregate_2p5d.py:65-81, for many AOIs in one plan.  A view is an FP32 height map with a
 * pixel -> UTM affine map in fixed point (units of 2^-VS_MAP_FRAC_BITS m):
 *   easting(i, j)  = (e0 + ej*(2j+1-W) + ei*(2i+1-H)) * 2^-28
 *   northing(i, j) = (n0 + nj*(2j+1-W) + ni*(2i+1-H)) * 2^-28
 *   height(i, j)   = heights[i*row_stride + j]   (NaN: no point)
 * for pixel row i < H, column j < W; the point index (first-of-equal order of the nanmax)
 * is i*W + j.  These coordinates are exact doubles, so the result is bit-identical to
 * materialising the FP64 point list and running proj_to_grid + the float32 3x3 median
 * blur per view, then the fusion per AOI.  The plan rejects (VS_ERR_ARG) grids whose
 * origin is not positive or whose extent crosses a power of two, and views whose
 * coordinates would not stay exact. */
#define VS_MAP_FRAC_BITS 28
typedef struct VsAoi {
    double xoff, yoff, xres, yres;   /* DSM grid, as proj_to_grid's arguments */
    int64_t xsize, ysize;
    int32_t first_view, n_views;     /* the AOI's views: consecutive entries of the view array */
} VsAoi;
typedef struct VsMapView {
    const float *heights;            /* device, row-major [height][row_stride] */
    int64_t row_stride;              /* elements, >= width */
    int32_t width, height;
    int32_t aoi, reserved;
    int64_t e0, n0;                  /* fixed-point origin terms (|.| < 2^53) */
    int32_t ej, ei, nj, ni;          /* fixed-point half-pixel steps */
    float *dsm;                      /* device output of this view's DSM; NULL: the run's
                                        view_dsm buffer at the view's offset */
} VsMapView;
/* Opaque host-side plan: validated descriptors and per-AOI binning tables uploaded into the
 * plan workspace.  Planning synchronises `stream`; running does not, and launches kernels
 * only (a run can be captured in a CUDA graph).  One plan serves one stream at a time. */
typedef struct VsAoiBatch VsAoiBatch;
size_t vs_aoi_batch_plan_workspace_size(const VsAoi *aois, int n_aois, int n_views);
int vs_aoi_batch_plan(const VsAoi *aois, int n_aois, const VsMapView *views, int n_views,
                      int tile, void *workspace, size_t workspace_bytes, VsAoiBatch **plan,
                      void *stream);
/* Cells of all views' DSMs (view v at the sum of the cells of views < v), of all fused
 * DSMs (AOI a at the sum of the cells of AOIs < a), and the scratch the fusion needs. */
int vs_aoi_batch_query(const VsAoiBatch *plan, int64_t *view_cells, int64_t *fused_cells,
                       size_t *scratch_bytes);
/* Rasterises views [view_begin, view_end) into their float32 DSMs in one persistent launch:
 * CTAs (at most blocks_per_sm per SM) take work items -- one tile x tile block of one
 * view's DSM, tile = 32 or 64 as planned -- from a device-side counter, bin the pixels that
 * can reach the block (plus a 2-cell halo) into shared memory and run the epilogue
 * (nanmax, hole fill, float32, blur) from there; no key grid is written to device memory.
 * A single view is the per-view form.  view_dsm may be NULL when every view of the plan
 * has its own `dsm` output. */
int vs_aoi_batch_run(const VsAoiBatch *plan, int view_begin, int view_end, int blocks_per_sm,
                     float *view_dsm, void *stream);
/* Fuses AOIs [aoi_begin, aoi_end) from their views' DSMs (vs_fuse_dsms per AOI). */
int vs_aoi_batch_fuse(const VsAoiBatch *plan, int aoi_begin, int aoi_end, const float *view_dsm,
                      float *fused, int median_blur, void *scratch, size_t scratch_bytes, void *stream);
void vs_aoi_batch_destroy(VsAoiBatch *plan);
/* Copies the width x height window of a height map in host memory (pinned for an
 * asynchronous copy; row stride host_row_stride floats) into device memory (row stride
 * row_stride floats) on `stream`: how a request's views reach the device when they are
 * not resident (the serving form's misses). */
int vs_map_upload(const float *host_heights, int64_t host_row_stride, int width, int height, float *heights,
                  int64_t row_stride, void *stream);

/* ---- (d) fusion ----------------------------------------------------------------------- */

/* FP64 point list (width*height rows of easting, northing, height, pixel order) of a float32
 * height map placed by a fixed-point affine map (units of 2^-28 m): pixel (i, j) at
 * easting = (e0 + ej (2j+1-W) + ei (2i+1-H)) 2^-28, northing likewise with n0, nj, ni.
 * The per-view point list the reference builds from a depth map (aggregate_2p5d_util.py:75-98,
 * vs_depth_to_points here) in the synthetic height-map form, for the plain per-view path
 * (points -> vs_proj_to_grid -> blur).  Requires |e0| + |ej| W + |ei| H < 2^52 (and the same
 * for n0, nj, ni), so that every coordinate is an exact double. */
int vs_map_points(const float *heights, int64_t row_stride, int width, int height, int64_t e0, int64_t n0,
                  int64_t ej, int64_t ei, int64_t nj, int64_t ni, double *points, void *stream);

/* Replaces the fusion block of run_fuse (aggregate_2p5d.py:65-81): per cell, reject
 * cells with <= 2 valid views, nanmedian, MAD rejection, nanmean (numpy's float32
 * pairwise order), then the 3x3 median blur when median_blur != 0.  dsm: device
 * float32 stack in `layout`; out: device float32 [h][w].  Bit-identical to the
 * reference's numpy arithmetic (NaN payloads aside). */
size_t vs_fuse_dsms_workspace_size(int64_t h, int64_t w);
int vs_fuse_dsms(const float *dsm, int layout, int64_t n_views, int64_t h, int64_t w, float *out,
                 int median_blur, void *workspace, size_t workspace_bytes, void *stream);

/* vs_fuse_dsms without a workspace, for callers that cannot allocate device memory where
 * they call it (a stream-ordered pipeline that forbids allocation after start-up, a
 * foreign host without a device allocator).  No counterpart in the reference: it is the
 * same fusion as vs_fuse_dsms, with the blur's intermediate grid in a library-owned
 * static device array of VS_FUSE_STATIC_MAX_CELLS floats (16 MiB, held by every GPU that
 * loads the library until exit); larger grids are rejected with VS_ERR_ARG.  The first
 * call on a device looks up the array's device address (cudaGetSymbolAddress), so make
 * that first call before any stream capture.  All calls share the array: calls whose
 * GPU work overlaps (different streams, concurrent threads) race on it.  The array needs
 * no clearing; each call overwrites what it reads.  No cudaMalloc/cudaFree is called. */
#define VS_FUSE_STATIC_MAX_CELLS 4194304
int vs_fuse_dsms_static(const float *dsm, int layout, int64_t n_views, int64_t h, int64_t w, float *out,
                        int median_blur, void *stream);

/* ---- (f1) depth maps -> UTM points -> DSM ---------------------------------------------------
 * The chain of aggregate_2p5d_util.py:75-98 (convert_depth_map_worker): depth <= 0 becomes
 * NaN; pixel (col, row) with depth d maps to inv_proj @ [col, row, 1, d] with a homogeneous
 * divide (ENU metres about the AOI origin); pixels whose z is NaN are dropped, pixel order
 * kept; ENU -> lat/lon/alt (coordinate_system.py:41-50, pymap3d.enu2geodetic) and lat/lon ->
 * UTM easting/northing (lib/latlon_utm_converter.py:38-52, utm + pyproj) in the zone of the
 * first point.  The geodesy restates the published algorithms (You 2000 for ECEF ->
 * geodetic, Krueger's series to n^6 for transverse Mercator); pymap3d and pyproj are not
 * bit-reproduced (their results agree to ~1e-8 m).
 *
 * A plan fixes the frame (ENU origin = the AOI centre and lowest altitude,
 * coordinate_system.py:44-47; UTM zone and hemisphere) and an ENU box.  Inside the box the
 * VS_GEO_FAST arithmetic evaluates the geodesy as a validated degree-4 polynomial (the plan
 * checks it against the FP64 chain; enabled only within VS_GEO_FAST_TOL_M metres); outside
 * it, and in VS_GEO_EXACT mode, every point takes the FP64 chain.  Creating a plan runs
 * three small kernels and synchronises `stream`; the device buffer (vs_geo_plan_device_bytes)
 * must stay allocated while the plan is used. */
#define VS_GEO_EXACT 0
#define VS_GEO_FAST 1
#define VS_GEO_FAST_TOL_M 2.5e-7
#define VS_GEO_FLAG_HEMISPHERE 1   /* a point lies in the other hemisphere (the reference asserts) */

typedef struct VsGeoFrame {
    double lat0, lon0, alt0;        /* ENU origin: degrees, degrees, metres */
    int32_t utm_zone;               /* 1..60 */
    int32_t south;                  /* 1: false northing 10,000 km */
    double box_lo[3], box_hi[3];    /* ENU box of the fast path (m); box_hi <= box_lo: none */
} VsGeoFrame;

typedef struct VsGeoPlan VsGeoPlan;

size_t vs_geo_plan_device_bytes(void);
int vs_geo_plan_create(const VsGeoFrame *frame, void *device_buffer, size_t device_bytes, VsGeoPlan **plan,
                       void *stream);
/* Largest |fast - exact| (m) seen by the validation, and whether the fast path is on. */
int vs_geo_plan_query(const VsGeoPlan *plan, double *max_err_m, int32_t *fast_enabled);
void vs_geo_plan_destroy(VsGeoPlan *plan);

/* coordinate_system.local_to_global: ENU points (point_stride doubles apart, xyz first) ->
 * lat, lon (degrees), alt (m), FP64 chain. */
int vs_enu_to_geodetic(const VsGeoPlan *plan, const double *enu, int64_t n, int64_t point_stride, double *lat,
                       double *lon, double *alt, void *stream);
/* lib/latlon_utm_converter.latlon_to_eastnorh in the plan's zone and hemisphere: lat, lon
 * (degrees) -> easting, northing (m).  flags (device int32, nullable): VS_GEO_FLAG_* or-ed. */
int vs_geodetic_to_utm(const VsGeoPlan *plan, const double *lat, const double *lon, int64_t n, double *east,
                       double *north, int32_t *flags, void *stream);

/* One depth map (height x width float32, row-major) -> points[n][3] = (easting, northing,
 * altitude) of its valid pixels in pixel order; *n_points (device) receives n.  points
 * must hold height * width rows.  inv_proj: host, 16 doubles, row-major. */
size_t vs_depth_to_points_workspace_size(int64_t height, int64_t width);
int vs_depth_to_points(const float *depth, int64_t height, int64_t width, const double *inv_proj,
                       const VsGeoPlan *plan, int32_t mode, double *points, int64_t *n_points, int32_t *flags,
                       void *workspace, size_t workspace_bytes, void *stream);

/* Depth maps -> per-view DSMs without materialising the points: the points of
 * vs_depth_to_points (the same bits) binned as vs_dsm_from_points does (nanmax, hole fill,
 * float32, 3x3 median blur) into dsm[n_views][ysize][xsize].  depths: host array of
 * n_views device pointers; heights, widths: host arrays; inv_projs: host, n_views x 16.
 * The grid must be positive and lie inside its origins' binades (the fast binning's
 * precondition; VS_ERR_ARG otherwise -- use vs_depth_to_points + vs_dsm_from_points). */
size_t vs_dsm_from_depth_maps_workspace_size(int64_t xsize, int64_t ysize);
int vs_dsm_from_depth_maps(const float *const *depths, const int64_t *heights, const int64_t *widths, int n_views,
                           const double *inv_projs, const VsGeoPlan *plan, int32_t mode, double xoff, double yoff,
                           double xresolution, double yresolution, int64_t xsize, int64_t ysize, float *dsm,
                           int32_t *flags, void *workspace, size_t workspace_bytes, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* VISSAT_GB300_H */
