/*
 * msplat_gb300.h -- C ABI of the GB300 (sm_103a) Gaussian-splatting rasteriser.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream, and
 * returns an msplat_status (0 = ok).  Nothing here allocates device memory:
 * outputs and scratch ("workspace") are owned by the caller.  Work is only
 * enqueued on `stream`; no function synchronises the host with the device.
 *
 * Each declaration names the reference interface it replaces
 * (pointrix-project/msplat, paths relative to that project).  The reference
 * exports these as a pybind11 module `msplat._C` (msplat/src/ext.cpp:13-26);
 * here they are `extern "C"` so ctypes / cgo / JNI can bind them directly.
 *
 * Conventions shared by all entry points
 *   - float tensors are fp32, contiguous, in the reference's layouts:
 *     xyz [P,3], uv [P,2], depth [P], scales [P,3], uquats [P,4] (r,x,y,z),
 *     cov3d [P,6] (upper triangle), conic [P,3], radius/tiles [P] int32,
 *     intr [4] = (fx,fy,cx,cy), extr [3,4] (or the first 12 floats of [4,4])
 *     row-major world-to-camera [R|t].
 *   - `visible` is a bool (1 byte) mask [P]; NULL means "all visible".
 *   - Tiles are 16x16 pixels; the tile grid is ceil(W/16) x ceil(H/16).
 *   - Outputs are fully written (elements the reference leaves at zero are
 *     written as zero), so callers may pass uninitialised buffers, except
 *     where a comment says "accumulated".
 */
#ifndef MSPLAT_GB300_H
#define MSPLAT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define MSPLAT_API __declspec(dllexport)
#else
#define MSPLAT_API __attribute__((visibility("default")))
#endif

typedef struct CUstream_st *msplat_stream_t; /* == cudaStream_t */

typedef enum {
    MSPLAT_OK = 0,
    MSPLAT_ERR_INVALID_ARGUMENT = 1, /* null pointer, negative size, bad shape */
    MSPLAT_ERR_WORKSPACE = 2,        /* workspace too small or misaligned */
    MSPLAT_ERR_LAUNCH = 3,           /* a kernel launch failed */
    MSPLAT_ERR_CAPACITY = 4,         /* more intersections than int32 / capacity */
    MSPLAT_ERR_UNSUPPORTED = 5,      /* e.g. SH degree > 10 */
    MSPLAT_ERR_TIMEOUT = 6           /* a bounded device-side wait gave up */
} msplat_status;

/* Human-readable text for a status, and the detail message of the last
 * failing call on this host thread. */
MSPLAT_API const char *msplat_status_string(int status);
MSPLAT_API const char *msplat_last_error(void);
/* Library version, e.g. "0.1.0". */
MSPLAT_API const char *msplat_version(void);
/* Number of kernels this library has launched in the process so far (all
 * host threads, all devices).  Instrumentation with no counterpart in the
 * reference: a caller reads it around a region to count the launches
 * inside. */
MSPLAT_API unsigned long long msplat_kernel_launches(void);

/* ------------------------------------------------------------------------ */
/* Projection: replaces projectPointsForward / projectPointsBackward
 * (msplat/src/project_point.cu:147-179, :181-228; bound as
 * _C.project_point_forward / _C.project_point_backward, ext.cpp:14-15).
 * uv = (fx*tx/tz + cx - 0.5, fy*ty/tz + cy - 0.5), depth = tz with
 * t = R*xyz + T.  Culled points (near / extent) get uv = 0, depth = 0.    */
MSPLAT_API int msplat_project_point_forward(int P, const float *xyz, const float *intr,
                                 const float *extr, int W, int H,
                                 float nearest, float extent, float *uv,
                                 float *depth, msplat_stream_t stream);

/* Scratch needed by the backward passes that reduce camera gradients. */
MSPLAT_API size_t msplat_camera_grad_workspace_size(int P);

/* dL_dxyz is written.  dL_dintr [4] / dL_dextr [12] may be NULL (the
 * reference skips them when intr/extr do not require grad); when given they
 * are written (not accumulated), reduced in a fixed order (deterministic). */
MSPLAT_API int msplat_project_point_backward(int P, const float *xyz, const float *intr,
                                  const float *extr, int W, int H,
                                  const float *uv, const float *depth,
                                  const float *dL_duv, const float *dL_ddepth,
                                  float *dL_dxyz, float *dL_dintr,
                                  float *dL_dextr, void *workspace,
                                  size_t workspace_bytes,
                                  msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* 3-D covariance: replaces computeCov3DForward / computeCov3DBackward
 * (msplat/src/compute_cov3d.cu:149-170, :172-200; ext.cpp:16-17).
 * Sigma = (S R)^T (S R) as [s00,s01,s02,s11,s12,s22].                      */
MSPLAT_API int msplat_compute_cov3d_forward(int P, const float *scales,
                                 const float *uquats, const uint8_t *visible,
                                 float *cov3d, msplat_stream_t stream);
MSPLAT_API int msplat_compute_cov3d_backward(int P, const float *scales,
                                  const float *uquats, const uint8_t *visible,
                                  const float *dL_dcov3d, float *dL_dscales,
                                  float *dL_duquats, msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* EWA splatting: replaces EWAProjectForward / EWAProjectBackward
 * (msplat/src/ewa_project.cu:254-297, :299-345; ext.cpp:18-19).
 * conic [P,3], radius [P], tiles [P] (tiles touched in the 16x16 grid).    */
MSPLAT_API int msplat_ewa_project_forward(int P, const float *xyz, const float *cov3d,
                               const float *intr, const float *extr,
                               const float *uv, int W, int H,
                               const uint8_t *visible, float *conic,
                               int32_t *radius, int32_t *tiles,
                               msplat_stream_t stream);
MSPLAT_API int msplat_ewa_project_backward(int P, const float *xyz, const float *cov3d,
                                const float *intr, const float *extr,
                                const int32_t *radius, const float *dL_dconic,
                                float *dL_dxyz, float *dL_dcov3d,
                                float *dL_dintr, float *dL_dextr,
                                void *workspace, size_t workspace_bytes,
                                msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Spherical harmonics, degrees 0..10 (D = (deg+1)^2 <= 121): replaces
 * computeSHForward / computeSHBackward (msplat/src/compute_sh.cu:1696-1753;
 * ext.cpp:22-23).  shs [P,C,D] channel-major, dirs [P,3], value [P,C].     */
MSPLAT_API int msplat_compute_sh_forward(int P, int C, int D, const float *shs,
                              const float *dirs, const uint8_t *visible,
                              float *value, msplat_stream_t stream);
MSPLAT_API int msplat_compute_sh_backward(int P, int C, int D, const float *shs,
                               const float *dirs, const uint8_t *visible,
                               const float *dL_dvalue, float *dL_dshs,
                               float *dL_ddirs, msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Sorting.  The reference sorts with torch.cumsum + its key kernel +
 * torch.sort + torch.gather + its range kernel (msplat/sort_gaussian.py:
 * 41-52).  The two native pieces are mirrored one-to-one:                  */

/* Replaces computeGaussianKey (msplat/src/sort_gaussian.cu:74-113;
 * ext.cpp:20).  `tiles_cumsum` is the inclusive int32 scan of tiles;
 * `num_intersects` = tiles_cumsum[P-1] (the reference reads it with a
 * blocking .item(); here the caller passes it).  key [I] int64 =
 * (tile << 32) | sign-extended depth bits; idx [I] int32.  Slots that no
 * Gaussian fills stay 0, like the reference's zero-initialised buffers.    */
MSPLAT_API int msplat_compute_gaussian_key(int P, const float *uv, const float *depth,
                                int W, int H, const int32_t *radius,
                                const int32_t *tiles_cumsum,
                                int64_t num_intersects, int64_t *key,
                                int32_t *idx, msplat_stream_t stream);

/* Replaces computeTileGaussianRange (msplat/src/sort_gaussian.cu:115-142;
 * ext.cpp:21).  tile_range [ntiles,2] int32 = [start,end) per tile, [0,0]
 * for empty tiles.  Keys whose tile id is outside the grid (negative-depth
 * keys) are skipped where the reference writes out of bounds.              */
MSPLAT_API int msplat_compute_tile_gaussian_range(int W, int H, int64_t num_intersects,
                                       const int64_t *key_sorted,
                                       int32_t *tile_range,
                                       msplat_stream_t stream);

/* Inclusive int32 scan (the reference's torch.cumsum(tiles, dtype=int32),
 * msplat/sort_gaussian.py:42).  Also writes out[n-1] widened to int64 into
 * *total (device pointer, may be NULL) for overflow-safe host reads.      */
MSPLAT_API size_t msplat_scan_workspace_size(int n);
MSPLAT_API int msplat_inclusive_scan_i32(int n, const int32_t *in, int32_t *out,
                              int64_t *total, void *workspace,
                              size_t workspace_bytes, msplat_stream_t stream);

/* Allocation-free variant of msplat_inclusive_scan_i32 (no counterpart in
 * the reference).  For callers that cannot allocate device memory where they
 * call the scan -- code running inside a CUDA stream capture, a host
 * application or plugin framework that owns every device allocation, or a
 * real-time loop that may not call an allocator -- and so cannot provide a
 * workspace.  Its scratch (the per-4096-element partial sums) is a fixed
 * array inside the library: every GPU that loads the library keeps those
 * 131 KB until the process exits.  n may not exceed
 * MSPLAT_SCAN_NOALLOC_MAX_N; larger n is rejected with MSPLAT_ERR_CAPACITY
 * before any work is enqueued.  All calls share the one array, so calls
 * that overlap on the GPU (different streams, or different host threads
 * without ordering) race and give wrong sums; serialise them.  The first
 * call on each device looks up the array's device address (with that device
 * current); make that first call before any stream capture.  The address is
 * cached for the life of the process: after cudaDeviceReset (or any reset of
 * the device's primary context) the library's module is loaded anew and the
 * cached address is stale, so do not call this entry point again in a
 * process that reset the device it ran on.  It never calls
 * cudaMalloc / cudaFree or any allocating routine.                         */
#define MSPLAT_SCAN_NOALLOC_MAX_N (64 * 1024 * 1024)
MSPLAT_API int msplat_inclusive_scan_i32_noalloc(int n, const int32_t *in,
                                                 int32_t *out, int64_t *total,
                                                 msplat_stream_t stream);

/* Stable LSD radix sort of (int64 key, int32 value) pairs in SIGNED int64
 * order (torch.sort on int64, msplat/sort_gaussian.py:49) that carries the
 * values along (the torch.gather of :50).  Only key bits [begin_bit,
 * end_bit) are sorted, 8 per pass; callers that know all keys are
 * non-negative pass end_bit < 64 to skip constant high digits, otherwise
 * end_bit must be 64.  vals_in == NULL means value = input index.  The
 * inputs are only read; outputs must not alias them.                      */
MSPLAT_API size_t msplat_radix_sort_i64_workspace_size(int64_t n);
MSPLAT_API int msplat_radix_sort_i64_pairs(int64_t n, const int64_t *keys_in,
                                const int32_t *vals_in, int64_t *keys_out,
                                int32_t *vals_out, int begin_bit,
                                int end_bit, void *workspace,
                                size_t workspace_bytes,
                                msplat_stream_t stream);

/* How every radix sort of the library runs its 8-bit passes (no
 * counterpart in the reference, which calls torch.sort,
 * msplat/sort_gaussian.py:42-50).  on == 0 (the default): three launches
 * per pass (upsweep, row scan, downsweep), no device-side waits.  on != 0:
 * one histogram kernel for all passes, then one kernel per pass that finds
 * its tile's output offsets by decoupled look-back; every look-back wait is
 * bounded by the limit of msplat_set_wait_limit and reported by
 * msplat_wait_error.  Results are identical either way; on GB300 the
 * three-launch passes are faster for the tile lists of a 1080p frame and
 * of a 64-camera batch.  Process-wide. */
MSPLAT_API int msplat_set_sort_onesweep(int on);

/* Fast drop-in for the whole of sort_gaussian (msplat/sort_gaussian.py:
 * 8-54) in two calls with one host read in between:
 *   1. _prepare: depth-sorts the Gaussians and scans their tile counts in
 *      depth order; writes counts[0] = number of intersections I and
 *      counts[1] = number of "filler" slots (tiles[i] larger than the
 *      Gaussian's rectangle, or radius <= 0 with tiles > 0).
 *   2. _finish (only valid when counts[1] == 0): emits (tile, id) pairs in
 *      depth order, stable-sorts them by tile, writes idx_sorted [I] (16-byte
 *      aligned) and tile_range [ntiles,2].  Bit-identical to the reference's
 *      output.
 * When counts[1] != 0 the caller uses the reference-layout path
 * (compute_gaussian_key + radix_sort_i64_pairs + tile range), which
 * reproduces the zero-filled slots exactly.                                */
MSPLAT_API size_t msplat_sort_prepare_workspace_size(int P, int W, int H);
MSPLAT_API size_t msplat_sort_finish_workspace_size(int P, int64_t num_intersects,
                                         int W, int H);
MSPLAT_API int msplat_sort_gaussian_prepare(int P, const float *depth,
                                 const int32_t *radius, const int32_t *tiles,
                                 const float *uv, int W, int H,
                                 int64_t *counts, void *workspace,
                                 size_t workspace_bytes,
                                 msplat_stream_t stream);
MSPLAT_API int msplat_sort_gaussian_finish(int P, const float *uv, const float *depth,
                                const int32_t *radius, int W, int H,
                                int64_t num_intersects,
                                const void *prepare_workspace,
                                int32_t *idx_sorted, int32_t *tile_range,
                                void *workspace, size_t workspace_bytes,
                                msplat_stream_t stream);

/* The prepare of the fused path's culled tile lists: as
 * msplat_sort_gaussian_prepare, but each Gaussian's tile rectangle is first
 * shrunk, side by side, while its outer row or column holds no pixel centre
 * the Gaussian (conic [P,3], opacity [P]) can take to alpha >= 1/255, and
 * negative-depth Gaussians (in no tile range) emit nothing.  The following
 * finish (either form) then writes lists without those entries: the blend
 * of them gives the same images and gradients as the reference's lists, but
 * idx_sorted, tile_range and the intersection count differ from the
 * reference's.  counts[1] still compares tiles[] with the unshrunk
 * rectangles.  Grids up to 32767 tiles a side.  No counterpart in the
 * reference. */
MSPLAT_API int msplat_sort_gaussian_prepare_culled(int P, const float *depth,
                                 const int32_t *radius, const int32_t *tiles,
                                 const float *uv, const float *conic,
                                 const float *opacity, int W, int H,
                                 int64_t *counts, void *workspace,
                                 size_t workspace_bytes,
                                 msplat_stream_t stream);

/* The finish without the host read of counts (for stream capture): the
 * buffers are sized for `capacity` intersections (idx_sorted [capacity],
 * workspace msplat_sort_finish_workspace_size(P, capacity, W, H)) and the
 * kernels take the count from `counts` on the device.  status[0] (int32,
 * device) is set to 1 when the result is not valid -- more intersections
 * than the capacity, or counts[1] != 0 (the reference layout is needed) --
 * and to 0 otherwise; the caller checks it later and redoes the frame with
 * msplat_sort_gaussian_finish then.  No counterpart in the reference. */
MSPLAT_API int msplat_sort_gaussian_finish_capacity(int P, const float *uv, const float *depth,
                                 const int32_t *radius, int W, int H, int64_t capacity,
                                 const int64_t *counts, const void *prepare_workspace,
                                 int32_t *idx_sorted, int32_t *tile_range, int32_t *status,
                                 void *workspace, size_t workspace_bytes,
                                 msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Alpha blending: replaces alphaBlendingForward / alphaBlendingBackward
 * (msplat/src/alpha_blending.cu:248-394, :396-573; ext.cpp:24-25).
 * feature [P,C] (any C >= 1, one pass, no chunking), out [C,H,W],
 * final_T [H,W], ncontrib [H,W] int32.                                     */
MSPLAT_API int msplat_alpha_blending_forward(int P, int C, const float *uv,
                                  const float *conic, const float *opacity,
                                  const float *feature,
                                  const int32_t *idx_sorted,
                                  const int32_t *tile_range, float bg, int W,
                                  int H, float *out, float *final_T,
                                  int32_t *ncontrib, msplat_stream_t stream);

/* Forward-blend variant and its bounded waits.  No counterpart in the
 * reference (its blend gathers each batch with a block barrier,
 * msplat/src/alpha_blending.cu:57-72).  With producer_warps = 2 or 4 the
 * C <= 4 forward runs as a producer / consumer ring: that many warps gather
 * each tile's batches into two shared-memory slots while eight warps blend,
 * handed off through mbarriers; 0 selects the block-barrier kernel.
 * batch_producer_warps does the same for the multi-camera grid.  Results
 * are identical either way; the default is the tuned choice.  Process-wide
 * setting (all devices, all threads). */
MSPLAT_API int msplat_set_blend_ring(int producer_warps, int batch_producer_warps);
/* The same for the C <= 4 backward: producer_warps = 1 or 2 runs it as a
 * ring (producer warps gather each tile's batches from the end of its list
 * while the backward's four consumer warps walk the other slot) on
 * single-camera images of at least 1,024 tiles, 0 the block-barrier kernel
 * everywhere.  Gradients agree up to the order of float atomics.
 * Process-wide. */
MSPLAT_API int msplat_set_blend_ring_bwd(int producer_warps, int batch_producer_warps);
/* Every device-side wait -- the ring's hand-offs, the sort's look-back,
 * the SH kernels' wait for a bulk copy of coefficient rows -- gives up
 * after `polls` polls of at most about 1 us each (default 2^21, about
 * 2 s), sets a device error word and lets the kernel finish with invalid
 * results instead of hanging.  Process-wide. */
MSPLAT_API int msplat_set_wait_limit(int polls);
/* Reads (after synchronising `stream`) the current device's error words of
 * the bounded waits into *error (1 if any is set; may be NULL), clears them
 * when reset != 0, and returns MSPLAT_ERR_TIMEOUT if one was set,
 * MSPLAT_OK otherwise. */
MSPLAT_API int msplat_wait_error(int reset, int *error, msplat_stream_t stream);

/* dL_duv [P,2], dL_dconic [P,3], dL_dopacity [P], dL_dfeature [P,C] must be
 * zero on entry (the kernels accumulate into them with atomics). */
MSPLAT_API int msplat_alpha_blending_backward(int P, int C, const float *uv,
                                   const float *conic, const float *opacity,
                                   const float *feature,
                                   const int32_t *idx_sorted,
                                   const int32_t *tile_range, float bg, int W,
                                   int H, const float *final_T,
                                   const int32_t *ncontrib,
                                   const float *dL_dout, float *dL_duv,
                                   float *dL_dconic, float *dL_dopacity,
                                   float *dL_dfeature, msplat_stream_t stream);

/* The same two calls keeping each list entry's warp-block mask from the
 * forward for the backward.  No counterpart in the reference (its backward
 * re-gathers and re-tests every entry, msplat/src/alpha_blending.cu:166-182).
 * entry_masks: one byte per entry of idx_sorted; the forward writes it for
 * every entry it gathers (every entry up to each tile's last contributor),
 * and the backward -- called with the same lists and C -- reads it instead
 * of repeating the tile and warp-block culls.  Results are those of the
 * plain calls.  For C > 4 (and builds that split tiles between blocks) the
 * masks are neither written nor read. */
MSPLAT_API int msplat_alpha_blending_forward_masks(int P, int C, const float *uv,
                                        const float *conic, const float *opacity,
                                        const float *feature,
                                        const int32_t *idx_sorted,
                                        const int32_t *tile_range, float bg,
                                        int W, int H, float *out,
                                        float *final_T, int32_t *ncontrib,
                                        unsigned char *entry_masks,
                                        msplat_stream_t stream);
MSPLAT_API int msplat_alpha_blending_backward_masks(int P, int C, const float *uv,
                                         const float *conic, const float *opacity,
                                         const float *feature,
                                         const int32_t *idx_sorted,
                                         const int32_t *tile_range, float bg,
                                         int W, int H, const float *final_T,
                                         const int32_t *ncontrib,
                                         const float *dL_dout, float *dL_duv,
                                         float *dL_dconic, float *dL_dopacity,
                                         float *dL_dfeature,
                                         const unsigned char *entry_masks,
                                         msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Fused preprocess of a rasterisation.  No single counterpart in the
 * reference: it is the composite project_point -> compute_cov3d ->
 * ewa_project of msplat/__init__.py:70-93 (visible = depth != 0), optionally
 * followed by compute_sh (msplat/compute_sh.py:8-64) on the view directions
 * d = (xyz - c) / |xyz - c|, c = -R^T T the camera centre of extr.  uv,
 * depth, conic, radius and tiles are bit-identical to the three stage calls.
 * shs [P,C,D] may be NULL (C = 0); color [P,C] is written when it is not. */
MSPLAT_API int msplat_rasterize_preprocess_forward(int P, const float *xyz, const float *scales,
                                  const float *uquats, const float *intr, const float *extr,
                                  int W, int H, float nearest, float extent, int C, int D,
                                  const float *shs, float *uv, float *depth, float *conic,
                                  int32_t *radius, int32_t *tiles, float *color,
                                  msplat_stream_t stream);

/* Scratch for the camera gradients of the backward (0 when P == 0). */
MSPLAT_API size_t msplat_rasterize_preprocess_workspace_size(int P, int C, int D);

/* Adjoint of the fused forward: from dL_duv [P,2] and dL_dconic [P,3] of
 * the blend (and dL_dcolor [P,C] when shs is given) writes dL_dxyz [P,3]
 * (projection + EWA + view direction), dL_dscales [P,3], dL_duquats [P,4],
 * dL_dshs [P,C,D], and dL_dintr [4] / dL_dextr [12] when not NULL (then
 * the workspace is required).  The covariance is recomputed, not stored. */
MSPLAT_API int msplat_rasterize_preprocess_backward(int P, const float *xyz, const float *scales,
                                  const float *uquats, const float *intr, const float *extr,
                                  int C, int D, const float *shs, const float *depth,
                                  const int32_t *radius, const float *dL_duv,
                                  const float *dL_dconic, const float *dL_dcolor,
                                  float *dL_dxyz, float *dL_dscales, float *dL_duquats,
                                  float *dL_dshs, float *dL_dintr, float *dL_dextr,
                                  void *workspace, size_t workspace_bytes,
                                  msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Batched preprocess of one scene for B cameras.  No counterpart in the
 * reference (one camera per call).  cams [B,16] = intr (fx, fy, cx, cy)
 * then extr (3x4 row-major); dims [B,2] int32 = (W, H).  Outputs are
 * camera-major: uv [B,P,2], depth [B,P,1], conic [B,P,3], radius [B,P],
 * tiles [B,P], color [B,P,C] (when shs [P,C,D] is given; C = 0 otherwise);
 * each camera's slice equals msplat_rasterize_preprocess_forward for that
 * camera bit for bit.  Each Gaussian and its SH rows are read once.
 * Rows of at most 1,599 floats (C * D; the adjoint: 795), else
 * MSPLAT_ERR_UNSUPPORTED. */
MSPLAT_API int msplat_batch_preprocess_forward(int P, int B, const float *xyz, const float *scales,
                                  const float *uquats, const float *cams, const int32_t *dims,
                                  float nearest, float extent, int C, int D, const float *shs,
                                  float *uv, float *depth, float *conic, int32_t *radius,
                                  int32_t *tiles, float *color, msplat_stream_t stream);

/* Scratch of the backward's camera gradients (B x blocks x 16 floats). */
MSPLAT_API size_t msplat_batch_preprocess_workspace_size(int P, int B, int C, int D);

/* Adjoint: from the per-camera blend gradients dL_duv [B,P,2], dL_dconic
 * [B,P,3], dL_dcolor [B,P,C] (with shs) and dL_dopacity_cam [B,P] (may be
 * NULL) writes the gradients summed over the cameras -- dL_dxyz [P,3],
 * dL_dscales [P,3], dL_duquats [P,4], dL_dshs [P,C,D], dL_dopacity [P]
 * (may be NULL) -- and, when dL_dcams [B,16] is not NULL, each camera's
 * (intr, extr) gradient (then the workspace is required). */
MSPLAT_API int msplat_batch_preprocess_backward(int P, int B, const float *xyz, const float *scales,
                                  const float *uquats, const float *cams, int C, int D,
                                  const float *shs, const float *depth, const int32_t *radius,
                                  const float *dL_duv, const float *dL_dconic,
                                  const float *dL_dcolor, const float *dL_dopacity_cam,
                                  float *dL_dxyz, float *dL_dscales, float *dL_duquats,
                                  float *dL_dshs, float *dL_dopacity, float *dL_dcams,
                                  void *workspace, size_t workspace_bytes,
                                  msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Multi-camera batches in one key space.  No counterpart in the reference,
 * which renders one camera per call (msplat/__init__.py:22-93) and sorts one
 * camera's intersections per call (msplat/sort_gaussian.py:8-54).  A batch
 * of B cameras (of one or several scenes) is sorted by (camera, tile,
 * depth) and blended by one grid over every camera's tiles.
 *
 * Layout: per-camera per-Gaussian arrays (uv [.,2], depth, conic [.,3],
 * radius, tiles, colour [.,C], and the blend's gradients) are stacked
 * camera after camera -- camera b's rows start at the sum of P over the
 * cameras before it; opacity (and shared features) are read at
 * opacity_offset[b] + g; tiles are numbered globally (tile_range has one
 * row per tile of all cameras); images are stacked: camera b's [C, H_b,
 * W_b] image starts at C * (pixels of the cameras before it), final_T and
 * ncontrib at (those pixels).  The order of each camera's list equals the
 * single-camera culled lists (msplat_sort_gaussian_prepare_culled), so
 * every camera's image is bit-identical to a single-camera call's. */

/* The plan: a host buffer of msplat_batch_plan_bytes(B) bytes built from the
 * cameras' dims [B,2] (W, H), npoints [B] (Gaussians of each camera's scene)
 * and opacity_offset [B] (may be NULL: all 0), all host arrays; the caller
 * copies it to device memory and passes that copy to the calls below.
 * sizes (host, 5 entries) receives: total tiles, total stacked rows, total
 * pixels, depth-key items (padded), tile-key passes. */
MSPLAT_API size_t msplat_batch_plan_bytes(int B);
MSPLAT_API int msplat_batch_plan(int B, const int32_t *dims, const int32_t *npoints,
                                 const int64_t *opacity_offset, void *plan, size_t plan_bytes,
                                 int64_t *sizes);

/* Depth sort of every camera's Gaussians (one segmented radix sort), the
 * culled rectangles and intersection counts.  counts (device, int64 [2 + B])
 * receives the intersections, the padded list length a finish needs (its
 * capacity) and each camera's intersections. */
MSPLAT_API size_t msplat_batch_sort_prepare_workspace_size(int B, int64_t depth_items);
MSPLAT_API int msplat_batch_sort_prepare(const void *plan, int B, int64_t depth_items, const float *uv,
                                         const float *depth, const int32_t *radius, const float *conic,
                                         const float *opacity, int64_t *counts, void *workspace,
                                         size_t workspace_bytes, msplat_stream_t stream);

/* Emission and a segmented stable sort by tile of every camera's list, and
 * the tile ranges [total_tiles, 2] (positions in idx_sorted [capacity],
 * 16-byte aligned).  capacity: a multiple of 3072, at least counts[1] of the prepare for a
 * valid result; no host read happens.  status (device int32, may be NULL)
 * is set to 1 when the capacity was too small (the result is then not
 * valid), else 0. */
MSPLAT_API size_t msplat_batch_sort_finish_workspace_size(int B, int64_t capacity, int passes);
MSPLAT_API int msplat_batch_sort_finish(const void *plan, int B, int64_t depth_items, int total_tiles, int passes,
                                        int64_t capacity, const void *prepare_workspace, int32_t *idx_sorted,
                                        int32_t *tile_range, int32_t *status, void *workspace,
                                        size_t workspace_bytes, msplat_stream_t stream);
/* The same, told the digit bits of the last tile-key pass: every camera's
 * local tile keys stay below 2^(8 (passes - 1) + last_pass_bits), so the
 * last pass ranks only those bits (1..8; bits_for(largest camera tile
 * count) - 8 (passes - 1)).  Same results as msplat_batch_sort_finish. */
MSPLAT_API int msplat_batch_sort_finish_bits(const void *plan, int B, int64_t depth_items, int total_tiles,
                                             int passes, int last_pass_bits, int64_t capacity,
                                             const void *prepare_workspace, int32_t *idx_sorted,
                                             int32_t *tile_range, int32_t *status, void *workspace,
                                             size_t workspace_bytes, msplat_stream_t stream);

/* One blend grid over every camera's tiles (the semantics of
 * msplat_alpha_blending_forward per camera).  feature_per_camera: 1 when
 * feature is stacked per camera (rows like uv), 0 when per scene (rows like
 * opacity). */
MSPLAT_API int msplat_batch_alpha_blending_forward(const void *plan, int B, int total_tiles, int C,
                                                   int feature_per_camera, const float *uv, const float *conic,
                                                   const float *opacity, const float *feature,
                                                   const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                                   float *out, float *final_T, int32_t *ncontrib,
                                                   msplat_stream_t stream);

/* Its adjoint: dL_duv [rows,2], dL_dconic [rows,3], dL_dopacity [rows] (the
 * camera's own opacity gradient) and dL_dfeature [rows,C] per stacked row,
 * zero on entry (accumulated). */
MSPLAT_API int msplat_batch_alpha_blending_backward(const void *plan, int B, int total_tiles, int64_t rows, int C,
                                                    int feature_per_camera, const float *uv, const float *conic,
                                                    const float *opacity, const float *feature,
                                                    const int32_t *idx_sorted, const int32_t *tile_range, float bg,
                                                    const float *final_T, const int32_t *ncontrib,
                                                    const float *dL_dout, float *dL_duv, float *dL_dconic,
                                                    float *dL_dopacity, float *dL_dfeature,
                                                    msplat_stream_t stream);

/* The same two calls keeping each list entry's warp-block mask from the
 * forward for the backward (as msplat_alpha_blending_forward_masks /
 * _backward_masks): entry_masks holds one byte per entry of idx_sorted. */
MSPLAT_API int msplat_batch_alpha_blending_forward_masks(const void *plan, int B, int total_tiles, int C,
                                                         int feature_per_camera, const float *uv, const float *conic,
                                                         const float *opacity, const float *feature,
                                                         const int32_t *idx_sorted, const int32_t *tile_range,
                                                         float bg, float *out, float *final_T, int32_t *ncontrib,
                                                         unsigned char *entry_masks, msplat_stream_t stream);
MSPLAT_API int msplat_batch_alpha_blending_backward_masks(const void *plan, int B, int total_tiles, int64_t rows,
                                                          int C, int feature_per_camera, const float *uv,
                                                          const float *conic, const float *opacity,
                                                          const float *feature, const int32_t *idx_sorted,
                                                          const int32_t *tile_range, float bg, const float *final_T,
                                                          const int32_t *ncontrib, const float *dL_dout,
                                                          float *dL_duv, float *dL_dconic, float *dL_dopacity,
                                                          float *dL_dfeature, const unsigned char *entry_masks,
                                                          msplat_stream_t stream);

/* ------------------------------------------------------------------------ */
/* Density-control statistics after a backward pass.  No kernel counterpart
 * in the reference; accumulates the screen-space gradient that its
 * alpha_blending returns for `ndc` (msplat/alpha_blending.py:107-110).
 * For every Gaussian with radius > 0: grad_accum += |dL_dndc| (2-norm of
 * the [P,2] row), count += 1, max_radius = max(max_radius, radius). */
MSPLAT_API int msplat_density_stats_update(int P, const float *dL_dndc, const int32_t *radius,
                                  float *grad_accum, int32_t *count, int32_t *max_radius,
                                  msplat_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* MSPLAT_GB300_H */
