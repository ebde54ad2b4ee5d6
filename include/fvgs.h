/*
 * fvgs.h -- C-ABI of the GB300 (sm_103a) Gaussian-splatting tracking and
 * mapping library.  Plain pointers and sizes only; every entry point returns
 * an int status (fvgs_status, 0 = FVGS_OK).
 *
 * This boundary replaces the device-side half of the reference's
 * GSSlam / GSCudaKernels path (jcevasco2003/f_vigs_slam).  Each entry point
 * names the reference interface it stands in for.  The reference's own
 * classes (GSSlam, RgbdPoseCostFunction) keep their interfaces: the bodies of
 * their member functions call these entry points.
 *
 * Memory: the library owns every device buffer of a session; caller arrays
 * are borrowed for the duration of a call and may be host (pageable or
 * pinned) or device pointers (CUDA unified addressing decides).
 * Threading: calls on one session are serialised by the caller; different
 * sessions are independent and may be driven from different threads.
 */
#ifndef FVGS_H
#define FVGS_H

#include "fvgs_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct fvgs_session fvgs_session;

/* Debug outputs (fvgs_session_set_debug). */
#define FVGS_DEBUG_PROJECTION 0x1u /* keep Sigma2D / inverse / visibility per Gaussian */
#define FVGS_DEBUG_IMAGES 0x2u     /* tracking kernel writes its forward-blend images */
#define FVGS_DEBUG_MAPPING 0x4u    /* mapping step keeps its 3D deltas */
#define FVGS_DEBUG_RADIX_SORT 0x8u /* bin with the global LSD radix sort instead of per-tile sorting
                                      (an independent implementation of the same order, for checking) */
#define FVGS_DEBUG_NO_CANDIDATES 0x10u /* project every Gaussian at every binning (no candidate list) */

/* Kernel classes for launch accounting and timing. */
enum {
    FVGS_K_PROJECT = 0, /* projection + tile count */
    FVGS_K_SCAN,        /* instance offsets (and mapping bucket offsets) */
    FVGS_K_EMIT,        /* tile-key emission */
    FVGS_K_SORT,        /* radix sort: histogram + digit passes */
    FVGS_K_RANGES,      /* per-tile ranges */
    FVGS_K_TRACK,       /* fused tracking blend + Jacobian */
    FVGS_K_REDUCE,      /* frame reduction of tile partials */
    FVGS_K_GN,          /* on-device Gauss-Newton pose update */
    FVGS_K_MAP_FWD,     /* mapping forward with checkpoints */
    FVGS_K_MAP_BWD,     /* mapping per-Gaussian backward */
    FVGS_K_MAP_UPDATE,  /* 2D->3D chain rule + Adam */
    FVGS_K_RENDER,      /* forward-only render */
    FVGS_K_MAINT,       /* map maintenance: visibility, outlier scores, marking, compaction */
    FVGS_K_COUNT
};

/* Human-readable name of a status code. */
const char* fvgs_status_string(int status);

/* Reference defaults of every tunable (see fvgs_params). */
int fvgs_params_default(fvgs_params* params);

/*
 * Create a session on CUDA device `device` holding up to `capacity_gaussians`
 * Gaussians and frames up to max_width x max_height (pyramid level 0).
 * Stands in for the device state that GSSlam owns
 * (include/f_vigs_slam/GSSlam.cuh:185-235: gaussians_, positions_2d_, ...,
 * hashes_, tile_ranges_).
 */
int fvgs_session_create(const fvgs_params* params, int device, uint32_t capacity_gaussians, int max_width,
                        int max_height, fvgs_session** out);
int fvgs_session_destroy(fvgs_session* s);
/* Run all further work of the session on this cudaStream_t (NULL = the
 * session's own stream). */
int fvgs_session_set_stream(fvgs_session* s, void* cuda_stream);
/* The cudaStream_t the session's work runs on and its CUDA device, for
 * callers that order their own copies or kernels against it. */
int fvgs_session_stream(fvgs_session* s, void** cuda_stream, int* device);
int fvgs_session_sync(fvgs_session* s);
int fvgs_session_set_debug(fvgs_session* s, uint32_t flags);
/* Time the kernel classes in class_mask (bit k = class k) with CUDA events on
 * the session's stream; 0 turns timing off.  Launch counts are always kept. */
int fvgs_session_set_timing(fvgs_session* s, uint32_t class_mask);
/* Per class: accumulated event time (ms), kernels launched, and timed calls
 * (one call = the kernels of one class enqueued together, e.g. a whole radix
 * sort) -- arrays of FVGS_K_COUNT, any may be null; reset != 0 clears them. */
int fvgs_session_get_timing(fvgs_session* s, double* ms, uint64_t* launches, uint64_t* timed_launches, int reset);
/* Bytes of device memory the session holds (admission accounting). */
int fvgs_session_footprint(const fvgs_session* s, uint64_t* bytes);

/*
 * Precision form.  FVGS_PRECISION_REDUCED stores the attributes the binning
 * reads in reduced precision -- scale and rotation in BF16, colour and
 * opacity in FP16, round to nearest even; means stay FP32 -- so a Gaussian
 * in view costs the projection 40 instead of 64 bytes.  Blending and the
 * Hessian accumulation stay FP32 (compensated), the 6x6 solve FP64.  The FP32
 * planes remain the master copy: mapping's Adam update works on them and
 * refreshes the reduced copy of every Gaussian it changes; uploads, removals
 * and seeding refresh it too.  Results are those of the FP32 path on the
 * rounded attributes.  No reference counterpart (the reference stores FP32).
 */
#define FVGS_PRECISION_FP32 0
#define FVGS_PRECISION_REDUCED 1
int fvgs_session_set_precision(fvgs_session* s, int precision);

/*
 * Launch autotuner of the Jacobian kernel (batching form).  The kernel has
 * eight launch variants with the same arithmetic in the same order:
 *   0: four CTAs of 256 threads per SM at 64 registers, batches of 256
 *      Gaussians staged in shared memory;
 *   1: three CTAs per SM at 80 registers;
 *   2: as 0, each batch of records gathered into shared memory by TMA while
 *      the previous batch is blended;
 *   3, 4: as 0 with batches of 128 and 512 Gaussians;
 *   5, 6: each 16 x 16 tile's list run by 2 CTAs of 16 x 8 pixels (5) or 4
 *      CTAs of 8 x 8 pixels (6), batches of 128 Gaussians: more CTAs for the
 *      few hundred tiles of a coarse pyramid level (16 x 16 tiles without
 *      compensated sums only; otherwise they run as 3);
 *   7: two CTAs per SM at 128 registers.
 * With the analytic Jacobian (whose single fused pass holds the colour
 * Jacobian's sums) every variant runs one CTA per SM fewer: 0, 3, 4 at three
 * CTAs and 80 registers, 1 at two CTAs and 128 registers, 7 at two CTAs with
 * batches of 128; 2 runs as 0.
 * Which is faster depends on the map and frame.  On the first frame of a new
 * frame shape of a pyramid level (fvgs_track_frame, fvgs_frame_submit) the
 * session bins the frame at the request's pose, times every variant on that
 * binning and keeps the fastest for that level and shape; results do not
 * depend on the choice.
 * fvgs_session_autotune runs the tuning explicitly (reps timed launches per
 * variant; variant and per-variant median ms (FVGS_TRACK_VARIANTS floats) may
 * be null); fvgs_session_set_autotune(s, 0) keeps variant 0 for untuned
 * shapes; fvgs_session_set_track_variant restores a known choice.  No
 * reference counterpart.
 */
#define FVGS_TRACK_VARIANTS 8
int fvgs_session_autotune(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, int reps,
                          int* variant, float* ms);
int fvgs_session_set_autotune(fvgs_session* s, int enabled);
int fvgs_session_set_track_variant(fvgs_session* s, int level, int variant);

/*
 * Gaussians in the reference's SoA layout (Gaussians,
 * include/f_vigs_slam/RepresentationClasses.hpp:53-99): positions[3n],
 * scales[3n], orientations[4n] as (x,y,z,w), colors[3n], opacities[n].
 */
int fvgs_upload_gaussians(fvgs_session* s, const float* positions, const float* scales,
                          const float* orientations, const float* colors, const float* opacities, uint32_t n);
int fvgs_download_gaussians(fvgs_session* s, float* positions, float* scales, float* orientations,
                            float* colors, float* opacities, uint32_t n);

/* Pyramid levels a session holds frames for (the reference uses three,
 * nb_pyr_levels_ = 3, include/f_vigs_slam/GSSlam.cuh:275). */
#define FVGS_MAX_LEVELS 4

/*
 * Observed frame of pyramid level `level` (0..FVGS_MAX_LEVELS-1): rgb[3P], depth[P],
 * grad_x[3P], grad_y[3P], dense row-major (the pyr_color_ / pyr_depth_ /
 * pyr_dx_ / pyr_dy_ images of GSSlam::initAndCopyImgs, src/GSSlam.cu:1913-1969).
 */
int fvgs_set_frame(fvgs_session* s, int level, const float* rgb, const float* depth, const float* grad_x,
                   const float* grad_y, int width, int height);
/* Observed frames of levels 0..levels-1 from one packed buffer: per level
 * rgb[3P], depth[P], grad_x[3P], grad_y[3P], level l of size
 * ceil(width / 2^l) x ceil(height / 2^l), level 0 first (the layout of
 * fvgs_server_request.pyr_frames).  A buffer in host memory crosses to the
 * device in one copy (into a staging buffer the session keeps), then each
 * level is copied on the device.  No reference counterpart (the reference
 * builds its pyramid from the camera frame; fvgs_preprocess_frame). */
int fvgs_set_frames_packed(fvgs_session* s, const float* frames, int levels, int width, int height);

/*
 * Projection, tile binning, stable depth-key sort and per-tile ranges for
 * `pose` (GSSlam::prepareRasterization, src/GSSlam.cu:408-646).  If
 * n_instances is non-null the call waits for the device and returns the
 * instance count.
 */
int fvgs_project_bin(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                     uint32_t* n_instances);
/* Results of the last fvgs_project_bin in the reference's buffer layout
 * (positions_2d_, covariances_2d_, inv_covariances_2d_, depths_, p_hats_,
 * tile_counts_); cov2d / inv2d / visible need FVGS_DEBUG_PROJECTION.  Any
 * pointer may be null. */
int fvgs_download_projection(fvgs_session* s, float* uv, float* cov2d, float* inv2d, float* depth, float* phat,
                             uint8_t* visible, uint32_t* tile_counts);
/* Sorted keys (hashes_), values (gaussian_indices_) and ranges[2T]
 * (tile_ranges_) of the last binning, T its tile count
 * (fvgs_session_binning_grid).  Any pointer may be null. */
int fvgs_download_binning(fvgs_session* s, uint64_t* keys, uint32_t* values, uint32_t* ranges,
                          uint64_t max_instances, uint32_t* n_instances);
/* How the last binning whose status the host has read (every call that
 * waits for the device reads it) was formed: its instance count, whether it
 * was incremental (1: built from the previous binning of the same tile grid,
 * 0: full), the instances that entered a tile since that binning, and the
 * Gaussians with such instances.  Any pointer may be null.  No reference counterpart: the
 * reference rebuilds every binning from scratch. */
int fvgs_session_binning_info(const fvgs_session* s, uint32_t* n_instances, int* incremental, uint32_t* n_entering,
                              uint32_t* n_changed);
/* Tile shape and tile count of the last binning (a tracking level may bin on
 * 8 x 8 or 32 x 8 tiles: fvgs_session_set_track_tiles).  Any pointer may be
 * null.  No reference counterpart (its tiles are always 16 x 16). */
int fvgs_session_binning_grid(const fvgs_session* s, int* tile_w, int* tile_h, int* num_tiles);
/* The projection's candidate list of the tile grid binned last, after the
 * work enqueued so far (waits for the session's stream): whether one is held,
 * its length, and the pose and view-cone half-angle (radians) it was built
 * at.  Every tile grid (frame size and tile shape; up to four, the least
 * recently binned one replaced) keeps its own list and binning history.  A
 * binning whose pose is within 2 degrees and 5 cm of its grid's list pose,
 * with a view cone no wider, projects only the listed Gaussians; any other
 * binning projects all of them and rebuilds the list; a change to the
 * Gaussians drops every list.  Any pointer may be null.  No reference
 * counterpart: the reference projects every Gaussian at every render. */
int fvgs_session_candidates(fvgs_session* s, int* valid, uint32_t* n, fvgs_pose* pose, float* cone);

/*
 * One RGB-D pose Jacobian evaluation at `pose` against the frame of `level`:
 * binning + fused tracking kernel + frame reduction.  Outputs the 6x6 JtJ
 * (row-major, symmetric) and Jtr[6] exactly as GSSlam::computeRgbdPoseJacobians
 * forms them before its IMU-extrinsic transform (src/GSSlam.cu:2103-2226):
 * camera frame, Jtr negated.  Replaces that function's device part and the
 * kernel getRgbdPoseJacobians (src/GSCudaKernels.cu:922-1392).
 */
int fvgs_track_jacobian(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level,
                        double* JtJ, double* Jtr);
/* Per-tile camera-frame partial sums of the last tracking evaluation:
 * tiles[27T] = Jtr[6] then JtJ upper triangle [21] (PoseOptimizationRgbdData). */
int fvgs_download_tile_partials(fvgs_session* s, float* tiles, int num_tiles);
/* Forward-blend images of the last tracking evaluation (FVGS_DEBUG_IMAGES). */
int fvgs_download_track_images(fvgs_session* s, float* color, float* depth, float* final_T, uint32_t* n_contrib);

/*
 * A whole tracking frame on the device: `iterations` Gauss-Newton steps, each
 * = binning + Jacobian + eigen-regularised pseudo-factor step + pose update
 * (the Ceres loop of GSSlam::optimizeWithCeres over RgbdPoseCostFunction with
 * PoseLocalParameterization, src/GSSlam.cu:2246-2297, as plain Gauss-Newton
 * with identity IMU-camera extrinsics).  pose is read and overwritten.
 * last_step[6] (nullable) receives the final update.
 */
int fvgs_track_frame(fvgs_session* s, fvgs_pose* pose, const fvgs_intrinsics* K, int level, int iterations,
                     double* last_step);
/*
 * A coarse-to-fine tracking frame, the level loop of
 * GSSlam::optimizeWithCeres (src/GSSlam.cu:2267-2297): for level = levels-1
 * down to 0, iterations[level] Gauss-Newton steps against that level's frame,
 * with the level's intrinsics K0 scaled by 2^-level as
 * GSSlam::computeRgbdPoseJacobians scales them (src/GSSlam.cu:2133-2138).
 * K0 are the level-0 intrinsics; levels <= FVGS_MAX_LEVELS.
 */
int fvgs_track_frame_pyramid(fvgs_session* s, fvgs_pose* pose, const fvgs_intrinsics* K0, const int* iterations,
                             int levels, double* last_step);

/*
 * Asynchronous frames, for serving and batching many sessions at once.
 * fvgs_frame_submit enqueues one frame on the session's stream and returns:
 * `iterations` Gauss-Newton steps from `pose` (as fvgs_track_frame), then,
 * when map_eta >= 0, one mapping step at the tracked pose (as fvgs_map_step).
 * A frame of a given shape (levels, iterations, intrinsics, mapping, and
 * whether its first binning continues the session's last one) is captured
 * as a CUDA graph on first use and replayed afterwards.  fvgs_frame_poll reports completion
 * without blocking; fvgs_frame_wait completes the frame (repeating it
 * eagerly if the instance buffers had to grow) and returns the pose and last
 * step (both nullable).  One frame per session may be in flight.  The
 * reference has no counterpart: it tracks one frame at a time on one map.
 */
int fvgs_frame_submit(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, int iterations,
                      float map_eta);
/* The same for a coarse-to-fine frame (as fvgs_track_frame_pyramid); the
 * optional mapping step runs at level 0. */
int fvgs_frame_submit_pyramid(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K0,
                              const int* iterations, int levels, float map_eta);
int fvgs_frame_poll(fvgs_session* s, int* done);
int fvgs_frame_wait(fvgs_session* s, fvgs_pose* pose, double* last_step);
/* Batched frames: submit one frame on each of n sessions (each on its own
 * stream, so their kernels overlap on the device), then wait for all;
 * poses[i] is read and overwritten, levels and map_etas nullable (level 0,
 * no mapping).  Returns the first error. */
int fvgs_frames_run(fvgs_session* const* sessions, fvgs_pose* poses, const fvgs_intrinsics* K, const int* levels,
                    int iterations, const float* map_etas, int n);
/* Batched coarse-to-fine frames: the same level schedule (iterations[levels])
 * on every session, K0[i] the level-0 intrinsics of session i. */
int fvgs_frames_run_pyramid(fvgs_session* const* sessions, fvgs_pose* poses, const fvgs_intrinsics* K0,
                            const int* iterations, int levels, const float* map_etas, int n);
/* Frames of the session that ran from a captured graph / eagerly. */
int fvgs_session_frame_stats(const fvgs_session* s, uint64_t* graphed, uint64_t* eager);

/*
 * Tile shape of one pyramid level's tracking (batching form): 16 x 16 (the
 * reference's TILE_SIZE, src/GSCudaKernels.cu:6, and the default), 8 x 8 or
 * 32 x 8.  That level's binnings and Jacobian kernel use the shape: tile
 * rectangles, tile-centre depth keys (src/GSCudaKernels.cu:617-639 with the
 * tile's own width and height) and tile lists follow it, so a pixel blends
 * its own tile's list -- another shape rasterizes the same map differently,
 * and parity holds against the oracle binned at the same shape.  Mapping,
 * rendering and map maintenance keep 16 x 16.  No reference counterpart.
 */
int fvgs_session_set_track_tiles(fvgs_session* s, int level, int tile_w, int tile_h);

/*
 * Keyframe batching in one persistent launch (batching form).  A batch holds
 * n sessions on one device, all with the same Jacobian mode.
 * fvgs_batch_run_pyramid runs one coarse-to-fine frame (iterations[levels],
 * as fvgs_track_frame_pyramid) on every session in lockstep: each
 * Gauss-Newton iteration bins every session (on the sessions' own streams,
 * concurrently), then ONE persistent launch blends and differentiates the
 * tiles of all sessions -- its CTAs take (session, tile) work items from a
 * shared counter, so uneven maps and frame sizes balance across the SMs --
 * and one launch reduces every session's tiles and applies its pose step.
 * The whole frame is captured once as one CUDA graph and replayed while the
 * sessions' binning state allows.  poses[i] is read and overwritten.  A
 * session whose instance buffers overflow is repeated alone on the plain
 * path after they grow.
 * Each level's tile shape and staging batch (128, 256 or 512 Gaussians per
 * shared-memory batch) belong to the batch and are pushed to its sessions
 * (fvgs_session_set_track_tiles and the launch variant), so a session's plain
 * frames give the batched result bit for bit.  fvgs_batch_set_level sets
 * them; fvgs_batch_autotune times the persistent launch for every shape x
 * batch (9 combinations) on every level the schedule uses, at the given
 * poses (reps launches each), and keeps the fastest per level; config_out
 * (nullable, 3 ints per level: tile_w, tile_h, batch) and ms_out (nullable,
 * 9 floats per level: shapes 16x16, 8x8, 32x8, each with batches 128, 256,
 * 512) report the outcome.  fvgs_batch_stats: frames replayed / enqueued
 * eagerly, batched kernel launches.  The reference tracks one frame of one
 * map per launch; no counterpart.
 */
typedef struct fvgs_batch fvgs_batch;
int fvgs_batch_create(fvgs_session* const* sessions, int n, fvgs_batch** out);
int fvgs_batch_destroy(fvgs_batch* b);
int fvgs_batch_set_level(fvgs_batch* b, int level, int tile_w, int tile_h, int batch_gaussians);
int fvgs_batch_autotune(fvgs_batch* b, const fvgs_pose* poses, const fvgs_intrinsics* K0, const int* iterations,
                        int levels, int reps, int* config_out, float* ms_out);
int fvgs_batch_run_pyramid(fvgs_batch* b, fvgs_pose* poses, const fvgs_intrinsics* K0, const int* iterations,
                           int levels);
int fvgs_batch_stats(const fvgs_batch* b, uint64_t* graphed, uint64_t* eager, uint64_t* batch_launches);

/*
 * The viewer's image: binning + the render-form forward pass
 * (GSSlam::rasterize / renderView, src/GSSlam.cu:648-799, kernel
 * forwardPassTileKernel, src/GSCudaKernels.cu:710-859), with its own
 * semantics: Sigma2D inverted in its true layout, every Gaussian of a tile
 * list blended without the tracking kernels' 0.99 / 1/255 thresholds, stop at
 * accumulated alpha >= 0.99, median depth at the 0.5 crossing (1e10 where
 * none), no background.  rgb[3P] float (the reference writes it into an 8-bit
 * image, overrunning it), depth[P]; rgb8[3P] (nullable) = round(255 c)
 * saturated.  Outputs may be host or device pointers; any may be null.
 */
int fvgs_render_view(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                     float* rgb, float* depth, uint8_t* rgb8);

/*
 * Frame preprocessing on the device (GSSlam::initAndCopyImgs,
 * src/GSSlam.cu:1913-1969, done on the host in the reference): from one camera
 * frame -- colour 8-bit, 3 channels, dense (channel order kept as given);
 * depth float metres, or uint16 millimetres when depth_u16_mm -- build pyramid
 * levels 0..levels-1 by pyrDown (5-tap binomial, reflect-101 borders; 8-bit
 * colour in integers, depth in float) and set each level's observed colour
 * (c / 255, and / 255 once more when double_scale, as computeRgbdPoseJacobians
 * scales it again, src/GSSlam.cu:2158), depth and 3x3 Sobel gradients of the
 * c / 255 colour, as fvgs_set_frame would.  Inputs may be host or device
 * pointers.
 */
int fvgs_preprocess_frame(fvgs_session* s, const uint8_t* color, const void* depth, int depth_u16_mm, int width,
                          int height, int levels, int double_scale);
/* A level's current frame (rgb[3P], depth[P], grad_x[3P], grad_y[3P], any
 * nullable) and its size. */
int fvgs_download_frame(fvgs_session* s, int level, float* rgb, float* depth, float* grad_x, float* grad_y,
                        int* width, int* height);

/*
 * Forward blend with the tracking kernel's semantics for every pixel of a
 * width x height view (observed depth treated as valid everywhere): colour
 * incl. background, median depth, final transmittance, contributor count.
 * Outputs may be host or device pointers; any may be null.
 */
int fvgs_render(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                float* rgb, float* depth, float* final_T, uint32_t* n_contrib);

/*
 * One mapping step against the frame of `level` seen from `pose`: binning,
 * forward blend with checkpoints, per-Gaussian backward to the 2D parameters,
 * 2D->3D chain rule and an Adam update of every Gaussian parameter
 * (GSSlam::optimizeGaussiansKeyframe, src/GSSlam.cu:1083-1320, and its
 * kernels src/GSCudaKernels.cu:2074-2882; eta as eta_gaussian_).  Adam state
 * lives in the session and starts at zero on upload.
 */
int fvgs_map_step(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, float eta);
/* Results of the last mapping step: forward images (final T, n_contrib,
 * colour incl. background, median depth) and per-Gaussian deltas with a
 * 16-float stride -- delta2d = DeltaGaussian2D fields (meanImg.xy,
 * invSigmaImg.xyz, color.xyz, depth, alpha, pHat.xy, n as uint32), delta3d =
 * DeltaGaussian3D fields (position, scale, orientation, color, alpha, n as
 * float; needs FVGS_DEBUG_MAPPING).  Any pointer may be null. */
int fvgs_download_map_state(fvgs_session* s, float* final_T, uint32_t* n_contrib, float* color, float* depth,
                            float* delta2d, float* delta3d);
/* Optimiser state of the first n Gaussians: nine planes of n float4 (plane p
 * at state + 4 n p): m and v of position, scale, orientation, colour, then
 * (m_alpha, v_alpha, step count, unused). */
int fvgs_download_adam_state(fvgs_session* s, float* state, uint32_t n);

/*
 * Map maintenance.  Removal keeps the survivors in their order at the front
 * and shrinks the session's Gaussian count, as the reference's
 * thrust::sort_by_key on the 0 / 0xff states followed by
 * n_Gaussians -= nb_removed (src/GSSlam.cu:1536-1569, 1668-1701); with
 * FVGS_Q_ADAM_STAY the optimiser state stays at its index.  Removing
 * Gaussians renumbers them, so the next binning is a full one.
 *
 * fvgs_remove_outliers: GSSlam::removeOutliers (src/GSSlam.cu:1581-1711) --
 * bin the view of `level` at `pose`, accumulate per Gaussian the alpha of
 * every (pixel, Gaussian) pair of its tiles with alpha >= 1/255 and rendered
 * depth > 0 (total_alpha) and the part of it where the observed depth is
 * > 0.1 and the rendered depth < 0.8 x observed (outlier_prob), and mark the
 * Gaussians with total_alpha > 1 and outlier_prob / total_alpha > threshold
 * (0.6 in the reference); computeOutliers_kernel / removeOutliers_kernel,
 * src/GSCudaKernels.cu:1620-1739.  remove = 0 only marks (fvgs_download_marks
 * reads the states and scores); *n_marked = number marked (= removed).
 */
int fvgs_remove_outliers(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level,
                         float threshold, int remove, uint32_t* n_marked);
/*
 * GSSlam::prune (src/GSSlam.cu:1467-1579), pruneGaussians_kernel
 * (src/GSCudaKernels.cu:1566-1618): mark Gaussians with opacity <
 * alpha_threshold, or whose middle scale / largest scale < scale_ratio_threshold
 * or largest scale < min_scale (0.05, 0.05, 0.005 in the reference).
 */
int fvgs_prune(fvgs_session* s, float alpha_threshold, float scale_ratio_threshold, float min_scale, int remove,
               uint32_t* n_marked);
/* States (0 keep, 0xff remove) of the last marking, and the outlier scores of
 * the last fvgs_remove_outliers, for its first n Gaussians (numbered as
 * before any removal).  Any pointer may be null. */
int fvgs_download_marks(fvgs_session* s, uint8_t* states, float* total_alpha, float* outlier_prob, uint32_t n);
/*
 * computeGaussiansVisibility_kernel (src/GSCudaKernels.cu:1455-1537) on the
 * view (pose, K, width x height): visibility[i] = 1 where some pixel blends
 * Gaussian i with alpha = min(0.99, opacity exp(-q/2)) >= 1/255 before its
 * transmittance falls below 0.5 (the first 256 Gaussians of each tile with
 * FVGS_Q_VIS_CAP256).  visibility (n bytes, host or device) may be null;
 * *n_visible = number of visible Gaussians.
 */
int fvgs_visibility(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                    uint8_t* visibility, uint32_t* n_visible);
/*
 * GSSlam::computeCovisibilityRatio (src/GSSlam.cu:1713-1904): visibility of
 * view a (the keyframe) and view b (the current frame), then
 * ratio = |a and b| / |a or b| (computeGaussiansCovisibility_kernel,
 * src/GSCudaKernels.cu:1539-1560); 1 for an empty map, 0 when a view has no
 * instances or the union is empty.
 */
int fvgs_covisibility(fvgs_session* s, const fvgs_pose* pose_a, const fvgs_intrinsics* K_a, int width_a,
                      int height_a, const fvgs_pose* pose_b, const fvgs_intrinsics* K_b, int width_b, int height_b,
                      uint32_t* n_inter, uint32_t* n_union, float* ratio);

/*
 * Seeding from the camera frame last given to fvgs_preprocess_frame (its
 * 8-bit colour, 3 bytes per pixel in the reference's (b, g, r) order, and its
 * depth in metres; FVGS_E_STATE if fvgs_set_frame has replaced level 0 since).
 * The pose's orientation is read as (w, x, y, z) and the seeds' orientations
 * are written in that order, as the reference's seeding kernels do (the
 * projection reads the same float4 as (x, y, z, w)).  The reference reserves
 * seed slots with an atomic counter, in no defined order; here seeds are
 * numbered in row-major order of their sample cell, and seeds beyond the
 * session's capacity are dropped.
 *
 * fvgs_init_gaussians: GSSlam::initializeGaussiansFromRgbd
 * (src/GSSlam.cu:271-407), computeNormalsFromDepth_kernel +
 * initGaussiansFromRgbd_kernel (src/GSCudaKernels.cu:87-315).  Replaces the
 * map: one Gaussian per sample pixel (every sample_px-th pixel in x and y)
 * with depth > 0 -- back-projected position, scale init_scale, orientation
 * turning +z onto the depth-map normal, colour / 255, opacity init_opacity
 * (reference defaults 10, 2.0, 0.8) -- and zeroes the optimiser state.
 *
 * fvgs_densify: GSSlam::densify (src/GSSlam.cu:1351-1465),
 * computeDensityMask_kernel + densifyGaussians_kernel
 * (src/GSCudaKernels.cu:1741-2066).  Bins the frame's view at `pose`, builds
 * the density mask (transmittance where the map leaves more than half the
 * light, 1 where the map's median depth lies more than 20% behind the
 * observed depth), and appends one Gaussian per sample cell of which at
 * least half the pixels are marked (sample_px = 1: per marked pixel).
 * mask (W x H floats, host or device) may be null; *n_added = Gaussians
 * appended.  With FVGS_Q_ADAM_STAY the new Gaussians keep the optimiser state
 * found at their slots (the reference's adam_states_ is never shrunk);
 * otherwise it is zeroed.
 */
int fvgs_init_gaussians(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int sample_px,
                        float init_scale, float init_opacity, uint32_t* n_gaussians);
int fvgs_densify(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int sample_px, float* mask,
                 uint32_t* n_added);

/*
 * Allocation-free pose Jacobian for callers that cannot call cudaMalloc -- a
 * tracking thread inside a host application whose own allocator owns the GPU
 * memory budget, or a real-time loop that must not pay cudaMalloc/cudaFree's
 * implicit synchronisation.  No counterpart in the reference: it is an
 * additional entry point of this library.
 *
 * Same result as fvgs_track_jacobian for an already-binned frame, with every
 * input a caller-owned device buffer in the reference's layout: ranges[2T]
 * (tile_ranges_), indices (sorted gaussian_indices_), positions_2d[2N],
 * depths[N], inv_covariances_2d[3N] stored (xx, yy, xy), p_hats[2N],
 * colors[3N], opacities[N], and the frame's grad_x / grad_y / observed_rgb
 * [3P] and observed_depth [P].  n_gaussians and n_instances are the lengths
 * of the per-Gaussian buffers and of indices: list entries past them are
 * skipped, as for the library's own buffers (0: not checked).  params may be
 * null (defaults); the Jacobian is the reference's approximate one whatever
 * its quirk bits (the screen-space buffers carry no camera-frame geometry for
 * the analytic one).  JtJ[36] and Jtr[6] may be host or device pointers; the
 * call returns after the stream (a cudaStream_t, NULL = legacy default
 * stream) has finished the work, so it cannot be called while that stream is
 * being captured into a CUDA graph.
 *
 * Its scratch is one static device array for at most FVGS_NOALLOC_MAX_TILES
 * 16x16 tiles (about 1.8 MB, held by every GPU that loads the library until
 * exit); larger frames return FVGS_E_CAPACITY.  The first call on a device
 * resolves that array's address in the device's primary context (the only
 * context supported).  Calls share the array: calls that overlap on the GPU
 * race.
 */
#define FVGS_NOALLOC_MAX_TILES 16384
int fvgs_rgbd_pose_jacobians_noalloc(const uint32_t* ranges, const uint32_t* indices, const float* positions_2d,
                                     const float* depths, const float* inv_covariances_2d, const float* p_hats,
                                     const float* colors, const float* opacities, const float* grad_x,
                                     const float* grad_y, const float* observed_rgb, const float* observed_depth,
                                     const fvgs_pose* pose, const fvgs_intrinsics* K, const fvgs_params* params,
                                     int width, int height, uint32_t n_gaussians, uint32_t n_instances, double* JtJ,
                                     double* Jtr, void* cuda_stream);

#ifdef __cplusplus
}
#endif
#endif /* FVGS_H */
