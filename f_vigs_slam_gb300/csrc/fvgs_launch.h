// fvgs_launch.h -- host-side launchers of the fvgs kernels (internal to the
// library; the public boundary is include/fvgs.h).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "../../include/fvgs_types.h"

namespace fvgs {

struct DevStatus;
struct DevPose;

#ifdef __CUDACC__
// Launch with programmatic stream serialisation (see pdl_begin): the kernel
// may be scheduled while its predecessor in the stream drains.
template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                           Args&&... args) {
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
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}
#endif

// Binning record of one Gaussian, 32 bytes so that one gather touches one
// sector: r = (x0 | y0 << 16, x1 | y1 << 16 (inclusive tile rectangle),
// instance count (0: none), phat.y bits), p = (u, v, z, phat.x).
struct __align__(32) BinRec {
    uint4 r;
    float4 p;
};

// The Gaussians a projection may find in view while the pose stays near the
// one they were culled at (the projection's candidate list, see
// project_count_kernel).  All zero = no list.
struct CandState {
    uint32_t valid;    // the list in cand[] holds n entries for pose (t, q) and cone
    uint32_t n;
    uint32_t n_build;  // entries appended by the building launch (0 between launches)
    uint32_t done;     // CTAs of the building launch that have finished (0 between launches)
    float t[3];
    float q[4];
    float cone;        // the view cone's half-angle (radians) the list was built for
};
// Pose change within which a candidate list stays complete, and the
// distance within which every Gaussian is a candidate.
constexpr float kCandMaxAngle = 0.0349066f;  // 2 degrees
constexpr float kCandMaxShift = 0.05f;       // metres
constexpr float kCandNear = 0.1f;            // metres

struct ProjectArgs {
    const float4* pos;
    const float4* scale;
    const float4* rot;
    const float4* col;
    // precision form: scale/rotation and colour/opacity from the reduced
    // planes instead of scale, rot, col (null: the FP32 planes)
    const uint4* attr_sr;
    const uint2* attr_c;
    int n;
    const DevPose* pose;
    fvgs_intrinsics K;
    int W, H, tw, th, ntx, nty;
    // 1/tw and 1/th when the tile sides are powers of two (x / 2^k == x * 2^-k
    // exactly in IEEE arithmetic), else 0 (divide)
    float inv_tw, inv_th;
    float radius_sigma;
    uint32_t quirks;
    float4* rec0;
    float4* rec1;
    float4* rec2;
    BinRec* bins;
    uint32_t* counts;
    int* tile_diff;    // optional: binning scratch (tile_diff_words): count grid, entering grid, counters
    // incremental binning (hist != 0): bins and counts still hold the previous
    // binning; the instances new to a tile go to the entering grid and the
    // Gaussians that have some to changed[] as (index, previous rectangle r.x,
    // r.y, previous count), at most changed_cap listed
    int hist;
    uint4* changed;
    uint32_t changed_cap;
    float* dbg_cov;    // optional: 3N Sigma2D (xx, yy, xy)
    float* dbg_inv;    // optional: 3N inverse, stored order (xx, yy, xy)
    uint8_t* dbg_vis;  // optional: N visibility
    // optional (analytic pose Jacobian): geometry record of every Gaussian
    // with instances, geo0 = (Sxx, Sxy, Sxz, Syy), geo1 = (Syz, Szz, x, y) --
    // the camera-frame 3D covariance and mean (z is rec0.z)
    float4* geo0;
    float4* geo1;
    // optional candidate list (capacity n) and its state; cone: the current
    // view's largest angle from the optical axis (its farthest image corner),
    // radians -- a list built for a cone at least as wide is reused
    uint32_t* cand;
    CandState* cst;
    float cone;
};

struct EmitArgs {
    const BinRec* bins;
    const uint32_t* offsets;
    int n;
    int ntx, tw, th;
    uint64_t capacity;
    uint64_t* keys;
    uint32_t* vals;
    // incremental mode (tile-bucket path): entering instances of the listed
    // Gaussians go to enter_keys at the enter_fill cursors
    const uint4* changed;  // DevStatus::n_changed entries
    uint64_t* enter_keys;
    uint32_t* enter_fill;
    uint32_t enter_cap;
};

// Copy a binning's ranges[T] and the sorted indices they cover into another
// buffer pair (same positions).
cudaError_t launch_copy_lists(const uint2* ranges, int T, const uint32_t* src, uint32_t* dst, uint2* ranges_dst,
                              uint64_t capacity, int max_ctas, cudaStream_t s);
// max_ctas caps the grid (the kernel strides over the Gaussians); <= 0: one thread per Gaussian.
cudaError_t launch_project_count(const ProjectArgs& a, int max_ctas, cudaStream_t s);
size_t scan_partials_size(int n);
cudaError_t launch_scan(const uint32_t* counts, int n, uint32_t* partials, uint32_t* offsets, DevStatus* st,
                        uint32_t capacity, cudaStream_t s);
cudaError_t launch_emit_keys(const EmitArgs& a, cudaStream_t s);
cudaError_t launch_ranges(const uint64_t* keys, const DevStatus* st, int num_tiles, uint32_t quirks,
                          uint2* ranges, int grid, cudaStream_t s);
// Tile-bucket binning: counts from the projection's difference grid, then
// ranges / cursors, then scatter of composite keys (depth bits << 32 | index).
// The binning scratch holds two (ntx+1) x (nty+1) difference grids (all
// instances, entering instances) and 8 counter words; one memset clears it.
size_t diff_grid_cells(int ntx, int nty);
size_t tile_diff_words(int ntx, int nty);
constexpr int kCounterWords = 8;  // [0] entering instances, [1] listed Gaussians
// hist: a previous binning on the same tile grid is valid; the kernel then
// also scans the entering grid and picks incremental mode when the entering
// instances fit enter_cap (DevStatus::mode).
// It also leaves the binning scratch zeroed for the next binning, and zeroes
// the scatter chunk counter and the sort's list counters (seg_ctrl[0..2]).
cudaError_t launch_tile_offsets(int* scratch, int ntx, int nty, bool hist, uint32_t enter_cap, uint2* ranges,
                                uint32_t* fill, uint2* enter_ranges, uint32_t* enter_fill, DevStatus* st,
                                uint32_t capacity, uint32_t* seg_ctrl, cudaStream_t s);
cudaError_t launch_emit_scatter(const EmitArgs& a, uint32_t* fill, uint32_t* chunk_counter, int grid,
                                const DevStatus* st, cudaStream_t s);
// Per-tile sort of the composite keys (segsort.cu): writes the sorted Gaussian
// indices to vals.  Tiles above 4096 instances go through a global merge sort
// that uses tmp (capacity u64) as scratch.
struct SegSortWork {
    uint32_t* large_list;  // [T] tiles too large for one CTA
    uint32_t* large_ctrl;  // [2]: count, next
};
// Incremental mode inputs: the previous binning's ranges and sorted indices,
// the entering instances per tile, and the current binning records.
struct SegSortIncr {
    const uint2* ranges_prev;
    const uint32_t* vals_prev;
    const uint2* enter_ranges;
    const uint64_t* enter_keys;
    const BinRec* bins;
    int ntx, tw, th;
    uint32_t n_gauss;    // indices at or above are rejected
    uint64_t capacity;   // instance buffer size: previous ranges are clamped to it
};
cudaError_t launch_segsort(uint64_t* comp, uint64_t* tmp, const uint2* ranges, int num_tiles, uint32_t* vals,
                           SegSortWork w, const DevStatus* st, int large_grid, const SegSortIncr& inc,
                           cudaStream_t s);
// Reference-format keys (tile << 32 | depth bits) of a tile-bucket binning,
// rebuilt from its ranges, sorted indices and binning records with the
// emission's arithmetic (the tracking path itself never reads them).
cudaError_t launch_make_keys(const BinRec* bins, const uint2* ranges, const uint32_t* vals, uint32_t n_gauss,
                             int num_tiles, int ntx, int tw, int th, const DevStatus* st, uint64_t* keys,
                             cudaStream_t s);

// ---- radix sort (sort.cu) ----
struct SortWorkspace {
    uint64_t* keys_alt;
    uint32_t* vals_alt;
    uint64_t* lookback;   // [max_tiles][256] 64-bit status words
    uint32_t* ctrl;       // [8 passes][256] histograms + [8] tile counters
    uint64_t max_items;
    uint32_t epoch;       // advanced per sort call; tags lookback words
    int persistent_ctas;  // resident CTAs of the onesweep kernel
    int num_sms;
};
size_t sort_lookback_words(uint64_t max_items);
size_t sort_ctrl_words();
int sort_num_passes(int key_bits);
cudaError_t sort_init(SortWorkspace* ws, int device);
// Stable LSD radix sort of (keys, vals) over key bits [0, key_bits); the item
// count is read from st->n_instances_clamped.  The result lands back in
// keys/vals (an even number of passes is always run; passes <= 8 so key_bits
// <= 64, and key_bits <= 56 whenever the padding pass is needed).
cudaError_t launch_radix_sort(uint64_t* keys, uint32_t* vals, const DevStatus* st, int key_bits,
                              SortWorkspace* ws, uint32_t* err_flags, cudaStream_t s);

// ---- tracking (track.cu) ----
struct TrackArgs {
    const float4* rec0;
    const float4* rec1;
    const float4* rec2;
    const uint2* ranges;
    const uint32_t* indices;
    // list entries at or beyond n_list and indices at or above n_gauss are
    // skipped (defensive: the binning never produces them)
    uint32_t n_list;
    uint32_t n_gauss;
    const float* obs_rgb;    // 3P
    const float* obs_depth;  // P
    const float* gx;         // 3P
    const float* gy;         // 3P
    const DevPose* pose;
    fvgs_intrinsics K;
    int W, H, ntx, nty;
    float bg[3];
    float alpha_thresh, color_thresh, depth_thresh;
    float* tile_out;  // [T][27] camera-frame partials
    // optional per-pixel outputs of the forward blend
    float* img_color;    // 3P
    float* img_depth;    // P
    float* img_T;        // P
    uint32_t* img_nc;    // P
    int render_only;     // 1: forward blend for every in-bounds pixel, no Jacobian
    // reference buffer layout (launch_track_ref_layout only): float2 uv,
    // float depth, float3 inverse covariance (stored xx, yy, xy), float2 p_hat,
    // float3 colour, float opacity per Gaussian
    const float* ref_uv;
    const float* ref_depth;
    const float* ref_inv;
    const float* ref_phat;
    const float* ref_col;
    const float* ref_opa;
    uint32_t quirks;
    // launch variant of the Jacobian kernel (the autotuner's choice): 0 = four
    // CTAs per SM (64 registers), 1 = three CTAs per SM (80 registers), 2 =
    // four CTAs per SM with the record batches gathered by TMA (needs the
    // record tensor maps); the arithmetic and its order are the same in all
    int variant;
    uint32_t* st_flags;  // status word for bounded-wait timeouts (variant 2)
    // analytic pose Jacobian (FVGS_Q_POSE_JAC_APPROX clear): the geometry
    // records written by the projection (ProjectArgs::geo0 / geo1)
    const float4* geo0;
    const float4* geo1;
    // tile shape of the binning the lists come from: 16 x 16 (also 0 x 0),
    // 8 x 8 or 32 x 8 (the TMA-staged variant only for 16 x 16)
    int tile_w, tile_h;
    // precision form: compensated accumulation of the per-pixel colour
    // Jacobian and of the in-tile sums (analytic Jacobian, 16 x 16 tiles)
    int compensated;
    // CTAs per list tile (0 or 1: one; 2: 16 x 8 pixel halves; 4: 8 x 8
    // quarters of a 16 x 16 list tile).  CTA c of list tile c / split writes
    // partial row c of tile_out; the frame reduction adds a tile's rows in
    // the fixed order of a whole tile's in-CTA sum, so the sums are the same
    // bits for every split.
    int split;
};
constexpr int kTrackVariants = 8;
// Whether the tracking kernel runs tiles of this shape.
inline bool track_tile_supported(int tw, int th) {
    return (tw == 16 && th == 16) || (tw == 8 && th == 8) || (tw == 32 && th == 8);
}
// Gaussians staged per shared-memory batch by a launch variant: 3, 5, 6 ->
// 128, 4 -> 512, otherwise 256.
inline int track_variant_batch(int variant) {
    return (variant == 3 || variant == 5 || variant == 6) ? 128 : (variant == 4 ? 512 : 256);
}
// CTAs per 16 x 16 list tile of a launch variant: 5 -> 2 (16 x 8 pixel
// halves), 6 -> 4 (8 x 8 quarters), otherwise 1.  More, smaller CTAs fill
// the SMs at the coarse pyramid levels, where a frame has a few hundred
// tiles with long lists; every CTA stages its tile's whole list.
inline int track_variant_split(int variant) { return variant == 5 ? 2 : (variant == 6 ? 4 : 1); }
// Set the dynamic shared-memory limits of the tracking kernels on the current
// device (their batches can exceed the 48 KB default); once per device,
// before any launch or capture.
cudaError_t track_configure_device();
// Tensor maps of the three record planes (2-D: 4 floats x capacity rows,
// 16-byte rows, one-row boxes) for the TMA-staged variant.
struct RecMaps {
    CUtensorMap rec[3];
};
cudaError_t launch_track(const TrackArgs& a, const RecMaps* maps, cudaStream_t s);
// The tracking kernel reading the reference's separate screen-space buffers
// instead of the packed record planes.
cudaError_t launch_track_ref_layout(const TrackArgs& a, cudaStream_t s);
// Sum tile partials in FP64, rotate to the world frame, write out[42] =
// JtJ[36] (symmetric) then Jtr[6] (negated, as the reference host code does).
// split: partial rows per tile (TrackArgs::split).
cudaError_t launch_track_reduce(const float* tile_out, int num_tiles, int split, DevPose* pose, double* out,
                                cudaStream_t s);
// The same reduction followed by one eigen-regularised Gauss-Newton update of
// the device pose (step_out[6] nullable).
cudaError_t launch_track_reduce_gn(const float* tile_out, int num_tiles, int split, DevPose* pose, double* out,
                                   double eig_eps, double* step_out, cudaStream_t s);
// One session's frame reduction + Gauss-Newton step in a batched launch.
struct ReduceJob {
    const float* tile_out;
    int num_tiles;
    int split;
    DevPose* pose;
    double* out;
    double eig_eps;
    double* step_out;
};
// launch_track_reduce_gn for n_jobs sessions at once (device array of jobs).
cudaError_t launch_track_reduce_batch(const ReduceJob* jobs, int n_jobs, cudaStream_t s);
// One session's tracking launch in a persistent batched launch: its
// arguments and the first work item (tile) of its range.
struct TrackJob {
    TrackArgs a;
};
// The tiles of n_jobs sessions in one persistent launch: work item i is tile
// i - begin[j] of job j for begin[j] <= i < begin[j + 1] (begin: n_jobs + 1
// device words).  Every job must use tile shape (tile_w, tile_h), the same
// Jacobian mode (analytic) and staging batch (variant).  counters: two
// device words, zero before the first launch; every launch leaves them zero.
cudaError_t launch_track_batch(const TrackJob* jobs, const uint32_t* begin, int n_jobs, uint32_t total_tiles,
                               int tile_w, int tile_h, bool analytic, int variant, uint32_t* counters, int num_sms,
                               cudaStream_t s);
// Kernel attributes of the persistent kernels on the current device.
cudaError_t track_batch_configure_device();

// ---- render form (render.cu) ----
struct RenderArgs {
    const float4* rec0;
    const float4* rec1;
    const float4* rec2;
    const uint2* ranges;
    const uint32_t* indices;
    uint32_t n_list, n_gauss;  // as TrackArgs
    int W, H, ntx, nty;
    uint32_t quirks;
    float* out_rgb;      // 3P
    float* out_depth;    // P
    uint8_t* out_rgb8;   // optional 3P
};
cudaError_t launch_render_view(const RenderArgs& a, cudaStream_t s);

// ---- frame preprocessing (preprocess.cu) ----
// Level 0 of a W x H camera frame: depth in metres (float, or uint16 mm), the
// colour (/255, twice with double_scale) and its Sobel derivatives.
cudaError_t launch_prep_level0(const uint8_t* img, const void* raw_depth, int u16_mm, int W, int H, int double_scale,
                               float* rgb, float* gx, float* gy, float* depth, cudaStream_t s);
// The next level from a Wp x Hp level: its 8-bit colour and depth by pyrDown,
// then the same colour, Sobel and depth outputs.
cudaError_t launch_prep_level(const uint8_t* prev, const float* prev_depth, int Wp, int Hp, int double_scale,
                              uint8_t* cur, float* rgb, float* gx, float* gy, float* depth, cudaStream_t s);

// ---- mapping (map.cu) ----
struct MapArgs {
    const float4* rec0;
    const float4* rec1;
    const float4* rec2;
    const uint2* ranges;
    const uint32_t* indices;
    uint32_t n_list;   // as TrackArgs
    uint32_t n_gauss;
    const float* obs_rgb;    // 3P
    const float* obs_depth;  // P
    int W, H, ntx, nty;
    float bg[3];
    const uint32_t* bucket_base;  // [T] exclusive bucket offsets (null with MAP_CAP256)
    float4* sampled;              // [buckets][256] (T, accumulated colour)
    float* final_T;               // P
    uint32_t* n_contrib;          // P
    float* color;                 // 3P, incl. background
    float* depth;                 // P
    float* color_err;             // 3P
    uint32_t* max_contrib;        // T
    float* delta2d;               // [N][16]: DeltaGaussian2D fields, n as u32 at 12
    float w_depth, w_dist;
};
struct MapUpdateArgs {
    float4* pos;
    float4* scale;
    float4* rot;
    float4* col;
    float4* adam;  // 9 planes of cap float4
    uint32_t cap;
    int n;
    const float* delta2d;
    const DevPose* pose;
    fvgs_intrinsics K;
    float lambda_iso, eta, beta1, beta2, eps;
    float* dbg_delta3d;  // optional [N][16]
    uint4* attr_sr;      // optional: refresh the reduced-precision planes of updated Gaussians
    uint2* attr_c;
    CandState* cst;      // optional: n_cst candidate-list states, all stale once positions move
    int n_cst;
};
cudaError_t launch_map_forward(const MapArgs& a, bool cap, cudaStream_t s);
cudaError_t launch_map_backward(const MapArgs& a, bool cap, cudaStream_t s);
cudaError_t launch_bucket_scan(const uint2* ranges, int T, uint32_t* bucket_base, uint32_t* total, cudaStream_t s);
cudaError_t launch_map_update(const MapUpdateArgs& a, const DevStatus* st, cudaStream_t s);
int map_cap_buckets();
// Reduced-precision planes from the FP32 master planes (precision form).
cudaError_t launch_pack_reduced(const float4* scale, const float4* rot, const float4* col, uint32_t n, uint4* sr,
                                uint2* c, cudaStream_t s);

// ---- map maintenance (maintenance.cu) ----
struct VisArgs {
    const float4* rec0;
    const float4* rec1;
    const uint2* ranges;
    const uint32_t* indices;
    uint32_t n_list, n_gauss;  // as TrackArgs
    int W, H, ntx, nty;
    int cap;       // Gaussians considered per tile (0: all)
    uint8_t* vis;  // [n_gauss], set to 1 where visible (cleared by the caller)
};
struct OutlierArgs {
    const float4* rec0;
    const float4* rec1;
    const float4* rec2;
    const uint2* ranges;
    const uint32_t* indices;
    uint32_t n_list, n_gauss;
    const float* obs_depth;  // P
    int W, H, ntx, nty;
    float* total_alpha;   // [n_gauss], zeroed by the caller
    float* outlier_prob;  // [n_gauss], zeroed by the caller
};
enum MarkMode { kMarkPrune = 0, kMarkOutliers = 1 };
struct MarkArgs {
    uint32_t n;
    const float4* scale;  // prune: scales and (col.w) opacities
    const float4* col;
    float alpha_thr, ratio_thr, min_scale;
    const float* total_alpha;  // outliers: accumulators and threshold
    const float* outlier_prob;
    float threshold;
    uint8_t* states;      // [n]: 0 keep, 0xff remove
    uint32_t* block_keep;  // [ceil(n / kCompactBlock)]
};
constexpr int kCompactBlock = 256;
struct CompactArgs {
    uint32_t n;
    const uint8_t* states;
    const uint32_t* block_base;  // exclusive survivors before each block
    const uint32_t* counters;    // [0] survivors, [1] removed
    const float4 *pos, *scale, *rot, *col;
    float4 *pos_out, *scale_out, *rot_out, *col_out;
    const float4* adam;  // 9 planes of cap (null: the optimiser state stays in place)
    float4* adam_out;
    uint32_t cap;
};
cudaError_t launch_visibility(const VisArgs& a, cudaStream_t s);
cudaError_t launch_outliers(const OutlierArgs& a, cudaStream_t s);
cudaError_t launch_mark(MarkMode mode, const MarkArgs& a, cudaStream_t s);
cudaError_t launch_compact_scan(const uint32_t* block_keep, uint32_t n, uint32_t* block_base, uint32_t* counters,
                                cudaStream_t s);
cudaError_t launch_compact_scatter(const CompactArgs& a, cudaStream_t s);
cudaError_t launch_covis_count(const uint8_t* va, const uint8_t* vb, uint32_t n, uint32_t* counters, cudaStream_t s);

// ---- seeding from an RGB-D frame (seed.cu) ----
enum SeedMode { kSeedInit = 0, kSeedDensify = 1 };
struct SeedArgs {
    const uint8_t* bgr;   // W x H x 3 bytes, (b, g, r)
    const float* depth;   // W x H, metres
    const float* mask;    // densify: W x H density mask
    int W, H;
    int sample;           // sample cell edge in pixels
    int ncx, ncy;         // sample cells
    fvgs_intrinsics K;
    float4 pose_q;        // raw, read as (w, x, y, z)
    float3 pose_t;
    float init_scale, init_opacity;
    uint32_t n0, cap;     // first slot written; slots >= cap are dropped
    uint32_t* block_keep;        // count: seeds per block of cells
    const uint32_t* block_base;  // emit: seeds before each block
    float4 *pos, *scale, *rot, *col;
    float4* adam;  // emit: zero the optimiser state of each seed (null: leave it)
};
struct DensityArgs {
    const float4* rec0;
    const float4* rec1;
    const float4* rec2;
    const uint2* ranges;
    const uint32_t* indices;
    uint32_t n_list, n_gauss;
    const float* obs_depth;  // P
    int W, H, ntx, nty;
    float* mask;  // P
};
cudaError_t launch_seed_count(SeedMode mode, const SeedArgs& a, cudaStream_t s);
cudaError_t launch_seed_emit(SeedMode mode, const SeedArgs& a, cudaStream_t s);
cudaError_t launch_density_mask(const DensityArgs& a, cudaStream_t s);

}  // namespace fvgs
