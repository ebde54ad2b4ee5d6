// capi.cu -- implementation of the fvgs C-ABI (include/fvgs.h): sessions that
// own all device state of one SLAM map, and the host-side orchestration of the
// binning / tracking kernels on the session's stream.
//
// The reference keeps this state as GSSlam members resized on every call
// (src/GSSlam.cu:408-471) and synchronises after every kernel
// (src/GSSlam.cu:47-66).  Here buffers are sized once per session, the
// instance count stays on the device, and a call synchronises once, when it
// has to hand results back to the host.  The instance buffers start at an
// estimate and grow when the device reports an overflow; the affected call is
// then re-run, so results never depend on the capacity.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <new>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/fvgs.h"
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

using namespace fvgs;

namespace {

constexpr int kMaxLevels = 4;
// binning contexts per session: one per tile grid in use (the pyramid levels)
constexpr int kBinCtx = 4;

struct FrameLevel {
    int W = 0, H = 0;
    size_t cap_px = 0;
    // launch variant of the Jacobian kernel chosen by the autotuner for
    // frames of tuned_w x tuned_h (0 until tuned)
    int track_variant = 0, tuned_w = 0, tuned_h = 0;
    float tuned_ms[kTrackVariants] = {};
    // tile shape of this level's tracking binnings (16 x 16, 8 x 8 or 32 x 8)
    int tile_w = 16, tile_h = 16;
    float* rgb = nullptr;
    float* depth = nullptr;
    float* gx = nullptr;
    float* gy = nullptr;
};

__global__ void set_pose_kernel(DevPose* dst, fvgs_pose p) {
    pdl_begin();
    for (int k = 0; k < 3; ++k) {
        dst->t[k] = p.position[k];
        dst->td[k] = (double)p.position[k];
    }
    for (int k = 0; k < 4; ++k) {
        dst->q[k] = p.orientation[k];
        dst->qd[k] = (double)p.orientation[k];
    }
}

// The same from a pose in device memory (filled by a host-to-device copy that
// a captured frame graph replays with the current request's pose).
__global__ void set_pose_dev_kernel(DevPose* dst, const fvgs_pose* src) {
    pdl_begin();
    for (int k = 0; k < 3; ++k) {
        dst->t[k] = src->position[k];
        dst->td[k] = (double)src->position[k];
    }
    for (int k = 0; k < 4; ++k) {
        dst->q[k] = src->orientation[k];
        dst->qd[k] = (double)src->orientation[k];
    }
}

__global__ void upload_pack_kernel(const float* pos, const float* scl, const float* rot, const float* col,
                                   const float* opa, uint32_t n, float4* gpos, float4* gscl, float4* grot,
                                   float4* gcol) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    gpos[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.f);
    gscl[i] = make_float4(scl[3 * i], scl[3 * i + 1], scl[3 * i + 2], 0.f);
    grot[i] = make_float4(rot[4 * i], rot[4 * i + 1], rot[4 * i + 2], rot[4 * i + 3]);
    gcol[i] = make_float4(col[3 * i], col[3 * i + 1], col[3 * i + 2], opa[i]);
}

__global__ void download_unpack_kernel(const float4* gpos, const float4* gscl, const float4* grot,
                                       const float4* gcol, uint32_t n, float* pos, float* scl, float* rot,
                                       float* col, float* opa) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = gpos[i], s = gscl[i], q = grot[i], c = gcol[i];
    pos[3 * i] = p.x; pos[3 * i + 1] = p.y; pos[3 * i + 2] = p.z;
    scl[3 * i] = s.x; scl[3 * i + 1] = s.y; scl[3 * i + 2] = s.z;
    rot[4 * i] = q.x; rot[4 * i + 1] = q.y; rot[4 * i + 2] = q.z; rot[4 * i + 3] = q.w;
    col[3 * i] = c.x; col[3 * i + 1] = c.y; col[3 * i + 2] = c.z;
    opa[i] = c.w;
}

int bits_for(int v) {  // bits needed to represent values 0..v-1
    int b = 0;
    while ((1 << b) < v) ++b;
    return b;
}

// A binning context: the state of the binnings of one tile grid (frame size
// and tile shape) -- its binning records, counts, candidate list, sorted
// lists (ping-pong) and history -- so the first binning at a pyramid level
// continues that level's previous binning instead of starting over.
struct BinCtx {
    int W = 0, H = 0, tw = 0, th = 0;  // the grid it is bound to (0: none)
    uint64_t last_use = 0;
    BinRec* bins = nullptr;
    uint32_t *counts = nullptr, *cand = nullptr;
    CandState* cst = nullptr;
    uint2 *ranges = nullptr, *ranges_prev = nullptr;
    uint32_t *vals = nullptr, *vals_alt = nullptr;
    // the pair member a frame leaves the current lists in (ctx_normalize)
    uint2* ranges_home = nullptr;
    uint32_t* vals_home = nullptr;
    bool hist_ok = false;
    int hist_ntx = 0, hist_nty = 0, hist_tw = 0, hist_th = 0;
};

// Host-side binning state of every context and the active one (graph entry
// and exit, capture fallback).
struct BinSnap {
    BinCtx c[kBinCtx];
    int cur = 0;
};

}  // namespace

struct fvgs_session {
    fvgs_params params{};
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    uint32_t debug = 0;
    uint32_t cap_g = 0, n_g = 0;
    int max_w = 0, max_h = 0;
    uint64_t footprint = 0;
    std::vector<void*> allocations;

    float4 *pos = nullptr, *scale = nullptr, *rot = nullptr, *col = nullptr;
    float4 *rec0 = nullptr, *rec1 = nullptr, *rec2 = nullptr;
    // geometry records of the analytic pose Jacobian (sessions whose quirks
    // clear FVGS_Q_POSE_JAC_APPROX): camera-frame covariance and mean
    float4 *geo0 = nullptr, *geo1 = nullptr;
    BinRec* bins = nullptr;  // binning records; bins[i].r.z == counts[i] after every binning
    uint32_t *counts = nullptr, *offsets = nullptr, *partials = nullptr;
    // the projection's candidate list (Gaussians that may be in view near the
    // pose it was built at) and its state; cleared when the Gaussians change
    uint32_t* cand = nullptr;
    CandState* cst = nullptr;
    float *dbg_cov = nullptr, *dbg_inv = nullptr;
    uint8_t* dbg_vis = nullptr;

    uint64_t cap_inst = 0;
    uint64_t* keys = nullptr;
    uint32_t* vals = nullptr;
    SortWorkspace sort{};

    int cap_tiles = 0;    // tiles of the largest frame at the smallest tracking tile (8 x 8)
    int cap_tiles16 = 0;  // tiles of the largest frame at 16 x 16 (mapping)
    uint2* ranges = nullptr;
    uint2* ranges_prev = nullptr;  // swapped with ranges per binning (vals with sort.vals_alt)
    float* tile_out = nullptr;
    int* tile_diff = nullptr;      // binning scratch: difference grids of tile counts + counters
    size_t tile_diff_cells = 0;
    bool diff_clean = false;       // the scratch is all zero (the tile-offsets kernel leaves it so)
    uint32_t* tile_fill = nullptr;  // scatter cursors
    SegSortWork seg{};
    // incremental binning: entering instances per tile and the Gaussians with some
    uint2* enter_ranges = nullptr;
    uint32_t* enter_fill = nullptr;
    uint64_t* enter_keys = nullptr;
    uint4* changed = nullptr;  // (index, previous rectangle, previous count) per changed Gaussian
    uint32_t enter_cap = 0;
    bool hist_ok = false;  // the last binning left valid (bins, counts, ranges, vals) for the next one
    bool keys_valid = false;  // keys[] holds the last binning's reference-format keys
    int hist_ntx = 0, hist_nty = 0, hist_tw = 0, hist_th = 0;
    int bin_tw = 16, bin_th = 16;  // tile shape of the last binning
    // Binning contexts, one per tile grid (frame size and tile shape) in use
    // (BinCtx).  The fields bins, counts, cand, cst, ranges, ranges_prev,
    // vals, sort.vals_alt and hist_* above are the active context's
    // (ctx_select).
    BinCtx bctx[kBinCtx];
    int bctx_cur = 0;
    uint64_t bctx_clock = 0;
    CandState* cst_all = nullptr;  // the contexts' candidate-list states, contiguous
    float* frame_stage = nullptr;  // packed frames from host memory (fvgs_set_frames_packed)
    size_t frame_stage_cap = 0;

    FrameLevel lv[kMaxLevels];
    // frame preprocessing: 8-bit colour pyramid and the raw depth of a frame
    uint8_t* pre_u8[kMaxLevels] = {};
    size_t pre_u8_px[kMaxLevels] = {};
    uint8_t* pre_raw = nullptr;  // camera depth as given (float or uint16)
    size_t pre_raw_bytes = 0;
    int pre_w = 0, pre_h = 0;
    bool pre_valid = false;  // pre_u8[0] and lv[0].depth hold the same camera frame

    DevPose* pose = nullptr;
    double* jj = nullptr;    // 42 doubles: JtJ[36], Jtr[6]
    double* step = nullptr;  // 6 doubles
    DevStatus* st = nullptr;
    double* h_jj = nullptr;  // pinned mirrors
    DevStatus* h_st = nullptr;
    fvgs_pose* h_pose = nullptr;
    DevPose* h_devpose = nullptr;

    float *img_color = nullptr, *img_depth = nullptr, *img_T = nullptr;
    uint32_t* img_nc = nullptr;
    size_t img_cap = 0;

    // mapping state and scratch
    float4* adam = nullptr;  // 9 planes x cap_g
    float* delta2d = nullptr;  // [cap_g][16]
    float* dbg_delta3d = nullptr;
    size_t map_px = 0;
    float *m_final_T = nullptr, *m_color = nullptr, *m_depth = nullptr, *m_color_err = nullptr;
    uint32_t* m_n_contrib = nullptr;
    uint32_t* m_max_contrib = nullptr;
    uint32_t* m_bucket_base = nullptr;
    uint32_t* m_bucket_total = nullptr;
    float4* m_sampled = nullptr;
    size_t m_sampled_slots = 0;
    int m_W = 0, m_H = 0;

    // map maintenance: second set of Gaussian planes (compaction target,
    // swapped in afterwards), its optimiser-state twin (allocated when the
    // moments move with their Gaussians), marks, scores and visibility masks
    float4 *pos_alt = nullptr, *scale_alt = nullptr, *rot_alt = nullptr, *col_alt = nullptr;
    float4* adam_alt = nullptr;
    uint8_t* mk_states = nullptr;
    uint8_t *vis_a = nullptr, *vis_b = nullptr;
    float *mk_total_alpha = nullptr, *mk_outlier_prob = nullptr;
    uint32_t *mk_block_keep = nullptr, *mk_block_base = nullptr;
    uint32_t* mk_ctr = nullptr;    // [0] survivors, [1] removed, [2] intersection, [3] union
    uint32_t* h_mk_ctr = nullptr;  // pinned mirror
    uint32_t mk_n = 0;             // Gaussians covered by the last marking
    bool mk_scores = false;        // the last marking was an outlier pass (scores valid)
    uint32_t *sd_block_keep = nullptr, *sd_block_base = nullptr;  // seeding: per block of sample cells
    size_t sd_blocks = 0;

    // precision form: reduced-precision copies of scale/rotation and
    // colour/opacity that the projection reads; the float4 planes stay the
    // master copy (mapping updates both)
    // tensor maps of the record planes (TMA-staged Jacobian variant)
    RecMaps rec_maps{};
    bool rec_maps_ok = false;

    int precision = FVGS_PRECISION_FP32;
    bool autotune = true;  // tune the Jacobian kernel's launch variant on a frame shape's first frame
    uint4* attr_sr = nullptr;
    uint2* attr_c = nullptr;

    // kernel accounting: launches per class (always), event timing (opt-in)
    uint32_t timing_mask = 0;
    uint64_t launches[FVGS_K_COUNT] = {};
    double kernel_ms[FVGS_K_COUNT] = {};
    uint64_t timed_launches[FVGS_K_COUNT] = {};
    std::vector<cudaEvent_t> ev_pool;
    size_t ev_used = 0;
    struct Pending {
        int cls;
        size_t a, b;
        uint32_t kernels;
    };
    std::vector<Pending> pending;

    int last_W = 0, last_H = 0, last_T = 0;
    int last_split = 1;  // partial rows per tile of the last tracking launch (TrackArgs::split)
    bool has_binning = false, has_track = false, dbg_proj_valid = false, has_map = false;

    // Asynchronous frames (fvgs_frame_submit / fvgs_frame_wait).  A frame
    // whose binning history is valid is captured once as a CUDA graph and
    // replayed; the request's pose reaches it through d_pose_in.  gen changes
    // with every device allocation (a graph holds buffer addresses).
    struct FrameGraph {
        bool valid = false;
        int iters[kMaxLevels] = {}, W[kMaxLevels] = {}, H[kMaxLevels] = {};
        int map_level = 0;
        uint32_t n_g = 0;  // launch shapes and kernel arguments depend on the Gaussian count
        fvgs_intrinsics K[kMaxLevels] = {};
        float eta = -1.f;
        uint64_t gen = 0;
        // the binning contexts the capture started from and left (buffers,
        // histories), and the frame's last binning
        BinSnap entry, exit;
        int exit_W = 0, exit_H = 0, exit_T = 0, exit_split = 1, exit_tw = 16, exit_th = 16;
        uint64_t launches[FVGS_K_COUNT] = {};
        uint64_t last_use = 0;
        cudaGraphExec_t exec = nullptr;
    };
    // frame shapes (regular frame, keyframe) x the binning histories they
    // start from (a frame leaves every context's lists at the same pair
    // member, ctx_normalize; after a reset the contexts regain their
    // histories over the first frames)
    static constexpr int kFrameGraphs = 6;
    FrameGraph graphs[kFrameGraphs];
    uint64_t graph_clock = 0;
    uint64_t gen = 1;
    fvgs_pose* d_pose_in = nullptr;
    cudaEvent_t frame_done = nullptr;
    bool frame_pending = false;
    // A frame: iters[l] Gauss-Newton iterations at pyramid level l with
    // intrinsics K[l], from the coarsest level down to level 0 (the loop of
    // GSSlam::optimizeWithCeres, src/GSSlam.cu:2269-2272), then optionally a
    // mapping step at map_level.
    struct FrameRequest {
        fvgs_pose pose{};
        fvgs_intrinsics K[kMaxLevels] = {};
        int iters[kMaxLevels] = {};
        int map_level = 0;
        float eta = -1.f;
    } req;
    uint64_t frames_graphed = 0, frames_eager = 0;
};

namespace {

thread_local char g_errbuf[256];

int cuda_fail(cudaError_t e, const char* what) {
    std::snprintf(g_errbuf, sizeof(g_errbuf), "%s: %s", what, cudaGetErrorString(e));
    return FVGS_E_CUDA;
}

#define FV_CK(call)                                     \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

template <typename T>
int dev_alloc(fvgs_session* s, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, sizeof(T) * count);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return FVGS_E_NOMEM;
    }
    s->allocations.push_back(v);
    s->footprint += sizeof(T) * count;
    ++s->gen;
    *p = static_cast<T*>(v);
    return FVGS_OK;
}

template <typename T>
void dev_free(fvgs_session* s, T*& p, size_t count) {
    if (!p) return;
    auto it = std::find(s->allocations.begin(), s->allocations.end(), (void*)p);
    if (it != s->allocations.end()) s->allocations.erase(it);
    cudaFree(p);
    s->footprint -= sizeof(T) * (count ? count : 1);
    ++s->gen;
    p = nullptr;
}

#define FV_TRY(expr)            \
    do {                        \
        int r_ = (expr);        \
        if (r_ != FVGS_OK) return r_; \
    } while (0)

// Tensor maps of the three record planes for the TMA-staged Jacobian kernel:
// 2-D, 4 floats x capacity rows of 16 bytes, one-row boxes (gather4 loads).
// The encoder comes from the driver through the runtime; without it the
// variant is simply not offered.
bool encode_record_maps(fvgs_session* s) {
    static PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    static bool looked = false;
    if (!looked) {
        looked = true;
        cudaDriverEntryPointQueryResult q{};
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        cudaGetLastError();
    }
    if (!enc) return false;
    float4* planes[3] = {s->rec0, s->rec1, s->rec2};
    const cuuint64_t dims[2] = {4, (cuuint64_t)s->cap_g};
    const cuuint64_t strides[1] = {sizeof(float4)};
    const cuuint32_t box[2] = {4, 1};
    const cuuint32_t elem[2] = {1, 1};
    for (int p = 0; p < 3; ++p)
        if (enc(&s->rec_maps.rec[p], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, planes[p], dims, strides, box, elem,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return false;
    return true;
}

// Bring the reduced-precision planes up to date with the master planes after
// a host-side map change (upload, removal, seeding).
int refresh_reduced(fvgs_session* s) {
    if (s->precision != FVGS_PRECISION_REDUCED || s->n_g == 0) return FVGS_OK;
    FV_CK(launch_pack_reduced(s->scale, s->rot, s->col, s->n_g, s->attr_sr, s->attr_c, s->stream));
    return FVGS_OK;
}

// ---- binning contexts -----------------------------------------------------
// The active context's state lives in the session's fields; these move it
// between the fields and the context table.
void ctx_store(fvgs_session* s) {
    BinCtx& c = s->bctx[s->bctx_cur];
    c.bins = s->bins;
    c.counts = s->counts;
    c.cand = s->cand;
    c.cst = s->cst;
    c.ranges = s->ranges;
    c.ranges_prev = s->ranges_prev;
    c.vals = s->vals;
    c.vals_alt = s->sort.vals_alt;
    c.hist_ok = s->hist_ok;
    c.hist_ntx = s->hist_ntx;
    c.hist_nty = s->hist_nty;
    c.hist_tw = s->hist_tw;
    c.hist_th = s->hist_th;
}

void ctx_load(fvgs_session* s, int i) {
    s->bctx_cur = i;
    const BinCtx& c = s->bctx[i];
    s->bins = c.bins;
    s->counts = c.counts;
    s->cand = c.cand;
    s->cst = c.cst;
    s->ranges = c.ranges;
    s->ranges_prev = c.ranges_prev;
    s->vals = c.vals;
    s->sort.vals_alt = c.vals_alt;
    s->hist_ok = c.hist_ok;
    s->hist_ntx = c.hist_ntx;
    s->hist_nty = c.hist_nty;
    s->hist_tw = c.hist_tw;
    s->hist_th = c.hist_th;
}

// Make the context of a W x H frame binned on tw x th tiles the active one:
// the context bound to that grid, else the least recently used one, rebound
// (its history is for another grid).
void ctx_select(fvgs_session* s, int W, int H, int tw, int th) {
    const auto bound = [&](const BinCtx& c) { return c.W == W && c.H == H && c.tw == tw && c.th == th; };
    if (bound(s->bctx[s->bctx_cur])) {
        s->bctx[s->bctx_cur].last_use = ++s->bctx_clock;
        return;
    }
    ctx_store(s);
    int pick = -1;
    for (int i = 0; i < kBinCtx && pick < 0; ++i)
        if (bound(s->bctx[i])) pick = i;
    if (pick < 0) {
        pick = 0;
        for (int i = 1; i < kBinCtx; ++i)
            if (s->bctx[i].last_use < s->bctx[pick].last_use) pick = i;
        BinCtx& c = s->bctx[pick];
        c.W = W;
        c.H = H;
        c.tw = tw;
        c.th = th;
        c.hist_ok = false;
    }
    s->bctx[pick].last_use = ++s->bctx_clock;
    ctx_load(s, pick);
    s->keys_valid = false;  // keys[] holds another context's binning
}

// Leave every context's current lists in its home pair member (copying them
// where the frame's binnings left them in the other): a frame with an odd
// number of binnings at a level would otherwise swap that context's
// ping-pong parity, and a captured frame holds the buffer addresses of the
// parity it was captured at.
int ctx_normalize(fvgs_session* s) {
    ctx_store(s);
    for (auto& c : s->bctx) {
        // a context without history needs no particular member (its next
        // binning is a full one, and graph keys ignore it); its lists may be
        // the last binning's, which downloads read
        if (!c.hist_ok || (c.vals == c.vals_home && c.ranges == c.ranges_home)) continue;
        // (a member already at home is copied onto itself: same values)
        FV_CK(launch_copy_lists(c.ranges, c.hist_ntx * c.hist_nty, c.vals, c.vals_home, c.ranges_home, s->cap_inst,
                                s->num_sms * 8, s->stream));
        if (c.vals != c.vals_home) std::swap(c.vals, c.vals_alt);
        if (c.ranges != c.ranges_home) std::swap(c.ranges, c.ranges_prev);
    }
    ctx_load(s, s->bctx_cur);
    return FVGS_OK;
}

// Every context's binning history is stale (the Gaussians or the instance
// buffers changed).
void ctx_drop_history(fvgs_session* s) {
    for (auto& c : s->bctx) c.hist_ok = false;
    s->hist_ok = false;
}

void snap_take(fvgs_session* s, BinSnap& b) {
    ctx_store(s);
    for (int i = 0; i < kBinCtx; ++i) b.c[i] = s->bctx[i];
    b.cur = s->bctx_cur;
}
void snap_put(fvgs_session* s, const BinSnap& b) {
    for (int i = 0; i < kBinCtx; ++i) {
        const uint64_t used = s->bctx[i].last_use;
        s->bctx[i] = b.c[i];
        s->bctx[i].last_use = used;
    }
    ctx_load(s, b.cur);
}
// Whether two snapshots bind the same grids to the same buffers with the same
// histories (what a captured frame's binnings depend on).
bool snap_same(const BinSnap& a, const BinSnap& b) {
    for (int i = 0; i < kBinCtx; ++i) {
        const BinCtx &x = a.c[i], &y = b.c[i];
        // a context without history is binned in full from whatever pair
        // member it holds, and the frame's exit state replaces it
        if (!x.hist_ok && !y.hist_ok) continue;
        if (x.W != y.W || x.H != y.H || x.tw != y.tw || x.th != y.th || x.bins != y.bins || x.ranges != y.ranges ||
            x.ranges_prev != y.ranges_prev || x.vals != y.vals || x.vals_alt != y.vals_alt || x.hist_ok != y.hist_ok ||
            x.hist_ntx != y.hist_ntx || x.hist_nty != y.hist_nty || x.hist_tw != y.hist_tw || x.hist_th != y.hist_th)
            return false;
    }
    return true;
}

int alloc_instances(fvgs_session* s, uint64_t cap) {
    ctx_store(s);
    ctx_drop_history(s);
    if (s->keys) {
        FV_CK(cudaStreamSynchronize(s->stream));
        dev_free(s, s->keys, s->cap_inst);
        for (auto& c : s->bctx) {
            dev_free(s, c.vals, s->cap_inst);
            dev_free(s, c.vals_alt, s->cap_inst);
        }
        dev_free(s, s->sort.keys_alt, s->cap_inst);
        dev_free(s, s->sort.lookback, sort_lookback_words(s->cap_inst));
    }
    s->cap_inst = cap;
    FV_TRY(dev_alloc(s, &s->keys, cap));
    for (auto& c : s->bctx) {
        FV_TRY(dev_alloc(s, &c.vals, cap));
        FV_TRY(dev_alloc(s, &c.vals_alt, cap));
        c.vals_home = c.vals;
        // the ranges pair in the same parity as the values
        if (c.ranges != c.ranges_home) std::swap(c.ranges, c.ranges_prev);
    }
    ctx_load(s, s->bctx_cur);
    FV_TRY(dev_alloc(s, &s->sort.keys_alt, cap));
    FV_TRY(dev_alloc(s, &s->sort.lookback, sort_lookback_words(cap)));
    FV_CK(cudaMemsetAsync(s->sort.lookback, 0, sizeof(uint64_t) * sort_lookback_words(cap), s->stream));
    s->sort.max_items = cap;
    s->sort.epoch = 1;
    return FVGS_OK;
}

int ensure_images(fvgs_session* s, size_t px) {
    if (px <= s->img_cap) return FVGS_OK;
    dev_free(s, s->img_color, 3 * s->img_cap);
    dev_free(s, s->img_depth, s->img_cap);
    dev_free(s, s->img_T, s->img_cap);
    dev_free(s, s->img_nc, s->img_cap);
    FV_TRY(dev_alloc(s, &s->img_color, 3 * px));
    FV_TRY(dev_alloc(s, &s->img_depth, px));
    FV_TRY(dev_alloc(s, &s->img_T, px));
    FV_TRY(dev_alloc(s, &s->img_nc, px));
    s->img_cap = px;
    return FVGS_OK;
}

int check_view(fvgs_session* s, int W, int H) {
    if (W <= 0 || H <= 0 || W > 65535 * s->params.tile_w || H > 65535 * s->params.tile_h) return FVGS_E_INVALID;
    const int ntx = (W + s->params.tile_w - 1) / s->params.tile_w;
    const int nty = (H + s->params.tile_h - 1) / s->params.tile_h;
    if (ntx * nty > s->cap_tiles) return FVGS_E_INVALID;
    return FVGS_OK;
}

cudaEvent_t next_event(fvgs_session* s) {
    if (s->ev_used == s->ev_pool.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
        s->ev_pool.push_back(e);
    }
    return s->ev_pool[s->ev_used++];
}

// Wraps the launches of one kernel class: counts kernels and, when the class
// is selected for timing, brackets them with CUDA events on the stream.
struct KScope {
    fvgs_session* s;
    int cls;
    uint32_t kernels;
    size_t a = (size_t)-1;
    KScope(fvgs_session* s_, int cls_, uint32_t kernels_) : s(s_), cls(cls_), kernels(kernels_) {
        s->launches[cls] += kernels;
        if (s->timing_mask & (1u << cls)) {
            cudaEvent_t e = next_event(s);
            if (e) {
                a = s->ev_used - 1;
                cudaEventRecord(e, s->stream);
            }
        }
    }
    ~KScope() {
        if (a != (size_t)-1) {
            cudaEvent_t e = next_event(s);
            if (e) {
                cudaEventRecord(e, s->stream);
                s->pending.push_back({cls, a, s->ev_used - 1, kernels});
            }
        }
    }
};

// Called after the stream has been synchronised.
void collect_timing(fvgs_session* s) {
    for (const auto& p : s->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, s->ev_pool[p.a], s->ev_pool[p.b]) == cudaSuccess) {
            s->kernel_ms[p.cls] += ms;
            s->timed_launches[p.cls] += 1;  // one timed call = one event pair
        } else {
            cudaGetLastError();
        }
    }
    s->pending.clear();
    s->ev_used = 0;
}

// Drop the projection's candidate list (the Gaussians changed).
cudaError_t cand_drop(fvgs_session* s) {
    return cudaMemsetAsync(s->cst_all, 0, sizeof(CandState) * kBinCtx, s->stream);
}

// The largest angle from the optical axis of a ray through the W x H image
// of K: the ray through its farthest corner.
float view_cone(const fvgs_intrinsics* K, int W, int H) {
    const double ex = std::max(std::fabs((double)K->cx), std::fabs((double)W - K->cx)) / K->fx;
    const double ey = std::max(std::fabs((double)K->cy), std::fabs((double)H - K->cy)) / K->fy;
    return (float)std::atan(std::sqrt(ex * ex + ey * ey));
}

// Enqueue binning for the pose already in s->pose.
int enqueue_bin(fvgs_session* s, const fvgs_intrinsics* K, int W, int H, int tw, int th) {
    const fvgs_params& P = s->params;
    if (!track_tile_supported(tw, th)) return FVGS_E_INVALID;
    const int ntx = (W + tw - 1) / tw;
    const int nty = (H + th - 1) / th;
    const int T = ntx * nty;
    const bool radix = (s->debug & FVGS_DEBUG_RADIX_SORT) != 0;
    ctx_select(s, W, H, tw, th);
    // Incremental binning needs the previous binning of the same Gaussians on
    // the same tile grid, with true per-tile ranges (not the reference's
    // culled-slot or range-launch behaviours).
    const bool literal = (s->params.quirks & (FVGS_Q_CULLED_SLOTS | FVGS_Q_RANGE_LAUNCH)) != 0;
    const bool hist = !radix && !literal && s->hist_ok && s->hist_ntx == ntx && s->hist_nty == nty &&
                      s->hist_tw == tw && s->hist_th == th;
    s->hist_ok = false;  // until this binning is fully enqueued
    if (!radix) {
        std::swap(s->ranges, s->ranges_prev);
        std::swap(s->vals, s->sort.vals_alt);
    }
    ProjectArgs pa{};
    pa.pos = s->pos;
    pa.scale = s->scale;
    pa.rot = s->rot;
    pa.col = s->col;
    if (s->precision == FVGS_PRECISION_REDUCED) {
        pa.attr_sr = s->attr_sr;
        pa.attr_c = s->attr_c;
    }
    pa.n = (int)s->n_g;
    pa.pose = s->pose;
    pa.K = *K;
    pa.W = W;
    pa.H = H;
    pa.tw = tw;
    pa.th = th;
    pa.inv_tw = (tw & (tw - 1)) == 0 ? 1.0f / (float)tw : 0.0f;
    pa.inv_th = (th & (th - 1)) == 0 ? 1.0f / (float)th : 0.0f;
    pa.ntx = ntx;
    pa.nty = nty;
    pa.radius_sigma = P.radius_sigma;
    pa.quirks = P.quirks;
    pa.rec0 = s->rec0;
    pa.rec1 = s->rec1;
    pa.rec2 = s->rec2;
    pa.bins = s->bins;
    pa.counts = s->counts;
    pa.geo0 = s->geo0;
    pa.geo1 = s->geo1;
    pa.cst = s->cst;
    if (!(s->debug & FVGS_DEBUG_NO_CANDIDATES)) pa.cand = s->cand;
    pa.cone = view_cone(K, W, H);
    if (s->debug & FVGS_DEBUG_PROJECTION) {
        pa.dbg_cov = s->dbg_cov;
        pa.dbg_inv = s->dbg_inv;
        pa.dbg_vis = s->dbg_vis;
    }
    if (!radix) {
        if (T > s->cap_tiles || tile_diff_words(ntx, nty) > s->tile_diff_cells) return FVGS_E_INVALID;
        if (!s->diff_clean) FV_CK(cudaMemsetAsync(s->tile_diff, 0, sizeof(int) * s->tile_diff_cells, s->stream));
        s->diff_clean = false;  // until the tile-offsets kernel of this binning is enqueued
        pa.tile_diff = s->tile_diff;
        if (hist) {
            pa.hist = 1;
            pa.changed = s->changed;
            pa.changed_cap = s->enter_cap;
        }
    }
    {
        KScope k(s, FVGS_K_PROJECT, 1);
        FV_CK(launch_project_count(pa, s->num_sms * 4, s->stream));
    }
    EmitArgs ea{};
    ea.bins = s->bins;
    ea.offsets = s->offsets;
    ea.n = (int)s->n_g;
    ea.ntx = ntx;
    ea.tw = tw;
    ea.th = th;
    ea.capacity = s->cap_inst;
    const uint32_t cap32 = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
    if (!radix) {
        // tile-bucket binning: counts -> ranges -> scatter -> per-tile sort
        {
            KScope k(s, FVGS_K_SCAN, 1);
            FV_CK(launch_tile_offsets(s->tile_diff, ntx, nty, hist, s->enter_cap, s->ranges, s->tile_fill,
                                      s->enter_ranges, s->enter_fill, s->st, cap32, s->seg.large_ctrl, s->stream));
            s->diff_clean = true;
        }
        ea.keys = s->sort.keys_alt;  // composite keys, tile-major
        ea.vals = nullptr;
        ea.changed = s->changed;
        ea.enter_keys = s->enter_keys;
        ea.enter_fill = s->enter_fill;
        ea.enter_cap = s->enter_cap;
        {
            KScope k(s, FVGS_K_EMIT, 1);
            FV_CK(launch_emit_scatter(ea, s->tile_fill, s->seg.large_ctrl + 2, s->num_sms * 8, s->st, s->stream));
        }
        SegSortIncr inc{};
        inc.ranges_prev = s->ranges_prev;
        inc.vals_prev = s->sort.vals_alt;
        inc.enter_ranges = s->enter_ranges;
        inc.enter_keys = s->enter_keys;
        inc.bins = s->bins;
        inc.ntx = ntx;
        inc.tw = tw;
        inc.th = th;
        inc.n_gauss = s->n_g;
        inc.capacity = s->cap_inst;
        {
            KScope k(s, FVGS_K_SORT, 2);
            FV_CK(launch_segsort(s->sort.keys_alt, s->keys, s->ranges, T, s->vals, s->seg, s->st, s->num_sms, inc,
                                 s->stream));
        }
        s->keys_valid = false;
        if (P.quirks & FVGS_Q_RANGE_LAUNCH) {
            // the literal range pass reads the reference-format keys
            KScope k(s, FVGS_K_RANGES, 2);
            FV_CK(launch_make_keys(s->bins, s->ranges, s->vals, s->n_g, T, ntx, tw, th, s->st, s->keys,
                                   s->stream));
            FV_CK(launch_ranges(s->keys, s->st, T, P.quirks, s->ranges, s->num_sms * 8, s->stream));
            s->keys_valid = true;
        }
    } else {
        // global path: offsets scan, generation-order keys, LSD radix sort, ranges
        {
            KScope k(s, FVGS_K_SCAN, 2);
            FV_CK(launch_scan(s->counts, (int)s->n_g, s->partials, s->offsets, s->st, cap32, s->stream));
        }
        ea.keys = s->keys;
        ea.vals = s->vals;
        {
            KScope k(s, FVGS_K_EMIT, 1);
            FV_CK(launch_emit_keys(ea, s->stream));
        }
        const int key_bits = 32 + std::max(1, bits_for(T));
        {
            KScope k(s, FVGS_K_SORT, 1 + (uint32_t)sort_num_passes(key_bits));
            FV_CK(launch_radix_sort(s->keys, s->vals, s->st, key_bits, &s->sort, &s->st->flags, s->stream));
        }
        {
            KScope k(s, FVGS_K_RANGES, 1);
            FV_CK(launch_ranges(s->keys, s->st, T, P.quirks, s->ranges, s->num_sms * 8, s->stream));
        }
        s->keys_valid = true;
    }
    s->last_W = W;
    s->last_H = H;
    s->last_T = T;
    s->hist_ok = !radix && !literal;
    s->hist_ntx = ntx;
    s->hist_nty = nty;
    s->hist_tw = s->bin_tw = tw;
    s->hist_th = s->bin_th = th;
    s->has_binning = true;
    s->dbg_proj_valid = (s->debug & FVGS_DEBUG_PROJECTION) != 0;
    return FVGS_OK;
}

// Whether a tracking launch may split its 16 x 16 list tiles over several CTAs.
bool split_ok(const TrackArgs& a) {
    return a.tile_w == 16 && a.tile_h == 16 && !a.compensated && !a.render_only;
}

// Arguments of the tracking kernel on the binning just enqueued.
TrackArgs make_track_args(fvgs_session* s, const fvgs_intrinsics* K, const FrameLevel& f, bool render_only,
                          bool images) {
    const fvgs_params& P = s->params;
    TrackArgs ta{};
    ta.rec0 = s->rec0;
    ta.rec1 = s->rec1;
    ta.rec2 = s->rec2;
    ta.ranges = s->ranges;
    ta.indices = s->vals;
    ta.n_list = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
    ta.n_gauss = s->n_g;
    ta.obs_rgb = f.rgb;
    ta.obs_depth = f.depth;
    ta.gx = f.gx;
    ta.gy = f.gy;
    ta.pose = s->pose;
    ta.K = *K;
    ta.W = f.W;
    ta.H = f.H;
    // the tile grid of the binning just enqueued
    ta.tile_w = s->bin_tw;
    ta.tile_h = s->bin_th;
    ta.ntx = (f.W + s->bin_tw - 1) / s->bin_tw;
    ta.nty = (f.H + s->bin_th - 1) / s->bin_th;
    ta.bg[0] = P.bg[0];
    ta.bg[1] = P.bg[1];
    ta.bg[2] = P.bg[2];
    ta.alpha_thresh = P.alpha_thresh;
    ta.color_thresh = P.color_thresh;
    ta.depth_thresh = P.depth_thresh;
    ta.tile_out = s->tile_out;
    if (images) {
        ta.img_color = s->img_color;
        ta.img_depth = s->img_depth;
        ta.img_T = s->img_T;
        ta.img_nc = s->img_nc;
    }
    ta.render_only = render_only ? 1 : 0;
    ta.quirks = P.quirks;
    ta.geo0 = s->geo0;
    ta.geo1 = s->geo1;
    // precision form: the analytic Jacobian's accumulations compensated (16 x 16 tiles)
    ta.compensated = (s->precision == FVGS_PRECISION_REDUCED && !render_only &&
                      !(P.quirks & FVGS_Q_POSE_JAC_APPROX) && ta.tile_w == 16 && ta.tile_h == 16)
                         ? 1
                         : 0;
    ta.variant = (f.tuned_w == f.W && f.tuned_h == f.H) ? f.track_variant : 0;
    if (ta.variant == 2 && !s->rec_maps_ok) ta.variant = 0;
    ta.split = 1;
    if (track_variant_split(ta.variant) > 1) {
        if (split_ok(ta)) ta.split = track_variant_split(ta.variant);
        else ta.variant = 3;  // the same staging batch, one CTA per tile
    }
    ta.st_flags = &s->st->flags;
    return ta;
}

int enqueue_track(fvgs_session* s, const fvgs_intrinsics* K, const FrameLevel& f, bool render_only,
                  bool images) {
    const TrackArgs ta = make_track_args(s, K, f, render_only, images);
    if (!render_only) s->last_split = ta.split;
    KScope k(s, render_only ? FVGS_K_RENDER : FVGS_K_TRACK, 1);
    FV_CK(launch_track(ta, s->rec_maps_ok ? &s->rec_maps : nullptr, s->stream));
    return FVGS_OK;
}

int set_pose(fvgs_session* s, const fvgs_pose* p) {
    FV_CK(launch_chained(set_pose_kernel, dim3(1), dim3(1), 0, s->stream, s->pose, *p));
    return FVGS_OK;
}

int reset_status(fvgs_session* s) {
    FV_CK(cudaMemsetAsync(s->st, 0, sizeof(DevStatus), s->stream));
    return FVGS_OK;
}

// After a synchronised step: grow on overflow (returns 1 = retry).
int check_status(fvgs_session* s, int* retry) {
    *retry = 0;
    const DevStatus st = *s->h_st;
    if (st.flags & kErrTimeout) return FVGS_E_TIMEOUT;
    if (st.flags & kErrBounds) {
        // an incremental binning did not find the instance count of a tile:
        // drop the histories and repeat the call with full binnings
        ctx_drop_history(s);
        *retry = 1;
        return FVGS_OK;
    }
    if (st.flags & kErrOverflow) {
        const uint64_t need = (uint64_t)st.n_instances;
        uint64_t cap = need + need / 4 + 65536;
        if (cap > 0xffffffffull) return FVGS_E_CAPACITY;
        FV_TRY(alloc_instances(s, cap));
        *retry = 1;
    }
    return FVGS_OK;
}

bool valid_pose(const fvgs_pose* p) { return p != nullptr; }

int ensure_map_buffers(fvgs_session* s, size_t px, bool cap) {
    if (px > s->map_px) {
        dev_free(s, s->m_final_T, s->map_px);
        dev_free(s, s->m_n_contrib, s->map_px);
        dev_free(s, s->m_color, 3 * s->map_px);
        dev_free(s, s->m_depth, s->map_px);
        dev_free(s, s->m_color_err, 3 * s->map_px);
        FV_TRY(dev_alloc(s, &s->m_final_T, px));
        FV_TRY(dev_alloc(s, &s->m_n_contrib, px));
        FV_TRY(dev_alloc(s, &s->m_color, 3 * px));
        FV_TRY(dev_alloc(s, &s->m_depth, px));
        FV_TRY(dev_alloc(s, &s->m_color_err, 3 * px));
        s->map_px = px;
    }
    // checkpoint slots: 8 per tile with MAP_CAP256, else one per 32 instances
    // of every tile (bounded by capacity/32 + tiles)
    const size_t slots = cap ? (size_t)s->cap_tiles16 * map_cap_buckets()
                             : (size_t)(s->cap_inst / 32 + 1) + (size_t)s->cap_tiles16;
    if (slots > s->m_sampled_slots) {
        dev_free(s, s->m_sampled, s->m_sampled_slots * 256);
        FV_TRY(dev_alloc(s, &s->m_sampled, slots * 256));
        s->m_sampled_slots = slots;
    }
    return FVGS_OK;
}

int enqueue_map(fvgs_session* s, const fvgs_intrinsics* K, const FrameLevel& f, float eta) {
    const fvgs_params& P = s->params;
    const bool cap = (P.quirks & FVGS_Q_MAP_CAP256) != 0;
    const int ntx = (f.W + P.tile_w - 1) / P.tile_w, nty = (f.H + P.tile_h - 1) / P.tile_h;
    MapArgs ma{};
    ma.rec0 = s->rec0;
    ma.rec1 = s->rec1;
    ma.rec2 = s->rec2;
    ma.ranges = s->ranges;
    ma.indices = s->vals;
    ma.n_list = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
    ma.n_gauss = s->n_g;
    ma.obs_rgb = f.rgb;
    ma.obs_depth = f.depth;
    ma.W = f.W;
    ma.H = f.H;
    ma.ntx = ntx;
    ma.nty = nty;
    ma.bg[0] = P.bg[0];
    ma.bg[1] = P.bg[1];
    ma.bg[2] = P.bg[2];
    ma.bucket_base = cap ? nullptr : s->m_bucket_base;
    ma.sampled = s->m_sampled;
    ma.final_T = s->m_final_T;
    ma.n_contrib = s->m_n_contrib;
    ma.color = s->m_color;
    ma.depth = s->m_depth;
    ma.color_err = s->m_color_err;
    ma.max_contrib = s->m_max_contrib;
    ma.delta2d = s->delta2d;
    ma.w_depth = P.w_depth;
    ma.w_dist = P.w_dist;
    if (!cap) {
        KScope k(s, FVGS_K_SCAN, 1);
        FV_CK(launch_bucket_scan(s->ranges, ntx * nty, s->m_bucket_base, s->m_bucket_total, s->stream));
    }
    FV_CK(cudaMemsetAsync(s->delta2d, 0, sizeof(float) * 16 * (size_t)s->n_g, s->stream));
    {
        KScope k(s, FVGS_K_MAP_FWD, 1);
        FV_CK(launch_map_forward(ma, cap, s->stream));
    }
    {
        KScope k(s, FVGS_K_MAP_BWD, 1);
        FV_CK(launch_map_backward(ma, cap, s->stream));
    }
    MapUpdateArgs ua{};
    ua.pos = s->pos;
    ua.scale = s->scale;
    ua.rot = s->rot;
    ua.col = s->col;
    ua.adam = s->adam;
    ua.cap = s->cap_g;
    ua.n = (int)s->n_g;
    ua.delta2d = s->delta2d;
    ua.pose = s->pose;
    ua.K = *K;
    ua.lambda_iso = P.lambda_iso;
    ua.eta = eta;
    ua.beta1 = P.adam_beta1;
    ua.beta2 = P.adam_beta2;
    ua.eps = P.adam_eps;
    ua.dbg_delta3d = (s->debug & FVGS_DEBUG_MAPPING) ? s->dbg_delta3d : nullptr;
    ua.cst = s->cst_all;
    ua.n_cst = kBinCtx;
    if (s->precision == FVGS_PRECISION_REDUCED) {
        ua.attr_sr = s->attr_sr;
        ua.attr_c = s->attr_c;
    }
    {
        KScope k(s, FVGS_K_MAP_UPDATE, 1);
        FV_CK(launch_map_update(ua, s->st, s->stream));
    }
    s->m_W = f.W;
    s->m_H = f.H;
    return FVGS_OK;
}

}  // namespace

extern "C" {

const char* fvgs_status_string(int status) {
    switch (status) {
        case FVGS_OK: return "ok";
        case FVGS_E_INVALID: return "invalid argument";
        case FVGS_E_NOMEM: return "out of memory";
        case FVGS_E_CUDA: return g_errbuf[0] ? g_errbuf : "CUDA error";
        case FVGS_E_CAPACITY: return "capacity exceeded";
        case FVGS_E_TIMEOUT: return "bounded device wait expired";
        case FVGS_E_STATE: return "call made in the wrong state";
        case FVGS_E_ADMISSION: return "not admitted";
        default: return "unknown status";
    }
}

int fvgs_params_default(fvgs_params* p) {
    if (!p) return FVGS_E_INVALID;
    std::memset(p, 0, sizeof(*p));
    p->tile_w = 16;
    p->tile_h = 16;
    p->radius_sigma = 3.0f;
    p->bg[0] = p->bg[1] = p->bg[2] = 0.0f;
    p->alpha_thresh = 0.2f;
    p->color_thresh = 0.1f;
    p->depth_thresh = 0.2f;
    p->w_depth = 1.0f;
    p->w_dist = 0.1f;
    p->lambda_iso = 0.01f;
    p->adam_beta1 = 0.9f;
    p->adam_beta2 = 0.999f;
    p->adam_eps = 1e-8f;
    p->quirks = FVGS_QUIRKS_DEFAULT;
    p->eig_eps = 1e-4;
    return FVGS_OK;
}

int fvgs_session_destroy(fvgs_session* s) {
    if (!s) return FVGS_E_INVALID;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (void* p : s->allocations) cudaFree(p);
    for (cudaEvent_t e : s->ev_pool) cudaEventDestroy(e);
    if (s->h_jj) cudaFreeHost(s->h_jj);
    if (s->h_st) cudaFreeHost(s->h_st);
    if (s->h_pose) cudaFreeHost(s->h_pose);
    if (s->h_devpose) cudaFreeHost(s->h_devpose);
    if (s->h_mk_ctr) cudaFreeHost(s->h_mk_ctr);
    for (auto& g : s->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (s->frame_done) cudaEventDestroy(s->frame_done);
    if (s->own_stream) cudaStreamDestroy(s->own_stream);
    delete s;
    return FVGS_OK;
}

int fvgs_session_create(const fvgs_params* params, int device, uint32_t capacity_gaussians, int max_width,
                        int max_height, fvgs_session** out) {
    if (!out || capacity_gaussians == 0 || max_width <= 0 || max_height <= 0) return FVGS_E_INVALID;
    *out = nullptr;
    fvgs_params P;
    if (params) P = *params;
    else fvgs_params_default(&P);
    // The sm_103a tracking kernel is written for 16x16 tiles (one thread per
    // pixel of a tile); other shapes are rejected rather than mis-rendered.
    if (P.tile_w != 16 || P.tile_h != 16) return FVGS_E_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return FVGS_E_INVALID;
    }
    FV_CK(cudaSetDevice(device));
    FV_CK(track_configure_device());
    fvgs_session* s = new (std::nothrow) fvgs_session();
    if (!s) return FVGS_E_NOMEM;
    s->params = P;
    s->device = device;
    s->cap_g = capacity_gaussians;
    s->max_w = max_width;
    s->max_h = max_height;
    int rc = FVGS_OK;
    auto fail = [&](int r) {
        fvgs_session_destroy(s);
        return r;
    };
    if (cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return fail(FVGS_E_CUDA);
    if (cudaStreamCreateWithFlags(&s->own_stream, cudaStreamNonBlocking) != cudaSuccess) return fail(FVGS_E_CUDA);
    s->stream = s->own_stream;
    const size_t N = capacity_gaussians;
#define FV_A(ptr, cnt) \
    if ((rc = dev_alloc(s, &(ptr), (cnt))) != FVGS_OK) return fail(rc)
    FV_A(s->pos, N);
    FV_A(s->scale, N);
    FV_A(s->rot, N);
    FV_A(s->col, N);
    FV_A(s->rec0, N);
    FV_A(s->rec1, N);
    FV_A(s->rec2, N);
    if (!(P.quirks & FVGS_Q_POSE_JAC_APPROX)) {
        FV_A(s->geo0, N);
        FV_A(s->geo1, N);
    }
    FV_A(s->offsets, N);
    FV_A(s->cst_all, kBinCtx);
    for (int c = 0; c < kBinCtx; ++c) {
        BinCtx& b = s->bctx[c];
        FV_A(b.bins, N);
        FV_A(b.counts, N);
        FV_A(b.cand, N);
        b.cst = s->cst_all + c;
    }
    FV_A(s->partials, scan_partials_size((int)N) + 1);
    // tile-indexed buffers hold the largest frame at the smallest tracking
    // tile (8 x 8); mapping runs on 16 x 16 tiles
    const int ntx = (max_width + 7) / 8, nty = (max_height + 7) / 8;
    s->cap_tiles = ntx * nty;
    s->cap_tiles16 = ((max_width + P.tile_w - 1) / P.tile_w) * ((max_height + P.tile_h - 1) / P.tile_h);
    for (int c = 0; c < kBinCtx; ++c) {
        FV_A(s->bctx[c].ranges, (size_t)s->cap_tiles);
        FV_A(s->bctx[c].ranges_prev, (size_t)s->cap_tiles);
        s->bctx[c].ranges_home = s->bctx[c].ranges;
    }
    ctx_load(s, 0);
    s->tile_diff_cells = tile_diff_words(ntx, nty);
    FV_A(s->tile_diff, s->tile_diff_cells);
    FV_A(s->tile_fill, (size_t)s->cap_tiles);
    FV_A(s->enter_ranges, (size_t)s->cap_tiles);
    FV_A(s->enter_fill, (size_t)s->cap_tiles);
    s->enter_cap = std::max<uint32_t>(1u << 16, capacity_gaussians);
    FV_A(s->enter_keys, (size_t)s->enter_cap);
    FV_A(s->changed, (size_t)s->enter_cap);
    FV_A(s->seg.large_list, (size_t)s->cap_tiles);
    FV_A(s->seg.large_ctrl, 4);  // [0..1] large-bucket list control, [2] scatter chunk counter
    // partial rows: a tile of the smallest tracking tile each, or four per
    // 16 x 16 tile split over 8 x 8 CTAs
    FV_A(s->tile_out, (size_t)std::max(s->cap_tiles, 4 * s->cap_tiles16) * FVGS_POSEDATA_FLOATS);
    FV_A(s->pose, 1);
    FV_A(s->d_pose_in, 1);
    FV_A(s->jj, 48);
    FV_A(s->step, 8);
    FV_A(s->st, 1);
    FV_A(s->sort.ctrl, sort_ctrl_words());
    FV_A(s->adam, 9 * N);
    FV_A(s->delta2d, 16 * N);
    FV_A(s->m_max_contrib, (size_t)s->cap_tiles);
    FV_A(s->m_bucket_base, (size_t)s->cap_tiles);
    FV_A(s->m_bucket_total, 1);
    FV_A(s->pos_alt, N);
    FV_A(s->scale_alt, N);
    FV_A(s->rot_alt, N);
    FV_A(s->col_alt, N);
    FV_A(s->mk_states, N);
    FV_A(s->vis_a, N);
    FV_A(s->vis_b, N);
    FV_A(s->mk_total_alpha, N);
    FV_A(s->mk_outlier_prob, N);
    FV_A(s->mk_block_keep, N / kCompactBlock + 1);
    FV_A(s->mk_block_base, N / kCompactBlock + 1);
    FV_A(s->mk_ctr, 4);
    s->sd_blocks = (size_t)max_width * max_height / kCompactBlock + 2;  // one sample cell per pixel at most
    FV_A(s->sd_block_keep, s->sd_blocks);
    FV_A(s->sd_block_base, s->sd_blocks);
#undef FV_A
    if (cudaMallocHost(&s->h_jj, sizeof(double) * 48) != cudaSuccess ||
        cudaMallocHost(&s->h_st, sizeof(DevStatus)) != cudaSuccess ||
        cudaMallocHost(&s->h_pose, sizeof(fvgs_pose)) != cudaSuccess ||
        cudaMallocHost(&s->h_devpose, sizeof(DevPose)) != cudaSuccess ||
        cudaMallocHost(&s->h_mk_ctr, sizeof(uint32_t) * 4) != cudaSuccess)
        return fail(FVGS_E_NOMEM);
    if (cudaEventCreateWithFlags(&s->frame_done, cudaEventDisableTiming) != cudaSuccess) return fail(FVGS_E_CUDA);
    if (sort_init(&s->sort, device) != cudaSuccess) return fail(FVGS_E_CUDA);
    s->rec_maps_ok = encode_record_maps(s);
    const uint64_t cap0 = std::max<uint64_t>(1u << 20, 8ull * N);
    if ((rc = alloc_instances(s, std::min<uint64_t>(cap0, 0xffffffffull))) != FVGS_OK) return fail(rc);
    if (cudaMemsetAsync(s->st, 0, sizeof(DevStatus), s->stream) != cudaSuccess) return fail(FVGS_E_CUDA);
    if (cudaMemsetAsync(s->cst_all, 0, sizeof(CandState) * kBinCtx, s->stream) != cudaSuccess)
        return fail(FVGS_E_CUDA);
    if (cudaStreamSynchronize(s->stream) != cudaSuccess) return fail(FVGS_E_CUDA);
    *out = s;
    return FVGS_OK;
}

int fvgs_session_set_stream(fvgs_session* s, void* stream) {
    if (!s) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    FV_CK(cudaStreamSynchronize(s->stream));
    s->stream = stream ? static_cast<cudaStream_t>(stream) : s->own_stream;
    return FVGS_OK;
}

int fvgs_session_stream(fvgs_session* s, void** stream, int* device) {
    if (!s) return FVGS_E_INVALID;
    if (stream) *stream = s->stream;
    if (device) *device = s->device;
    return FVGS_OK;
}

int fvgs_session_sync(fvgs_session* s) {
    if (!s) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

int fvgs_session_set_debug(fvgs_session* s, uint32_t flags) {
    if (!s) return FVGS_E_INVALID;
    ++s->gen;  // captured frames follow the debug outputs of their capture
    FV_CK(cudaSetDevice(s->device));
    if ((flags & FVGS_DEBUG_PROJECTION) && !s->dbg_cov) {
        FV_TRY(dev_alloc(s, &s->dbg_cov, 3 * (size_t)s->cap_g));
        FV_TRY(dev_alloc(s, &s->dbg_inv, 3 * (size_t)s->cap_g));
        FV_TRY(dev_alloc(s, &s->dbg_vis, (size_t)s->cap_g));
    }
    if (flags & FVGS_DEBUG_IMAGES) FV_TRY(ensure_images(s, (size_t)s->max_w * s->max_h));
    if ((flags & FVGS_DEBUG_MAPPING) && !s->dbg_delta3d) FV_TRY(dev_alloc(s, &s->dbg_delta3d, 16 * (size_t)s->cap_g));
    s->debug = flags;
    return FVGS_OK;
}

int fvgs_session_set_precision(fvgs_session* s, int precision) {
    if (!s || (precision != FVGS_PRECISION_FP32 && precision != FVGS_PRECISION_REDUCED)) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    if (precision == s->precision) return FVGS_OK;
    if (precision == FVGS_PRECISION_REDUCED && !s->attr_sr) {
        FV_TRY(dev_alloc(s, &s->attr_sr, s->cap_g));
        FV_TRY(dev_alloc(s, &s->attr_c, s->cap_g));
    }
    s->precision = precision;
    ++s->gen;  // captured frame graphs read the other planes
    FV_TRY(refresh_reduced(s));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

int fvgs_session_binning_info(const fvgs_session* s, uint32_t* n_instances, int* incremental, uint32_t* n_entering,
                              uint32_t* n_changed) {
    if (!s) return FVGS_E_INVALID;
    const DevStatus& st = *s->h_st;
    if (n_instances) *n_instances = st.n_instances;
    if (incremental) *incremental = st.mode == kBinIncremental ? 1 : 0;
    if (n_entering) *n_entering = st.n_enter;
    if (n_changed) *n_changed = st.n_changed;
    return FVGS_OK;
}

int fvgs_session_binning_grid(const fvgs_session* s, int* tile_w, int* tile_h, int* num_tiles) {
    if (!s) return FVGS_E_INVALID;
    if (!s->has_binning) return FVGS_E_STATE;
    if (tile_w) *tile_w = s->bin_tw;
    if (tile_h) *tile_h = s->bin_th;
    if (num_tiles) *num_tiles = s->last_T;
    return FVGS_OK;
}

int fvgs_session_candidates(fvgs_session* s, int* valid, uint32_t* n, fvgs_pose* pose, float* cone) {
    if (!s) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    CandState c{};
    FV_CK(cudaMemcpyAsync(&c, s->cst, sizeof(CandState), cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    if (valid) *valid = c.valid ? 1 : 0;
    if (n) *n = c.valid ? c.n : 0u;
    if (pose) {
        for (int k = 0; k < 3; ++k) pose->position[k] = c.t[k];
        for (int k = 0; k < 4; ++k) pose->orientation[k] = c.q[k];
    }
    if (cone) *cone = c.cone;
    return FVGS_OK;
}

int fvgs_session_footprint(const fvgs_session* s, uint64_t* bytes) {
    if (!s || !bytes) return FVGS_E_INVALID;
    *bytes = s->footprint;
    return FVGS_OK;
}

int fvgs_upload_gaussians(fvgs_session* s, const float* positions, const float* scales, const float* orientations,
                          const float* colors, const float* opacities, uint32_t n) {
    if (!s || n > s->cap_g || (n && (!positions || !scales || !orientations || !colors || !opacities)))
        return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    s->n_g = n;
    s->has_binning = s->has_track = false;
    ctx_drop_history(s);
    FV_CK(cand_drop(s));
    if (n == 0) return FVGS_OK;
    // Stage through rec planes (free until the next binning) so host arrays of
    // the reference's float3 layout become 16-byte vectors on the device.
    float* tmp = reinterpret_cast<float*>(s->rec0);  // 4N floats
    float* tmp2 = reinterpret_cast<float*>(s->rec1);
    float* tmp3 = reinterpret_cast<float*>(s->rec2);
    float* tmp4 = reinterpret_cast<float*>(s->bins);       // 8N floats
    float* tmp5 = reinterpret_cast<float*>(s->offsets);
    FV_CK(cudaMemcpyAsync(tmp, positions, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(tmp2, scales, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(tmp3, orientations, sizeof(float) * 4 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(tmp4, colors, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(tmp5, opacities, sizeof(float) * n, cudaMemcpyDefault, s->stream));
    upload_pack_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(tmp, tmp2, tmp3, tmp4, tmp5, n, s->pos, s->scale,
                                                               s->rot, s->col);
    FV_CK(cudaGetLastError());
    // fresh map: Adam moments and step counters start at zero
    FV_CK(cudaMemsetAsync(s->adam, 0, sizeof(float4) * 9 * (size_t)s->cap_g, s->stream));
    FV_TRY(refresh_reduced(s));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

int fvgs_download_gaussians(fvgs_session* s, float* positions, float* scales, float* orientations, float* colors,
                            float* opacities, uint32_t n) {
    if (!s || n > s->n_g || (n && (!positions || !scales || !orientations || !colors || !opacities)))
        return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    if (n == 0) return FVGS_OK;
    float* tmp = reinterpret_cast<float*>(s->rec0);
    float* tmp2 = reinterpret_cast<float*>(s->rec1);
    float* tmp3 = reinterpret_cast<float*>(s->rec2);
    float* tmp4 = reinterpret_cast<float*>(s->bins);       // 8N floats
    float* tmp5 = reinterpret_cast<float*>(s->offsets);
    download_unpack_kernel<<<(n + 255) / 256, 256, 0, s->stream>>>(s->pos, s->scale, s->rot, s->col, n, tmp, tmp2,
                                                                   tmp3, tmp4, tmp5);
    FV_CK(cudaGetLastError());
    FV_CK(cudaMemcpyAsync(positions, tmp, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(scales, tmp2, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(orientations, tmp3, sizeof(float) * 4 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(colors, tmp4, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(opacities, tmp5, sizeof(float) * n, cudaMemcpyDefault, s->stream));
    FV_CK(cand_drop(s));  // out-of-view Gaussians' records are no longer cleared
    FV_CK(cudaStreamSynchronize(s->stream));
    s->has_binning = s->has_track = false;  // staging overwrote the records
    s->hist_ok = false;
    return FVGS_OK;
}

namespace {

int ensure_level(fvgs_session* s, int level, int width, int height) {
    FrameLevel& f = s->lv[level];
    const size_t px = (size_t)width * height;
    if (px > f.cap_px) {
        dev_free(s, f.rgb, 3 * f.cap_px);
        dev_free(s, f.depth, f.cap_px);
        dev_free(s, f.gx, 3 * f.cap_px);
        dev_free(s, f.gy, 3 * f.cap_px);
        FV_TRY(dev_alloc(s, &f.rgb, 3 * px));
        FV_TRY(dev_alloc(s, &f.depth, px));
        FV_TRY(dev_alloc(s, &f.gx, 3 * px));
        FV_TRY(dev_alloc(s, &f.gy, 3 * px));
        f.cap_px = px;
    }
    f.W = width;
    f.H = height;
    return FVGS_OK;
}

}  // namespace

int fvgs_preprocess_frame(fvgs_session* s, const uint8_t* color, const void* depth, int depth_u16_mm, int width,
                          int height, int levels, int double_scale) {
    if (!s || !color || !depth || levels < 1 || levels > kMaxLevels) return FVGS_E_INVALID;
    if (check_view(s, width, height) != FVGS_OK) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    const size_t px0 = (size_t)width * height;
    const size_t raw_bytes = px0 * (depth_u16_mm ? sizeof(uint16_t) : sizeof(float));
    if (raw_bytes > s->pre_raw_bytes) {
        dev_free(s, s->pre_raw, s->pre_raw_bytes);
        FV_TRY(dev_alloc(s, &s->pre_raw, raw_bytes));
        s->pre_raw_bytes = raw_bytes;
    }
    int W = width, H = height;
    for (int l = 0; l < levels; ++l) {
        if (l > 0) {
            W = (W + 1) / 2;
            H = (H + 1) / 2;
        }
        const size_t px = (size_t)W * H;
        if (px > s->pre_u8_px[l]) {
            dev_free(s, s->pre_u8[l], 3 * s->pre_u8_px[l]);
            FV_TRY(dev_alloc(s, &s->pre_u8[l], 3 * px));
            s->pre_u8_px[l] = px;
        }
        FV_TRY(ensure_level(s, l, W, H));
    }
    s->pre_valid = true;
    s->pre_w = width;
    s->pre_h = height;
    FV_CK(cudaMemcpyAsync(s->pre_u8[0], color, 3 * px0, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(s->pre_raw, depth, raw_bytes, cudaMemcpyDefault, s->stream));
    // one launch per level (pyrDown, colour, Sobel and depth together), chained
    FV_CK(launch_prep_level0(s->pre_u8[0], s->pre_raw, depth_u16_mm, width, height, double_scale, s->lv[0].rgb,
                             s->lv[0].gx, s->lv[0].gy, s->lv[0].depth, s->stream));
    for (int l = 1; l < levels; ++l) {
        FrameLevel& f = s->lv[l];
        const FrameLevel& g = s->lv[l - 1];
        FV_CK(launch_prep_level(s->pre_u8[l - 1], g.depth, g.W, g.H, double_scale, s->pre_u8[l], f.rgb, f.gx, f.gy,
                                f.depth, s->stream));
    }
    return FVGS_OK;
}

int fvgs_download_frame(fvgs_session* s, int level, float* rgb, float* depth, float* grad_x, float* grad_y,
                        int* width, int* height) {
    if (!s || level < 0 || level >= kMaxLevels) return FVGS_E_INVALID;
    const FrameLevel& f = s->lv[level];
    if (!f.rgb) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    const size_t px = (size_t)f.W * f.H;
    if (width) *width = f.W;
    if (height) *height = f.H;
    if (rgb) FV_CK(cudaMemcpyAsync(rgb, f.rgb, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    if (depth) FV_CK(cudaMemcpyAsync(depth, f.depth, sizeof(float) * px, cudaMemcpyDefault, s->stream));
    if (grad_x) FV_CK(cudaMemcpyAsync(grad_x, f.gx, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    if (grad_y) FV_CK(cudaMemcpyAsync(grad_y, f.gy, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

int fvgs_set_frame(fvgs_session* s, int level, const float* rgb, const float* depth, const float* grad_x,
                   const float* grad_y, int width, int height) {
    if (!s || level < 0 || level >= kMaxLevels || !rgb || !depth || !grad_x || !grad_y) return FVGS_E_INVALID;
    if (check_view(s, width, height) != FVGS_OK) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    FrameLevel& f = s->lv[level];
    const size_t px = (size_t)width * height;
    FV_TRY(ensure_level(s, level, width, height));
    if (level == 0) s->pre_valid = false;  // level 0 no longer holds the preprocessed camera frame
    FV_CK(cudaMemcpyAsync(f.rgb, rgb, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(f.depth, depth, sizeof(float) * px, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(f.gx, grad_x, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    FV_CK(cudaMemcpyAsync(f.gy, grad_y, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    return FVGS_OK;
}

int fvgs_set_frames_packed(fvgs_session* s, const float* frames, int levels, int width, int height) {
    if (!s || !frames || levels < 1 || levels > kMaxLevels || width <= 0 || height <= 0) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    size_t total = 0;
    for (int l = 0, w = width, h = height; l < levels; ++l, w = (w + 1) / 2, h = (h + 1) / 2)
        total += 10 * (size_t)w * h;
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, frames) != cudaSuccess) {
        cudaGetLastError();
        attr.type = cudaMemoryTypeUnregistered;
    }
    const float* src = frames;
    if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged) {
        // host memory: one copy to the device, then the levels from there
        if (total > s->frame_stage_cap) {
            dev_free(s, s->frame_stage, s->frame_stage_cap);
            s->frame_stage_cap = 0;
            FV_TRY(dev_alloc(s, &s->frame_stage, total));
            s->frame_stage_cap = total;
        }
        FV_CK(cudaMemcpyAsync(s->frame_stage, frames, sizeof(float) * total, cudaMemcpyDefault, s->stream));
        src = s->frame_stage;
    }
    for (int l = 0, w = width, h = height; l < levels; ++l, w = (w + 1) / 2, h = (h + 1) / 2) {
        const size_t px = (size_t)w * h;
        FV_TRY(fvgs_set_frame(s, l, src, src + 3 * px, src + 4 * px, src + 7 * px, w, h));
        src += 10 * px;
    }
    return FVGS_OK;
}

int fvgs_project_bin(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                     uint32_t* n_instances) {
    if (!s || !valid_pose(pose) || !K) return FVGS_E_INVALID;
    FV_TRY(check_view(s, width, height));
    FV_CK(cudaSetDevice(s->device));
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, width, height, s->params.tile_w, s->params.tile_h));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;
        if (n_instances) *n_instances = s->h_st->n_instances;
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

int fvgs_download_projection(fvgs_session* s, float* uv, float* cov2d, float* inv2d, float* depth, float* phat,
                             uint8_t* visible, uint32_t* tile_counts) {
    if (!s) return FVGS_E_INVALID;
    if (!s->has_binning) return FVGS_E_STATE;
    if ((cov2d || inv2d || visible) && !s->dbg_proj_valid) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    const size_t n = s->n_g;
    std::vector<float4> r0(n), r1(n), r2(n);
    FV_CK(cudaMemcpyAsync(r0.data(), s->rec0, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaMemcpyAsync(r1.data(), s->rec1, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaMemcpyAsync(r2.data(), s->rec2, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
    if (cov2d) FV_CK(cudaMemcpyAsync(cov2d, s->dbg_cov, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    if (inv2d) FV_CK(cudaMemcpyAsync(inv2d, s->dbg_inv, sizeof(float) * 3 * n, cudaMemcpyDefault, s->stream));
    if (visible) FV_CK(cudaMemcpyAsync(visible, s->dbg_vis, n, cudaMemcpyDefault, s->stream));
    std::vector<uint32_t> cnt(n);
    FV_CK(cudaMemcpyAsync(cnt.data(), s->counts, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    if (tile_counts) std::memcpy(tile_counts, cnt.data(), sizeof(uint32_t) * n);
    for (size_t i = 0; i < n; ++i) {
        // Gaussians without instances keep no record on the device; the
        // reference's buffers hold zeros for them
        if (cnt[i] == 0) r0[i] = r1[i] = r2[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (uv) {
            uv[2 * i] = r0[i].x;
            uv[2 * i + 1] = r0[i].y;
        }
        if (depth) depth[i] = r0[i].z;
        if (phat) {
            phat[2 * i] = r1[i].w;
            phat[2 * i + 1] = r2[i].x;
        }
    }
    return FVGS_OK;
}

int fvgs_download_binning(fvgs_session* s, uint64_t* keys, uint32_t* values, uint32_t* ranges,
                          uint64_t max_instances, uint32_t* n_instances) {
    if (!s) return FVGS_E_INVALID;
    if (!s->has_binning) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    const uint32_t n = s->h_st->n_instances_clamped;
    if (n_instances) *n_instances = n;
    if ((keys || values) && n > max_instances) return FVGS_E_CAPACITY;
    if (keys && n && !s->keys_valid) {
        const int ntx = (s->last_W + s->bin_tw - 1) / s->bin_tw;
        FV_CK(launch_make_keys(s->bins, s->ranges, s->vals, s->n_g, s->last_T, ntx, s->bin_tw,
                               s->bin_th, s->st, s->keys, s->stream));
        s->keys_valid = true;
    }
    if (keys && n) FV_CK(cudaMemcpyAsync(keys, s->keys, sizeof(uint64_t) * n, cudaMemcpyDefault, s->stream));
    if (values && n) FV_CK(cudaMemcpyAsync(values, s->vals, sizeof(uint32_t) * n, cudaMemcpyDefault, s->stream));
    if (ranges) FV_CK(cudaMemcpyAsync(ranges, s->ranges, sizeof(uint2) * s->last_T, cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

int fvgs_track_jacobian(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, double* JtJ,
                        double* Jtr) {
    if (!s || !valid_pose(pose) || !K || level < 0 || level >= kMaxLevels || !JtJ || !Jtr) return FVGS_E_INVALID;
    const FrameLevel& f = s->lv[level];
    if (!f.rgb) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    const bool images = (s->debug & FVGS_DEBUG_IMAGES) != 0;
    if (images) FV_TRY(ensure_images(s, (size_t)f.W * f.H));
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, f.W, f.H, f.tile_w, f.tile_h));
        FV_TRY(enqueue_track(s, K, f, false, images));
        {
            KScope k(s, FVGS_K_REDUCE, 1);
            FV_CK(launch_track_reduce(s->tile_out, s->last_T, s->last_split, s->pose, s->jj, s->stream));
        }
        FV_CK(cudaMemcpyAsync(s->h_jj, s->jj, sizeof(double) * 42, cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;
        std::memcpy(JtJ, s->h_jj, sizeof(double) * 36);
        std::memcpy(Jtr, s->h_jj + 36, sizeof(double) * 6);
        s->has_track = true;
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

int fvgs_download_tile_partials(fvgs_session* s, float* tiles, int num_tiles) {
    if (!s || !tiles) return FVGS_E_INVALID;
    if (!s->has_track) return FVGS_E_STATE;
    if (num_tiles < s->last_T) return FVGS_E_CAPACITY;
    FV_CK(cudaSetDevice(s->device));
    const int split = std::max(1, s->last_split);
    if (split == 1) {
        FV_CK(cudaMemcpyAsync(tiles, s->tile_out, sizeof(float) * 27 * s->last_T, cudaMemcpyDefault, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        return FVGS_OK;
    }
    // tiles split over several CTAs: add each tile's partial rows in the
    // frame reduction's order (FP32 adds, the same on host and device)
    std::vector<float> rows((size_t)27 * s->last_T * split);
    FV_CK(cudaMemcpyAsync(rows.data(), s->tile_out, sizeof(float) * rows.size(), cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    for (int t = 0; t < s->last_T; ++t)
        for (int c = 0; c < 27; ++c) {
            const float* r = rows.data() + ((size_t)t * split) * 27 + c;
            tiles[(size_t)t * 27 + c] = split == 2 ? r[0] + r[27] : (r[0] + r[27]) + (r[54] + r[81]);
        }
    return FVGS_OK;
}

int fvgs_download_track_images(fvgs_session* s, float* color, float* depth, float* final_T, uint32_t* n_contrib) {
    if (!s) return FVGS_E_INVALID;
    if (!s->has_track || !(s->debug & FVGS_DEBUG_IMAGES)) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    const size_t px = (size_t)s->last_W * s->last_H;
    if (color) FV_CK(cudaMemcpyAsync(color, s->img_color, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    if (depth) FV_CK(cudaMemcpyAsync(depth, s->img_depth, sizeof(float) * px, cudaMemcpyDefault, s->stream));
    if (final_T) FV_CK(cudaMemcpyAsync(final_T, s->img_T, sizeof(float) * px, cudaMemcpyDefault, s->stream));
    if (n_contrib) FV_CK(cudaMemcpyAsync(n_contrib, s->img_nc, sizeof(uint32_t) * px, cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

namespace {

// Launch-variant autotuner of the Jacobian kernel: bin the level's frame at
// `pose`, run every variant `reps` times in turn on that binning (timed with
// CUDA events on the session's stream), keep the fastest median for frames
// of this shape.  Every variant computes the same values in the same order,
// so the choice changes only the time.
// Whether launch variant v is a distinct choice for the level's frames: the
// TMA-staged one needs the record tensor maps; the split ones need 16 x 16
// tiles without compensated sums.
bool variant_applies(const fvgs_session* s, const FrameLevel& f, int v) {
    if (v == 2) return s->rec_maps_ok;
    if (track_variant_split(v) > 1) {
        TrackArgs a{};
        a.tile_w = f.tile_w ? f.tile_w : 16;
        a.tile_h = f.tile_h ? f.tile_h : 16;
        a.compensated = s->precision == FVGS_PRECISION_REDUCED && !(s->params.quirks & FVGS_Q_POSE_JAC_APPROX);
        return split_ok(a);
    }
    return true;
}

int autotune_track(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, int reps) {
    FrameLevel& f = s->lv[level];
    if (!f.rgb) return FVGS_E_STATE;
    reps = std::max(1, std::min(reps, 16));
    for (int attempt = 0;; ++attempt) {
        if (attempt == 4) return FVGS_E_CAPACITY;
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, f.W, f.H, f.tile_w, f.tile_h));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (!retry) break;
    }
    std::vector<cudaEvent_t> ev(2 * (size_t)reps * kTrackVariants, nullptr);
    int rc = FVGS_OK;
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) rc = FVGS_E_CUDA;
    FrameLevel saved = f;
    if (rc == FVGS_OK) {
        f.tuned_w = f.W;
        f.tuned_h = f.H;
        for (int r = 0; r < reps && rc == FVGS_OK; ++r)
            for (int v = 0; v < kTrackVariants && rc == FVGS_OK; ++v) {
                if (!variant_applies(s, f, v)) continue;
                f.track_variant = v;
                const size_t k = 2 * ((size_t)r * kTrackVariants + v);
                if (cudaEventRecord(ev[k], s->stream) != cudaSuccess) rc = FVGS_E_CUDA;
                if (rc == FVGS_OK) rc = enqueue_track(s, K, f, false, false);
                if (rc == FVGS_OK && cudaEventRecord(ev[k + 1], s->stream) != cudaSuccess) rc = FVGS_E_CUDA;
            }
        if (rc == FVGS_OK && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = FVGS_E_CUDA;
    }
    float med[kTrackVariants] = {};
    if (rc == FVGS_OK) {
        for (int v = 0; v < kTrackVariants; ++v) {
            std::vector<float> t(reps);
            for (int r = 0; r < reps; ++r) {
                const size_t k = 2 * ((size_t)r * kTrackVariants + v);
                cudaEventElapsedTime(&t[r], ev[k], ev[k + 1]);
            }
            std::sort(t.begin(), t.end());
            med[v] = t[reps / 2];
        }
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    if (rc != FVGS_OK) {
        cudaGetLastError();
        f = saved;
        return rc;
    }
    int best = 0;
    for (int v = 1; v < kTrackVariants; ++v)
        if (variant_applies(s, f, v) && med[v] < med[best]) best = v;
    f.track_variant = best;
    for (int v = 0; v < kTrackVariants; ++v) f.tuned_ms[v] = med[v];
    ++s->gen;  // captured frame graphs hold the previous kernel
    return FVGS_OK;
}

static_assert(kTrackVariants == FVGS_TRACK_VARIANTS, "launch variants of the Jacobian kernel");

bool needs_tuning(const fvgs_session* s, int level) {
    const FrameLevel& f = s->lv[level];
    return s->autotune && (f.tuned_w != f.W || f.tuned_h != f.H);
}

}  // namespace

int fvgs_session_autotune(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, int reps,
                          int* variant, float* ms) {
    if (!s || !valid_pose(pose) || !K || level < 0 || level >= kMaxLevels) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    FV_TRY(autotune_track(s, pose, K, level, reps));
    if (variant) *variant = s->lv[level].track_variant;
    if (ms)
        for (int v = 0; v < kTrackVariants; ++v) ms[v] = s->lv[level].tuned_ms[v];
    return FVGS_OK;
}

int fvgs_session_set_autotune(fvgs_session* s, int enabled) {
    if (!s) return FVGS_E_INVALID;
    s->autotune = enabled != 0;
    return FVGS_OK;
}

int fvgs_session_set_track_variant(fvgs_session* s, int level, int variant) {
    if (!s || level < 0 || level >= kMaxLevels || variant < 0 || variant >= kTrackVariants) return FVGS_E_INVALID;
    FrameLevel& f = s->lv[level];
    if (!f.rgb || (variant == 2 && !s->rec_maps_ok)) return FVGS_E_STATE;
    f.track_variant = variant;
    f.tuned_w = f.W;
    f.tuned_h = f.H;
    ++s->gen;
    return FVGS_OK;
}

namespace {

// One frame on the session's stream: the request's pose (already in the
// pinned staging s->h_pose) to the device, the Gauss-Newton steps of every
// level from the coarsest down, optionally a mapping step at the tracked
// pose, then the result pose, last step and status back to pinned host memory.
int enqueue_frame(fvgs_session* s, const fvgs_session::FrameRequest& r) {
    FV_TRY(reset_status(s));
    FV_CK(cudaMemcpyAsync(s->d_pose_in, s->h_pose, sizeof(fvgs_pose), cudaMemcpyHostToDevice, s->stream));
    FV_CK(launch_chained(set_pose_dev_kernel, dim3(1), dim3(1), 0, s->stream, s->pose,
                         static_cast<const fvgs_pose*>(s->d_pose_in)));
    for (int l = kMaxLevels - 1; l >= 0; --l) {
        const FrameLevel& f = s->lv[l];
        for (int it = 0; it < r.iters[l]; ++it) {
            FV_TRY(enqueue_bin(s, &r.K[l], f.W, f.H, f.tile_w, f.tile_h));
            FV_TRY(enqueue_track(s, &r.K[l], f, false, false));
            KScope k(s, FVGS_K_GN, 1);
            FV_CK(launch_track_reduce_gn(s->tile_out, s->last_T, s->last_split, s->pose, s->jj, s->params.eig_eps,
                                         s->step, s->stream));
        }
    }
    if (r.eta >= 0.f) {
        const FrameLevel& f = s->lv[r.map_level];
        FV_TRY(enqueue_bin(s, &r.K[r.map_level], f.W, f.H, s->params.tile_w, s->params.tile_h));
        FV_TRY(enqueue_map(s, &r.K[r.map_level], f, r.eta));
    }
    FV_TRY(ctx_normalize(s));
    FV_CK(cudaMemcpyAsync(s->h_devpose, s->pose, sizeof(DevPose), cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaMemcpyAsync(s->h_jj + 42, s->step, sizeof(double) * 6, cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
    return FVGS_OK;
}

// Level of the frame's first binning (-1: none).
int first_level(const fvgs_session::FrameRequest& r) {
    for (int l = kMaxLevels - 1; l >= 0; --l)
        if (r.iters[l] > 0) return l;
    return r.eta >= 0.f ? r.map_level : -1;
}

bool frame_key_matches(const fvgs_session::FrameGraph& g, fvgs_session* s, const fvgs_session::FrameRequest& r) {
    if (!(g.valid && g.gen == s->gen && g.map_level == r.map_level && g.eta == r.eta && g.n_g == s->n_g))
        return false;
    BinSnap now;
    snap_take(s, now);
    if (!snap_same(g.entry, now)) return false;
    for (int l = 0; l < kMaxLevels; ++l) {
        const bool used = r.iters[l] > 0 || (r.eta >= 0.f && l == r.map_level);
        if (g.iters[l] != r.iters[l]) return false;
        if (!used) continue;
        const FrameLevel& f = s->lv[l];
        if (g.W[l] != f.W || g.H[l] != f.H || g.K[l].fx != r.K[l].fx || g.K[l].fy != r.K[l].fy ||
            g.K[l].cx != r.K[l].cx || g.K[l].cy != r.K[l].cy)
            return false;
    }
    return true;
}

// Whether a frame may run from a captured graph: no per-call host work may
// be involved (the binning scratch is clean, so no binning needs a host-side
// memset; no event timing; the tile-bucket binning without the reference's
// literal range / culled-slot behaviours).  A captured frame holds the
// binning decisions of its capture, so the graph key records whether its
// first binning continued the previous one.
bool frame_graphable(const fvgs_session* s, const fvgs_session::FrameRequest& r) {
    const bool literal = (s->params.quirks & (FVGS_Q_CULLED_SLOTS | FVGS_Q_RANGE_LAUNCH)) != 0;
    return first_level(r) >= 0 && s->diff_clean && s->timing_mask == 0 && !(s->debug & FVGS_DEBUG_RADIX_SORT) &&
           !literal;
}

int launch_frame(fvgs_session* s) {
    const fvgs_session::FrameRequest& r = s->req;
    *s->h_pose = r.pose;
    if (!frame_graphable(s, r)) {
        ++s->frames_eager;
        return enqueue_frame(s, r);
    }
    for (auto& g : s->graphs) {
        if (!frame_key_matches(g, s, r)) continue;
        FV_CK(cudaGraphLaunch(g.exec, s->stream));
        g.last_use = ++s->graph_clock;
        snap_put(s, g.exit);
        for (int c = 0; c < FVGS_K_COUNT; ++c) s->launches[c] += g.launches[c];
        s->bin_tw = g.exit_tw;
        s->bin_th = g.exit_th;
        s->last_W = g.exit_W;
        s->last_H = g.exit_H;
        s->last_T = g.exit_T;
        s->last_split = g.exit_split;
        s->keys_valid = false;
        s->has_binning = true;
        ++s->frames_graphed;
        return FVGS_OK;
    }
    // capture this frame shape into a free or the least recently used slot
    int victim = 0;
    for (int i = 0; i < fvgs_session::kFrameGraphs; ++i) {
        if (!s->graphs[i].valid || s->graphs[i].gen != s->gen) {
            victim = i;
            break;
        }
        if (s->graphs[i].last_use < s->graphs[victim].last_use) victim = i;
    }
    fvgs_session::FrameGraph& g = s->graphs[victim];
    if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    g.valid = false;
    // host-side binning state before the capture: a capture enqueues nothing,
    // so if it fails the frame runs eagerly from exactly this state
    uint64_t before[FVGS_K_COUNT];
    std::memcpy(before, s->launches, sizeof(before));
    snap_take(s, g.entry);
    const bool clean0 = s->diff_clean, keys0 = s->keys_valid, binned0 = s->has_binning;
    const int lw0 = s->last_W, lh0 = s->last_H, lt0 = s->last_T, ls0 = s->last_split;
    const int btw0 = s->bin_tw, bth0 = s->bin_th;
    g.n_g = s->n_g;
    cudaGraph_t graph = nullptr;
    int rc = FVGS_OK;
    cudaError_t ec = cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal);
    if (ec == cudaSuccess) {
        rc = enqueue_frame(s, r);
        ec = cudaStreamEndCapture(s->stream, &graph);
    }
    if (rc == FVGS_OK && ec == cudaSuccess && graph) ec = cudaGraphInstantiate(&g.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc != FVGS_OK || ec != cudaSuccess || !g.exec) {
        cudaGetLastError();
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        std::memcpy(s->launches, before, sizeof(before));
        snap_put(s, g.entry);
        s->diff_clean = clean0;
        s->keys_valid = keys0;
        s->has_binning = binned0;
        s->bin_tw = btw0;
        s->bin_th = bth0;
        s->last_W = lw0;
        s->last_H = lh0;
        s->last_T = lt0;
        s->last_split = ls0;
        ++s->frames_eager;
        return enqueue_frame(s, r);
    }
    for (int l = 0; l < kMaxLevels; ++l) {
        g.iters[l] = r.iters[l];
        g.W[l] = s->lv[l].W;
        g.H[l] = s->lv[l].H;
        g.K[l] = r.K[l];
    }
    g.map_level = r.map_level;
    g.eta = r.eta;
    g.gen = s->gen;
    snap_take(s, g.exit);
    g.exit_tw = s->bin_tw;
    g.exit_th = s->bin_th;
    g.exit_W = s->last_W;
    g.exit_H = s->last_H;
    g.exit_T = s->last_T;
    g.exit_split = s->last_split;
    for (int c = 0; c < FVGS_K_COUNT; ++c) g.launches[c] = s->launches[c] - before[c];
    g.valid = true;
    g.last_use = ++s->graph_clock;
    FV_CK(cudaGraphLaunch(g.exec, s->stream));
    ++s->frames_graphed;
    return FVGS_OK;
}

}  // namespace

namespace {

// Intrinsics of pyramid level l from those of level 0: focal lengths and
// principal point scaled by 2^-l (GSSlam::computeRgbdPoseJacobians,
// src/GSSlam.cu:2133-2138).
fvgs_intrinsics level_intrinsics(const fvgs_intrinsics& K0, int l) {
    const float sc = 1.0f / (float)(1 << l);
    fvgs_intrinsics K = K0;
    K.fx *= sc;
    K.fy *= sc;
    K.cx *= sc;
    K.cy *= sc;
    return K;
}

using Request = fvgs_session::FrameRequest;

Request single_level_request(const fvgs_pose* pose, const fvgs_intrinsics* K, int level, int iterations,
                             float map_eta) {
    Request r;
    r.pose = *pose;
    r.K[level] = *K;
    r.iters[level] = iterations;
    r.map_level = level;
    r.eta = map_eta >= 0.f ? map_eta : -1.f;
    return r;
}

int pyramid_request(const fvgs_pose* pose, const fvgs_intrinsics* K0, const int* iterations, int levels,
                    float map_eta, Request* r) {
    if (!pose || !K0 || !iterations || levels < 1 || levels > kMaxLevels || !(map_eta == map_eta))
        return FVGS_E_INVALID;
    *r = Request{};
    r->pose = *pose;
    for (int l = 0; l < levels; ++l) {
        if (iterations[l] < 0) return FVGS_E_INVALID;
        r->K[l] = level_intrinsics(*K0, l);
        r->iters[l] = iterations[l];
    }
    r->map_level = 0;
    r->eta = map_eta >= 0.f ? map_eta : -1.f;
    return FVGS_OK;
}

// Checks and one-time preparations of a frame: every level it uses holds an
// observed frame, mapping buffers exist, launch variants are tuned.
int prepare_request(fvgs_session* s, const Request& r) {
    if (s->n_g == 0) return FVGS_E_STATE;
    for (int l = 0; l < kMaxLevels; ++l) {
        const bool used = r.iters[l] > 0 || (r.eta >= 0.f && l == r.map_level);
        if (used && !s->lv[l].rgb) return FVGS_E_STATE;
    }
    if (r.eta >= 0.f) {
        const FrameLevel& f = s->lv[r.map_level];
        FV_TRY(ensure_map_buffers(s, (size_t)f.W * f.H, (s->params.quirks & FVGS_Q_MAP_CAP256) != 0));
    }
    for (int l = kMaxLevels - 1; l >= 0; --l)
        if (r.iters[l] > 0 && needs_tuning(s, l)) FV_TRY(autotune_track(s, &r.pose, &r.K[l], l, 5));
    return FVGS_OK;
}

int total_iterations(const Request& r) {
    int n = 0;
    for (int l = 0; l < kMaxLevels; ++l) n += r.iters[l];
    return n;
}

// The plain per-frame path: the frame enqueued eagerly, then waited for.
int run_request_eager(fvgs_session* s, const Request& r, fvgs_pose* pose, double* last_step) {
    FV_TRY(prepare_request(s, r));
    for (int attempt = 0; attempt < 4; ++attempt) {
        *s->h_pose = r.pose;
        FV_TRY(enqueue_frame(s, r));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;
        for (int k = 0; k < 3; ++k) pose->position[k] = s->h_devpose->t[k];
        for (int k = 0; k < 4; ++k) pose->orientation[k] = s->h_devpose->q[k];
        if (last_step) std::memcpy(last_step, s->h_jj + 42, sizeof(double) * 6);
        s->has_track = total_iterations(r) > 0;
        if (r.eta >= 0.f) s->has_map = true;
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

int submit_request(fvgs_session* s, const Request& r) {
    if (s->frame_pending) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    FV_TRY(prepare_request(s, r));
    s->req = r;
    FV_TRY(launch_frame(s));
    FV_CK(cudaEventRecord(s->frame_done, s->stream));
    s->frame_pending = true;
    return FVGS_OK;
}

}  // namespace

int fvgs_track_frame(fvgs_session* s, fvgs_pose* pose, const fvgs_intrinsics* K, int level, int iterations,
                     double* last_step) {
    if (!s || !valid_pose(pose) || !K || level < 0 || level >= kMaxLevels || iterations < 0) return FVGS_E_INVALID;
    if (!s->lv[level].rgb) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    return run_request_eager(s, single_level_request(pose, K, level, iterations, -1.f), pose, last_step);
}

int fvgs_track_frame_pyramid(fvgs_session* s, fvgs_pose* pose, const fvgs_intrinsics* K0, const int* iterations,
                             int levels, double* last_step) {
    if (!s) return FVGS_E_INVALID;
    Request r;
    FV_TRY(pyramid_request(pose, K0, iterations, levels, -1.f, &r));
    FV_CK(cudaSetDevice(s->device));
    return run_request_eager(s, r, pose, last_step);
}

int fvgs_frame_submit(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, int iterations,
                      float map_eta) {
    if (!s || !valid_pose(pose) || !K || level < 0 || level >= kMaxLevels || iterations < 0 || !(map_eta == map_eta))
        return FVGS_E_INVALID;
    return submit_request(s, single_level_request(pose, K, level, iterations, map_eta));
}

int fvgs_frame_submit_pyramid(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K0,
                              const int* iterations, int levels, float map_eta) {
    if (!s) return FVGS_E_INVALID;
    Request r;
    FV_TRY(pyramid_request(pose, K0, iterations, levels, map_eta, &r));
    return submit_request(s, r);
}

int fvgs_frame_poll(fvgs_session* s, int* done) {
    if (!s || !done) return FVGS_E_INVALID;
    if (!s->frame_pending) return FVGS_E_STATE;
    const cudaError_t e = cudaEventQuery(s->frame_done);
    if (e == cudaErrorNotReady) {
        *done = 0;
        return FVGS_OK;
    }
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventQuery");
    *done = 1;
    return FVGS_OK;
}

int fvgs_frame_wait(fvgs_session* s, fvgs_pose* pose, double* last_step) {
    if (!s) return FVGS_E_INVALID;
    if (!s->frame_pending) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    s->frame_pending = false;
    FV_CK(cudaEventSynchronize(s->frame_done));
    collect_timing(s);
    int retry = 0;
    FV_TRY(check_status(s, &retry));
    // An instance overflow (the buffers have grown) or an inconsistent
    // incremental binning: run the frame again, eagerly, from the same pose.
    for (int attempt = 0; retry && attempt < 4; ++attempt) {
        if (s->req.eta >= 0.f) {
            const FrameLevel& f = s->lv[s->req.map_level];
            FV_TRY(ensure_map_buffers(s, (size_t)f.W * f.H, (s->params.quirks & FVGS_Q_MAP_CAP256) != 0));
        }
        *s->h_pose = s->req.pose;
        ++s->frames_eager;
        FV_TRY(enqueue_frame(s, s->req));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        FV_TRY(check_status(s, &retry));
    }
    if (retry) return FVGS_E_CAPACITY;
    if (pose) {
        for (int k = 0; k < 3; ++k) pose->position[k] = s->h_devpose->t[k];
        for (int k = 0; k < 4; ++k) pose->orientation[k] = s->h_devpose->q[k];
    }
    if (last_step) std::memcpy(last_step, s->h_jj + 42, sizeof(double) * 6);
    s->has_track = total_iterations(s->req) > 0;
    if (s->req.eta >= 0.f) s->has_map = true;
    return FVGS_OK;
}

namespace {

// Submit every session's frame (each on its own stream), then wait for all.
int run_batched(fvgs_session* const* sessions, fvgs_pose* poses, int n, const std::function<int(int)>& submit) {
    int first_error = FVGS_OK;
    int submitted = 0;
    for (; submitted < n; ++submitted) {
        const int rc = submit(submitted);
        if (rc != FVGS_OK) {
            first_error = rc;
            break;
        }
    }
    for (int i = 0; i < submitted; ++i) {
        const int rc = fvgs_frame_wait(sessions[i], &poses[i], nullptr);
        if (rc != FVGS_OK && first_error == FVGS_OK) first_error = rc;
    }
    return first_error;
}

}  // namespace

int fvgs_frames_run(fvgs_session* const* sessions, fvgs_pose* poses, const fvgs_intrinsics* K, const int* levels,
                    int iterations, const float* map_etas, int n) {
    if (!sessions || !poses || !K || n < 0) return FVGS_E_INVALID;
    return run_batched(sessions, poses, n, [&](int i) {
        return fvgs_frame_submit(sessions[i], &poses[i], &K[i], levels ? levels[i] : 0, iterations,
                                 map_etas ? map_etas[i] : -1.f);
    });
}

int fvgs_frames_run_pyramid(fvgs_session* const* sessions, fvgs_pose* poses, const fvgs_intrinsics* K0,
                            const int* iterations, int levels, const float* map_etas, int n) {
    if (!sessions || !poses || !K0 || !iterations || n < 0) return FVGS_E_INVALID;
    return run_batched(sessions, poses, n, [&](int i) {
        return fvgs_frame_submit_pyramid(sessions[i], &poses[i], &K0[i], iterations, levels,
                                         map_etas ? map_etas[i] : -1.f);
    });
}

int fvgs_session_set_track_tiles(fvgs_session* s, int level, int tile_w, int tile_h) {
    if (!s || level < 0 || level >= kMaxLevels || !track_tile_supported(tile_w, tile_h)) return FVGS_E_INVALID;
    FrameLevel& f = s->lv[level];
    f.tile_w = tile_w;
    f.tile_h = tile_h;
    ++s->gen;  // captured frames bin on the previous grid
    return FVGS_OK;
}

// ---------------------------------------------------------------------------
// Batching form: the frames of many sessions in lockstep, each Gauss-Newton
// iteration binning every session on its own stream and then blending and
// differentiating the tiles of all of them in one persistent launch.
// ---------------------------------------------------------------------------
struct fvgs_batch {
    std::vector<fvgs_session*> s;
    int device = 0, num_sms = 0;
    bool analytic = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_fork = nullptr;
    std::vector<cudaEvent_t> ev_join;
    int tw[kMaxLevels], th[kMaxLevels], variant[kMaxLevels];
    uint32_t* counters = nullptr;  // the persistent kernel's work counters
    // job tables, one region per Gauss-Newton iteration: host (pinned)
    // staging, the eager path's device copy and the captured frame's
    int cap_iters = 0;
    TrackJob* h_jobs = nullptr;
    uint32_t* h_begin = nullptr;
    ReduceJob* h_rjobs = nullptr;
    TrackJob *d_jobs = nullptr, *g_jobs = nullptr;
    uint32_t *d_begin = nullptr, *g_begin = nullptr;
    ReduceJob *d_rjobs = nullptr, *g_rjobs = nullptr;
    struct Exit {  // one session's key and the host-side binning state its captured frame leaves
        uint64_t gen = 0;
        uint32_t n_g = 0;
        BinSnap entry, exit;  // the session's binning contexts before and after the frame
        int W[kMaxLevels] = {}, H[kMaxLevels] = {};
        fvgs_intrinsics K[kMaxLevels] = {};
        int tw = 0, th = 0, last_W = 0, last_H = 0, last_T = 0;
        uint64_t launches[FVGS_K_COUNT] = {};
    };
    struct Graph {
        bool valid = false;
        int iters[kMaxLevels] = {};
        int tw[kMaxLevels] = {}, th[kMaxLevels] = {}, variant[kMaxLevels] = {};
        std::vector<Exit> exit;
        uint64_t batch_launches = 0;
        cudaGraphExec_t exec = nullptr;
    } graph;
    uint64_t graphed = 0, eager = 0, batch_launches = 0;
};

namespace {

void batch_free_tables(fvgs_batch* b) {
    if (b->h_jobs) cudaFreeHost(b->h_jobs);
    if (b->h_begin) cudaFreeHost(b->h_begin);
    if (b->h_rjobs) cudaFreeHost(b->h_rjobs);
    for (void* p : {(void*)b->d_jobs, (void*)b->g_jobs, (void*)b->d_begin, (void*)b->g_begin, (void*)b->d_rjobs,
                    (void*)b->g_rjobs})
        if (p) cudaFree(p);
    b->h_jobs = nullptr;
    b->h_begin = nullptr;
    b->h_rjobs = nullptr;
    b->d_jobs = b->g_jobs = nullptr;
    b->d_begin = b->g_begin = nullptr;
    b->d_rjobs = b->g_rjobs = nullptr;
    b->cap_iters = 0;
}

void batch_drop_graph(fvgs_batch* b) {
    if (b->graph.exec) cudaGraphExecDestroy(b->graph.exec);
    b->graph.exec = nullptr;
    b->graph.valid = false;
}

int batch_ensure_tables(fvgs_batch* b, int iters) {
    if (iters <= b->cap_iters) return FVGS_OK;
    batch_drop_graph(b);
    batch_free_tables(b);
    const size_t n = b->s.size(), it = (size_t)iters;
    if (cudaMallocHost(&b->h_jobs, sizeof(TrackJob) * n * it) != cudaSuccess ||
        cudaMallocHost(&b->h_begin, sizeof(uint32_t) * (n + 1) * it) != cudaSuccess ||
        cudaMallocHost(&b->h_rjobs, sizeof(ReduceJob) * n * it) != cudaSuccess ||
        cudaMalloc(&b->d_jobs, sizeof(TrackJob) * n * it) != cudaSuccess ||
        cudaMalloc(&b->g_jobs, sizeof(TrackJob) * n * it) != cudaSuccess ||
        cudaMalloc(&b->d_begin, sizeof(uint32_t) * (n + 1) * it) != cudaSuccess ||
        cudaMalloc(&b->g_begin, sizeof(uint32_t) * (n + 1) * it) != cudaSuccess ||
        cudaMalloc(&b->d_rjobs, sizeof(ReduceJob) * n * it) != cudaSuccess ||
        cudaMalloc(&b->g_rjobs, sizeof(ReduceJob) * n * it) != cudaSuccess) {
        cudaGetLastError();
        batch_free_tables(b);
        return FVGS_E_NOMEM;
    }
    b->cap_iters = iters;
    return FVGS_OK;
}

// Push a level's tile shape and staging batch to every session, so each one's
// plain frames blend exactly as the batch does.
void batch_apply_level(fvgs_batch* b, int l) {
    for (fvgs_session* s : b->s) {
        FrameLevel& f = s->lv[l];
        f.tile_w = b->tw[l];
        f.tile_h = b->th[l];
        f.track_variant = b->variant[l];
        f.tuned_w = f.W;
        f.tuned_h = f.H;
        ++s->gen;
    }
    batch_drop_graph(b);
}

// Fork the sessions' streams off the batch stream / join them back.
int batch_fork(fvgs_batch* b) {
    FV_CK(cudaEventRecord(b->ev_fork, b->stream));
    for (fvgs_session* s : b->s) FV_CK(cudaStreamWaitEvent(s->stream, b->ev_fork, 0));
    return FVGS_OK;
}

int batch_join(fvgs_batch* b) {
    for (size_t i = 0; i < b->s.size(); ++i) {
        FV_CK(cudaEventRecord(b->ev_join[i], b->s[i]->stream));
        FV_CK(cudaStreamWaitEvent(b->stream, b->ev_join[i], 0));
    }
    return FVGS_OK;
}

// Bin every session at level l (pose already on the device) and fill job
// table region `it`; returns the iteration's tile total in *total.
int batch_bin_level(fvgs_batch* b, const Request* reqs, int l, int it, uint32_t* total) {
    const size_t n = b->s.size();
    uint32_t t = 0;
    for (size_t i = 0; i < n; ++i) {
        fvgs_session* s = b->s[i];
        const FrameLevel& f = s->lv[l];
        FV_TRY(enqueue_bin(s, &reqs[i].K[l], f.W, f.H, b->tw[l], b->th[l]));
        TrackJob& j = b->h_jobs[(size_t)it * n + i];
        j.a = make_track_args(s, &reqs[i].K[l], f, false, false);
        j.a.variant = b->variant[l];
        j.a.split = 1;  // the persistent launch runs one work item per tile
        b->h_begin[(size_t)it * (n + 1) + i] = t;
        t += (uint32_t)s->last_T;
        ReduceJob& r = b->h_rjobs[(size_t)it * n + i];
        r.tile_out = s->tile_out;
        r.num_tiles = s->last_T;
        r.split = 1;
        r.pose = s->pose;
        r.out = s->jj;
        r.eig_eps = s->params.eig_eps;
        r.step_out = s->step;
    }
    b->h_begin[(size_t)it * (n + 1) + n] = t;
    *total = t;
    return FVGS_OK;
}

// One batched frame: the sessions' start poses (their pinned h_pose) to the
// device, the Gauss-Newton iterations of every level from the coarsest down,
// then every session's pose, last step and status back to pinned memory.
// Job tables: uploaded per iteration (eager) or read from the captured
// frame's tables (capture: filled on the host, uploaded after the capture).
int enqueue_batch_frame(fvgs_batch* b, const Request* reqs, bool capture) {
    const size_t n = b->s.size();
    TrackJob* jobs = capture ? b->g_jobs : b->d_jobs;
    uint32_t* begin = capture ? b->g_begin : b->d_begin;
    ReduceJob* rjobs = capture ? b->g_rjobs : b->d_rjobs;
    FV_TRY(batch_fork(b));
    for (fvgs_session* s : b->s) {
        FV_TRY(reset_status(s));
        FV_CK(cudaMemcpyAsync(s->d_pose_in, s->h_pose, sizeof(fvgs_pose), cudaMemcpyHostToDevice, s->stream));
        FV_CK(launch_chained(set_pose_dev_kernel, dim3(1), dim3(1), 0, s->stream, s->pose,
                             static_cast<const fvgs_pose*>(s->d_pose_in)));
    }
    int it = 0;
    for (int l = kMaxLevels - 1; l >= 0; --l) {
        for (int k = 0; k < reqs[0].iters[l]; ++k, ++it) {
            uint32_t total = 0;
            FV_TRY(batch_bin_level(b, reqs, l, it, &total));
            FV_TRY(batch_join(b));
            if (!capture) {
                FV_CK(cudaMemcpyAsync(jobs + (size_t)it * n, b->h_jobs + (size_t)it * n, sizeof(TrackJob) * n,
                                      cudaMemcpyHostToDevice, b->stream));
                FV_CK(cudaMemcpyAsync(begin + (size_t)it * (n + 1), b->h_begin + (size_t)it * (n + 1),
                                      sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, b->stream));
                FV_CK(cudaMemcpyAsync(rjobs + (size_t)it * n, b->h_rjobs + (size_t)it * n, sizeof(ReduceJob) * n,
                                      cudaMemcpyHostToDevice, b->stream));
            }
            FV_CK(launch_track_batch(jobs + (size_t)it * n, begin + (size_t)it * (n + 1), (int)n, total, b->tw[l],
                                     b->th[l], b->analytic, b->variant[l], b->counters, b->num_sms, b->stream));
            FV_CK(launch_track_reduce_batch(rjobs + (size_t)it * n, (int)n, b->stream));
            b->batch_launches += 2;
            FV_TRY(batch_fork(b));
        }
    }
    for (fvgs_session* s : b->s) {
        FV_TRY(ctx_normalize(s));
        FV_CK(cudaMemcpyAsync(s->h_devpose, s->pose, sizeof(DevPose), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaMemcpyAsync(s->h_jj + 42, s->step, sizeof(double) * 6, cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
    }
    return batch_join(b);
}

bool batch_key_matches(fvgs_batch* b, const Request* reqs) {
    const fvgs_batch::Graph& g = b->graph;
    if (!g.valid) return false;
    for (int l = 0; l < kMaxLevels; ++l)
        if (g.iters[l] != reqs[0].iters[l] || g.tw[l] != b->tw[l] || g.th[l] != b->th[l] ||
            g.variant[l] != b->variant[l])
            return false;
    for (size_t i = 0; i < b->s.size(); ++i) {
        fvgs_session* s = b->s[i];
        const fvgs_batch::Exit& e = g.exit[i];
        if (e.gen != s->gen || e.n_g != s->n_g) return false;
        BinSnap now;
        snap_take(s, now);
        if (!snap_same(e.entry, now)) return false;
        for (int l = 0; l < kMaxLevels; ++l) {
            if (reqs[i].iters[l] == 0) continue;
            const FrameLevel& f = s->lv[l];
            if (e.W[l] != f.W || e.H[l] != f.H || e.K[l].fx != reqs[i].K[l].fx || e.K[l].fy != reqs[i].K[l].fy ||
                e.K[l].cx != reqs[i].K[l].cx || e.K[l].cy != reqs[i].K[l].cy)
                return false;
        }
    }
    return true;
}

// Host-side binning state of a session (restored when a capture fails).
struct HostBinState {
    BinSnap snap;
    bool clean, keys, binned;
    int btw, bth, lw, lh, lt, ls;
    uint64_t launches[FVGS_K_COUNT];
    void save(fvgs_session* s) {
        snap_take(s, snap);
        clean = s->diff_clean;
        keys = s->keys_valid;
        binned = s->has_binning;
        btw = s->bin_tw;
        bth = s->bin_th;
        lw = s->last_W;
        lh = s->last_H;
        lt = s->last_T;
        ls = s->last_split;
        std::memcpy(launches, s->launches, sizeof(launches));
    }
    void restore(fvgs_session* s) const {
        snap_put(s, snap);
        s->diff_clean = clean;
        s->keys_valid = keys;
        s->has_binning = binned;
        s->bin_tw = btw;
        s->bin_th = bth;
        s->last_W = lw;
        s->last_H = lh;
        s->last_T = lt;
        s->last_split = ls;
        std::memcpy(s->launches, launches, sizeof(launches));
    }
};

// Launch the batched frame: replay the captured graph, or capture it, or
// (when some session cannot run from a graph) enqueue it eagerly.
int batch_launch(fvgs_batch* b, const Request* reqs) {
    const size_t n = b->s.size();
    bool graphable = true;
    for (size_t i = 0; i < n; ++i) graphable = graphable && frame_graphable(b->s[i], reqs[i]);
    if (!graphable) {
        ++b->eager;
        return enqueue_batch_frame(b, reqs, false);
    }
    if (batch_key_matches(b, reqs)) {
        FV_CK(cudaGraphLaunch(b->graph.exec, b->stream));
        for (size_t i = 0; i < n; ++i) {
            fvgs_session* s = b->s[i];
            const fvgs_batch::Exit& e = b->graph.exit[i];
            snap_put(s, e.exit);
            s->bin_tw = e.tw;
            s->bin_th = e.th;
            s->last_W = e.last_W;
            s->last_H = e.last_H;
            s->last_T = e.last_T;
            s->last_split = 1;  // batched launches run one CTA per tile
            s->keys_valid = false;
            s->has_binning = true;
            for (int c = 0; c < FVGS_K_COUNT; ++c) s->launches[c] += e.launches[c];
        }
        b->batch_launches += b->graph.batch_launches;
        ++b->graphed;
        return FVGS_OK;
    }
    batch_drop_graph(b);
    std::vector<HostBinState> before(n);
    std::vector<fvgs_batch::Exit> exit(n);
    for (size_t i = 0; i < n; ++i) {
        fvgs_session* s = b->s[i];
        before[i].save(s);
        fvgs_batch::Exit& e = exit[i];
        e.gen = s->gen;
        e.n_g = s->n_g;
        snap_take(s, e.entry);
        for (int l = 0; l < kMaxLevels; ++l) {
            e.W[l] = s->lv[l].W;
            e.H[l] = s->lv[l].H;
            e.K[l] = reqs[i].K[l];
        }
    }
    const uint64_t launches0 = b->batch_launches;
    cudaGraph_t graph = nullptr;
    int rc = FVGS_OK;
    cudaError_t ec = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (ec == cudaSuccess) {
        rc = enqueue_batch_frame(b, reqs, true);
        ec = cudaStreamEndCapture(b->stream, &graph);
    }
    if (rc == FVGS_OK && ec == cudaSuccess && graph) ec = cudaGraphInstantiate(&b->graph.exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (rc == FVGS_OK && ec == cudaSuccess && b->graph.exec) {
        // the captured launches read the tables filled on the host during the capture
        const int iters = total_iterations(reqs[0]);
        if (cudaMemcpy(b->g_jobs, b->h_jobs, sizeof(TrackJob) * n * iters, cudaMemcpyHostToDevice) != cudaSuccess ||
            cudaMemcpy(b->g_begin, b->h_begin, sizeof(uint32_t) * (n + 1) * iters, cudaMemcpyHostToDevice) !=
                cudaSuccess ||
            cudaMemcpy(b->g_rjobs, b->h_rjobs, sizeof(ReduceJob) * n * iters, cudaMemcpyHostToDevice) != cudaSuccess)
            ec = cudaErrorUnknown;
    }
    if (rc != FVGS_OK || ec != cudaSuccess || !b->graph.exec) {
        cudaGetLastError();
        batch_drop_graph(b);
        for (size_t i = 0; i < n; ++i) before[i].restore(b->s[i]);
        b->batch_launches = launches0;
        ++b->eager;
        return enqueue_batch_frame(b, reqs, false);
    }
    for (size_t i = 0; i < n; ++i) {
        fvgs_session* s = b->s[i];
        fvgs_batch::Exit& e = exit[i];
        snap_take(s, e.exit);
        e.tw = s->bin_tw;
        e.th = s->bin_th;
        e.last_W = s->last_W;
        e.last_H = s->last_H;
        e.last_T = s->last_T;
        for (int c = 0; c < FVGS_K_COUNT; ++c) e.launches[c] = s->launches[c] - before[i].launches[c];
    }
    fvgs_batch::Graph& g = b->graph;
    for (int l = 0; l < kMaxLevels; ++l) {
        g.iters[l] = reqs[0].iters[l];
        g.tw[l] = b->tw[l];
        g.th[l] = b->th[l];
        g.variant[l] = b->variant[l];
    }
    g.exit = exit;
    g.batch_launches = b->batch_launches - launches0;
    g.valid = true;
    FV_CK(cudaGraphLaunch(g.exec, b->stream));
    ++b->graphed;
    return FVGS_OK;
}

int batch_requests(fvgs_batch* b, const fvgs_pose* poses, const fvgs_intrinsics* K0, const int* iterations,
                   int levels, std::vector<Request>& reqs) {
    const size_t n = b->s.size();
    reqs.resize(n);
    for (size_t i = 0; i < n; ++i) {
        FV_TRY(pyramid_request(&poses[i], &K0[i], iterations, levels, -1.f, &reqs[i]));
        fvgs_session* s = b->s[i];
        // the persistent kernel has no compensated (precision-form) variant
        if (s->n_g == 0 || s->frame_pending || s->precision != FVGS_PRECISION_FP32) return FVGS_E_STATE;
        for (int l = 0; l < kMaxLevels; ++l)
            if (reqs[i].iters[l] > 0 && !s->lv[l].rgb) return FVGS_E_STATE;
    }
    return FVGS_OK;
}

}  // namespace

int fvgs_batch_create(fvgs_session* const* sessions, int n, fvgs_batch** out) {
    if (!sessions || n <= 0 || !out) return FVGS_E_INVALID;
    *out = nullptr;
    for (int i = 0; i < n; ++i) {
        if (!sessions[i] || sessions[i]->device != sessions[0]->device) return FVGS_E_INVALID;
        if ((sessions[i]->params.quirks ^ sessions[0]->params.quirks) & FVGS_Q_POSE_JAC_APPROX) return FVGS_E_INVALID;
        for (int k = 0; k < i; ++k)
            if (sessions[k] == sessions[i]) return FVGS_E_INVALID;
    }
    FV_CK(cudaSetDevice(sessions[0]->device));
    fvgs_batch* b = new (std::nothrow) fvgs_batch();
    if (!b) return FVGS_E_NOMEM;
    b->s.assign(sessions, sessions + n);
    b->device = sessions[0]->device;
    b->num_sms = sessions[0]->num_sms;
    b->analytic = !(sessions[0]->params.quirks & FVGS_Q_POSE_JAC_APPROX);
    for (int l = 0; l < kMaxLevels; ++l) {
        b->tw[l] = b->th[l] = 16;
        b->variant[l] = 0;
    }
    b->ev_join.assign(n, nullptr);
    bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess &&
              cudaMalloc(&b->counters, 2 * sizeof(uint32_t)) == cudaSuccess &&
              cudaMemset(b->counters, 0, 2 * sizeof(uint32_t)) == cudaSuccess;
    for (int i = 0; ok && i < n; ++i) ok = cudaEventCreateWithFlags(&b->ev_join[i], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        fvgs_batch_destroy(b);
        return FVGS_E_CUDA;
    }
    for (int l = 0; l < kMaxLevels; ++l) batch_apply_level(b, l);
    *out = b;
    return FVGS_OK;
}

int fvgs_batch_destroy(fvgs_batch* b) {
    if (!b) return FVGS_E_INVALID;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    batch_drop_graph(b);
    batch_free_tables(b);
    if (b->counters) cudaFree(b->counters);
    for (cudaEvent_t e : b->ev_join)
        if (e) cudaEventDestroy(e);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return FVGS_OK;
}

int fvgs_batch_set_level(fvgs_batch* b, int level, int tile_w, int tile_h, int batch_gaussians) {
    if (!b || level < 0 || level >= kMaxLevels || !track_tile_supported(tile_w, tile_h)) return FVGS_E_INVALID;
    if (batch_gaussians != 128 && batch_gaussians != 256 && batch_gaussians != 512) return FVGS_E_INVALID;
    b->tw[level] = tile_w;
    b->th[level] = tile_h;
    b->variant[level] = batch_gaussians == 128 ? 3 : (batch_gaussians == 512 ? 4 : 0);
    batch_apply_level(b, level);
    return FVGS_OK;
}

int fvgs_batch_run_pyramid(fvgs_batch* b, fvgs_pose* poses, const fvgs_intrinsics* K0, const int* iterations,
                           int levels) {
    if (!b || !poses || !K0 || !iterations) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(b->device));
    std::vector<Request> reqs;
    FV_TRY(batch_requests(b, poses, K0, iterations, levels, reqs));
    const size_t n = b->s.size();
    FV_TRY(batch_ensure_tables(b, std::max(1, total_iterations(reqs[0]))));
    for (size_t i = 0; i < n; ++i) *b->s[i]->h_pose = reqs[i].pose;
    FV_TRY(batch_launch(b, reqs.data()));
    FV_CK(cudaStreamSynchronize(b->stream));
    int first_error = FVGS_OK;
    for (size_t i = 0; i < n; ++i) {
        fvgs_session* s = b->s[i];
        collect_timing(s);
        int retry = 0;
        int rc = check_status(s, &retry);
        if (rc == FVGS_OK && retry) {
            // instance overflow (buffers grown) or an inconsistent incremental
            // binning: this session's frame again, alone, with the same tiles
            ++s->frames_eager;
            rc = run_request_eager(s, reqs[i], &poses[i], nullptr);
        } else if (rc == FVGS_OK) {
            for (int k = 0; k < 3; ++k) poses[i].position[k] = s->h_devpose->t[k];
            for (int k = 0; k < 4; ++k) poses[i].orientation[k] = s->h_devpose->q[k];
            s->has_track = true;
        }
        if (rc != FVGS_OK && first_error == FVGS_OK) first_error = rc;
    }
    return first_error;
}

int fvgs_batch_autotune(fvgs_batch* b, const fvgs_pose* poses, const fvgs_intrinsics* K0, const int* iterations,
                        int levels, int reps, int* config_out, float* ms_out) {
    if (!b || !poses || !K0 || !iterations) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(b->device));
    std::vector<Request> reqs;
    FV_TRY(batch_requests(b, poses, K0, iterations, levels, reqs));
    FV_TRY(batch_ensure_tables(b, std::max(1, total_iterations(reqs[0]))));
    reps = std::max(1, std::min(reps, 16));
    const size_t n = b->s.size();
    const int shapes[3][2] = {{16, 16}, {8, 8}, {32, 8}};
    const int variants[3] = {3, 0, 4};  // batches of 128, 256, 512
    std::vector<cudaEvent_t> ev(2 * (size_t)reps, nullptr);
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            for (auto& e2 : ev)
                if (e2) cudaEventDestroy(e2);
            return FVGS_E_CUDA;
        }
    int rc = FVGS_OK;
    for (int l = 0; l < levels && l < kMaxLevels && rc == FVGS_OK; ++l) {
        if (reqs[0].iters[l] == 0) continue;
        float best = INFINITY;
        int best_shape = 0, best_variant = 0;
        for (int sh = 0; sh < 3 && rc == FVGS_OK; ++sh) {
            b->tw[l] = shapes[sh][0];
            b->th[l] = shapes[sh][1];
            uint32_t total = 0;
            // bin every session at its pose with this tile shape (again after an overflow)
            for (int attempt = 0;; ++attempt) {
                if (attempt == 4) {
                    rc = FVGS_E_CAPACITY;
                    break;
                }
                if ((rc = batch_fork(b)) != FVGS_OK) break;
                for (size_t i = 0; i < n && rc == FVGS_OK; ++i) {
                    rc = reset_status(b->s[i]);
                    if (rc == FVGS_OK) rc = set_pose(b->s[i], &reqs[i].pose);
                }
                if (rc == FVGS_OK) rc = batch_bin_level(b, reqs.data(), l, 0, &total);
                if (rc == FVGS_OK) rc = batch_join(b);
                for (size_t i = 0; i < n && rc == FVGS_OK; ++i)
                    if (cudaMemcpyAsync(b->s[i]->h_st, b->s[i]->st, sizeof(DevStatus), cudaMemcpyDeviceToHost,
                                        b->stream) != cudaSuccess)
                        rc = FVGS_E_CUDA;
                if (rc == FVGS_OK && cudaStreamSynchronize(b->stream) != cudaSuccess) rc = FVGS_E_CUDA;
                if (rc != FVGS_OK) break;
                int any = 0;
                for (size_t i = 0; i < n && rc == FVGS_OK; ++i) {
                    collect_timing(b->s[i]);
                    int retry = 0;
                    rc = check_status(b->s[i], &retry);
                    any |= retry;
                }
                if (rc != FVGS_OK || !any) break;
            }
            if (rc != FVGS_OK) break;
            if (cudaMemcpy(b->d_jobs, b->h_jobs, sizeof(TrackJob) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
                cudaMemcpy(b->d_begin, b->h_begin, sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice) !=
                    cudaSuccess) {
                rc = FVGS_E_CUDA;
                break;
            }
            for (int vi = 0; vi < 3 && rc == FVGS_OK; ++vi) {
                const int v = variants[vi];
                for (int r = 0; r < reps && rc == FVGS_OK; ++r) {
                    if (cudaEventRecord(ev[2 * r], b->stream) != cudaSuccess ||
                        launch_track_batch(b->d_jobs, b->d_begin, (int)n, total, b->tw[l], b->th[l], b->analytic, v,
                                           b->counters, b->num_sms, b->stream) != cudaSuccess ||
                        cudaEventRecord(ev[2 * r + 1], b->stream) != cudaSuccess)
                        rc = FVGS_E_CUDA;
                }
                if (rc == FVGS_OK && cudaStreamSynchronize(b->stream) != cudaSuccess) rc = FVGS_E_CUDA;
                if (rc != FVGS_OK) break;
                std::vector<float> t(reps);
                for (int r = 0; r < reps; ++r) cudaEventElapsedTime(&t[r], ev[2 * r], ev[2 * r + 1]);
                std::sort(t.begin(), t.end());
                const float med = t[reps / 2];
                if (ms_out) ms_out[l * 9 + sh * 3 + vi] = med;
                if (med < best) {
                    best = med;
                    best_shape = sh;
                    best_variant = v;
                }
            }
        }
        if (rc != FVGS_OK) break;
        b->tw[l] = shapes[best_shape][0];
        b->th[l] = shapes[best_shape][1];
        b->variant[l] = best_variant;
        if (config_out) {
            config_out[3 * l] = b->tw[l];
            config_out[3 * l + 1] = b->th[l];
            config_out[3 * l + 2] = track_variant_batch(best_variant);
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int l = 0; l < kMaxLevels; ++l) batch_apply_level(b, l);
    if (rc != FVGS_OK) cudaGetLastError();
    return rc;
}

int fvgs_batch_stats(const fvgs_batch* b, uint64_t* graphed, uint64_t* eager, uint64_t* batch_launches) {
    if (!b) return FVGS_E_INVALID;
    if (graphed) *graphed = b->graphed;
    if (eager) *eager = b->eager;
    if (batch_launches) *batch_launches = b->batch_launches;
    return FVGS_OK;
}

int fvgs_session_frame_stats(const fvgs_session* s, uint64_t* graphed, uint64_t* eager) {
    if (!s) return FVGS_E_INVALID;
    if (graphed) *graphed = s->frames_graphed;
    if (eager) *eager = s->frames_eager;
    return FVGS_OK;
}

int fvgs_render(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height, float* rgb,
                float* depth, float* final_T, uint32_t* n_contrib) {
    if (!s || !valid_pose(pose) || !K) return FVGS_E_INVALID;
    FV_TRY(check_view(s, width, height));
    FV_CK(cudaSetDevice(s->device));
    const size_t px = (size_t)width * height;
    FV_TRY(ensure_images(s, px));
    FrameLevel view;
    view.W = width;
    view.H = height;
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, width, height, s->params.tile_w, s->params.tile_h));
        FV_TRY(enqueue_track(s, K, view, true, true));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;
        if (rgb) FV_CK(cudaMemcpyAsync(rgb, s->img_color, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
        if (depth) FV_CK(cudaMemcpyAsync(depth, s->img_depth, sizeof(float) * px, cudaMemcpyDefault, s->stream));
        if (final_T) FV_CK(cudaMemcpyAsync(final_T, s->img_T, sizeof(float) * px, cudaMemcpyDefault, s->stream));
        if (n_contrib) FV_CK(cudaMemcpyAsync(n_contrib, s->img_nc, sizeof(uint32_t) * px, cudaMemcpyDefault, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

int fvgs_render_view(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                     float* rgb, float* depth, uint8_t* rgb8) {
    if (!s || !valid_pose(pose) || !K) return FVGS_E_INVALID;
    FV_TRY(check_view(s, width, height));
    FV_CK(cudaSetDevice(s->device));
    const size_t px = (size_t)width * height;
    FV_TRY(ensure_images(s, px));
    // the 8-bit copy lives in the contributor-count image (4 bytes per pixel)
    uint8_t* rgb8_dev = rgb8 ? reinterpret_cast<uint8_t*>(s->img_nc) : nullptr;
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, width, height, s->params.tile_w, s->params.tile_h));
        RenderArgs ra{};
        ra.rec0 = s->rec0;
        ra.rec1 = s->rec1;
        ra.rec2 = s->rec2;
        ra.ranges = s->ranges;
        ra.indices = s->vals;
        ra.n_list = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
        ra.n_gauss = s->n_g;
        ra.W = width;
        ra.H = height;
        ra.ntx = (width + s->params.tile_w - 1) / s->params.tile_w;
        ra.nty = (height + s->params.tile_h - 1) / s->params.tile_h;
        ra.quirks = s->params.quirks;
        ra.out_rgb = s->img_color;
        ra.out_depth = s->img_depth;
        ra.out_rgb8 = rgb8_dev;
        {
            KScope k(s, FVGS_K_RENDER, 1);
            FV_CK(launch_render_view(ra, s->stream));
        }
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;
        if (rgb) FV_CK(cudaMemcpyAsync(rgb, s->img_color, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
        if (depth) FV_CK(cudaMemcpyAsync(depth, s->img_depth, sizeof(float) * px, cudaMemcpyDefault, s->stream));
        if (rgb8) FV_CK(cudaMemcpyAsync(rgb8, rgb8_dev, 3 * px, cudaMemcpyDefault, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

int fvgs_session_set_timing(fvgs_session* s, uint32_t class_mask) {
    if (!s) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    FV_CK(cudaStreamSynchronize(s->stream));
    collect_timing(s);
    s->timing_mask = class_mask;
    ++s->gen;
    return FVGS_OK;
}

int fvgs_session_get_timing(fvgs_session* s, double* ms, uint64_t* launches, uint64_t* timed_launches, int reset) {
    if (!s) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    FV_CK(cudaStreamSynchronize(s->stream));
    collect_timing(s);
    for (int k = 0; k < FVGS_K_COUNT; ++k) {
        if (ms) ms[k] = s->kernel_ms[k];
        if (launches) launches[k] = s->launches[k];
        if (timed_launches) timed_launches[k] = s->timed_launches[k];
        if (reset) {
            s->kernel_ms[k] = 0.0;
            s->launches[k] = 0;
            s->timed_launches[k] = 0;
        }
    }
    return FVGS_OK;
}

int fvgs_map_step(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level, float eta) {
    if (!s || !valid_pose(pose) || !K || level < 0 || level >= kMaxLevels || !(eta >= 0.f)) return FVGS_E_INVALID;
    const FrameLevel& f = s->lv[level];
    if (!f.rgb) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    const bool cap = (s->params.quirks & FVGS_Q_MAP_CAP256) != 0;
    FV_TRY(ensure_map_buffers(s, (size_t)f.W * f.H, cap));
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, f.W, f.H, s->params.tile_w, s->params.tile_h));
        FV_TRY(enqueue_map(s, K, f, eta));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) {
            // the instance buffers grew; checkpoint slots follow capacity
            FV_TRY(ensure_map_buffers(s, (size_t)f.W * f.H, cap));
            continue;
        }
        s->has_map = true;
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

int fvgs_download_map_state(fvgs_session* s, float* final_T, uint32_t* n_contrib, float* color, float* depth,
                            float* delta2d, float* delta3d) {
    if (!s) return FVGS_E_INVALID;
    if (!s->has_map) return FVGS_E_STATE;
    if (delta3d && !(s->debug & FVGS_DEBUG_MAPPING)) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    const size_t px = (size_t)s->m_W * s->m_H, n = s->n_g;
    if (final_T) FV_CK(cudaMemcpyAsync(final_T, s->m_final_T, sizeof(float) * px, cudaMemcpyDefault, s->stream));
    if (n_contrib) FV_CK(cudaMemcpyAsync(n_contrib, s->m_n_contrib, sizeof(uint32_t) * px, cudaMemcpyDefault, s->stream));
    if (color) FV_CK(cudaMemcpyAsync(color, s->m_color, sizeof(float) * 3 * px, cudaMemcpyDefault, s->stream));
    if (depth) FV_CK(cudaMemcpyAsync(depth, s->m_depth, sizeof(float) * px, cudaMemcpyDefault, s->stream));
    if (delta2d) FV_CK(cudaMemcpyAsync(delta2d, s->delta2d, sizeof(float) * 16 * n, cudaMemcpyDefault, s->stream));
    if (delta3d) FV_CK(cudaMemcpyAsync(delta3d, s->dbg_delta3d, sizeof(float) * 16 * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}


// ---------------------------------------------------------------------------
// Map maintenance (GSSlam::removeOutliers, prune, computeCovisibilityRatio,
// src/GSSlam.cu:1467-1904).
namespace {

// Bin one view and flag the Gaussians that some pixel of it sees.  vis must be
// cleared first; returns the view's instance count in *n_inst.
int visibility_pass(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int W, int H, uint8_t* vis,
                    uint32_t* n_inst) {
    FV_TRY(check_view(s, W, H));
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, W, H, s->params.tile_w, s->params.tile_h));
        FV_CK(cudaMemsetAsync(vis, 0, s->n_g, s->stream));
        VisArgs va{};
        va.rec0 = s->rec0;
        va.rec1 = s->rec1;
        va.ranges = s->ranges;
        va.indices = s->vals;
        va.n_list = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
        va.n_gauss = s->n_g;
        va.W = W;
        va.H = H;
        va.ntx = (W + s->params.tile_w - 1) / s->params.tile_w;
        va.nty = (H + s->params.tile_h - 1) / s->params.tile_h;
        va.cap = (s->params.quirks & FVGS_Q_VIS_CAP256) ? 256 : 0;
        va.vis = vis;
        {
            KScope k(s, FVGS_K_MAINT, 1);
            FV_CK(launch_visibility(va, s->stream));
        }
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;
        *n_inst = s->h_st->n_instances;
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

// Enqueue marking (prune criteria or outlier scores), the survivor scan and,
// when remove is set, the scatter into the second set of planes.
int enqueue_mark_compact(fvgs_session* s, MarkMode mode, const MarkArgs& proto, bool remove) {
    const uint32_t n = s->n_g;
    MarkArgs ma = proto;
    ma.n = n;
    ma.states = s->mk_states;
    ma.block_keep = s->mk_block_keep;
    KScope k(s, FVGS_K_MAINT, remove ? 3 : 2);
    FV_CK(launch_mark(mode, ma, s->stream));
    FV_CK(launch_compact_scan(s->mk_block_keep, n, s->mk_block_base, s->mk_ctr, s->stream));
    if (remove) {
        const bool move_adam = !(s->params.quirks & FVGS_Q_ADAM_STAY);
        if (move_adam && !s->adam_alt) FV_TRY(dev_alloc(s, &s->adam_alt, 9 * (size_t)s->cap_g));
        CompactArgs ca{};
        ca.n = n;
        ca.states = s->mk_states;
        ca.block_base = s->mk_block_base;
        ca.counters = s->mk_ctr;
        ca.pos = s->pos;
        ca.scale = s->scale;
        ca.rot = s->rot;
        ca.col = s->col;
        ca.pos_out = s->pos_alt;
        ca.scale_out = s->scale_alt;
        ca.rot_out = s->rot_alt;
        ca.col_out = s->col_alt;
        ca.adam = move_adam ? s->adam : nullptr;
        ca.adam_out = move_adam ? s->adam_alt : nullptr;
        ca.cap = s->cap_g;
        FV_CK(launch_compact_scatter(ca, s->stream));
    }
    FV_CK(cudaMemcpyAsync(s->h_mk_ctr, s->mk_ctr, sizeof(uint32_t) * 2, cudaMemcpyDeviceToHost, s->stream));
    s->mk_n = n;
    return FVGS_OK;
}

// After the stream is synchronised: adopt the compacted planes.
int finish_compact(fvgs_session* s, bool remove, uint32_t* n_marked) {
    const uint32_t removed = s->h_mk_ctr[1];
    if (n_marked) *n_marked = removed;
    if (!remove || removed == 0) return FVGS_OK;
    std::swap(s->pos, s->pos_alt);
    std::swap(s->scale, s->scale_alt);
    std::swap(s->rot, s->rot_alt);
    std::swap(s->col, s->col_alt);
    if (!(s->params.quirks & FVGS_Q_ADAM_STAY)) std::swap(s->adam, s->adam_alt);
    s->n_g = s->h_mk_ctr[0];
    FV_CK(cand_drop(s));
    // every per-Gaussian index of the last binning is stale now
    s->has_binning = s->has_track = s->has_map = false;
    ctx_drop_history(s);
    s->keys_valid = false;
    s->dbg_proj_valid = false;
    ++s->gen;  // captured frame graphs hold the old plane addresses
    return refresh_reduced(s);
}

}  // namespace

int fvgs_visibility(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int width, int height,
                    uint8_t* visibility, uint32_t* n_visible) {
    if (!s || !valid_pose(pose) || !K) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    if (s->n_g == 0) {
        if (n_visible) *n_visible = 0;
        return FVGS_OK;
    }
    uint32_t n_inst = 0;
    FV_TRY(visibility_pass(s, pose, K, width, height, s->vis_a, &n_inst));
    FV_CK(cudaMemsetAsync(s->mk_ctr + 2, 0, sizeof(uint32_t) * 2, s->stream));
    {
        KScope k(s, FVGS_K_MAINT, 1);
        FV_CK(launch_covis_count(s->vis_a, s->vis_a, s->n_g, s->mk_ctr + 2, s->stream));
    }
    FV_CK(cudaMemcpyAsync(s->h_mk_ctr + 2, s->mk_ctr + 2, sizeof(uint32_t) * 2, cudaMemcpyDeviceToHost, s->stream));
    if (visibility) FV_CK(cudaMemcpyAsync(visibility, s->vis_a, s->n_g, cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    collect_timing(s);
    if (n_visible) *n_visible = s->h_mk_ctr[3];
    return FVGS_OK;
}

int fvgs_covisibility(fvgs_session* s, const fvgs_pose* pose_a, const fvgs_intrinsics* K_a, int width_a,
                      int height_a, const fvgs_pose* pose_b, const fvgs_intrinsics* K_b, int width_b, int height_b,
                      uint32_t* n_inter, uint32_t* n_union, float* ratio) {
    if (!s || !valid_pose(pose_a) || !K_a || !valid_pose(pose_b) || !K_b) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    if (n_inter) *n_inter = 0;
    if (n_union) *n_union = 0;
    if (s->n_g == 0) {  // the reference returns 1 for an empty map
        if (ratio) *ratio = 1.0f;
        return FVGS_OK;
    }
    if (ratio) *ratio = 0.0f;
    uint32_t n_inst = 0;
    FV_TRY(visibility_pass(s, pose_a, K_a, width_a, height_a, s->vis_a, &n_inst));
    if (n_inst == 0) return FVGS_OK;  // no instances in a view: ratio 0, as the reference
    FV_TRY(visibility_pass(s, pose_b, K_b, width_b, height_b, s->vis_b, &n_inst));
    if (n_inst == 0) return FVGS_OK;
    FV_CK(cudaMemsetAsync(s->mk_ctr + 2, 0, sizeof(uint32_t) * 2, s->stream));
    {
        KScope k(s, FVGS_K_MAINT, 1);
        FV_CK(launch_covis_count(s->vis_a, s->vis_b, s->n_g, s->mk_ctr + 2, s->stream));
    }
    FV_CK(cudaMemcpyAsync(s->h_mk_ctr + 2, s->mk_ctr + 2, sizeof(uint32_t) * 2, cudaMemcpyDeviceToHost, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    collect_timing(s);
    const uint32_t inter = s->h_mk_ctr[2], uni = s->h_mk_ctr[3];
    if (n_inter) *n_inter = inter;
    if (n_union) *n_union = uni;
    if (ratio) *ratio = uni == 0 ? 0.0f : (float)inter / (float)uni;
    return FVGS_OK;
}

int fvgs_remove_outliers(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int level,
                         float threshold, int remove, uint32_t* n_marked) {
    if (!s || !valid_pose(pose) || !K || level < 0 || level >= kMaxLevels) return FVGS_E_INVALID;
    const FrameLevel& f = s->lv[level];
    if (!f.depth || f.W <= 0 || f.H <= 0) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    if (n_marked) *n_marked = 0;
    s->mk_n = 0;
    if (s->n_g == 0) return FVGS_OK;
    FV_TRY(check_view(s, f.W, f.H));
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, f.W, f.H, s->params.tile_w, s->params.tile_h));
        FV_CK(cudaMemsetAsync(s->mk_total_alpha, 0, sizeof(float) * s->n_g, s->stream));
        FV_CK(cudaMemsetAsync(s->mk_outlier_prob, 0, sizeof(float) * s->n_g, s->stream));
        OutlierArgs oa{};
        oa.rec0 = s->rec0;
        oa.rec1 = s->rec1;
        oa.rec2 = s->rec2;
        oa.ranges = s->ranges;
        oa.indices = s->vals;
        oa.n_list = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
        oa.n_gauss = s->n_g;
        oa.obs_depth = f.depth;
        oa.W = f.W;
        oa.H = f.H;
        oa.ntx = (f.W + s->params.tile_w - 1) / s->params.tile_w;
        oa.nty = (f.H + s->params.tile_h - 1) / s->params.tile_h;
        oa.total_alpha = s->mk_total_alpha;
        oa.outlier_prob = s->mk_outlier_prob;
        {
            KScope k(s, FVGS_K_MAINT, 1);
            FV_CK(launch_outliers(oa, s->stream));
        }
        MarkArgs ma{};
        ma.total_alpha = s->mk_total_alpha;
        ma.outlier_prob = s->mk_outlier_prob;
        ma.threshold = threshold;
        FV_TRY(enqueue_mark_compact(s, kMarkOutliers, ma, remove != 0));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;  // the planes were only read: repeat from the start
        s->mk_scores = true;
        return finish_compact(s, remove != 0, n_marked);
    }
    return FVGS_E_CAPACITY;
}

int fvgs_prune(fvgs_session* s, float alpha_threshold, float scale_ratio_threshold, float min_scale, int remove,
               uint32_t* n_marked) {
    if (!s) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    if (n_marked) *n_marked = 0;
    s->mk_n = 0;
    if (s->n_g == 0) return FVGS_OK;
    MarkArgs ma{};
    ma.scale = s->scale;
    ma.col = s->col;
    ma.alpha_thr = alpha_threshold;
    ma.ratio_thr = scale_ratio_threshold;
    ma.min_scale = min_scale;
    FV_TRY(enqueue_mark_compact(s, kMarkPrune, ma, remove != 0));
    FV_CK(cudaStreamSynchronize(s->stream));
    collect_timing(s);
    s->mk_scores = false;
    return finish_compact(s, remove != 0, n_marked);
}

int fvgs_download_marks(fvgs_session* s, uint8_t* states, float* total_alpha, float* outlier_prob, uint32_t n) {
    if (!s || n > s->mk_n) return FVGS_E_INVALID;
    if ((total_alpha || outlier_prob) && !s->mk_scores) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    if (n == 0) return FVGS_OK;
    if (states) FV_CK(cudaMemcpyAsync(states, s->mk_states, n, cudaMemcpyDefault, s->stream));
    if (total_alpha)
        FV_CK(cudaMemcpyAsync(total_alpha, s->mk_total_alpha, sizeof(float) * n, cudaMemcpyDefault, s->stream));
    if (outlier_prob)
        FV_CK(cudaMemcpyAsync(outlier_prob, s->mk_outlier_prob, sizeof(float) * n, cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}

int fvgs_download_adam_state(fvgs_session* s, float* state, uint32_t n) {
    if (!s || n > s->n_g || (n && !state)) return FVGS_E_INVALID;
    FV_CK(cudaSetDevice(s->device));
    if (n == 0) return FVGS_OK;
    // nine planes of n float4, plane p at state + 4 n p
    for (int p = 0; p < 9; ++p)
        FV_CK(cudaMemcpyAsync(state + (size_t)4 * n * p, s->adam + (size_t)p * s->cap_g, sizeof(float4) * n,
                              cudaMemcpyDefault, s->stream));
    FV_CK(cudaStreamSynchronize(s->stream));
    return FVGS_OK;
}


// ---------------------------------------------------------------------------
// Seeding from the camera frame (GSSlam::initializeGaussiansFromRgbd,
// src/GSSlam.cu:271-407; GSSlam::densify, src/GSSlam.cu:1351-1465).
namespace {

SeedArgs seed_args(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int sample) {
    SeedArgs a{};
    a.bgr = s->pre_u8[0];
    a.depth = s->lv[0].depth;
    a.W = s->pre_w;
    a.H = s->pre_h;
    a.sample = sample;
    a.ncx = (a.W + sample - 1) / sample;
    a.ncy = (a.H + sample - 1) / sample;
    a.K = *K;
    a.pose_q = make_float4(pose->orientation[0], pose->orientation[1], pose->orientation[2], pose->orientation[3]);
    a.pose_t = make_float3(pose->position[0], pose->position[1], pose->position[2]);
    a.cap = s->cap_g;
    a.block_keep = s->sd_block_keep;
    a.block_base = s->sd_block_base;
    a.pos = s->pos;
    a.scale = s->scale;
    a.rot = s->rot;
    a.col = s->col;
    return a;
}

int enqueue_seed(fvgs_session* s, SeedMode mode, const SeedArgs& a) {
    const uint32_t cells = (uint32_t)a.ncx * (uint32_t)a.ncy;
    if ((cells + kCompactBlock - 1) / kCompactBlock > s->sd_blocks) return FVGS_E_INVALID;
    KScope k(s, FVGS_K_MAINT, 3);
    FV_CK(launch_seed_count(mode, a, s->stream));
    FV_CK(launch_compact_scan(s->sd_block_keep, cells, s->sd_block_base, s->mk_ctr, s->stream));
    FV_CK(launch_seed_emit(mode, a, s->stream));
    FV_CK(cudaMemcpyAsync(s->h_mk_ctr, s->mk_ctr, sizeof(uint32_t) * 2, cudaMemcpyDeviceToHost, s->stream));
    return FVGS_OK;
}

int map_grew(fvgs_session* s, uint32_t n) {
    s->n_g = n;
    FV_CK(cand_drop(s));
    s->has_binning = s->has_track = s->has_map = false;
    ctx_drop_history(s);  // the new Gaussians have no previous binning
    s->keys_valid = false;
    s->dbg_proj_valid = false;
    ++s->gen;
    return refresh_reduced(s);
}

}  // namespace

int fvgs_init_gaussians(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int sample_px,
                        float init_scale, float init_opacity, uint32_t* n_gaussians) {
    if (!s || !valid_pose(pose) || !K || sample_px < 1) return FVGS_E_INVALID;
    if (!s->pre_valid) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    SeedArgs a = seed_args(s, pose, K, sample_px);
    a.init_scale = init_scale;
    a.init_opacity = init_opacity;
    a.n0 = 0;
    // a new map: optimiser state starts at zero, as the reference's empty adam_states_
    FV_CK(cudaMemsetAsync(s->adam, 0, sizeof(float4) * 9 * (size_t)s->cap_g, s->stream));
    FV_TRY(enqueue_seed(s, kSeedInit, a));
    FV_CK(cudaStreamSynchronize(s->stream));
    collect_timing(s);
    FV_TRY(map_grew(s, std::min<uint32_t>(s->h_mk_ctr[0], s->cap_g)));
    if (n_gaussians) *n_gaussians = s->n_g;
    return FVGS_OK;
}

int fvgs_densify(fvgs_session* s, const fvgs_pose* pose, const fvgs_intrinsics* K, int sample_px, float* mask,
                 uint32_t* n_added) {
    if (!s || !valid_pose(pose) || !K || sample_px < 1) return FVGS_E_INVALID;
    if (!s->pre_valid) return FVGS_E_STATE;
    FV_CK(cudaSetDevice(s->device));
    if (n_added) *n_added = 0;
    if (s->n_g == 0) return FVGS_OK;  // as the reference: nothing to densify against
    const int W = s->pre_w, H = s->pre_h;
    FV_TRY(check_view(s, W, H));
    const size_t px = (size_t)W * H;
    FV_TRY(ensure_images(s, px));
    for (int attempt = 0; attempt < 4; ++attempt) {
        FV_TRY(reset_status(s));
        FV_TRY(set_pose(s, pose));
        FV_TRY(enqueue_bin(s, K, W, H, s->params.tile_w, s->params.tile_h));
        DensityArgs da{};
        da.rec0 = s->rec0;
        da.rec1 = s->rec1;
        da.rec2 = s->rec2;
        da.ranges = s->ranges;
        da.indices = s->vals;
        da.n_list = (uint32_t)std::min<uint64_t>(s->cap_inst, 0xffffffffu);
        da.n_gauss = s->n_g;
        da.obs_depth = s->lv[0].depth;
        da.W = W;
        da.H = H;
        da.ntx = (W + s->params.tile_w - 1) / s->params.tile_w;
        da.nty = (H + s->params.tile_h - 1) / s->params.tile_h;
        da.mask = s->img_T;  // the density mask lives in the final-transmittance image
        {
            KScope k(s, FVGS_K_MAINT, 1);
            FV_CK(launch_density_mask(da, s->stream));
        }
        SeedArgs a = seed_args(s, pose, K, sample_px);
        a.mask = s->img_T;
        a.n0 = s->n_g;
        a.adam = (s->params.quirks & FVGS_Q_ADAM_STAY) ? nullptr : s->adam;
        FV_TRY(enqueue_seed(s, kSeedDensify, a));
        FV_CK(cudaMemcpyAsync(s->h_st, s->st, sizeof(DevStatus), cudaMemcpyDeviceToHost, s->stream));
        if (mask) FV_CK(cudaMemcpyAsync(mask, s->img_T, sizeof(float) * px, cudaMemcpyDefault, s->stream));
        FV_CK(cudaStreamSynchronize(s->stream));
        collect_timing(s);
        int retry = 0;
        FV_TRY(check_status(s, &retry));
        if (retry) continue;  // seeds past the map were written but not adopted
        const uint64_t total = (uint64_t)s->n_g + s->h_mk_ctr[0];
        const uint32_t n_new = (uint32_t)std::min<uint64_t>(total, s->cap_g);
        if (n_added) *n_added = n_new - s->n_g;
        if (n_new != s->n_g) FV_TRY(map_grew(s, n_new));
        return FVGS_OK;
    }
    return FVGS_E_CAPACITY;
}

}  // extern "C"
