// binning.cu -- projection, tile counting, instance offsets, key emission and
// per-tile ranges for sm_103a.
//
// Reference path: GSSlam::prepareRasterization (src/GSSlam.cu:408-646) with
// projectGaussiansWorldToScreen_kernel (src/GSCudaKernels.cu:345-476),
// countTilesPerGaussian_kernel (549-593), thrust::exclusive_scan
// (src/GSSlam.cu:556-572), generateTileHashes_kernel (596-667) and
// computeIndicesRanges_kernel (669-707).
//
// Differences in structure (same results):
//  * projection and counting are one kernel; the tile rectangle is computed
//    once and kept in a 32-byte binning record;
//  * the instance total never leaves the device: later kernels read it from
//    DevStatus, so a tracking iteration needs no host round trip;
//  * keys are emitted by whole warps over the concatenated tile lists of 32
//    Gaussians, so writes are contiguous and a large splat does not stall a
//    thread while its neighbours idle.
// All key-critical arithmetic uses explicit round-to-nearest intrinsics in the
// fixed order that the CPU restatement mirrors, so keys are bit-exact.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

// Add the inclusive tile rectangle [x0..x1] x [y0..y1] to a 2-D difference
// grid of row pitch gw = ntx + 1; tile counts are the grid's 2-D prefix sums.
__device__ __forceinline__ void add_rect(int* d, int gw, int x0, int y0, int x1, int y1) {
    atomicAdd(&d[y0 * gw + x0], 1);
    atomicAdd(&d[y0 * gw + x1 + 1], -1);
    atomicAdd(&d[(y1 + 1) * gw + x0], -1);
    atomicAdd(&d[(y1 + 1) * gw + x1 + 1], 1);
}

// One Gaussian: p is its position, prev_count its instance count in the
// previous binning (incremental mode), R and tw the camera pose; grid: the
// count and entering difference grids (a.tile_diff, or the CTA's copy in
// shared memory).
__device__ __forceinline__ void project_one(const ProjectArgs& a, int i, float4 p, uint32_t prev_count,
                                            const float (&R)[3][3], const float (&tw)[3], int* grid) {
    const fvgs_intrinsics K = a.K;

    float u = 0.f, v = 0.f, z = 0.f, cxx = 0.f, cyy = 0.f, cxy = 0.f;
    float ixx = 0.f, iyy = 0.f, ixy = 0.f, phx = 0.f, phy = 0.f;
    float4 geo0 = make_float4(0.f, 0.f, 0.f, 0.f), geo1 = geo0;  // camera-frame covariance and mean
    bool visible = false;
    {
        const float d0 = __fsub_rn(p.x, tw[0]);
        const float d1 = __fsub_rn(p.y, tw[1]);
        const float d2 = __fsub_rn(p.z, tw[2]);
        // a*b + c*d + e*f as nvcc contracts the reference's expression
        const float pcx = __fmaf_rn(R[2][0], d2, __fmaf_rn(R[0][0], d0, __fmul_rn(R[1][0], d1)));
        const float pcy = __fmaf_rn(R[2][1], d2, __fmaf_rn(R[0][1], d0, __fmul_rn(R[1][1], d1)));
        const float pcz = __fmaf_rn(R[2][2], d2, __fmaf_rn(R[0][2], d0, __fmul_rn(R[1][2], d1)));
        if (pcz > 0.0f) {
            const float inv_z = __fdiv_rn(1.0f, pcz);
            const float uu = __fmaf_rn(K.fx, __fmul_rn(pcx, inv_z), K.cx);
            const float vv = __fmaf_rn(K.fy, __fmul_rn(pcy, inv_z), K.cy);
            if (!(uu < 0.0f || uu >= (float)a.W || vv < 0.0f || vv >= (float)a.H)) {
                visible = true;
                u = uu;
                v = vv;
                z = pcz;
                float4 s, qg4;
                if (a.attr_sr) {
                    unpack_sr(a.attr_sr[i], s, qg4);
                } else {
                    s = a.scale[i];
                    qg4 = a.rot[i];
                }
                const float qg[4] = {qg4.x, qg4.y, qg4.z, qg4.w};
                float Rg[3][3];
                quat_to_R(qg, Rg);
                float M[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    M[r][0] = __fmul_rn(Rg[r][0], s.x);
                    M[r][1] = __fmul_rn(Rg[r][1], s.y);
                    M[r][2] = __fmul_rn(Rg[r][2], s.z);
                }
                float S[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = r; c < 3; ++c) {
                        S[r][c] = __fmaf_rn(M[r][2], M[c][2], __fmaf_rn(M[r][0], M[c][0], __fmul_rn(M[r][1], M[c][1])));
                        S[c][r] = S[r][c];
                    }
                // Sigma_cam[r][c] = sum_k sum_l R[k][r] Sigma[k][l] R[l][c]: every entry by the
                // reference's own 9-term accumulation (src/GSCudaKernels.cu:423-433)
                float C[3][3];
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        float acc = 0.0f;
#pragma unroll
                        for (int k = 0; k < 3; ++k)
#pragma unroll
                            for (int l = 0; l < 3; ++l) acc = __fmaf_rn(__fmul_rn(R[k][r], S[k][l]), R[l][c], acc);
                        C[r][c] = acc;
                    }
                const float Jm[2][3] = {
                    {__fmul_rn(K.fx, inv_z), 0.0f, __fmul_rn(__fmul_rn(__fmul_rn(-K.fx, pcx), inv_z), inv_z)},
                    {0.0f, __fmul_rn(K.fy, inv_z), __fmul_rn(__fmul_rn(__fmul_rn(-K.fy, pcy), inv_z), inv_z)}};
                // Sigma_2d = J Sigma_cam J^T by the same 9-term accumulation, zero entries of J included
                float S2[2][2];
#pragma unroll
                for (int r = 0; r < 2; ++r)
#pragma unroll
                    for (int c = r; c < 2; ++c) {
                        float acc = 0.0f;
#pragma unroll
                        for (int k = 0; k < 3; ++k)
#pragma unroll
                            for (int l = 0; l < 3; ++l) acc = __fmaf_rn(__fmul_rn(Jm[r][k], C[k][l]), Jm[c][l], acc);
                        S2[r][c] = acc;
                    }
                cxx = S2[0][0];
                cyy = S2[1][1];
                cxy = S2[0][1];
                const float det = __fmaf_rn(cxx, cyy, -__fmul_rn(cxy, cxy));
                if (det == 0.0f) {
                    ixx = 1.0f;
                    iyy = 1.0f;
                    ixy = 0.0f;
                } else {
                    const float inv_det = __fdiv_rn(1.0f, det);
                    ixx = __fmul_rn(cyy, inv_det);
                    iyy = __fmul_rn(cxx, inv_det);
                    ixy = __fmul_rn(-cxy, inv_det);
                }
                phx = __fmul_rn(__fmul_rn(pcx, inv_z), inv_z);
                phy = __fmul_rn(__fmul_rn(pcy, inv_z), inv_z);
                geo0 = make_float4(C[0][0], C[0][1], C[0][2], C[1][1]);
                geo1 = make_float4(C[1][2], C[2][2], pcx, pcy);
            }
        }
    }
    // Tile rectangle (countTilesPerGaussian_kernel).  Culled slots see the
    // zero record and land on tile 0, as the reference's zeroed buffers do.
    const float rx = __fmul_rn(a.radius_sigma, __fsqrt_rn(cxx));
    const float ry = __fmul_rn(a.radius_sigma, __fsqrt_rn(cyy));
    const float bx0 = fmaxf(0.0f, __fsub_rn(u, rx));
    const float bx1 = fminf((float)(a.W - 1), __fadd_rn(u, rx));
    const float by0 = fmaxf(0.0f, __fsub_rn(v, ry));
    const float by1 = fminf((float)(a.H - 1), __fadd_rn(v, ry));
    // bx / tw of the reference; a multiplication by 2^-k when tw = 2^k (exact)
    auto tdiv = [](float x, int t, float inv) { return inv != 0.0f ? __fmul_rn(x, inv) : __fdiv_rn(x, (float)t); };
    int x0 = __float2int_rz(tdiv(bx0, a.tw, a.inv_tw));
    int x1 = __float2int_rz(tdiv(bx1, a.tw, a.inv_tw));
    int y0 = __float2int_rz(tdiv(by0, a.th, a.inv_th));
    int y1 = __float2int_rz(tdiv(by1, a.th, a.inv_th));
    x0 = max(0, min(x0, a.ntx - 1));
    x1 = max(0, min(x1, a.ntx - 1));
    y0 = max(0, min(y0, a.nty - 1));
    y1 = max(0, min(y1, a.nty - 1));
    uint32_t count = (uint32_t)((x1 - x0 + 1) * (y1 - y0 + 1));
    if (!visible && !(a.quirks & FVGS_Q_CULLED_SLOTS)) count = 0;

    // The previous binning's rectangle (incremental mode: bins and counts
    // still hold it; read before anything of Gaussian i is overwritten).
    const uint32_t old_count = a.hist ? prev_count : 0u;
    uint4 old_r = make_uint4(0, 0, 0, 0);
    if (old_count) old_r = a.bins[i].r;
    // Records of Gaussians without instances are never read by the blending
    // kernels; they are written only where the culled-slot behaviour makes
    // culled Gaussians blend (with the zero record), and the host reports
    // zeros for them.
    if (count && (visible || (a.quirks & FVGS_Q_CULLED_SLOTS))) {
        const float4 co = a.attr_c ? unpack_c(a.attr_c[i]) : a.col[i];
        const bool swap = (a.quirks & FVGS_Q_INVSIGMA_SWAP) != 0;
        a.rec0[i] = make_float4(u, v, z, co.w);
        a.rec1[i] = make_float4(ixx, swap ? iyy : ixy, swap ? ixy : iyy, phx);
        a.rec2[i] = make_float4(phy, co.x, co.y, co.z);
        a.bins[i].p = make_float4(u, v, z, phx);
        if (a.geo0) {
            a.geo0[i] = geo0;
            a.geo1[i] = geo1;
        }
    }
    // bins[i].r.z == counts[i] after every binning; a Gaussian without
    // instances before and now needs no write (most of a large map).
    if (!a.hist || count || old_count) {
        a.bins[i].r = make_uint4((uint32_t)x0 | ((uint32_t)y0 << 16), (uint32_t)x1 | ((uint32_t)y1 << 16), count,
                                 __float_as_uint(phy));
        a.counts[i] = count;
    }
    if (a.tile_diff) {
        const int gw = a.ntx + 1;
        const size_t cells = (size_t)gw * (a.nty + 1);
        if (count) add_rect(grid, gw, x0, y0, x1, y1);
        if (a.hist) {
            // instances entering a tile: the new rectangle minus the previous one
            uint32_t n_enter = 0;
            if (count) {
                const EnterSplit es = enter_split(x0, y0, x1, y1, old_count != 0, (int)(old_r.x & 0xffffu),
                                                  (int)(old_r.x >> 16), (int)(old_r.y & 0xffffu), (int)(old_r.y >> 16));
                n_enter = entering_count(es);
                int* e = grid + cells;
                if (es.whole) {
                    add_rect(e, gw, x0, y0, x1, y1);
                } else {
                    if (es.iy0 > y0) add_rect(e, gw, x0, y0, x1, es.iy0 - 1);
                    if (es.iy1 < y1) add_rect(e, gw, x0, es.iy1 + 1, x1, y1);
                    if (es.ix0 > x0) add_rect(e, gw, x0, es.iy0, es.ix0 - 1, es.iy1);
                    if (es.ix1 < x1) add_rect(e, gw, es.ix1 + 1, es.iy0, x1, es.iy1);
                }
            }
            // warp-aggregated: entering total and the list of changed Gaussians
            uint32_t* ctr = reinterpret_cast<uint32_t*>(a.tile_diff + 2 * cells);
            const unsigned act = __activemask();
            const unsigned want = __ballot_sync(act, n_enter != 0u);
            if (want) {
                const int leader = __ffs(want) - 1;
                const uint32_t sum = __reduce_add_sync(act, n_enter);
                uint32_t base = 0;
                if ((int)(threadIdx.x & 31) == leader) {
                    atomicAdd(&ctr[0], sum);
                    base = atomicAdd(&ctr[1], (uint32_t)__popc(want));
                }
                base = __shfl_sync(act, base, leader);
                if (n_enter) {
                    const uint32_t idx = base + (uint32_t)__popc(want & lanemask_lt());
                    if (idx < a.changed_cap) a.changed[idx] = make_uint4((uint32_t)i, old_r.x, old_r.y, old_count);
                }
            }
        }
    }
    if (a.dbg_cov) {
        a.dbg_cov[3 * i] = cxx;
        a.dbg_cov[3 * i + 1] = cyy;
        a.dbg_cov[3 * i + 2] = cxy;
        a.dbg_inv[3 * i] = ixx;
        a.dbg_inv[3 * i + 1] = iyy;
        a.dbg_inv[3 * i + 2] = ixy;
        a.dbg_vis[i] = visible ? 1 : 0;
    }
}

// Whether Gaussian i at position p lands in the image (the reference's
// culling, src/GSCudaKernels.cu:381,391), with project_one's arithmetic;
// pc: its camera-frame position.
__device__ __forceinline__ bool in_view(const ProjectArgs& a, float4 p, const float (&R)[3][3], const float (&tw)[3],
                                        float3& pc) {
    const float d0 = __fsub_rn(p.x, tw[0]);
    const float d1 = __fsub_rn(p.y, tw[1]);
    const float d2 = __fsub_rn(p.z, tw[2]);
    const float pcx = __fmaf_rn(R[2][0], d2, __fmaf_rn(R[0][0], d0, __fmul_rn(R[1][0], d1)));
    const float pcy = __fmaf_rn(R[2][1], d2, __fmaf_rn(R[0][1], d0, __fmul_rn(R[1][1], d1)));
    const float pcz = __fmaf_rn(R[2][2], d2, __fmaf_rn(R[0][2], d0, __fmul_rn(R[1][2], d1)));
    pc = make_float3(pcx, pcy, pcz);
    if (!(pcz > 0.0f)) return false;
    const float inv_z = __fdiv_rn(1.0f, pcz);
    const float uu = __fmaf_rn(a.K.fx, __fmul_rn(pcx, inv_z), a.K.cx);
    const float vv = __fmaf_rn(a.K.fy, __fmul_rn(pcy, inv_z), a.K.cy);
    return !(uu < 0.0f || uu >= (float)a.W || vv < 0.0f || vv >= (float)a.H);
}

// Chunks of kProjChunk Gaussians per CTA round.  Phase 1: every thread loads
// the positions (and previous counts) of its Gaussians, all loads in flight
// together, and culls them; a Gaussian out of view is finished right there
// (count 0, its binning record cleared where it had instances), the others
// are queued in shared memory.  Phase 2: the CTA runs project_one over the
// queue with full warps -- most of a large map is out of view, so in Gaussian
// order only a few lanes of a warp would take the projection's long path.
// Queue order does not matter: every output is indexed by the Gaussian, the
// tile counts are sums, and the changed list is consumed order-free.
// Culled-slot binning and the debug outputs take project_one for every
// Gaussian.
constexpr int kProjThreads = 256, kProjPerThread = 2, kProjChunk = kProjThreads * kProjPerThread;
// Difference grids of at most this many cells (both grids together) are
// accumulated in shared memory and added to the global ones once per CTA: at
// the coarse pyramid levels every Gaussian in view adds its rectangle's
// corners to a few dozen cells, and same-address global atomics from every
// SM serialise (level 3 of a 1280x720 frame: 77 cells).
constexpr int kProjSmemCells = 2048;

// A list is built for the current view cone widened by this margin, so that
// the pyramid levels of one camera (whose corner half-angles differ by a
// fraction of a pixel) share it.
constexpr float kCandConeMargin = 0.0174533f;  // 1 degree

// Candidate test of a Gaussian at camera-frame position pc for the view cone
// of half-angle cone: in it, widened by the largest rotation kCandMaxAngle
// and by the bearing change asin(kCandMaxShift / |pc|) of the largest shift,
// or within kCandNear of the camera.  A Gaussian in view at any pose within
// that rotation and shift of this one, with a view cone no wider, passes:
// its bearing at this pose is within cone + rotation + asin(shift / |pc|) of
// the optical axis.  An extra 0.5 degree covers the FP32 evaluation.
__device__ __forceinline__ bool candidate(float3 pc, float cone) {
    const float r = sqrtf(pc.x * pc.x + pc.y * pc.y + pc.z * pc.z);
    if (!(r > kCandNear)) return true;
    const float ang = cone + kCandMaxAngle + 0.0087f + asinf(fminf(1.0f, kCandMaxShift / r));
    if (ang >= 3.14159f) return true;
    return pc.z >= r * cosf(ang);
}

// Whether the current pose is within the candidate list's bounds of the pose
// the list was built at (rotation angle and shift), and the view cone no
// wider: every Gaussian in view now is on the list.
__device__ __forceinline__ bool cand_reusable(const CandState& c, const DevPose& P, float cone) {
    if (!c.valid || !(cone <= c.cone)) return false;
    const float dx = P.t[0] - c.t[0], dy = P.t[1] - c.t[1], dz = P.t[2] - c.t[2];
    if (!(dx * dx + dy * dy + dz * dz <= kCandMaxShift * kCandMaxShift)) return false;
    // angle between the two rotations: 2 acos |q0 . q1| for unit quaternions
    const float n0 = c.q[0] * c.q[0] + c.q[1] * c.q[1] + c.q[2] * c.q[2] + c.q[3] * c.q[3];
    const float n1 = P.q[0] * P.q[0] + P.q[1] * P.q[1] + P.q[2] * P.q[2] + P.q[3] * P.q[3];
    const float d = c.q[0] * P.q[0] + c.q[1] * P.q[1] + c.q[2] * P.q[2] + c.q[3] * P.q[3];
    return fabsf(d) * rsqrtf(n0 * n1) >= cosf(0.5f * kCandMaxAngle);
}

__global__ void __launch_bounds__(kProjThreads, 4) project_count_kernel(ProjectArgs a) {
    pdl_begin();
    __shared__ uint32_t q_i[kProjChunk], q_prev[kProjChunk];
    __shared__ int q_n;
    __shared__ int s_grid[kProjSmemCells];
    const int cells = a.tile_diff ? (a.ntx + 1) * (a.nty + 1) : 0;
    const int grid_cells = (a.hist ? 2 : 1) * cells;
    const bool smem_grid = a.tile_diff && grid_cells <= kProjSmemCells;
    int* grid = smem_grid ? s_grid : a.tile_diff;
    if (smem_grid)
        for (int c = threadIdx.x; c < grid_cells; c += kProjThreads) s_grid[c] = 0;
    const DevPose* P = a.pose;
    const float qc[4] = {P->q[0], P->q[1], P->q[2], P->q[3]};
    float R[3][3];
    quat_to_R(qc, R);
    const float tw[3] = {P->t[0], P->t[1], P->t[2]};
    const bool all_slow = (a.quirks & FVGS_Q_CULLED_SLOTS) || a.dbg_cov;
    const int lane = threadIdx.x & 31;
    // Candidate list: while the pose stays within its bounds, only the
    // Gaussians on it are projected (the others stay out of view, with count
    // 0 since the launch that built it); otherwise every Gaussian is, and
    // the list is rebuilt.  Every CTA reads the same state (it changes only
    // when the last CTA of a building launch has finished).
    const bool use_cand = a.cand && a.cst && !all_slow;
    const bool reuse = use_cand && cand_reusable(*a.cst, *P, a.cone);
    const bool build = use_cand && !reuse;
    const float cone_b = a.cone + kCandConeMargin;
    // A launch that projects every Gaussian without building a list drops
    // the one held: Gaussians off it may have records from this pose.
    if (a.cst && !use_cand && blockIdx.x == 0 && threadIdx.x == 0) a.cst->valid = 0;
    const int n_items = reuse ? (int)a.cst->n : a.n;
    // every CTA takes one contiguous span of the items (a multiple of a warp),
    // in chunks: a short candidate list then spreads over the whole grid
    // instead of filling a few CTAs' chunks
    const int span = ((n_items + (int)gridDim.x - 1) / (int)gridDim.x + 31) & ~31;
    const int b1 = min(n_items, (int)blockIdx.x * span + span);
    for (int base = (int)blockIdx.x * span; base < b1; base += kProjChunk) {
        if (threadIdx.x == 0) q_n = 0;
        __syncthreads();
        float4 p[kProjPerThread];
        uint32_t c[kProjPerThread];
        int gi[kProjPerThread];
#pragma unroll
        for (int k = 0; k < kProjPerThread; ++k) {
            const int item = base + k * kProjThreads + (int)threadIdx.x;
            gi[k] = item < b1 ? (reuse ? (int)a.cand[item] : item) : a.n;
        }
#pragma unroll
        for (int k = 0; k < kProjPerThread; ++k) {
            const int i = gi[k];
            p[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            c[k] = 0;
            if (i < a.n) {
                p[k] = a.pos[i];
                if (a.hist) c[k] = a.counts[i];
            }
        }
#pragma unroll
        for (int k = 0; k < kProjPerThread; ++k) {
            const int i = gi[k];
            const bool valid = i < a.n;
            float3 pc;
            const bool seen = valid && in_view(a, p[k], R, tw, pc);
            const bool queue = valid && (all_slow || seen);
            if (build) {
                // warp-aggregated append of the Gaussians that may come into view
                const bool cand = valid && (seen || candidate(pc, cone_b));
                const uint32_t cb = __ballot_sync(kFullMask, cand);
                if (cb) {
                    const int leader = __ffs(cb) - 1;
                    uint32_t slot = 0;
                    if (lane == leader) slot = atomicAdd(&a.cst->n_build, (uint32_t)__popc(cb));
                    slot = __shfl_sync(kFullMask, slot, leader) + (uint32_t)__popc(cb & lanemask_lt());
                    if (cand) a.cand[slot] = (uint32_t)i;
                }
            }
            if (valid && !queue && (!a.hist || c[k])) {
                // out of view, no instances now: project_one's record for it
                a.bins[i].r = make_uint4(0u, 0u, 0u, 0u);
                a.counts[i] = 0;
            }
            const uint32_t bal = __ballot_sync(kFullMask, queue);
            if (bal) {
                const int leader = __ffs(bal) - 1;
                int slot = 0;
                if (lane == leader) slot = atomicAdd(&q_n, __popc(bal));
                slot = __shfl_sync(kFullMask, slot, leader) + __popc(bal & lanemask_lt());
                if (queue) {
                    q_i[slot] = (uint32_t)i;
                    q_prev[slot] = c[k];
                }
            }
        }
        __syncthreads();
        const int nq = q_n;
        for (int k = threadIdx.x; k < nq; k += kProjThreads) {
            const uint32_t i = q_i[k];
            project_one(a, (int)i, a.pos[i], q_prev[k], R, tw, grid);
        }
        __syncthreads();  // the queue is consumed before the next chunk's
    }
    if (smem_grid) {
        __syncthreads();
        for (int c = threadIdx.x; c < grid_cells; c += kProjThreads) {
            const int v = s_grid[c];
            if (v) atomicAdd(&a.tile_diff[c], v);
        }
    }
    if (build && threadIdx.x == 0) {
        // the last CTA to finish publishes the list for the pose it was built at
        __threadfence();
        if (atomicAdd(&a.cst->done, 1u) == gridDim.x - 1) {
            CandState* cs = a.cst;
            cs->n = atomicExch(&cs->n_build, 0u);
            for (int k = 0; k < 3; ++k) cs->t[k] = P->t[k];
            for (int k = 0; k < 4; ++k) cs->q[k] = P->q[k];
            cs->cone = cone_b;
            cs->done = 0;
            __threadfence();
            cs->valid = 1;
        }
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan of counts: kernel 1 sums 4096-element blocks; kernel 2 lets
// every block reduce the sums before it (at most a few hundred values) and
// scan its own block.  Two launches, no inter-block waits, deterministic.
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanBlock = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t block_reduce_sum(uint32_t v, uint32_t* smem) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) smem[w] = v;
    __syncthreads();
    uint32_t r = 0;
    if (w == 0) {
        r = (l < (int)(blockDim.x >> 5)) ? smem[l] : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_xor_sync(kFullMask, r, o);
    }
    __syncthreads();
    return r;  // valid in warp 0
}

__global__ void __launch_bounds__(kScanThreads) scan_partials_kernel(const uint32_t* counts, int n,
                                                                     uint32_t* partials) {
    __shared__ uint32_t sm[32];
    const int base = blockIdx.x * kScanBlock;
    uint32_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += counts[i];
    }
    s = block_reduce_sum(s, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(kScanThreads) scan_final_kernel(const uint32_t* counts, int n,
                                                                  const uint32_t* partials, int n_blocks,
                                                                  uint32_t* offsets, DevStatus* st,
                                                                  uint32_t capacity) {
    __shared__ uint32_t sm[32];
    __shared__ uint32_t s_warp[32];
    __shared__ uint32_t s_base;
    // prefix of all earlier blocks
    uint32_t pre = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += kScanThreads) pre += partials[b];
    pre = block_reduce_sum(pre, sm);
    if (threadIdx.x == 0) s_base = pre;
    __syncthreads();
    const uint32_t block_base = s_base;
    // blocked arrangement: thread t owns items base + t*4 .. +3 (contiguous)
    const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanItems;
    uint32_t c[kScanItems];
    uint32_t tsum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        c[k] = (base + k < n) ? counts[base + k] : 0u;
        tsum += c[k];
    }
    // block exclusive scan of tsum
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    uint32_t incl = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
        if (l >= o) incl += y;
    }
    if (l == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        uint32_t x = s_warp[l];
        uint32_t xi = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, xi, o);
            if (l >= o) xi += y;
        }
        s_warp[l] = xi - x;  // exclusive warp prefix
    }
    __syncthreads();
    uint32_t run = block_base + s_warp[w] + (incl - tsum);
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        if (base + k < n) offsets[base + k] = run;
        run += c[k];
    }
    if (blockIdx.x == n_blocks - 1 && threadIdx.x == kScanThreads - 1) {
        st->n_instances = run;
        st->n_instances_clamped = run < capacity ? run : capacity;
        if (run > capacity) atomicOr(&st->flags, kErrOverflow);
    }
}

// ---------------------------------------------------------------------------
// Key emission: a warp takes 32 consecutive Gaussians, whose instances are
// contiguous in the output, and walks their concatenated tile lists 32 at a
// time.  Each lane finds its owning Gaussian by a 5-step shuffle search.
// key = tile << 32 | bits(fmaf(phx, dx, z) + phy * dy), dx = tile centre - u
// (tile_depth).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) emit_keys_kernel(EmitArgs a) {
    const int gbase = (blockIdx.x * blockDim.x + threadIdx.x) & ~31;
    const int lane = threadIdx.x & 31;
    if (gbase >= a.n) return;  // whole warp leaves together
    const int g = gbase + lane;
    const bool valid = g < a.n;
    uint4 b0 = make_uint4(0, 0, 0, 0);
    float4 b1 = make_float4(0, 0, 0, 0);
    uint32_t off = 0;
    if (valid) {
        b0 = a.bins[g].r;
        off = a.offsets[g];
        if (b0.z) b1 = a.bins[g].p;
    }
    const uint32_t cnt = valid ? b0.z : 0u;
    // warp-local exclusive prefix of counts
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t excl = incl - cnt;
    const uint32_t total = __shfl_sync(kFullMask, incl, 31);
    const uint32_t warp_off = __shfl_sync(kFullMask, off, 0);
    const uint64_t cap = a.capacity;
    for (uint32_t m0 = 0; m0 < total; m0 += 32) {
        const uint32_t m = m0 + lane;
        // largest l with excl[l] <= m
        int lo = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
            const uint32_t e = __shfl_sync(kFullMask, excl, lo + step);
            if (e <= m) lo += step;
        }
        const uint32_t r0 = __shfl_sync(kFullMask, b0.x, lo);
        const uint32_t r1 = __shfl_sync(kFullMask, b0.y, lo);
        const uint32_t phy_bits = __shfl_sync(kFullMask, b0.w, lo);
        const float u = __shfl_sync(kFullMask, b1.x, lo);
        const float v = __shfl_sync(kFullMask, b1.y, lo);
        const float z = __shfl_sync(kFullMask, b1.z, lo);
        const float phx = __shfl_sync(kFullMask, b1.w, lo);
        const uint32_t e_lo = __shfl_sync(kFullMask, excl, lo);
        if (m < total) {
            const uint32_t local = m - e_lo;
            const int x0 = (int)(r0 & 0xffffu), y0 = (int)(r0 >> 16);
            const int x1 = (int)(r1 & 0xffffu);
            const int w = x1 - x0 + 1;
            const int tx = x0 + (int)(local % (uint32_t)w);
            const int ty = y0 + (int)(local / (uint32_t)w);
            const float d = tile_depth(tx, ty, a.tw, a.th, u, v, z, phx, phy_bits);
            const uint32_t tile = (uint32_t)(ty * a.ntx + tx);
            const uint64_t dst = (uint64_t)warp_off + m;
            if (dst < cap) {
                a.keys[dst] = ((uint64_t)tile << 32) | (uint64_t)__float_as_uint(d);
                a.vals[dst] = (uint32_t)(gbase + lo);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Per-tile ranges over the sorted keys (ranges zeroed beforehand).
// Intended: every boundary.  RANGE_LAUNCH: the reference's literal launch,
// which only visits the first 256*ceil(T/256) instances and whose first
// instance never closes its tile.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) ranges_kernel(const uint64_t* keys, const DevStatus* st, int num_tiles,
                                                     uint32_t quirks, uint2* ranges) {
    const uint32_t n = st->n_instances_clamped;
    uint32_t limit = n;
    if (quirks & FVGS_Q_RANGE_LAUNCH) {
        const uint32_t launched = (uint32_t)((num_tiles + 255) / 256) * 256u;
        limit = min(limit, launched);
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < limit; i += gridDim.x * blockDim.x) {
        // Tile ids are range-checked: after an instance overflow (the call is
        // then repeated with larger buffers) unwritten slots hold stale keys.
        const uint32_t t = (uint32_t)(keys[i] >> 32);
        if (t >= (uint32_t)num_tiles) continue;
        if (quirks & FVGS_Q_RANGE_LAUNCH) {
            if (i == 0) {
                ranges[t].x = 0;
                continue;
            }
            const uint32_t pt = (uint32_t)(keys[i - 1] >> 32);
            if (pt != t) {
                if (pt < (uint32_t)num_tiles) ranges[pt].y = i;
                ranges[t].x = i;
            }
            if (i == n - 1) ranges[t].y = n;
        } else {
            if (i == 0 || (uint32_t)(keys[i - 1] >> 32) != t) ranges[t].x = i;
            if (i == n - 1 || (uint32_t)(keys[i + 1] >> 32) != t) ranges[t].y = i + 1;
        }
    }
}

// ---------------------------------------------------------------------------
// Tile offsets from the difference grids (one CTA): 2-D prefix sums give the
// instance count of every tile; an exclusive scan in row-major tile order gives
// each tile's [start, end) in the tile-major instance array -- these are the
// per-tile ranges, and the starts seed the scatter cursors.  With a valid
// previous binning the entering grid is scanned the same way (into a compact
// array of entering instances) and the binning mode is chosen.
// ---------------------------------------------------------------------------
constexpr int kOffThreads = 1024;
constexpr int kOffSmemCells = 48 * 1024;  // 192 KB of grid staged in shared memory

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

__global__ void __launch_bounds__(kOffThreads) tile_offsets_kernel(int* scratch, int ntx, int nty, int hist,
                                                                   uint32_t enter_cap, uint2* ranges, uint32_t* fill,
                                                                   uint2* enter_ranges, uint32_t* enter_fill,
                                                                   DevStatus* st, uint32_t capacity,
                                                                   uint32_t* seg_ctrl) {
    pdl_begin();
    extern __shared__ int s_grid[];
    __shared__ uint32_t s_w[2][32];
    __shared__ uint32_t s_carry[2];
    __shared__ uint32_t s_ctr[2];
    const int gw = ntx + 1, gh = nty + 1, cells = gw * gh;
    const int ng = hist ? 2 : 1;
    const bool staged = ng * cells <= kOffSmemCells;
    int* g = staged ? s_grid : scratch;
    uint32_t* ctr = reinterpret_cast<uint32_t*>(scratch + 2 * (size_t)cells);
    if (threadIdx.x == 0) {
        s_ctr[0] = ctr[0];
        s_ctr[1] = ctr[1];
    }
    if (staged)
        for (int i = threadIdx.x; i < ng * cells; i += kOffThreads) s_grid[i] = scratch[i];
    __syncthreads();
    // the scratch is left zeroed for the next binning (staged: right away)
    if (staged) {
        for (int i = threadIdx.x; i < ng * cells; i += kOffThreads) scratch[i] = 0;
        if (threadIdx.x < kCounterWords) ctr[threadIdx.x] = 0u;
    }
    // row prefix sums (one thread per grid row), then column prefix sums
    for (int r = threadIdx.x; r < ng * gh; r += kOffThreads) {
        int* row = g + (size_t)(r / gh) * cells + (r % gh) * gw;
        int acc = 0;
        for (int c = 0; c < gw; ++c) {
            acc += row[c];
            row[c] = acc;
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < ng * gw; c += kOffThreads) {
        int* col = g + (size_t)(c / gw) * cells + (c % gw);
        int acc = 0;
        for (int r = 0; r < gh; ++r) {
            acc += col[r * gw];
            col[r * gw] = acc;
        }
    }
    __syncthreads();
    // exclusive scans of both grids over tiles in row-major order
    const int T = ntx * nty;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x < 2) s_carry[threadIdx.x] = 0;
    __syncthreads();
    for (int base = 0; base < T; base += kOffThreads) {
        const int t = base + threadIdx.x;
        const int cell = (t / ntx) * gw + (t % ntx);
        const uint32_t c0 = t < T ? (uint32_t)g[cell] : 0u;
        const uint32_t c1 = (hist && t < T) ? (uint32_t)g[cells + cell] : 0u;
        const uint32_t i0 = warp_incl_scan(c0, lane);
        const uint32_t i1 = warp_incl_scan(c1, lane);
        if (lane == 31) {
            s_w[0][w] = i0;
            s_w[1][w] = i1;
        }
        __syncthreads();
        if (w < 2) {
            const uint32_t v = s_w[w][lane];
            s_w[w][lane] = warp_incl_scan(v, lane) - v;
        }
        __syncthreads();
        const uint32_t start0 = s_carry[0] + s_w[0][w] + i0 - c0;
        const uint32_t start1 = s_carry[1] + s_w[1][w] + i1 - c1;
        if (t < T) {
            fill[t] = start0;
            // empty tiles keep the (0, 0) of the reference's zeroed range buffer
            ranges[t] = c0 ? make_uint2(start0, start0 + c0) : make_uint2(0u, 0u);
            if (hist) {
                enter_fill[t] = start1;
                enter_ranges[t] = make_uint2(start1, start1 + c1);
            }
        }
        __syncthreads();
        if (threadIdx.x == kOffThreads - 1) {
            s_carry[0] = start0 + c0;
            s_carry[1] = start1 + c1;
        }
        __syncthreads();
    }
    if (!staged) {
        __syncthreads();
        for (int i = threadIdx.x; i < ng * cells; i += kOffThreads) scratch[i] = 0;
        if (threadIdx.x < kCounterWords) ctr[threadIdx.x] = 0u;
    }
    if (threadIdx.x == 0) {
        const uint32_t total = s_carry[0];
        // list counters of the per-tile sort and the scatter's chunk counter
        seg_ctrl[0] = 0u;
        seg_ctrl[1] = 0u;
        seg_ctrl[2] = 0u;
        st->n_instances = total;
        st->n_instances_clamped = total < capacity ? total : capacity;
        if (total > capacity) atomicOr(&st->flags, kErrOverflow);
        const uint32_t n_enter = hist ? s_ctr[0] : total;
        const uint32_t n_changed = hist ? s_ctr[1] : 0u;
        const bool incr = hist && n_enter == s_carry[1] && n_enter <= enter_cap && n_changed <= enter_cap;
        st->mode = incr ? kBinIncremental : kBinFull;
        st->n_enter = n_enter;
        st->n_changed = n_changed;
    }
}

// ---------------------------------------------------------------------------
// Scatter emission.  A warp takes 32 Gaussians and walks their concatenated
// tile lists 32 instances per lane-round (a 5-step shuffle search finds each
// lane's Gaussian); every instance yields its tile and the composite key
// depth_bits << 32 | Gaussian index.  The order inside a tile bucket is
// arbitrary here; the per-tile sort on these unique keys restores the
// reference's (depth, generation order).
// Full mode walks Gaussians chunk * 32 + lane and emits every instance.
// Incremental mode walks the listed (changed) Gaussians and emits only the
// tiles outside their previous rectangle.
// ---------------------------------------------------------------------------
constexpr int kWalkBatch = 4;  // instances per lane per round, memory ops in flight together

template <bool INCR, typename F>
__device__ __forceinline__ void walk_instances(const EmitArgs& a, uint32_t first, uint32_t n_items, F&& visit) {
    const int lane = threadIdx.x & 31;
    const uint32_t item = first + (uint32_t)lane;
    const bool valid = item < n_items;
    uint32_t g = 0;
    uint4 b0 = make_uint4(0, 0, 0, 0);
    float4 b1 = make_float4(0, 0, 0, 0);
    uint4 prev = make_uint4(0, 0, 0, 0);  // incremental: (index, previous rectangle, previous count)
    uint32_t cnt = 0;
    if (valid) {
        if (INCR) {
            prev = a.changed[item];
            g = prev.x;
        } else {
            g = item;
        }
        b0 = a.bins[g].r;
        if (b0.z) b1 = a.bins[g].p;
        if (INCR) {
            cnt = b0.z ? entering_count(enter_split((int)(b0.x & 0xffffu), (int)(b0.x >> 16), (int)(b0.y & 0xffffu),
                                                    (int)(b0.y >> 16), prev.w != 0u, (int)(prev.y & 0xffffu),
                                                    (int)(prev.y >> 16), (int)(prev.z & 0xffffu),
                                                    (int)(prev.z >> 16)))
                       : 0u;
        } else {
            cnt = b0.z;
        }
    }
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t excl = incl - cnt;
    const uint32_t total = __shfl_sync(kFullMask, incl, 31);
    for (uint32_t m0 = 0; m0 < total; m0 += 32 * kWalkBatch) {
        uint32_t tiles[kWalkBatch];
        uint64_t keys[kWalkBatch];
        bool ok[kWalkBatch];
#pragma unroll
        for (int q = 0; q < kWalkBatch; ++q) {
            const uint32_t m = m0 + 32 * q + lane;
            int lo = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const uint32_t e = __shfl_sync(kFullMask, excl, lo + step);
                if (e <= m) lo += step;
            }
            const uint32_t r0 = __shfl_sync(kFullMask, b0.x, lo);
            const uint32_t r1 = __shfl_sync(kFullMask, b0.y, lo);
            const uint32_t phy_bits = __shfl_sync(kFullMask, b0.w, lo);
            const float u = __shfl_sync(kFullMask, b1.x, lo);
            const float v = __shfl_sync(kFullMask, b1.y, lo);
            const float z = __shfl_sync(kFullMask, b1.z, lo);
            const float phx = __shfl_sync(kFullMask, b1.w, lo);
            const uint32_t e_lo = __shfl_sync(kFullMask, excl, lo);
            const uint32_t g_lo = __shfl_sync(kFullMask, g, lo);
            const uint32_t local = m - e_lo;
            const int x0 = (int)(r0 & 0xffffu), y0 = (int)(r0 >> 16);
            const int x1 = (int)(r1 & 0xffffu), y1 = (int)(r1 >> 16);
            int tx, ty;
            if (INCR) {
                const uint32_t p0 = __shfl_sync(kFullMask, prev.y, lo);
                const uint32_t p1 = __shfl_sync(kFullMask, prev.z, lo);
                const uint32_t pc = __shfl_sync(kFullMask, prev.w, lo);
                entering_tile(enter_split(x0, y0, x1, y1, pc != 0u, (int)(p0 & 0xffffu), (int)(p0 >> 16),
                                          (int)(p1 & 0xffffu), (int)(p1 >> 16)),
                              local, tx, ty);
            } else {
                const int w = max(1, x1 - x0 + 1);
                tx = x0 + (int)(local % (uint32_t)w);
                ty = y0 + (int)(local / (uint32_t)w);
            }
            ok[q] = m < total;
            const float d = tile_depth(tx, ty, a.tw, a.th, u, v, z, phx, phy_bits);
            tiles[q] = (uint32_t)(ty * a.ntx + tx);
            keys[q] = ((uint64_t)__float_as_uint(d) << 32) | (uint64_t)g_lo;
        }
        visit(tiles, keys, ok);
    }
}

template <bool INCR>
__device__ __forceinline__ void scatter_chunks(const EmitArgs& a, uint32_t* fill, uint64_t* out, uint64_t cap,
                                               uint32_t n_items, uint32_t* chunk_counter) {
    const int lane = threadIdx.x & 31;
    const uint32_t n_chunks = (n_items + 31) / 32;
    // Incremental mode has a few chunks: static assignment, so the idle warps
    // leave without touching the shared counter.
    const uint32_t warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    uint32_t next = warp_id;
    for (;;) {
        uint32_t chunk = next;
        if (INCR) {
            next += n_warps;
        } else {
            if (lane == 0) chunk = atomicAdd(chunk_counter, 1u);
            chunk = __shfl_sync(kFullMask, chunk, 0);
        }
        if (chunk >= n_chunks) return;
        walk_instances<INCR>(a, chunk * 32, n_items, [&](const uint32_t* tiles, const uint64_t* keys, const bool* ok) {
            uint32_t slot[kWalkBatch];
#pragma unroll
            for (int q = 0; q < kWalkBatch; ++q)
                if (ok[q]) slot[q] = atomicAdd(&fill[tiles[q]], 1u);
#pragma unroll
            for (int q = 0; q < kWalkBatch; ++q)
                if (ok[q] && slot[q] < cap) out[slot[q]] = keys[q];
        });
    }
}

// Scatter with persistent warps: each warp takes chunks of 32 Gaussians from a
// global counter, so warps whose chunks hold few instances (culled or small
// Gaussians) simply take more chunks; every instance takes the next slot of
// its tile with one global atomic.
__global__ void __launch_bounds__(256) emit_scatter_kernel(EmitArgs a, uint32_t* fill, uint32_t* chunk_counter,
                                                           const DevStatus* st) {
    pdl_begin();
    if (st->flags & kErrOverflow) return;
    if (st->mode == kBinIncremental)
        scatter_chunks<true>(a, a.enter_fill, a.enter_keys, a.enter_cap, st->n_changed, chunk_counter);
    else
        scatter_chunks<false>(a, fill, a.keys, a.capacity, (uint32_t)a.n, chunk_counter);
}

// Copy a binning's sorted lists (the instances of every tile's range) and its
// ranges into the other buffer pair; positions are unchanged.
__global__ void __launch_bounds__(256) copy_lists_kernel(const uint2* __restrict__ ranges, int T,
                                                         const uint32_t* __restrict__ src, uint32_t* __restrict__ dst,
                                                         uint2* __restrict__ ranges_dst, uint64_t capacity) {
    pdl_begin();
    for (int t = blockIdx.x; t < T; t += gridDim.x) {
        const uint2 r = ranges[t];
        if (threadIdx.x == 0) ranges_dst[t] = r;
        const uint64_t end = min((uint64_t)r.y, capacity);
        for (uint64_t i = (uint64_t)r.x + threadIdx.x; i < end; i += blockDim.x) dst[i] = src[i];
    }
}

// ------------------------------- launchers ---------------------------------
cudaError_t launch_copy_lists(const uint2* ranges, int T, const uint32_t* src, uint32_t* dst, uint2* ranges_dst,
                              uint64_t capacity, int max_ctas, cudaStream_t s) {
    if (T <= 0) return cudaSuccess;
    const int grid = T < max_ctas ? T : max_ctas;
    return launch_chained(copy_lists_kernel, dim3(grid), dim3(256), 0, s, ranges, T, src, dst, ranges_dst, capacity);
}

cudaError_t launch_project_count(const ProjectArgs& a, int max_ctas, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const int need = (a.n + kProjChunk - 1) / kProjChunk;
    return launch_chained(project_count_kernel, dim3(max_ctas > 0 && max_ctas < need ? max_ctas : need), dim3(256), 0,
                          s, a);
}

size_t scan_partials_size(int n) { return (size_t)((n + kScanBlock - 1) / kScanBlock); }

cudaError_t launch_scan(const uint32_t* counts, int n, uint32_t* partials, uint32_t* offsets, DevStatus* st,
                        uint32_t capacity, cudaStream_t s) {
    const int nb = (n + kScanBlock - 1) / kScanBlock;
    if (nb == 0) return cudaSuccess;
    scan_partials_kernel<<<nb, kScanThreads, 0, s>>>(counts, n, partials);
    scan_final_kernel<<<nb, kScanThreads, 0, s>>>(counts, n, partials, nb, offsets, st, capacity);
    return cudaGetLastError();
}

cudaError_t launch_emit_keys(const EmitArgs& a, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    emit_keys_kernel<<<(a.n + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_ranges(const uint64_t* keys, const DevStatus* st, int num_tiles, uint32_t quirks,
                          uint2* ranges, int grid, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(ranges, 0, sizeof(uint2) * (size_t)num_tiles, s);
    if (e != cudaSuccess) return e;
    ranges_kernel<<<grid, 256, 0, s>>>(keys, st, num_tiles, quirks, ranges);
    return cudaGetLastError();
}

}  // namespace fvgs

namespace fvgs {

size_t diff_grid_cells(int ntx, int nty) { return (size_t)(ntx + 1) * (nty + 1); }
size_t tile_diff_words(int ntx, int nty) { return 2 * diff_grid_cells(ntx, nty) + kCounterWords; }

cudaError_t launch_tile_offsets(int* scratch, int ntx, int nty, bool hist, uint32_t enter_cap, uint2* ranges,
                                uint32_t* fill, uint2* enter_ranges, uint32_t* enter_fill, DevStatus* st,
                                uint32_t capacity, uint32_t* seg_ctrl, cudaStream_t s) {
    // set on every launch: cheap, and correct for whichever device is current
    const cudaError_t e = cudaFuncSetAttribute(tile_offsets_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)(sizeof(int) * kOffSmemCells));
    if (e != cudaSuccess) return e;
    const size_t cells = (hist ? 2 : 1) * diff_grid_cells(ntx, nty);
    const size_t smem = cells <= (size_t)kOffSmemCells ? sizeof(int) * cells : 0;
    return launch_chained(tile_offsets_kernel, dim3(1), dim3(kOffThreads), smem, s, scratch, ntx, nty, hist ? 1 : 0,
                          enter_cap, ranges, fill, enter_ranges, enter_fill, st, capacity, seg_ctrl);
}

cudaError_t launch_emit_scatter(const EmitArgs& a, uint32_t* fill, uint32_t* chunk_counter, int grid,
                                const DevStatus* st, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    const int needed = (a.n + 255) / 256;
    return launch_chained(emit_scatter_kernel, dim3(grid < needed ? grid : needed), dim3(256), 0, s, a, fill,
                          chunk_counter, st);
}

}  // namespace fvgs
