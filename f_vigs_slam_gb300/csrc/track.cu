// track.cu -- fused tracking kernel (forward blend + RGB-D pose Jacobian +
// per-tile J^T J / J^T r reduction), the frame reduction, and the on-device
// Gauss-Newton pose update, for sm_103a.
//
// Reference: getRgbdPoseJacobians (src/GSCudaKernels.cu:922-1392), the host
// reduction and sign convention of GSSlam::computeRgbdPoseJacobians
// (src/GSSlam.cu:2205-2226), the eigen-regularised pseudo factor of
// RgbdPoseCostFunction::Evaluate (src/RgbdPoseCost.cu:57-106) and the pose
// update PoseLocalParameterization::Plus (src/PoseLocalParameterization.cpp:22-44).
//
// Per-pixel semantics are the reference's (each pixel scans its tile list,
// thresholds 0.99 / 1/255 / 1e-4 / 0.5 / 1e-3, the pass-1-only v<=0 skip, the
// second pass over the first n_contrib entries).  The arithmetic is
// reorganised for the GPU without changing the mathematics:
//  * every per-Gaussian colour term is rank one (Jt_cam = jt_dl (x) alpha*dC),
//    so J_pose * JtJ_cam * J_pose^T becomes one 21-FMA update with
//    u = (jt_dl, d * (ray x jt_dl)) instead of the reference's 3x3 and 6x3
//    products; with jt_dl = g / d that is u = (g / d, ray x g), so the
//    per-pixel depth enters through one reciprocal;
//  * per-Gaussian factors of u (the mean's ray, -f * ray) are computed once
//    per staged batch; the per-pixel depth takes the compensated evaluation
//    only where its two-FMA value may have cancelled; reciprocals are the
//    one-ulp rcp.approx;
//  * terms are accumulated in the camera frame (translation rows without R)
//    and rotated once per frame, in FP64, by diag(R, I);
//  * the 27 per-thread sums are reduced by a 31-shuffle butterfly
//    reduce-scatter, then across the 8 warps in a fixed order, and written
//    once per tile (no atomics: results are run-to-run deterministic).
#include <cooperative_groups.h>

#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace cg = cooperative_groups;

namespace fvgs {

constexpr int kTW = 16, kTH = 16, kPix = kTW * kTH;
constexpr int kBatch = 256;
constexpr float kInv255 = 1.0f / 255.0f;

// z + dx*phx + dy*phy with compensated arithmetic (error-free products via
// FMA, error-free sums via TwoSum): the per-Gaussian depth cancels to values
// near zero for distant pixels, and its reciprocal enters the Jacobian, so a
// plain FP32 evaluation would cost several digits there.
__device__ __forceinline__ float depth_at(float z, float dx, float phx, float dy, float phy) {
    const float p1 = __fmul_rn(dx, phx);
    const float e1 = __fmaf_rn(dx, phx, -p1);
    const float p2 = __fmul_rn(dy, phy);
    const float e2 = __fmaf_rn(dy, phy, -p2);
    const float s1 = __fadd_rn(z, p1);
    const float b1 = __fsub_rn(s1, z);
    const float r1 = __fadd_rn(__fsub_rn(z, __fsub_rn(s1, b1)), __fsub_rn(p1, b1));
    const float s2 = __fadd_rn(s1, p2);
    const float b2 = __fsub_rn(s2, s1);
    const float r2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, b2)), __fsub_rn(p2, b2));
    return __fadd_rn(s2, __fadd_rn(__fadd_rn(r1, r2), __fadd_rn(e1, e2)));
}

// z + dx*phx + dy*phy by two FMAs when that is accurate, else depth_at.  Each
// FMA rounds once, so the error is at most 2^-24 (|t| + |s|) with t the first
// FMA's result and s the second's; when |t| <= 8 |s| that is under 6e-7 |s|.
// Cancellation (|s| small against |t|) and non-finite values take the
// compensated path.
__device__ __forceinline__ float depth_fast(float z, float dx, float phx, float dy, float phy) {
    const float t = __fmaf_rn(dx, phx, z);
    const float s = __fmaf_rn(dy, phy, t);
    if (fabsf(t) <= 8.0f * fabsf(s)) return s;
    return depth_at(z, dx, phx, dy, phy);
}

__device__ __forceinline__ void rank1_update(float A[21], float w, float a0, float a1, float a2, float d,
                                             float r0, float r1, float r2) {
    // u = (a, d * (r x a))
    const float u[6] = {a0, a1, a2, d * (r1 * a2 - r2 * a1), d * (r2 * a0 - r0 * a2), d * (r0 * a1 - r1 * a0)};
    int idx = 0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float wu = w * u[i];
#pragma unroll
        for (int j = i; j < 6; ++j) A[idx++] += wu * u[j];
    }
}

// Butterfly reduce-scatter of 32 values over a warp: lane l ends with the warp
// sum of value l.
__device__ __forceinline__ float warp_reduce_scatter32(float (&v)[32]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < o; ++k) {
            const float send = upper ? v[k] : v[k + o];
            const float keep = upper ? v[k + o] : v[k];
            v[k] = keep + __shfl_xor_sync(kFullMask, send, o);
        }
    }
    return v[0];
}

// Stage one Gaussian's blending record: from the packed record planes, or
// (REF_LAYOUT) built from the reference's separate screen-space buffers.
template <bool REF_LAYOUT>
__device__ __forceinline__ void load_record(const TrackArgs& a, uint32_t g, float4& r0, float4& r1, float4& r2) {
    if (!REF_LAYOUT) {
        r0 = a.rec0[g];
        r1 = a.rec1[g];
        r2 = a.rec2[g];
    } else {
        const float2 uv = reinterpret_cast<const float2*>(a.ref_uv)[g];
        const float ixx = a.ref_inv[3 * (size_t)g], iyy = a.ref_inv[3 * (size_t)g + 1],
                    ixy = a.ref_inv[3 * (size_t)g + 2];
        const float2 ph = reinterpret_cast<const float2*>(a.ref_phat)[g];
        const bool swap = (a.quirks & FVGS_Q_INVSIGMA_SWAP) != 0;
        r0 = make_float4(uv.x, uv.y, a.ref_depth[g], a.ref_opa[g]);
        r1 = make_float4(ixx, swap ? iyy : ixy, swap ? ixy : iyy, ph.x);
        r2 = make_float4(ph.y, a.ref_col[3 * (size_t)g], a.ref_col[3 * (size_t)g + 1], a.ref_col[3 * (size_t)g + 2]);
    }
}

// Minimum of q(dx, dy) = a dx^2 + 2 b dx dy + c dy^2 over the rectangle
// [dxlo, dxhi] x [dylo, dyhi].  A positive definite q has its minimum at the
// origin when the rectangle contains it; otherwise (and for any indefinite or
// negative q) the minimum lies on the boundary, where each edge is a 1-D
// quadratic: its endpoints, plus the clamped stationary point when convex.
__device__ __forceinline__ float quad_min_rect(float a, float b, float c, float dxlo, float dxhi, float dylo,
                                               float dyhi) {
    if (a > 0.f && c > 0.f && a * c - b * b > 0.f && dxlo <= 0.f && dxhi >= 0.f && dylo <= 0.f && dyhi >= 0.f)
        return 0.f;
    float m = INFINITY;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const float X = e ? dxhi : dxlo;
        const float Y = e ? dyhi : dylo;
        // corners (each corner is visited once: (X, dylo), (X, dyhi))
        m = fminf(m, a * X * X + 2.0f * b * X * dylo + c * dylo * dylo);
        m = fminf(m, a * X * X + 2.0f * b * X * dyhi + c * dyhi * dyhi);
        if (c > 0.f) {
            const float dy = fminf(fmaxf(-b * X / c, dylo), dyhi);
            m = fminf(m, a * X * X + 2.0f * b * X * dy + c * dy * dy);
        }
        if (a > 0.f) {
            const float dx = fminf(fmaxf(-b * Y / a, dxlo), dxhi);
            m = fminf(m, a * dx * dx + 2.0f * b * dx * Y + c * Y * Y);
        }
    }
    return m;
}

// Tile-level rejection, done once per staged Gaussian.  A pixel skips a
// Gaussian when v > vreject (alpha < 1/255, both passes) or, in the forward
// pass only, when v <= 0.  If the extremes of v over the tile's pixel
// rectangle prove one of these for every pixel -- min v > vreject, or (forward
// pass) max v < 0 -- with a margin covering FP32 rounding at the magnitude of
// the terms, the Gaussian is dropped from the staged batch.  Kept Gaussians
// carry their original list index, so contributor counts and all results are
// unchanged.  Non-finite records are always kept.
template <bool FORWARD>
__device__ __forceinline__ bool tile_prunable(float u, float v, float ca, float cb, float cc, float vrej, float x0,
                                              float y0) {
    if (vrej == -INFINITY) return true;  // zero opacity: alpha is 0 everywhere
    if (!(isfinite(u) && isfinite(v) && isfinite(ca) && isfinite(cb) && isfinite(cc) && isfinite(vrej))) return false;
    const float dxlo = u - (x0 + (float)(kTW - 1)), dxhi = u - x0;
    const float dylo = v - (y0 + (float)(kTH - 1)), dyhi = v - y0;
    const float mx = fmaxf(fabsf(dxlo), fabsf(dxhi)), my = fmaxf(fabsf(dylo), fabsf(dyhi));
    const float margin = 1e-5f * (fabsf(ca) * mx * mx + 2.0f * fabsf(cb) * mx * my + fabsf(cc) * my * my) + 1e-3f;
    if (quad_min_rect(ca, cb, cc, dxlo, dxhi, dylo, dyhi) > vrej + margin) return true;
    if (FORWARD && -quad_min_rect(-ca, -cb, -cc, dxlo, dxhi, dylo, dyhi) < -margin) return true;
    return false;
}

// Shared-memory batch of Gaussians, repacked so a rejected pair needs two
// loads: sA = (u, v, c.x, c.y), sB = (c.z, vreject, log2(opacity), z),
// sC = (phat.x, phat.y, r, g), sD = b, s_orig = index in the tile's list;
// for the Jacobian pass also NX planes sX: the reference Jacobian stages
// sX[0] = (rgx, rgy, -fx rgx, -fy rgy), the mean's normalised ray and the
// third row of the projection Jacobian without 1/d; the analytic Jacobian
// stages eight planes with the derivatives of (u, v, a, b, c) with respect to
// the camera-frame pose update and the mean's (x, y) (see stage_deriv).
template <int BATCH = kBatch, int NX = 1>
struct TrackBatch {
    float4 A[BATCH];
    float4 B[BATCH];
    float4 C[BATCH];
    float4 X[NX][BATCH];
    float D[BATCH];
    int orig[BATCH];
    int wcnt[kPix / 32];
};

// What a staging round stores besides the blending record.
enum StageExtra { kStageNone = 0, kStageRay = 1, kStageDeriv = 2 };

// Derivatives of one Gaussian's screen mean (u, v) and consumed conic slots
// (a, b, c) with respect to the camera-frame pose update delta = (dp_c,
// dtheta): t' = t + R dp_c, R' = R exp(dtheta), so d p_cam / d dp_c = -I,
// d p_cam / d dtheta = [p_cam]x and d Sigma_cam / d dtheta_j =
// -[e_j]x Sigma_cam + Sigma_cam [e_j]x.  With J the projection's Jacobian
// (rows J0, J1), M = Sigma_cam J^T and Q = Sigma2D^-1:
//   d Sigma2D = dJ M + (dJ M)^T (+ the rotated-covariance terms
//   2 J0 x M0, J0 x M1 + J1 x M0, 2 J1 x M1 for dtheta), dQ = -Q dSigma2D Q.
// r0, r1: the blending record; g0, g1: the geometry record (camera-frame
// covariance and mean).  out: du[6], dv[6], da[6], db[6], dc[6], x, y.
__device__ __forceinline__ void stage_deriv(const TrackArgs& a, const float4& r0, const float4& r1, const float4& g0,
                                            const float4& g1, float4 (&out)[8]) {
    const bool swap = (a.quirks & FVGS_Q_INVSIGMA_SWAP) != 0;
    const float fx = a.K.fx, fy = a.K.fy;
    const float z = r0.z, x = g1.z, y = g1.w;
    const float sxx = g0.x, sxy = g0.y, sxz = g0.z, syy = g0.w, syz = g1.x, szz = g1.y;
    const float q00 = r1.x, q01 = swap ? r1.z : r1.y, q11 = swap ? r1.y : r1.z;
    const float iz = __frcp_rn(z), iz2 = iz * iz, iz3 = iz2 * iz;
    // J0 = (j00, 0, j02), J1 = (0, j11, j12)
    const float j00 = fx * iz, j02 = -fx * x * iz2, j11 = fy * iz, j12 = -fy * y * iz2;
    const float m0x = sxx * j00 + sxz * j02, m0y = sxy * j00 + syz * j02, m0z = sxz * j00 + szz * j02;
    const float m1x = sxy * j11 + sxz * j12, m1y = syy * j11 + syz * j12, m1z = syz * j11 + szz * j12;
    // rotated-covariance terms: w00 = 2 J0 x M0, w01 = J0 x M1 + J1 x M0, w11 = 2 J1 x M1
    const float w00[3] = {2.f * (-j02 * m0y), 2.f * (j02 * m0x - j00 * m0z), 2.f * (j00 * m0y)};
    const float w01[3] = {-j02 * m1y + (j11 * m0z - j12 * m0y), (j02 * m1x - j00 * m1z) + j12 * m0x,
                          j00 * m1y - j11 * m0x};
    const float w11[3] = {2.f * (j11 * m1z - j12 * m1y), 2.f * (j12 * m1x), 2.f * (-j11 * m1x)};
    const float qa = q00 * q00, qb = 2.f * q00 * q01, qc = q01 * q01;
    const float qd = q00 * q01, qe = q00 * q11 + q01 * q01, qf = q01 * q11;
    const float qg = 2.f * q01 * q11, qh = q11 * q11;
    float du[6], dv[6], da[6], db[6], dc[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        // d p_cam for tangent direction k
        const float dpx = k == 0 ? -1.f : (k == 4 ? -z : (k == 5 ? y : 0.f));
        const float dpy = k == 1 ? -1.f : (k == 3 ? z : (k == 5 ? -x : 0.f));
        const float dpz = k == 2 ? -1.f : (k == 3 ? -y : (k == 4 ? x : 0.f));
        const float dj00 = -fx * iz2 * dpz;
        const float dj02 = -fx * iz2 * dpx + 2.f * fx * x * iz3 * dpz;
        const float dj11 = -fy * iz2 * dpz;
        const float dj12 = -fy * iz2 * dpy + 2.f * fy * y * iz3 * dpz;
        float ds00 = 2.f * (dj00 * m0x + dj02 * m0z);
        float ds01 = (dj00 * m1x + dj02 * m1z) + (dj11 * m0y + dj12 * m0z);
        float ds11 = 2.f * (dj11 * m1y + dj12 * m1z);
        if (k >= 3) {
            ds00 += w00[k - 3];
            ds01 += w01[k - 3];
            ds11 += w11[k - 3];
        }
        const float dq00 = -(qa * ds00 + qb * ds01 + qc * ds11);
        const float dq01 = -(qd * ds00 + qe * ds01 + qf * ds11);
        const float dq11 = -(qc * ds00 + qg * ds01 + qh * ds11);
        du[k] = j00 * dpx + j02 * dpz;
        dv[k] = j11 * dpy + j12 * dpz;
        da[k] = dq00;
        db[k] = swap ? dq11 : dq01;
        dc[k] = swap ? dq01 : dq11;
    }
    out[0] = make_float4(du[0], du[1], du[2], du[3]);
    out[1] = make_float4(du[4], du[5], dv[0], dv[1]);
    out[2] = make_float4(dv[2], dv[3], dv[4], dv[5]);
    out[3] = make_float4(da[0], da[1], da[2], da[3]);
    out[4] = make_float4(da[4], da[5], db[0], db[1]);
    out[5] = make_float4(db[2], db[3], db[4], db[5]);
    out[6] = make_float4(dc[0], dc[1], dc[2], dc[3]);
    out[7] = make_float4(dc[4], dc[5], x, y);
}

template <int STAGE, int BATCH, int NX>
__device__ __forceinline__ void put_staged(const TrackArgs& a, TrackBatch<BATCH, NX>& sb, int pos, const float4& r0,
                                           const float4& r1, const float4& r2, float vrej, int li, uint32_t g) {
    sb.A[pos] = make_float4(r0.x, r0.y, r1.x, r1.y);
    sb.B[pos] = make_float4(r1.z, vrej, log2_opacity(r0.w), r0.z);
    sb.C[pos] = make_float4(r1.w, r2.x, r2.y, r2.z);
    sb.D[pos] = r2.w;
    sb.orig[pos] = li;
    if constexpr (STAGE == kStageRay) {
        const float rgx = (r0.x - a.K.cx) * __frcp_rn(a.K.fx), rgy = (r0.y - a.K.cy) * __frcp_rn(a.K.fy);
        sb.X[0][pos] = make_float4(rgx, rgy, -a.K.fx * rgx, -a.K.fy * rgy);
    } else if constexpr (STAGE == kStageDeriv) {
        static_assert(NX == 8, "the analytic Jacobian stages eight derivative planes");
        float4 d[8];
        stage_deriv(a, r0, r1, a.geo0[g], a.geo1[g], d);
#pragma unroll
        for (int k = 0; k < 8; ++k) sb.X[k][pos] = d[k];
    }
}

// Stage entries [base, min(base+BATCH, limit)) of the tile's list, dropping
// the ones tile_prunable rejects; returns the number kept.  The CTA takes the
// entries 256 at a time (one per thread; BATCH = 128 uses half the threads),
// each round compacted after the previous one, so the staged order is the
// list order.  Ends with a barrier.
template <bool REF_LAYOUT, bool FORWARD, int STAGE, int BATCH, int NX>
__device__ __forceinline__ int stage_batch(const TrackArgs& a, TrackBatch<BATCH, NX>& sb, uint32_t list0, int base,
                                           int limit, float x0, float y0) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int total = 0;
#pragma unroll
    for (int r0 = 0; r0 < BATCH; r0 += kPix) {
        const int li = base + r0 + tid;
        bool keep = false;
        float4 r0v, r1, r2;
        float vrej = 0.f;
        uint32_t g = 0;
        if (r0 + tid < BATCH && li < limit) {
            g = a.indices[list0 + li];
            if (g < a.n_gauss) {
                load_record<REF_LAYOUT>(a, g, r0v, r1, r2);
                vrej = reject_bound(r0v.w);
                keep = !tile_prunable<FORWARD>(r0v.x, r0v.y, r1.x, r1.y, r1.z, vrej, x0, y0);
            }
        }
        const uint32_t bal = __ballot_sync(kFullMask, keep);
        if (lane == 0) sb.wcnt[w] = __popc(bal);
        __syncthreads();
        int wbase = 0, round_total = 0;
#pragma unroll
        for (int k = 0; k < kPix / 32; ++k) {
            const int c = sb.wcnt[k];
            wbase += (k < w) ? c : 0;
            round_total += c;
        }
        if (keep)
            put_staged<STAGE>(a, sb, total + wbase + __popc(bal & lanemask_lt()), r0v, r1, r2, vrej, li, g);
        total += round_total;
        __syncthreads();
    }
    return total;
}

// ---------------------------------------------------------------------------
// TMA staging (launch variant 2).  The records of a batch are gathered into
// shared memory by tile::gather4 tensor copies -- four Gaussians' 16-byte rows
// of one record plane per copy, 192 copies per batch -- completing on an
// mbarrier.  The next batch is gathered while the current one is blended, so
// the records' load latency leaves the blending warps.  The staging itself
// (rejection test, compaction into TrackBatch) is the same as stage_batch's.
// Row indices outside the map (past the list, or defensive out-of-range
// values) are replaced by row 0 and the row is not staged, so every copy
// reads inside the record planes and transfers exactly 64 bytes.
constexpr int kGroups = kBatch / 4;
constexpr uint32_t kTmaBatchBytes = 3u * kGroups * 64u;

struct TmaStage {
    float4 raw[3][kGroups][8];  // plane, group of 4 Gaussians (128-byte slots, first 64 bytes used)
    uint32_t gid[kBatch];       // the batch's Gaussian indices (0xffffffff past the list)
    unsigned long long bar;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_bar_init(unsigned long long* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void tma_bar_expect(unsigned long long* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait for the completion of the phase with the given parity.
__device__ __forceinline__ bool tma_bar_wait(unsigned long long* bar, uint32_t parity) {
    uint32_t done = 0;
    for (uint32_t it = 0; it < kSpinLimit && !done; ++it)
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
    return done != 0;
}

__device__ __forceinline__ void tma_gather4(float4* dst, const CUtensorMap* map, uint32_t r0, uint32_t r1,
                                            uint32_t r2, uint32_t r3, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_u32(bar))
        : "memory");
}

// Issue the gathers of entries [base, base + kBatch) of the tile's list (the
// expected bytes were announced before the preceding barrier).
__device__ __forceinline__ void tma_issue(const TrackArgs& a, const RecMaps& maps, TmaStage& ts, uint32_t list0,
                                          int base, int limit) {
    const int tid = threadIdx.x;
    {
        const int li = base + tid;
        ts.gid[tid] = li < limit ? a.indices[list0 + li] : 0xffffffffu;
    }
    if (tid < 3 * kGroups) {
        // the rows of the previous batch were read through the generic proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const int plane = tid / kGroups, grp = tid % kGroups;
        uint32_t r[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int li = base + 4 * grp + j;
            const uint32_t g = li < limit ? a.indices[list0 + li] : 0u;
            r[j] = g < a.n_gauss ? g : 0u;
        }
        tma_gather4(&ts.raw[plane][grp][0], &maps.rec[plane], r[0], r[1], r[2], r[3], &ts.bar);
    }
}

// stage_batch with the records taken from the gathered batch; also announces
// and issues the gathers of the next batch once this one is consumed.
// parity / pending / broken track the mbarrier (uniform across the CTA).  A
// wait that gives up flags kErrTimeout and leaves the copy pending: nothing
// more is staged or issued, and the end of the pass waits for it once more.
struct TmaState {
    uint32_t parity = 0;
    bool pending = false;
    bool broken = false;
};

template <bool FORWARD>
__device__ __forceinline__ int stage_batch_tma(const TrackArgs& a, const RecMaps& maps, TrackBatch<>& sb, TmaStage& ts,
                                               uint32_t list0, int base, int limit, float x0, float y0,
                                               TmaState& tm) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    bool ready = !tm.broken;
    if (ready && tm.pending) {
        ready = tma_bar_wait(&ts.bar, tm.parity);
        if (ready) {
            tm.parity ^= 1u;
            tm.pending = false;
        } else {
            tm.broken = true;
            if (tid == 0) atomicOr(&a.st_flags[0], kErrTimeout);
        }
    }
    const int li = base + tid;
    bool keep = false;
    float4 r0, r1, r2;
    float vrej = 0.f;
    const uint32_t g = ts.gid[tid];
    if (ready && li < limit && g < a.n_gauss) {
        r0 = ts.raw[0][tid >> 2][tid & 3];
        r1 = ts.raw[1][tid >> 2][tid & 3];
        r2 = ts.raw[2][tid >> 2][tid & 3];
        vrej = reject_bound(r0.w);
        keep = !tile_prunable<FORWARD>(r0.x, r0.y, r1.x, r1.y, r1.z, vrej, x0, y0);
    }
    const uint32_t bal = __ballot_sync(kFullMask, keep);
    if (lane == 0) sb.wcnt[w] = __popc(bal);
    __syncthreads();  // the batch's raw rows and indices are consumed
    int wbase = 0, total = 0;
#pragma unroll
    for (int k = 0; k < kPix / 32; ++k) {
        const int c = sb.wcnt[k];
        wbase += (k < w) ? c : 0;
        total += c;
    }
    if (keep) put_staged<FORWARD ? kStageNone : kStageRay>(a, sb, wbase + __popc(bal & lanemask_lt()), r0, r1, r2, vrej, li, g);
    const bool next = ready && base + kBatch < limit;
    if (next && tid == 0) tma_bar_expect(&ts.bar, kTmaBatchBytes);
    __syncthreads();
    if (next) {
        tma_issue(a, maps, ts, list0, base + kBatch, limit);
        tm.pending = true;
    }
    return total;
}

// Start a pass: announce and gather its first batch.
__device__ __forceinline__ void tma_begin(const TrackArgs& a, const RecMaps& maps, TmaStage& ts, uint32_t list0,
                                          int limit, TmaState& tm) {
    if (limit <= 0 || tm.broken) return;
    if (threadIdx.x == 0) tma_bar_expect(&ts.bar, kTmaBatchBytes);
    __syncthreads();
    tma_issue(a, maps, ts, list0, 0, limit);
    tm.pending = true;
}

// End a pass: wait (bounded) for a gather still in flight, since the buffer
// is reused or the CTA exits.
__device__ __forceinline__ void tma_drain(const TrackArgs& a, TmaStage& ts, TmaState& tm) {
    if (!tm.pending) return;
    if (tma_bar_wait(&ts.bar, tm.parity)) {
        tm.parity ^= 1u;
        tm.pending = false;
    } else {
        tm.broken = true;
        if (threadIdx.x == 0) atomicOr(&a.st_flags[0], kErrTimeout);
    }
}

// Depth weight of a pixel's depth residual: the reference's
// (|e| < thr ? 1 : thr / |e|) / z_obs (src/GSCudaKernels.cu:1120-1121) with
// FVGS_Q_DEPTH_HUBER, else Tukey's biweight (1 - (e / thr)^2)^2 / z_obs, zero
// beyond thr.
__device__ __forceinline__ float depth_weight(float derr, float thr, float z_obs, bool huber) {
    const float ld = fabsf(derr);
    float w;
    if (huber) {
        w = (ld < thr) ? 1.0f : thr / ld;
    } else {
        const float r = ld / thr, t = 1.0f - r * r;
        w = (ld < thr) ? t * t : 0.0f;
    }
    return w / z_obs;
}

template <bool RENDER_ONLY, bool REF_LAYOUT = false, int MIN_CTAS = 4, bool TMA = false, int BATCH = kBatch,
          bool ANALYTIC = false>
__global__ void __launch_bounds__(kPix, MIN_CTAS) track_tile_kernel(TrackArgs a, const __grid_constant__ RecMaps maps) {
    static_assert(!TMA || BATCH == kBatch, "the TMA staging gathers batches of kBatch records");
    static_assert(BATCH % 128 == 0 && BATCH <= 2 * kPix, "batch of 128, 256 or 512 Gaussians");
    static_assert(!ANALYTIC || (!TMA && !REF_LAYOUT && BATCH <= kBatch), "analytic Jacobian: packed records, plain staging");
    pdl_begin();
    __shared__ TrackBatch<BATCH, ANALYTIC ? 8 : 1> sb;
    __shared__ float s_red[kPix / 32][32];
    __shared__ uint32_t s_nmax;
    extern __shared__ __align__(128) unsigned char s_dyn[];  // TMA variant: the gathered batch
    TmaStage& ts = *reinterpret_cast<TmaStage*>((reinterpret_cast<uintptr_t>(s_dyn) + 127) & ~uintptr_t(127));
    TmaState tm;
    if (TMA) {
        if (threadIdx.x == 0) tma_bar_init(&ts.bar);
        __syncthreads();
    }

    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int tid = threadIdx.x;
    // each warp covers an 8 x 4 pixel block (compact footprint: less divergence)
    const int wq = tid >> 5, lq = tid & 31;
    const int x = tx * kTW + (wq & 1) * 8 + (lq & 7), y = ty * kTH + (wq >> 1) * 4 + (lq >> 3);
    const float x0 = (float)(tx * kTW), y0 = (float)(ty * kTH);
    const bool in_bounds = (x < a.W && y < a.H);
    const size_t p = (size_t)y * a.W + x;
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    const int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    const float xf = (float)x, yf = (float)y;

    float img_depth = 0.f;
    if (!RENDER_ONLY && in_bounds) img_depth = a.obs_depth[p];
    const bool inside = RENDER_ONLY ? in_bounds : (in_bounds && img_depth > 0.1f);

    // ------------------------- pass 1: forward blend -------------------------
    float T = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, depth = 0.f;
    uint32_t last = 0;
    bool done = !inside;
    float final_T = 1.f;
    uint32_t n_contrib = 0;
    if (n > 0) {
        if (TMA) tma_begin(a, maps, ts, range.x, n, tm);
        for (int base = 0; base < n; base += BATCH) {
            if (__syncthreads_and(done)) break;
            int cnt;
            if constexpr (TMA)
                cnt = stage_batch_tma<true>(a, maps, sb, ts, range.x, base, n, x0, y0, tm);
            else
                cnt = stage_batch<REF_LAYOUT, true, kStageNone>(a, sb, range.x, base, n, x0, y0);
            if (!done) {
                int last_j = -1;  // staged slot of the last blended Gaussian in this batch
                // one staged Gaussian: returns false when the pixel terminates
                auto blend = [&](int j, float dx, float dy, float v) -> bool {
                    const float4 rB = sb.B[j];
                    const float alpha = gauss_alpha(rB.z, v);
                    if (alpha < kInv255) return true;
                    const float test_T = T * (1.0f - alpha);
                    if (test_T < 0.0001f) return false;
                    const float4 rC = sb.C[j];
                    const float aT = alpha * T;
                    cr += rC.z * aT;
                    cg += rC.w * aT;
                    cb += sb.D[j] * aT;
                    if (T > 0.5f && test_T < 0.5f) depth = depth_at(rB.w, dx, rC.x, dy, rC.y);
                    T = test_T;
                    last_j = j;
                    return true;
                };
                int j = 0;
                // two Gaussians per iteration: both quadratic forms are evaluated
                // before the (mostly rejecting) branches, in list order
                for (; j + 1 < cnt; j += 2) {
                    const float4 rA0 = sb.A[j], rA1 = sb.A[j + 1];
                    const float2 rB0 = *reinterpret_cast<const float2*>(&sb.B[j]);
                    const float2 rB1 = *reinterpret_cast<const float2*>(&sb.B[j + 1]);
                    const float dx0 = rA0.x - xf, dy0 = rA0.y - yf;
                    const float dx1 = rA1.x - xf, dy1 = rA1.y - yf;
                    float q0, q1;
                    const float v0 = conic_form(rA0.z, rA0.w, rB0.x, dx0, dy0, q0, q1);
                    const float v1 = conic_form(rA1.z, rA1.w, rB1.x, dx1, dy1, q0, q1);
                    const bool k0 = !(v0 > rB0.y || v0 <= 0.0f);
                    const bool k1 = !(v1 > rB1.y || v1 <= 0.0f);
                    if (k0 && !blend(j, dx0, dy0, v0)) {
                        done = true;
                        break;
                    }
                    if (k1 && !blend(j + 1, dx1, dy1, v1)) {
                        done = true;
                        break;
                    }
                }
                if (!done && j < cnt) {
                    const float4 rA = sb.A[j];
                    const float2 rB = *reinterpret_cast<const float2*>(&sb.B[j]);
                    const float dx = rA.x - xf, dy = rA.y - yf;
                    float q0, q1;
                    const float v = conic_form(rA.z, rA.w, rB.x, dx, dy, q0, q1);
                    if (!(v > rB.y || v <= 0.0f) && !blend(j, dx, dy, v)) done = true;
                }
                if (last_j >= 0) last = (uint32_t)sb.orig[last_j] + 1u;
            }
        }
        if (TMA) tma_drain(a, ts, tm);
        if (inside) {
            final_T = T;
            n_contrib = last;
            cr += T * a.bg[0];
            cg += T * a.bg[1];
            cb += T * a.bg[2];
        }
    }
    if (a.img_color && in_bounds) {
        a.img_color[3 * p] = cr;
        a.img_color[3 * p + 1] = cg;
        a.img_color[3 * p + 2] = cb;
        a.img_depth[p] = depth;
        a.img_T[p] = final_T;
        a.img_nc[p] = n_contrib;
    }
    if (RENDER_ONLY) return;

    // ------------------------- per-pixel term -------------------------------
    const bool do_jac = inside && (final_T < a.alpha_thresh);
    float A[21];
    float bv[6];
#pragma unroll
    for (int k = 0; k < 21; ++k) A[k] = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) bv[k] = 0.f;
    const float fx = a.K.fx, fy = a.K.fy, cx = a.K.cx, cy = a.K.cy;
    const bool huber = (a.quirks & FVGS_Q_DEPTH_HUBER) != 0;
    float e0 = 0.f, e1 = 0.f, e2 = 0.f, wc = 0.f, derr = 0.f, wd = 0.f;
    if (ANALYTIC && do_jac) {
        e0 = cr - a.obs_rgb[3 * p];
        e1 = cg - a.obs_rgb[3 * p + 1];
        e2 = cb - a.obs_rgb[3 * p + 2];
        derr = depth - img_depth;
        const float closs = sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
        wc = (closs < a.color_thresh) ? 1.0f : a.color_thresh / closs;
        wd = depth_weight(derr, a.depth_thresh, img_depth, huber);
    }
    if (!ANALYTIC && do_jac) {
        e0 = cr - a.obs_rgb[3 * p];
        e1 = cg - a.obs_rgb[3 * p + 1];
        e2 = cb - a.obs_rgb[3 * p + 2];
        derr = (img_depth > 0.1f) ? (depth - img_depth) : 0.0f;
        const float closs = sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
        wc = (closs < a.color_thresh) ? 1.0f : a.color_thresh / closs;
        const float rx = (xf - cx) / fx, ry = (yf - cy) / fy;
        const float inv_id = __frcp_rn(img_depth);
        const float j0 = fx * inv_id, j3 = fy * inv_id, j4 = -fx * rx * inv_id, j5 = -fy * ry * inv_id;
        const float gX[3] = {a.gx[3 * p], a.gx[3 * p + 1], a.gx[3 * p + 2]};
        const float gY[3] = {a.gy[3 * p], a.gy[3 * p + 1], a.gy[3 * p + 2]};
        const float ee[3] = {e0, e1, e2};
        float Jr0 = 0.f, Jr1 = 0.f, Jr2 = 0.f;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float c0 = j0 * gX[k], c1 = j3 * gY[k], c2 = j4 * gX[k] + j5 * gY[k];
            rank1_update(A, wc, c0, c1, c2, img_depth, rx, ry, 1.0f);
            Jr0 += c0 * ee[k];
            Jr1 += c1 * ee[k];
            Jr2 += c2 * ee[k];
        }
        Jr0 *= -wc;
        Jr1 *= -wc;
        Jr2 *= -wc;
        wd = depth_weight(derr, a.depth_thresh, img_depth, huber);
        // wd * ray ray^T: the rotation block gets ray x ray = 0
        {
            const float r[3] = {rx, ry, 1.0f};
            int idx = 0;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
#pragma unroll
                for (int j = i; j < 6; ++j) {
                    if (j < 3) A[idx] += wd * r[i] * r[j];
                    ++idx;
                }
            }
        }
        Jr0 += wd * derr * rx;
        Jr1 += wd * derr * ry;
        Jr2 += wd * derr;
        bv[0] += Jr0;
        bv[1] += Jr1;
        bv[2] += Jr2;
        bv[3] += img_depth * (ry * Jr2 - 1.0f * Jr1);
        bv[4] += img_depth * (1.0f * Jr0 - rx * Jr2);
        bv[5] += img_depth * (rx * Jr1 - ry * Jr0);
    }

    // ------------------- pass 2: per-Gaussian terms --------------------------
    if (tid == 0) s_nmax = 0;
    __syncthreads();
    if (do_jac && n_contrib > 0) atomicMax(&s_nmax, n_contrib);
    __syncthreads();
    const int nmax = (int)min((uint32_t)n, s_nmax);
    if constexpr (ANALYTIC) {
        // Colour Jacobian jc (3 x 6) and depth Jacobian jd of the pixel over
        // the Gaussians the forward pass blended, in its order: for each,
        // dC/dalpha = c T - (C - A) / (1 - alpha) (A: colour accumulated up
        // to and including it, C: final colour with background), dalpha/dv =
        // -alpha / 2 (0 where alpha is clamped at 0.99) and dv/ddelta from
        // the staged derivatives; jd is the derivative of
        // d = z + dx phat.x + dy phat.y of the Gaussian where T crosses 0.5.
        float jc[3][6], jd[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            jc[0][k] = jc[1][k] = jc[2][k] = 0.f;
            jd[k] = 0.f;
        }
        float prod = 1.f, remr = cr, remg = cg, remb = cb;
        bool done2 = !do_jac;
        for (int base = 0; base < nmax; base += BATCH) {
            if (__syncthreads_and(done2)) break;
            const int cnt = stage_batch<false, true, kStageDeriv>(a, sb, range.x, base, nmax, x0, y0);
            if (done2) continue;
            for (int j = 0; j < cnt; ++j) {
                if (sb.orig[j] >= (int)n_contrib) {
                    done2 = true;
                    break;
                }
                const float4 rA = sb.A[j];
                const float4 rB = sb.B[j];
                const float dx = rA.x - xf, dy = rA.y - yf;
                float dl0, dl1;
                const float v = conic_form(rA.z, rA.w, rB.x, dx, dy, dl0, dl1);
                if (v > rB.y || v <= 0.0f) continue;
                const float raw = gauss_weight(rB.z, v);
                const float alpha = fminf(0.99f, raw);
                if (alpha < kInv255) continue;
                const float4 rC = sb.C[j];
                float d0 = rC.z * prod, d1 = rC.w * prod, d2 = sb.D[j] * prod;
                remr -= alpha * d0;
                remg -= alpha * d1;
                remb -= alpha * d2;
                const float inv1m = rcp_approx(1.0f - alpha);
                const float kf = (raw > 0.99f) ? 0.0f : -0.5f * alpha;
                const float k0 = kf * (d0 - remr * inv1m), k1 = kf * (d1 - remg * inv1m),
                            k2 = kf * (d2 - remb * inv1m);
                const float cu = 2.0f * dl0, cv = 2.0f * dl1, ca = dx * dx, cb2 = 2.0f * dx * dy, cc = dy * dy;
                const float4 X0 = sb.X[0][j], X1 = sb.X[1][j], X2 = sb.X[2][j], X3 = sb.X[3][j];
                const float4 X4 = sb.X[4][j], X5 = sb.X[5][j], X6 = sb.X[6][j], X7 = sb.X[7][j];
                const float du[6] = {X0.x, X0.y, X0.z, X0.w, X1.x, X1.y};
                const float dv[6] = {X1.z, X1.w, X2.x, X2.y, X2.z, X2.w};
                const float da[6] = {X3.x, X3.y, X3.z, X3.w, X4.x, X4.y};
                const float db[6] = {X4.z, X4.w, X5.x, X5.y, X5.z, X5.w};
                const float dc[6] = {X6.x, X6.y, X6.z, X6.w, X7.x, X7.y};
                float gv[6];
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    gv[k] = cu * du[k] + cv * dv[k] + ca * da[k] + cb2 * db[k] + cc * dc[k];
                    jc[0][k] += k0 * gv[k];
                    jc[1][k] += k1 * gv[k];
                    jc[2][k] += k2 * gv[k];
                }
                const float np = prod * (1.0f - alpha);
                if (prod > 0.5f && np < 0.5f) {
                    // d phat = (dp_x / z^2 - 2 x dp_z / z^3, dp_y / z^2 - 2 y dp_z / z^3)
                    const float z = rB.w, x = X7.z, y = X7.w;
                    const float iz = __frcp_rn(z), iz2 = iz * iz, iz3 = iz2 * iz;
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const float dpx = k == 0 ? -1.f : (k == 4 ? -z : (k == 5 ? y : 0.f));
                        const float dpy = k == 1 ? -1.f : (k == 3 ? z : (k == 5 ? -x : 0.f));
                        const float dpz = k == 2 ? -1.f : (k == 3 ? -y : (k == 4 ? x : 0.f));
                        const float dphx = dpx * iz2 - 2.f * x * iz3 * dpz;
                        const float dphy = dpy * iz2 - 2.f * y * iz3 * dpz;
                        jd[k] = dpz + rC.x * du[k] + dx * dphx + rC.y * dv[k] + dy * dphy;
                    }
                }
                prod = np;
            }
        }
        if (do_jac) {
            int idx = 0;
#pragma unroll
            for (int i = 0; i < 6; ++i) {
#pragma unroll
                for (int k = i; k < 6; ++k)
                    A[idx++] = wc * (jc[0][i] * jc[0][k] + jc[1][i] * jc[1][k] + jc[2][i] * jc[2][k]) +
                               wd * jd[i] * jd[k];
                bv[i] = -(wc * (jc[0][i] * e0 + jc[1][i] * e1 + jc[2][i] * e2) + wd * jd[i] * derr);
            }
        }
    } else {
        // rem = final colour minus the colour accumulated so far (running)
        float prod_alpha = 1.f, remr = cr, remg = cg, remb = cb;
        bool depth_pending = img_depth > 0.5f;  // the depth term is added once, where T first falls to 0.5
        bool done2 = !do_jac;
        if (TMA) tma_begin(a, maps, ts, range.x, nmax, tm);
        for (int base = 0; base < nmax; base += BATCH) {
            if (__syncthreads_and(done2)) break;
            int cnt;
            if constexpr (TMA)
                cnt = stage_batch_tma<false>(a, maps, sb, ts, range.x, base, nmax, x0, y0, tm);
            else
                cnt = stage_batch<REF_LAYOUT, false, kStageRay>(a, sb, range.x, base, nmax, x0, y0);
            if (!done2) {
                for (int j = 0; j < cnt; ++j) {
                    if (sb.orig[j] >= (int)n_contrib) {
                        done2 = true;
                        break;
                    }
                    const float4 rA = sb.A[j];
                    const float4 rB = sb.B[j];
                    const float dx = rA.x - xf, dy = rA.y - yf;
                    float dl0, dl1;
                    const float v = conic_form(rA.z, rA.w, rB.x, dx, dy, dl0, dl1);
                    if (v > rB.y) continue;
                    const float alpha = gauss_alpha(rB.z, v);
                    if (alpha < kInv255) continue;
                    const float4 rC = sb.C[j];
                    const float4 rE = sb.X[0][j];
                    const float d = depth_fast(rB.w, dx, rC.x, dy, rC.y);
                    float da0 = rC.z * prod_alpha, da1 = rC.w * prod_alpha, da2 = sb.D[j] * prod_alpha;
                    remr -= alpha * da0;
                    remg -= alpha * da1;
                    remb -= alpha * da2;
                    const float inv1m = rcp_approx(1.0f - alpha);
                    da0 -= remr * inv1m;
                    da1 -= remg * inv1m;
                    da2 -= remb * inv1m;
                    // The reference's per-Gaussian row is u = (jt, d (r x jt)) with
                    // jt = g / d, g = (fx dl0, fy dl1, -fx rgx dl0 - fy rgy dl1) and
                    // r = (rgx, rgy, 1): the same vector as (g / d, r x g).
                    const float g0 = fx * dl0, g1 = fy * dl1, g2 = rE.z * dl0 + rE.w * dl1;
                    const float inv_d = rcp_approx(d);
                    const float u0 = g0 * inv_d, u1 = g1 * inv_d, u2 = g2 * inv_d;
                    const float u3 = rE.y * g2 - g1, u4 = g0 - rE.x * g2, u5 = rE.x * g1 - rE.y * g0;
                    const float w = wc * alpha * alpha * (da0 * da0 + da1 * da1 + da2 * da2);
                    {
                        const float u[6] = {u0, u1, u2, u3, u4, u5};
                        int idx = 0;
    #pragma unroll
                        for (int i = 0; i < 6; ++i) {
                            const float wu = w * u[i];
    #pragma unroll
                            for (int k = i; k < 6; ++k) A[idx++] += wu * u[k];
                        }
                    }
                    const float coef = -wc * alpha * (da0 * e0 + da1 * e1 + da2 * e2);
                    bv[0] += coef * u0;
                    bv[1] += coef * u1;
                    bv[2] += coef * u2;
                    bv[3] += coef * u3;
                    bv[4] += coef * u4;
                    bv[5] += coef * u5;
                    prod_alpha *= (1.0f - alpha);
                    if (depth_pending && prod_alpha <= 0.5f) {
                        // the depth term wd * derr * r: its rotation part d (r x r) is zero
                        depth_pending = false;
                        const float r[3] = {rE.x, rE.y, 1.0f};
                        int idx = 0;
    #pragma unroll
                        for (int i = 0; i < 3; ++i) {
    #pragma unroll
                            for (int jj = i; jj < 6; ++jj) {
                                if (jj < 3) A[idx] += wd * r[i] * r[jj];
                                ++idx;
                            }
                        }
                        bv[0] += wd * derr * rE.x;
                        bv[1] += wd * derr * rE.y;
                        bv[2] += wd * derr;
                    }
                    if (prod_alpha < 0.001f) {
                        done2 = true;
                        break;
                    }
                }
            }
        }
    }
    if (TMA) tma_drain(a, ts, tm);

    // --------------------------- tile reduction ------------------------------
    float vals[32];
#pragma unroll
    for (int k = 0; k < 6; ++k) vals[k] = bv[k];
#pragma unroll
    for (int k = 0; k < 21; ++k) vals[6 + k] = A[k];
#pragma unroll
    for (int k = 27; k < 32; ++k) vals[k] = 0.f;
    const float mine = warp_reduce_scatter32(vals);
    s_red[tid >> 5][tid & 31] = mine;
    __syncthreads();
    if (tid < FVGS_POSEDATA_FLOATS) {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < kPix / 32; ++w) s += s_red[w][tid];
        a.tile_out[(size_t)tile * FVGS_POSEDATA_FLOATS + tid] = s;
    }
}

// Cholesky of a symmetric 6x6 (lower factor in L); false if not positive
// definite.  Fully unrolled so everything stays in registers.
__device__ __forceinline__ bool chol6(const double A[6][6], double L[6][6]) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double s = A[j][j];
#pragma unroll
        for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
        if (!(s > 0.0)) return false;
        const double ljj = sqrt(s);
        L[j][j] = ljj;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            double t = A[i][j];
#pragma unroll
            for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
            L[i][j] = t / ljj;
        }
#pragma unroll
        for (int i = 0; i < j; ++i) L[i][j] = 0.0;
    }
    return true;
}

// delta = -sum_{lambda_i > eps} (u_i . g / lambda_i) u_i for symmetric H:
// the Gauss-Newton step of the pseudo residual / Jacobian pair that
// RgbdPoseCostFunction::Evaluate builds from the eigen-decomposition of JtJ
// (src/RgbdPoseCost.cu:57-78).  When H - eps*I is positive definite every
// eigenvalue is kept and the step is exactly -H^-1 g (Cholesky); otherwise a
// cyclic Jacobi eigen-decomposition drops the small eigenvalues.
__device__ __noinline__ void pseudo_step(const double H[6][6], const double g[6], double eps, double delta[6]) {
    double L[6][6];
    double He[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) He[i][j] = H[i][j] - (i == j ? eps : 0.0);
    if (chol6(He, L) && chol6(H, L)) {
        double y[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            double s = g[i];
#pragma unroll
            for (int k = 0; k < i; ++k) s -= L[i][k] * y[k];
            y[i] = s / L[i][i];
        }
#pragma unroll
        for (int i = 5; i >= 0; --i) {
            double s = y[i];
#pragma unroll
            for (int k = i + 1; k < 6; ++k) s -= L[k][i] * delta[k];
            delta[i] = s / L[i][i];
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) delta[i] = -delta[i];
        return;
    }
    double A[6][6], V[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            A[i][j] = H[i][j];
            V[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0, tot = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                tot += A[i][j] * A[i][j];
                if (i != j) off += A[i][j] * A[i][j];
            }
        if (off <= 1e-30 * tot) break;
#pragma unroll
        for (int p = 0; p < 5; ++p)
#pragma unroll
            for (int q = p + 1; q < 6; ++q) {
                const double apq = A[p][q];
                if (apq != 0.0) {
                    const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                    const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                    const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const double akp = A[k][p], akq = A[k][q];
                        A[k][p] = cs * akp - sn * akq;
                        A[k][q] = sn * akp + cs * akq;
                    }
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const double apk = A[p][k], aqk = A[q][k];
                        A[p][k] = cs * apk - sn * aqk;
                        A[q][k] = sn * apk + cs * aqk;
                    }
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const double vkp = V[k][p], vkq = V[k][q];
                        V[k][p] = cs * vkp - sn * vkq;
                        V[k][q] = sn * vkp + cs * vkq;
                    }
                }
            }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) delta[k] = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const double lam = A[i][i];
        if (lam > eps) {
            double ug = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) ug += V[k][i] * g[k];
#pragma unroll
            for (int k = 0; k < 6; ++k) delta[k] -= (ug / lam) * V[k][i];
        }
    }
}

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(kFullMask, v, src); }

// 1/x for finite positive x: the PTX rcp.approx.ftz.f64 estimate refined by
// two Newton steps r += r (1 - x r), each doubling the correct bits, to within
// an ulp or two of the correctly rounded reciprocal.  FP64 division is a long
// dependent sequence on this part, and the factorisation and pose step below
// are latency chains.
__device__ __forceinline__ double rcp_newton(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    r = fma(r, fma(-x, r, 1.0), r);
    return fma(r, fma(-x, r, 1.0), r);
}

// Lower-triangle lane map: lane l < 21 holds entry (i, j), i >= j,
// l = i (i + 1) / 2 + j.
__device__ __forceinline__ int tri_index(int i, int j) { return i * (i + 1) / 2 + j; }

// Warp-parallel LDL^T factorisation of a symmetric 6x6 held as one
// lower-triangle entry per lane (lanes >= 21 idle), without square roots: on
// return lane tri_index(i, j) holds L[i][j] (i > j, unit diagonal implied) or
// D[i] (i == j).  Returns false (uniformly) when a pivot is not positive, i.e.
// the matrix is not positive definite.  Lane k < 6 also ends with 1 / D[k]
// in inv_d.
__device__ __forceinline__ bool warp_ldl6(double& m, int li, int lj, double& inv_d) {
    const int lane = threadIdx.x & 31;
    const bool act = lane < 21;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double dk = shfl_d(m, tri_index(k, k));
        if (!(dk > 0.0 && dk <= 1e300)) return false;
        const double inv = rcp_newton(dk);
        if (lane == k) inv_d = inv;
        // entries still holding L(i, k) D(k) for i > k
        const double lik = shfl_d(m, (act && li > k) ? tri_index(li, k) : 0);
        const double ljk = shfl_d(m, (act && lj > k) ? tri_index(lj, k) : 0);
        if (act && lj > k) m = fma(-lik * inv, ljk, m);
        if (act && lj == k && li > k) m *= inv;
    }
    return true;
}

// Frame reduction + (optionally) the Gauss-Newton pose update, one cluster of
// kRedCtas CTAs: warp k of the cluster sums tiles k, k + 8 kRedCtas, ... with
// lane l < 27 holding column l (Kahan-compensated FP32, fixed order), the
// CTA combines its warps in FP64, and CTA 0 gathers the CTAs' sums over
// distributed shared memory in rank order (deterministic).  The total is
// rotated to the world frame by diag(R, I) and written as out[42] = JtJ[36]
// symmetric, Jtr[6] negated (src/GSSlam.cu:2205-2226); then the pseudo-factor
// step of RgbdPoseCostFunction (src/RgbdPoseCost.cu:57-78) and
// PoseLocalParameterization::Plus on the device pose.
//
// FP64 is issued slowly on this part, so the 6x6 work is spread over lanes:
// warp 0 factors H - eps*I (all eigenvalues > eps exactly when it is positive
// definite, and then the eigen-regularised step equals -H^-1 g), warp 1 factors
// H and solves; only a failed test falls back to a one-thread Jacobi
// eigen-decomposition that drops the small eigenvalues.
constexpr int kRedCtas = 8;
constexpr int kRedUnroll = 28;
template <bool DO_GN>
__global__ void __cluster_dims__(kRedCtas, 1, 1) __launch_bounds__(256)
    track_reduce_kernel(const float* __restrict__ tile_out, int num_tiles, DevPose* pose, double* out,
                        double eig_eps, double* step_out) {
    pdl_begin();
    __shared__ double s_w[8][32];
    __shared__ double s_part[32];
    __shared__ double s_tot[27];
    __shared__ double s_R[9];
    __shared__ int s_pd;
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank();
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int col = lane < FVGS_POSEDATA_FLOATS ? lane : 0;
    const int stride = kRedCtas * 8;
    // the pose the step is applied to, loaded now so its latency overlaps the sums
    float pq[4] = {0.f, 0.f, 0.f, 0.f};
    double pqd[4] = {0.0, 0.0, 0.0, 0.0}, ptd[3] = {0.0, 0.0, 0.0};
    if (DO_GN && rank == 0 && w == 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            pq[k] = pose->q[k];
            pqd[k] = pose->qd[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) ptd[k] = pose->td[k];
    }
    // every load of a round is issued before the (ordered) compensated adds
    float sum = 0.f, comp = 0.f;
    for (int t0 = (int)rank * 8 + w; t0 < num_tiles; t0 += kRedUnroll * stride) {
        float x[kRedUnroll];
#pragma unroll
        for (int u = 0; u < kRedUnroll; ++u) {
            const int t = t0 + u * stride;
            x[u] = t < num_tiles ? tile_out[(size_t)t * FVGS_POSEDATA_FLOATS + col] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kRedUnroll; ++u) {
            if (t0 + u * stride < num_tiles) {
                const float y = __fsub_rn(x[u], comp);
                const float s = __fadd_rn(sum, y);
                comp = __fsub_rn(__fsub_rn(s, sum), y);
                sum = s;
            }
        }
    }
    s_w[w][lane] = lane < FVGS_POSEDATA_FLOATS ? (double)sum - (double)comp : 0.0;
    __syncthreads();
    if (w == 0) {
        double c = 0.0;
#pragma unroll
        for (int ww = 0; ww < 8; ++ww) c += s_w[ww][lane];
        s_part[lane] = c;
    }
    cluster.sync();  // every CTA's column sums are visible cluster-wide
    if (rank == 0 && w == 0 && lane < FVGS_POSEDATA_FLOATS) {
        double c = 0.0;
#pragma unroll
        for (int r = 0; r < kRedCtas; ++r) c += cluster.map_shared_rank(s_part, r)[lane];
        s_tot[lane] = c;
    }
    cluster.sync();  // CTA 0 has read the remote sums; the others may leave
    if (rank != 0) return;
    if (w >= 2) return;
    // ---- CTA 0, warps 0 and 1 only; named barrier 1 over 64 threads ----
    // lane l < 21 holds lower-triangle entry (li, lj) of a symmetric 6x6
    int li = 0, lj = 0;
    if (lane < 21) {
        while (tri_index(li + 1, 0) <= lane) ++li;
        lj = lane - tri_index(li, 0);
    }
    auto Ac = [&](int a, int b) {
        const int hi = a > b ? a : b, lo = a > b ? b : a;
        // upper-triangle row-major index of (lo, hi) among the 21 JtJ sums
        return s_tot[6 + lo * 6 - lo * (lo - 1) / 2 + (hi - lo)];
    };
    if (!DO_GN) {
        // world-frame JtJ = D A D^T and Jtr = -(D b), D = diag(R, I)
        if (w == 1 && lane < 9) {
            const double qx = pose->q[0], qy = pose->q[1], qz = pose->q[2], qw = pose->q[3];
            const int i = lane / 3, j = lane % 3;
            const double q[3] = {qx, qy, qz};
            double r;
            if (i == j) {
                const double a = q[(i + 1) % 3], b2 = q[(i + 2) % 3];
                r = 1.0 - 2.0 * (a * a + b2 * b2);
            } else {
                // off-diagonal: 2 (q_i q_j -/+ w q_k), sign + when (i, j) is (1,0), (2,1), (0,2)
                const int k = 3 - i - j;
                const bool plus = (i == (j + 1) % 3);
                r = 2.0 * (q[i] * q[j] + (plus ? qw * q[k] : -qw * q[k]));
            }
            s_R[lane] = r;
        }
        asm volatile("bar.sync 1, 64;" ::: "memory");
        if (w != 0) return;
        if (lane < 21) {
            double m;
            if (li < 3) {  // then lj < 3
                double s = 0.0;
#pragma unroll
                for (int a2 = 0; a2 < 3; ++a2)
#pragma unroll
                    for (int b2 = 0; b2 < 3; ++b2) s = fma(s_R[li * 3 + a2] * Ac(a2, b2), s_R[lj * 3 + b2], s);
                m = s;
            } else if (lj < 3) {
                double s = 0.0;
#pragma unroll
                for (int b2 = 0; b2 < 3; ++b2) s = fma(Ac(li, b2), s_R[lj * 3 + b2], s);
                m = s;
            } else {
                m = Ac(li, lj);
            }
            out[li * 6 + lj] = m;
            out[lj * 6 + li] = m;
        } else if (lane < 27) {
            const int i = lane - 21;
            out[36 + i] = i < 3 ? -(s_R[i * 3] * s_tot[0] + s_R[i * 3 + 1] * s_tot[1] + s_R[i * 3 + 2] * s_tot[2])
                                : -s_tot[i];
        }
        return;
    }
    // Gauss-Newton step.  With H = D A D^T and g = -(D b) the step
    // -H^-1 g equals D x for A x = b, and H, A share their eigenvalues, so the
    // camera-frame system is factored and only the step is rotated.
    double m = lane < 21 ? Ac(li, lj) : 0.0;
    if (w == 0) {
        if (lane < 21 && li == lj) m -= eig_eps;
        double inv_d;
        const bool pd = warp_ldl6(m, li, lj, inv_d);
        if (lane == 0) s_pd = pd ? 1 : 0;
        asm volatile("bar.sync 1, 64;" ::: "memory");
        return;
    }
    // warp 1
    double inv_d = 0.0;
    const bool pdh = warp_ldl6(m, li, lj, inv_d);
    asm volatile("bar.sync 1, 64;" ::: "memory");
    double xv = lane < 6 ? s_tot[lane] : 0.0;  // lane k < 6 ends with x[k]
    if (s_pd && pdh) {
        // L y = b (unit lower)
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double yk = shfl_d(xv, k);
            const double lik = shfl_d(m, (lane < 6 && lane > k) ? tri_index(lane, k) : 0);
            if (lane < 6 && lane > k) xv = fma(-lik, yk, xv);
        }
        // D z = y
        if (lane < 6) xv *= inv_d;
        // L^T x = z (unit upper)
#pragma unroll
        for (int k = 5; k >= 0; --k) {
            const double xk = shfl_d(xv, k);
            const double lki = shfl_d(m, (lane < k) ? tri_index(k, lane) : 0);
            if (lane < k) xv = fma(-lki, xk, xv);
        }
    } else {
        // rare: some eigenvalue <= eps -- exact eigen-decomposition on one lane
        double dl[6] = {0, 0, 0, 0, 0, 0};
        if (lane == 0) {
            double A[6][6], g[6];
            for (int i = 0; i < 6; ++i) {
                for (int j = 0; j < 6; ++j) A[i][j] = Ac(i, j);
                g[i] = -s_tot[i];
            }
            pseudo_step(A, g, eig_eps, dl);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double d = shfl_d(dl[k], 0);
            if (lane == k) xv = d;
        }
    }
    double x[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) x[k] = shfl_d(xv, k);
    if (lane != 0) return;
    // delta = (R x_t, x_r), R of the pose the Jacobians were taken at
    const double qx = pq[0], qy = pq[1], qz = pq[2], qw = pq[3];
    const double R[3][3] = {
        {1.0 - 2.0 * (qy * qy + qz * qz), 2.0 * (qx * qy - qw * qz), 2.0 * (qx * qz + qw * qy)},
        {2.0 * (qx * qy + qw * qz), 1.0 - 2.0 * (qx * qx + qz * qz), 2.0 * (qy * qz - qw * qx)},
        {2.0 * (qx * qz - qw * qy), 2.0 * (qy * qz + qw * qx), 1.0 - 2.0 * (qx * qx + qy * qy)}};
    double delta[6];
#pragma unroll
    for (int i = 0; i < 3; ++i) delta[i] = R[i][0] * x[0] + R[i][1] * x[1] + R[i][2] * x[2];
#pragma unroll
    for (int i = 3; i < 6; ++i) delta[i] = x[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        ptd[k] += delta[k];
        pose->td[k] = ptd[k];
    }
    const double ax = pqd[0], ay = pqd[1], az = pqd[2], aw = pqd[3];
    const double bx = 0.5 * delta[3], by = 0.5 * delta[4], bz = 0.5 * delta[5];
    double nx = aw * bx + ax + (ay * bz - az * by);
    double ny = aw * by + ay + (az * bx - ax * bz);
    double nz = aw * bz + az + (ax * by - ay * bx);
    double nw = aw - (ax * bx + ay * by + az * bz);
    // 1 / |n| by the FP32 estimate and two Newton steps r *= (3 - n2 r^2) / 2
    // (about 2^-22, 2^-44, then rounding): the quaternion is within O(|delta|^2)
    // of unit length, and FP64 square root and division are long chains here
    const double n2 = nx * nx + ny * ny + nz * nz + nw * nw;
    double inn = (double)rsqrtf((float)n2);
    inn = inn * fma(-0.5 * n2, inn * inn, 1.5);
    inn = inn * fma(-0.5 * n2, inn * inn, 1.5);
    nx *= inn;
    ny *= inn;
    nz *= inn;
    nw *= inn;
    pose->qd[0] = nx;
    pose->qd[1] = ny;
    pose->qd[2] = nz;
    pose->qd[3] = nw;
#pragma unroll
    for (int k = 0; k < 3; ++k) pose->t[k] = (float)ptd[k];
    pose->q[0] = (float)nx;
    pose->q[1] = (float)ny;
    pose->q[2] = (float)nz;
    pose->q[3] = (float)nw;
    if (step_out)
#pragma unroll
        for (int k = 0; k < 6; ++k) step_out[k] = delta[k];
}

cudaError_t launch_track(const TrackArgs& a, const RecMaps* maps, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    RecMaps m{};
    if (maps) m = *maps;
    if (a.render_only) return launch_chained(track_tile_kernel<true>, dim3(T), dim3(kPix), 0, s, a, m);
    if (!(a.quirks & FVGS_Q_POSE_JAC_APPROX)) {
        // analytic Jacobian: plain staging of up to 256 Gaussians per batch
        // (the derivative planes fill the rest of the shared memory)
        if (!a.geo0 || !a.geo1) return cudaErrorInvalidValue;
        if (a.variant == 1)
            return launch_chained(track_tile_kernel<false, false, 3, false, kBatch, true>, dim3(T), dim3(kPix), 0, s,
                                  a, m);
        if (a.variant == 3)
            return launch_chained(track_tile_kernel<false, false, 4, false, 128, true>, dim3(T), dim3(kPix), 0, s, a,
                                  m);
        return launch_chained(track_tile_kernel<false, false, 4, false, kBatch, true>, dim3(T), dim3(kPix), 0, s, a,
                              m);
    }
    if (a.variant == 1) return launch_chained(track_tile_kernel<false, false, 3>, dim3(T), dim3(kPix), 0, s, a, m);
    if (a.variant == 3)
        return launch_chained(track_tile_kernel<false, false, 4, false, 128>, dim3(T), dim3(kPix), 0, s, a, m);
    if (a.variant == 4)
        return launch_chained(track_tile_kernel<false, false, 4, false, 512>, dim3(T), dim3(kPix), 0, s, a, m);
    if (a.variant == 2) {
        if (!maps || !a.st_flags) return cudaErrorInvalidValue;
        return launch_chained(track_tile_kernel<false, false, 4, true>, dim3(T), dim3(kPix), sizeof(TmaStage) + 128,
                              s, a, m);
    }
    return launch_chained(track_tile_kernel<false>, dim3(T), dim3(kPix), 0, s, a, m);
}

cudaError_t launch_track_ref_layout(const TrackArgs& a, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    return launch_chained(track_tile_kernel<false, true>, dim3(T), dim3(kPix), 0, s, a, RecMaps{});
}

cudaError_t launch_track_reduce(const float* tile_out, int num_tiles, DevPose* pose, double* out,
                                cudaStream_t s) {
    return launch_chained(track_reduce_kernel<false>, dim3(kRedCtas), dim3(256), 0, s, tile_out, num_tiles, pose, out,
                          0.0, static_cast<double*>(nullptr));
}

cudaError_t launch_track_reduce_gn(const float* tile_out, int num_tiles, DevPose* pose, double* out,
                                   double eig_eps, double* step_out, cudaStream_t s) {
    return launch_chained(track_reduce_kernel<true>, dim3(kRedCtas), dim3(256), 0, s, tile_out, num_tiles, pose, out,
                          eig_eps, step_out);
}

}  // namespace fvgs
