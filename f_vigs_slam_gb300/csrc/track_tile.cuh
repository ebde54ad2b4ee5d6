// track_tile.cuh -- the per-tile body of the fused tracking kernel (forward
// blend + RGB-D pose Jacobian + per-tile J^T J / J^T r reduction) and its
// helpers, shared by the per-frame kernel (track.cu) and the persistent
// kernel that runs the tiles of many sessions in one launch (track_batch.cu).
//
// Reference: getRgbdPoseJacobians (src/GSCudaKernels.cu:922-1392); the
// arithmetic and its reorganisation are described at the top of track.cu.
#pragma once

#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

// The default tile (16 x 16, one thread per pixel) -- the reference's TILE_SIZE
// (src/GSCudaKernels.cu:6) -- and the only one of the TMA-staged variant.
constexpr int kTW = 16, kTH = 16, kPix = kTW * kTH;
constexpr int kBatch = 256;
constexpr float kInv255 = 1.0f / 255.0f;

// Error-free difference: hi + lo == a - b exactly (TwoSum).
__device__ __forceinline__ void two_diff(float a, float b, float& hi, float& lo) {
    hi = __fsub_rn(a, b);
    const float bb = __fsub_rn(hi, a);
    lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fsub_rn(-b, bb));
}

// z + dx*phx + dy*phy, dx = u - x and dy = v - y taken exactly, with
// compensated arithmetic (error-free differences and products via TwoSum and
// FMA, error-free sums via TwoSum): the per-Gaussian depth cancels to values
// near zero for distant pixels, and its reciprocal enters the Jacobian, so a
// plain FP32 evaluation -- or one that rounds dx, which happens when |dx|
// exceeds |u| -- would cost several digits there.
__device__ __forceinline__ float depth_at(float z, float u, float x, float phx, float v, float y, float phy) {
    float dx, dxl, dy, dyl;
    two_diff(u, x, dx, dxl);
    two_diff(v, y, dy, dyl);
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
    const float lo = __fmaf_rn(dxl, phx, __fmul_rn(dyl, phy));
    return __fadd_rn(s2, __fadd_rn(__fadd_rn(r1, r2), __fadd_rn(__fadd_rn(e1, e2), lo)));
}

// z + dx*phx + dy*phy by two FMAs on the rounded dx = u - x, dy = v - y when
// that is accurate, else depth_at.  Each FMA rounds once and dx, dy carry at
// most half an ulp each, so the error is at most 2^-24 (|t| + |s| + |dx phx|
// + |dy phy|) with t the first FMA's result and s the second's; when |t|, |dx
// phx| and |dy phy| are all within 8 |s| that is under 1.2e-6 |s|.
// Cancellation and non-finite values take the compensated path.
__device__ __forceinline__ float depth_fast(float z, float dx, float phx, float dy, float phy, float u, float x,
                                           float v, float y) {
    const float t = __fmaf_rn(dx, phx, z);
    const float s = __fmaf_rn(dy, phy, t);
    const float m = 8.0f * fabsf(s);
    if (fabsf(t) <= m && fabsf(dx * phx) <= m && fabsf(dy * phy) <= m) return s;
    return depth_at(z, u, x, phx, v, y, phy);
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

// Kahan-compensated s += x: c carries the running rounding error.
__device__ __forceinline__ void kahan_add(float& s, float& c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// Error-free sum: hi + lo == a + b exactly (TwoSum).
__device__ __forceinline__ void two_sum(float a, float b, float& hi, float& lo) {
    hi = __fadd_rn(a, b);
    const float bb = __fsub_rn(hi, a);
    lo = __fadd_rn(__fsub_rn(a, __fsub_rn(hi, bb)), __fsub_rn(b, bb));
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

// The same with every value an unevaluated sum v + e (precision form): each
// add is a TwoSum whose error joins the low parts, so the warp sum of value l
// is returned as hi + lo with the rounding of the butterfly compensated.
__device__ __forceinline__ void warp_reduce_scatter32_comp(float (&v)[32], float (&e)[32], float& hi, float& lo) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const bool upper = (lane & o) != 0;
#pragma unroll
        for (int k = 0; k < o; ++k) {
            const float send = upper ? v[k] : v[k + o], send_e = upper ? e[k] : e[k + o];
            const float keep = upper ? v[k + o] : v[k], keep_e = upper ? e[k + o] : e[k];
            const float rv = __shfl_xor_sync(kFullMask, send, o), re = __shfl_xor_sync(kFullMask, send_e, o);
            float err;
            two_sum(keep, rv, v[k], err);
            e[k] = __fadd_rn(__fadd_rn(keep_e, re), err);
        }
    }
    hi = v[0];
    lo = e[0];
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
template <bool FORWARD, int TW = kTW, int TH = kTH>
__device__ __forceinline__ bool tile_prunable(float u, float v, float ca, float cb, float cc, float vrej, float x0,
                                              float y0) {
    if (vrej == -INFINITY) return true;  // zero opacity: alpha is 0 everywhere
    if (!(isfinite(u) && isfinite(v) && isfinite(ca) && isfinite(cb) && isfinite(cc) && isfinite(vrej))) return false;
    const float dxlo = u - (x0 + (float)(TW - 1)), dxhi = u - x0;
    const float dylo = v - (y0 + (float)(TH - 1)), dyhi = v - y0;
    const float mx = fmaxf(fabsf(dxlo), fabsf(dxhi)), my = fmaxf(fabsf(dylo), fabsf(dyhi));
    const float margin = 1e-5f * (fabsf(ca) * mx * mx + 2.0f * fabsf(cb) * mx * my + fabsf(cc) * my * my) + 1e-3f;
    if (quad_min_rect(ca, cb, cc, dxlo, dxhi, dylo, dyhi) > vrej + margin) return true;
    if (FORWARD && -quad_min_rect(-ca, -cb, -cc, dxlo, dxhi, dylo, dyhi) < -margin) return true;
    return false;
}

// The warps of a TW x TH tile (8 x 4 pixel blocks, row-major) whose pixels a
// staged Gaussian can reach: those whose block meets the axis-aligned box of
// the ellipse v <= vreject (v = a dx^2 + 2 b dx dy + c dy^2, half-widths
// sqrt(V c / det) and sqrt(V a / det)).  Every pixel outside it rejects the
// Gaussian in both passes (v > vreject), so a warp whose block misses the box
// may skip it without changing any result.  V = 1.05 vreject + 1e-3 and the
// widths grow by 1% + 0.01 px: when det >= 1e-4 a c the FP32 evaluation of v
// errs by less than 1.6% of v, so no pixel the kernel would keep falls
// outside.  Forms that are not positive definite, nearly singular ones and
// non-finite values reach every warp.
template <int TW, int TH>
__device__ __forceinline__ uint32_t warp_block_mask(float u, float v, float a, float b, float c, float vrej,
                                                    float x0, float y0) {
    constexpr int NW = TW * TH / 32, WX = TW / 8;
    constexpr uint32_t kAll = (1u << NW) - 1u;
    const float det = a * c - b * b;
    const float vm = fmaf(vrej, 1.05f, 1e-3f);
    if (!(a > 0.f && c > 0.f && det > 1e-4f * (a * c) && vm > 0.f && vm < INFINITY && isfinite(u) && isfinite(v)))
        return kAll;
    const float inv = __frcp_rn(det);
    const float hx = fmaf(sqrtf(vm * c * inv), 1.01f, 0.01f), hy = fmaf(sqrtf(vm * a * inv), 1.01f, 0.01f);
    if (!(hx < INFINITY && hy < INFINITY)) return kAll;
    uint32_t m = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        const float bx = x0 + (float)((w % WX) * 8), by = y0 + (float)((w / WX) * 4);
        if (bx <= u + hx && bx + 7.0f >= u - hx && by <= v + hy && by + 3.0f >= v - hy) m |= 1u << w;
    }
    return m;
}

// Shared-memory batch of Gaussians, repacked so a rejected pair needs two
// loads: sA = (u, v, c.x, c.y), sB = (c.z, vreject, log2(opacity), z),
// sC = (phat.x, phat.y, r, g), sD = b, s_orig = index in the tile's list;
// for the Jacobian pass also NX planes sX: the reference Jacobian stages
// sX[0] = (rgx, rgy, -fx rgx, -fy rgy), the mean's normalised ray and the
// third row of the projection Jacobian without 1/d; the analytic Jacobian
// stages eight planes with the derivatives of (u, v, a, b, c) with respect to
// the camera-frame pose update and the mean's (x, y) (see stage_deriv).
template <int BATCH = kBatch, int NX = 1, int NT = kPix>
struct TrackBatch {
    // wm[j]: the warps (8 x 4 pixel blocks) whose pixels staged Gaussian j
    // can reach (warp_block_mask); bm[w][g]: bit k set when entry 32 g + k
    // is in warp w's mask -- each warp walks only its own entries
    uint8_t wm[BATCH];
    uint32_t bm[NT / 32][BATCH / 32];
    float4 A[BATCH];
    float4 B[BATCH];
    float4 C[BATCH];
    float4 X[NX][BATCH];
    float D[BATCH];
    int orig[BATCH];
    int wcnt[NT / 32];
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
// covariance and mean).  out: du, dv, da, db, dc grouped by pairs of pose
// coordinates (2m, 2m + 1), each quantity's pair adjacent (the order the
// fused pass reads them in, deriv_pairs), then the mean's x, y.
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
    out[0] = make_float4(du[0], du[1], dv[0], dv[1]);
    out[1] = make_float4(da[0], da[1], db[0], db[1]);
    out[2] = make_float4(dc[0], dc[1], du[2], du[3]);
    out[3] = make_float4(dv[2], dv[3], da[2], da[3]);
    out[4] = make_float4(db[2], db[3], dc[2], dc[3]);
    out[5] = make_float4(du[4], du[5], dv[4], dv[5]);
    out[6] = make_float4(da[4], da[5], db[4], db[5]);
    out[7] = make_float4(dc[4], dc[5], x, y);
}

// The derivatives of pose-coordinate pair m (2m, 2m + 1) of staged Gaussian
// j (stage_deriv's layout): du, dv, da, db, dc as float2 (register pairs).
struct DerivPair {
    float2 du, dv, da, db, dc;
};
// One pair at a time (three or two 16-byte and one 8-byte shared load), so
// the fused pass holds one pair's ten values rather than all thirty.
template <int BATCH, int NX>
__device__ __forceinline__ DerivPair deriv_pair(const float4 (&X)[NX][BATCH], int j, int m) {
    auto lo = [&](int plane) { return *reinterpret_cast<const float2*>(&X[plane][j].x); };
    auto hi = [&](int plane) { return *reinterpret_cast<const float2*>(&X[plane][j].z); };
    if (m == 0) {
        const float4 p0 = X[0][j], p1 = X[1][j];
        return {make_float2(p0.x, p0.y), make_float2(p0.z, p0.w), make_float2(p1.x, p1.y), make_float2(p1.z, p1.w),
                lo(2)};
    }
    if (m == 1) {
        const float4 p3 = X[3][j], p4 = X[4][j];
        return {hi(2), make_float2(p3.x, p3.y), make_float2(p3.z, p3.w), make_float2(p4.x, p4.y),
                make_float2(p4.z, p4.w)};
    }
    const float4 p5 = X[5][j], p6 = X[6][j];
    return {make_float2(p5.x, p5.y), make_float2(p5.z, p5.w), make_float2(p6.x, p6.y), make_float2(p6.z, p6.w),
            lo(7)};
}

template <int STAGE, int TW, int TH, int BATCH, int NX, int NT>
__device__ __forceinline__ void put_staged(const TrackArgs& a, TrackBatch<BATCH, NX, NT>& sb, int pos, const float4& r0,
                                           const float4& r1, const float4& r2, float vrej, int li, uint32_t g,
                                           float x0, float y0) {
    static_assert(TW * TH == NT, "tile shape of the staged batch");
    sb.wm[pos] = (uint8_t)warp_block_mask<TW, TH>(r0.x, r0.y, r1.x, r1.y, r1.z, vrej, x0, y0);
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
// entries TW * TH at a time (one per thread; a smaller BATCH uses part of them),
// each round compacted after the previous one, so the staged order is the
// list order.  Ends with a barrier.
template <bool REF_LAYOUT, bool FORWARD, int STAGE, int TW, int TH, int BATCH, int NX>
__device__ __forceinline__ int stage_batch(const TrackArgs& a, TrackBatch<BATCH, NX, TW * TH>& sb, uint32_t list0, int base,
                                           int limit, float x0, float y0) {
    constexpr int NT = TW * TH;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    int total = 0;
#pragma unroll
    for (int r0 = 0; r0 < BATCH; r0 += NT) {
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
                keep = !tile_prunable<FORWARD, TW, TH>(r0v.x, r0v.y, r1.x, r1.y, r1.z, vrej, x0, y0);
            }
        }
        const uint32_t bal = __ballot_sync(kFullMask, keep);
        if (lane == 0) sb.wcnt[w] = __popc(bal);
        __syncthreads();
        int wbase = 0, round_total = 0;
#pragma unroll
        for (int k = 0; k < NT / 32; ++k) {
            const int c = sb.wcnt[k];
            wbase += (k < w) ? c : 0;
            round_total += c;
        }
        if (keep)
            put_staged<STAGE, TW, TH>(a, sb, total + wbase + __popc(bal & lanemask_lt()), r0v, r1, r2, vrej, li, g,
                                      x0, y0);
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
    if (keep)
        put_staged<FORWARD ? kStageNone : kStageRay, kTW, kTH>(a, sb, wbase + __popc(bal & lanemask_lt()), r0, r1, r2,
                                                             vrej, li, g, x0, y0);
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

// Per-warp bitmaps of a staged batch of cnt entries (after its barrier; every
// lane of the CTA takes part).  A warp writes and reads only its own rows.
template <int BATCH, int NX, int NT>
__device__ __forceinline__ void build_warp_bitmaps(TrackBatch<BATCH, NX, NT>& sb, int cnt) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int g = 0; g * 32 < cnt; ++g) {
        const int j = g * 32 + lane;
        const bool rel = j < cnt && ((sb.wm[j] >> w) & 1u);
        const uint32_t b = __ballot_sync(kFullMask, rel);
        if (lane == 0) sb.bm[w][g] = b;
    }
    __syncwarp();
}

// Shared-memory batch of the body below (dynamic shared memory: the analytic
// Jacobian's batch of 512 exceeds the static limit).
template <int TW, int TH, int BATCH, bool ANALYTIC>
using BodyBatch = TrackBatch<BATCH, ANALYTIC ? 8 : 1, TW * TH>;

// Dynamic shared memory of one CTA running the body: the staged batch, then
// (TMA variant) the gathered batch at a 128-byte boundary.
template <int TW, int TH, int BATCH, bool ANALYTIC, bool TMA>
constexpr size_t body_smem_bytes() {
    return sizeof(BodyBatch<TW, TH, BATCH, ANALYTIC>) + (TMA ? sizeof(TmaStage) + 128 : 0);
}

template <int TW, int TH, int BATCH, bool ANALYTIC>
__device__ __forceinline__ TmaStage& body_tma_stage(unsigned char* dyn) {
    const uintptr_t p = reinterpret_cast<uintptr_t>(dyn) + sizeof(BodyBatch<TW, TH, BATCH, ANALYTIC>);
    return *reinterpret_cast<TmaStage*>((p + 127) & ~uintptr_t(127));
}

// One tile of the fused tracking kernel, run by a CTA of TW * TH threads (one
// per pixel; each warp covers an 8 x 4 pixel block).  Tile shapes: 16 x 16
// (the reference's), 8 x 8 and 32 x 8; the binning must use the same shape,
// except that a 16 x 16 list tile may be split over a.split CTAs of 16 x 8
// or 8 x 8 pixels (CTA `tile` covers part (tile % split) of list tile
// tile / split).  Ends with the CTA's 27 partials written to
// a.tile_out[tile]: the sum over its warps in the order of tile_partial_sum.
// COMP (precision form, analytic Jacobian only): the forward blend's colour
// accumulated with Kahan summation, and the in-tile sums of the 27 J^T J /
// J^T r partials compensated (warp_reduce_scatter32_comp, then TwoSum across
// warps); the tile-to-frame sum is compensated in every form.
// The sum of a CTA's warp partials (column col of s_red).  16 pixels wide:
// per 8-row band, (left 8 x 8 quadrant + right quadrant), each quadrant its
// upper + lower warp, then band 0 + band 1 -- so a 16 x 16 tile's sum is
// ((q00 + q10) + (q01 + q11)) whether one CTA forms it or the frame
// reduction adds the partials of 16 x 8 or 8 x 8 CTAs (tile_partial_sum).
// Other widths: the warps in order.
template <int TW, int TH>
__device__ __forceinline__ float cta_partial_sum(const float (*s_red)[32], int col) {
    constexpr int NW = TW * TH / 32;
    if constexpr (TW == 16) {
        float s = __fadd_rn(__fadd_rn(s_red[0][col], s_red[2][col]), __fadd_rn(s_red[1][col], s_red[3][col]));
        if constexpr (TH == 16)
            s = __fadd_rn(s, __fadd_rn(__fadd_rn(s_red[4][col], s_red[6][col]),
                                       __fadd_rn(s_red[5][col], s_red[7][col])));
        return s;
    } else if constexpr (TW == 8 && TH == 8) {
        return __fadd_rn(s_red[0][col], s_red[1][col]);
    } else {
        float s = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) s += s_red[w][col];
        return s;
    }
}

template <int TW, int TH, bool RENDER_ONLY, bool REF_LAYOUT, bool TMA, int BATCH, bool ANALYTIC,
          bool COMP = false>
__device__ __forceinline__ void track_tile_body(const TrackArgs& a, const RecMaps& maps, int tile,
                                                unsigned char* dyn) {
    constexpr int NT = TW * TH;
    static_assert(!COMP || ANALYTIC, "compensated accumulation: analytic Jacobian");
    static_assert(TW % 8 == 0 && TH % 4 == 0 && NT % 32 == 0 && NT <= 256, "tile of 8 x 4 pixel warps");
    static_assert(TW != 16 || TH == 8 || TH == 16, "16-wide CTAs: 8-row bands");
    static_assert(!TMA || (BATCH == kBatch && TW == kTW && TH == kTH),
                  "the TMA staging gathers batches of kBatch records for 16 x 16 tiles");
    static_assert(BATCH % 128 == 0 && BATCH <= 512, "batch of 128, 256 or 512 Gaussians");
    static_assert(!ANALYTIC || (!TMA && !REF_LAYOUT), "analytic Jacobian: packed records, plain staging");
    BodyBatch<TW, TH, BATCH, ANALYTIC>& sb = *reinterpret_cast<BodyBatch<TW, TH, BATCH, ANALYTIC>*>(dyn);
    __shared__ float s_red[NT / 32][32];
    __shared__ float s_red_lo[COMP ? NT / 32 : 1][32];
    __shared__ uint32_t s_nmax;
    TmaStage& ts = body_tma_stage<TW, TH, BATCH, ANALYTIC>(dyn);
    TmaState tm;

    // the list tile and this CTA's pixel block in it
    const int split = a.split > 1 ? a.split : 1;
    const int lt = split == 1 ? tile : tile / split;
    int bx = 0, by = 0, ltw = TW, lth = TH;
    if (split > 1) {
        const int sub = tile - lt * split;
        bx = (sub % (16 / TW)) * TW;
        by = (sub / (16 / TW)) * TH;
        ltw = lth = 16;
    }
    const int tx = lt % a.ntx, ty = lt / a.ntx;
    const int px0 = tx * ltw + bx, py0 = ty * lth + by;
    const int tid = threadIdx.x;
    // each warp covers an 8 x 4 pixel block (compact footprint: less divergence)
    const int wq = tid >> 5, lq = tid & 31;
    const int x = px0 + (wq % (TW / 8)) * 8 + (lq & 7), y = py0 + (wq / (TW / 8)) * 4 + (lq >> 3);
    const float x0 = (float)px0, y0 = (float)py0;
    const bool in_bounds = (x < a.W && y < a.H);
    const size_t p = (size_t)y * a.W + x;
    uint2 range = a.ranges[lt];
    range.y = min(range.y, a.n_list);
    const int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    const float xf = (float)x, yf = (float)y;

    float img_depth = 0.f;
    if (!RENDER_ONLY && in_bounds) img_depth = a.obs_depth[p];
    const bool inside = RENDER_ONLY ? in_bounds : (in_bounds && img_depth > 0.1f);

    // ------------------------- pass 1: forward blend -------------------------
    // FUSED (analytic Jacobian): the colour and depth Jacobians are
    // accumulated in this pass, so there is no second pass over the list.
    // Each blended Gaussian contributes
    //   kf (c T - (C - A) / (1 - alpha)) dv/dpose
    // per channel (A: colour accumulated up to and including it, C: the final
    // colour with background, kf = dalpha/dv = -alpha / 2, 0 where alpha is
    // clamped at 0.99); C is known only at the end, so with it factored out
    //   S1 += (kf c T + kf A / (1 - alpha)) dv/dpose,  S2 += kf / (1 - alpha) dv/dpose,
    // and the colour Jacobian is S1 - C S2.  (The reference's second pass
    // walks the list again with the remaining colour C - A.)
    constexpr bool FUSED = ANALYTIC && !RENDER_ONLY;
    float T = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, depth = 0.f;
    float ccr = 0.f, ccg = 0.f, ccb = 0.f;  // Kahan carries of the colour (COMP)
    uint32_t last = 0;
    bool done = !inside;
    float final_T = 1.f;
    uint32_t n_contrib = 0;
    float2 fs1[3][3], fs2[3];  // FUSED: S1 (channel, pose pair) and S2 (pose pair)
#pragma unroll
    for (int m = 0; m < 3; ++m) fs1[0][m] = fs1[1][m] = fs1[2][m] = fs2[m] = make_float2(0.f, 0.f);
    // FUSED: the depth Jacobian, written once where T crosses 0.5 (each
    // thread its own column: no barrier needed)
    __shared__ float s_jd[FUSED ? 6 : 1][FUSED ? NT : 1];
    if constexpr (FUSED) {
#pragma unroll
        for (int k = 0; k < 6; ++k) s_jd[k][tid] = 0.f;
    }
    if (n > 0) {
        if (TMA) tma_begin(a, maps, ts, range.x, n, tm);
        for (int base = 0; base < n; base += BATCH) {
            if (__syncthreads_and(done)) break;
            int cnt;
            if constexpr (TMA)
                cnt = stage_batch_tma<true>(a, maps, sb, ts, range.x, base, n, x0, y0, tm);
            else
                cnt = stage_batch<REF_LAYOUT, true, FUSED ? kStageDeriv : kStageNone, TW, TH>(a, sb, range.x,
                                                                                                 base, n, x0, y0);
            build_warp_bitmaps(sb, cnt);
            if (FUSED && !done) {
                int last_j = -1;
                // one staged Gaussian with its conic-form gradient (dl0, dl1):
                // returns false when the pixel terminates
                auto blend_jac = [&](int j, float dx, float dy, float dl0, float dl1, float v) -> bool {
                    const float4 rB = sb.B[j];
                    const float raw = gauss_weight(rB.z, v);
                    const float alpha = fminf(0.99f, raw);
                    if (alpha < kInv255) return true;
                    const float test_T = T * (1.0f - alpha);
                    if (test_T < 0.0001f) return false;
                    const float4 rC = sb.C[j];
                    const float cB = sb.D[j];
                    const float aT = alpha * T;
                    if constexpr (COMP) {
                        kahan_add(cr, ccr, rC.z * aT);
                        kahan_add(cg, ccg, rC.w * aT);
                        kahan_add(cb, ccb, cB * aT);
                    } else {
                        cr += rC.z * aT;
                        cg += rC.w * aT;
                        cb += cB * aT;
                    }
                    const float inv1m = rcp_approx(1.0f - alpha);
                    const float kf = (raw > 0.99f) ? 0.0f : -0.5f * alpha;
                    const float kfi = kf * inv1m;
                    const float kT = kf * T;
                    const float2 w0 = make_float2(kT * rC.z + kfi * cr, kT * rC.z + kfi * cr);
                    const float2 w1 = make_float2(kT * rC.w + kfi * cg, kT * rC.w + kfi * cg);
                    const float2 w2 = make_float2(kT * cB + kfi * cb, kT * cB + kfi * cb);
                    const float2 wi = make_float2(kfi, kfi);
                    const float cu = 2.0f * dl0, cv = 2.0f * dl1, ca = dx * dx, cb2 = 2.0f * dx * dy, cc = dy * dy;
                    const float2 cu2 = make_float2(cu, cu), cv2 = make_float2(cv, cv), ca2 = make_float2(ca, ca),
                                 cb22 = make_float2(cb2, cb2), cc2 = make_float2(cc, cc);
#pragma unroll
                    for (int m = 0; m < 3; ++m) {
                        // dv/dpose = cu du + cv dv + ca da + cb2 db + cc dc for pose pair m
                        const DerivPair d = deriv_pair(sb.X, j, m);
                        float2 gv = __fmul2_rn(cu2, d.du);
                        gv = __ffma2_rn(cv2, d.dv, gv);
                        gv = __ffma2_rn(ca2, d.da, gv);
                        gv = __ffma2_rn(cb22, d.db, gv);
                        gv = __ffma2_rn(cc2, d.dc, gv);
                        fs1[0][m] = __ffma2_rn(w0, gv, fs1[0][m]);
                        fs1[1][m] = __ffma2_rn(w1, gv, fs1[1][m]);
                        fs1[2][m] = __ffma2_rn(w2, gv, fs1[2][m]);
                        fs2[m] = __ffma2_rn(wi, gv, fs2[m]);
                    }
                    if (T > 0.5f && test_T < 0.5f) {
                        const float4 rA = sb.A[j];
                        depth = depth_at(rB.w, rA.x, xf, rC.x, rA.y, yf, rC.y);
                        // d depth = d z + phat . d(dx, dy) + (dx, dy) . d phat, with
                        // d phat = (dp_x / z^2 - 2 x dp_z / z^3, dp_y / z^2 - 2 y dp_z / z^3)
                        const float z = rB.w, x = sb.X[7][j].z, y = sb.X[7][j].w;
                        const float iz = __frcp_rn(z), iz2 = iz * iz, iz3 = iz2 * iz;
#pragma unroll
                        for (int k = 0; k < 6; ++k) {
                            const float dpx = k == 0 ? -1.f : (k == 4 ? -z : (k == 5 ? y : 0.f));
                            const float dpy = k == 1 ? -1.f : (k == 3 ? z : (k == 5 ? -x : 0.f));
                            const float dpz = k == 2 ? -1.f : (k == 3 ? -y : (k == 4 ? x : 0.f));
                            const float dphx = dpx * iz2 - 2.f * x * iz3 * dpz;
                            const float dphy = dpy * iz2 - 2.f * y * iz3 * dpz;
                            const DerivPair d = deriv_pair(sb.X, j, k >> 1);
                            const float du_k = (k & 1) ? d.du.y : d.du.x;
                            const float dv_k = (k & 1) ? d.dv.y : d.dv.x;
                            s_jd[k][tid] = dpz + rC.x * du_k + dx * dphx + rC.y * dv_k + dy * dphy;
                        }
                    }
                    T = test_T;
                    last_j = j;
                    return true;
                };
                for (int g = 0; g * 32 < cnt && !done; ++g) {
                    uint32_t bits = sb.bm[wq][g];
                    while (bits) {
                        const int j0 = g * 32 + __ffs(bits) - 1;
                        bits &= bits - 1;
                        if (bits) {
                            const int j1 = g * 32 + __ffs(bits) - 1;
                            bits &= bits - 1;
                            const float4 rA0 = sb.A[j0], rA1 = sb.A[j1];
                            const float2 rB0 = *reinterpret_cast<const float2*>(&sb.B[j0]);
                            const float2 rB1 = *reinterpret_cast<const float2*>(&sb.B[j1]);
                            const float dx0 = rA0.x - xf, dy0 = rA0.y - yf;
                            const float dx1 = rA1.x - xf, dy1 = rA1.y - yf;
                            float l00, l01, l10, l11;
                            const float v0 = conic_form(rA0.z, rA0.w, rB0.x, dx0, dy0, l00, l01);
                            const float v1 = conic_form(rA1.z, rA1.w, rB1.x, dx1, dy1, l10, l11);
                            const bool k0 = !(v0 > rB0.y || v0 <= 0.0f);
                            const bool k1 = !(v1 > rB1.y || v1 <= 0.0f);
                            if (k0 && !blend_jac(j0, dx0, dy0, l00, l01, v0)) {
                                done = true;
                                break;
                            }
                            if (k1 && !blend_jac(j1, dx1, dy1, l10, l11, v1)) {
                                done = true;
                                break;
                            }
                        } else {
                            const float4 rA = sb.A[j0];
                            const float2 rB = *reinterpret_cast<const float2*>(&sb.B[j0]);
                            const float dx = rA.x - xf, dy = rA.y - yf;
                            float l0, l1;
                            const float v = conic_form(rA.z, rA.w, rB.x, dx, dy, l0, l1);
                            if (!(v > rB.y || v <= 0.0f) && !blend_jac(j0, dx, dy, l0, l1, v)) {
                                done = true;
                                break;
                            }
                        }
                    }
                }
                if (last_j >= 0) last = (uint32_t)sb.orig[last_j] + 1u;
            }
            if (!FUSED && !done) {
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
                    if (T > 0.5f && test_T < 0.5f) depth = depth_at(rB.w, sb.A[j].x, xf, rC.x, sb.A[j].y, yf, rC.y);
                    T = test_T;
                    last_j = j;
                    return true;
                };
                // the warp's own entries (its bitmap), two per iteration: both
                // quadratic forms are evaluated before the (mostly rejecting)
                // branches, in list order
                for (int g = 0; g * 32 < cnt && !done; ++g) {
                    uint32_t bits = sb.bm[wq][g];
                    while (bits) {
                        const int j0 = g * 32 + __ffs(bits) - 1;
                        bits &= bits - 1;
                        if (bits) {
                            const int j1 = g * 32 + __ffs(bits) - 1;
                            bits &= bits - 1;
                            const float4 rA0 = sb.A[j0], rA1 = sb.A[j1];
                            const float2 rB0 = *reinterpret_cast<const float2*>(&sb.B[j0]);
                            const float2 rB1 = *reinterpret_cast<const float2*>(&sb.B[j1]);
                            const float dx0 = rA0.x - xf, dy0 = rA0.y - yf;
                            const float dx1 = rA1.x - xf, dy1 = rA1.y - yf;
                            float q0, q1;
                            const float v0 = conic_form(rA0.z, rA0.w, rB0.x, dx0, dy0, q0, q1);
                            const float v1 = conic_form(rA1.z, rA1.w, rB1.x, dx1, dy1, q0, q1);
                            const bool k0 = !(v0 > rB0.y || v0 <= 0.0f);
                            const bool k1 = !(v1 > rB1.y || v1 <= 0.0f);
                            if (k0 && !blend(j0, dx0, dy0, v0)) {
                                done = true;
                                break;
                            }
                            if (k1 && !blend(j1, dx1, dy1, v1)) {
                                done = true;
                                break;
                            }
                        } else {
                            const float4 rA = sb.A[j0];
                            const float2 rB = *reinterpret_cast<const float2*>(&sb.B[j0]);
                            const float dx = rA.x - xf, dy = rA.y - yf;
                            float q0, q1;
                            const float v = conic_form(rA.z, rA.w, rB.x, dx, dy, q0, q1);
                            if (!(v > rB.y || v <= 0.0f) && !blend(j0, dx, dy, v)) {
                                done = true;
                                break;
                            }
                        }
                    }
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

    // ------------------- pass 2 (reference Jacobian): per-Gaussian terms ---
    int nmax = 0;
    if constexpr (!FUSED) {
        if (tid == 0) s_nmax = 0;
        __syncthreads();
        if (do_jac && n_contrib > 0) atomicMax(&s_nmax, n_contrib);
        __syncthreads();
        nmax = (int)min((uint32_t)n, s_nmax);
    }
    if constexpr (ANALYTIC) {
        // Colour Jacobian jc (3 x 6) of the pixel from the fused pass's sums:
        // jc = S1 - C S2 (C: the final colour with background); jd: the depth
        // Jacobian of the Gaussian where T crossed 0.5.  Pose coordinates in
        // pairs (2m, 2m + 1), packed FP32 FMAs (two IEEE round-to-nearest
        // FMAs each, the results of __fmaf_rn).
        float2 jc2[3][3];
        const float2 nr = make_float2(-cr, -cr), ng = make_float2(-cg, -cg), nb = make_float2(-cb, -cb);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            jc2[0][m] = __ffma2_rn(nr, fs2[m], fs1[0][m]);
            jc2[1][m] = __ffma2_rn(ng, fs2[m], fs1[1][m]);
            jc2[2][m] = __ffma2_rn(nb, fs2[m], fs1[2][m]);
        }
        float jd[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) jd[k] = s_jd[k][tid];
        if (do_jac) {
            float jc[3][6];
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int m = 0; m < 3; ++m) {
                    jc[c][2 * m] = jc2[c][m].x;
                    jc[c][2 * m + 1] = jc2[c][m].y;
                }
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
                    cnt = stage_batch<REF_LAYOUT, false, kStageRay, TW, TH>(a, sb, range.x, base, nmax, x0, y0);
                build_warp_bitmaps(sb, cnt);
                if (!done2) {
                    for (int g = 0; g * 32 < cnt && !done2; ++g) {
                        for (uint32_t bits = sb.bm[wq][g]; bits; bits &= bits - 1) {
                            const int j = g * 32 + __ffs(bits) - 1;
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
                        const float d = depth_fast(rB.w, dx, rC.x, dy, rC.y, rA.x, xf, rA.y, yf);
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
    if constexpr (COMP) {
        float errs[32];
#pragma unroll
        for (int k = 0; k < 32; ++k) errs[k] = 0.f;
        float hi, lo;
        warp_reduce_scatter32_comp(vals, errs, hi, lo);
        s_red[tid >> 5][tid & 31] = hi;
        s_red_lo[tid >> 5][tid & 31] = lo;
        __syncthreads();
        if (tid < FVGS_POSEDATA_FLOATS) {
            float s = 0.f, e = 0.f;
#pragma unroll
            for (int w = 0; w < NT / 32; ++w) {
                float err;
                two_sum(s, s_red[w][tid], s, err);
                e = __fadd_rn(e, __fadd_rn(err, s_red_lo[w][tid]));
            }
            a.tile_out[(size_t)tile * FVGS_POSEDATA_FLOATS + tid] = __fadd_rn(s, e);
        }
    } else {
        const float mine = warp_reduce_scatter32(vals);
        s_red[tid >> 5][tid & 31] = mine;
        __syncthreads();
        if (tid < FVGS_POSEDATA_FLOATS)
            a.tile_out[(size_t)tile * FVGS_POSEDATA_FLOATS + tid] = cta_partial_sum<TW, TH>(s_red, tid);
    }
}

}  // namespace fvgs
