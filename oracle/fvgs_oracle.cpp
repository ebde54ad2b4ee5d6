/*
 * fvgs_oracle.cpp -- CPU restatement of the reference's Gaussian-splatting hot
 * path (jcevasco2003/f_vigs_slam, src/GSCudaKernels.cu + src/GSSlam.cu +
 * src/RgbdPoseCost.cu).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the restatement the CUDA library is
 * compared against, and the timed CPU baseline.  No product code path may
 * call it.
 *
 * PARITY STATUS: the binning is pinned to the reference's own code.  The
 * reference ships no tests, golden vectors or fixtures and cannot be built
 * whole here (its device code needs Eigen, its host code OpenCV-CUDA, Ceres
 * and ROS 2), but its binning kernels can: oracle/ref_build.py compiles them
 * from its sources for the host (compared with this file's no-FMA build in
 * every field, tests/test_ref_pin.py) and with nvcc for the GPU (keys, sorted
 * indices and ranges compared bit for bit, tests/test_ref_pin_gpu.py).  The
 * FP64 paths downstream are pinned by known-answer tests derived by hand from
 * the reference source (tests/test_oracle_kat.py) and by finite differences.
 *
 * Two precisions:
 *  - FP32, reference operation order, for projection, tile counts and tile
 *    keys.  Every multiply-add that the CUDA kernels fuse is written here as
 *    an explicit fmaf and the file is compiled with -ffp-contract=off, so the
 *    results are bit-identical to the GPU's.
 *  - FP64 for everything downstream (blending, pose Jacobian, mapping
 *    gradients, Adam), consuming the FP32 2D records and tile lists so that
 *    both sides blend the same Gaussians in the same order.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/fvgs_types.h"

namespace {

// ---------------------------------------------------------------------------
// FP32 projection (src/GSCudaKernels.cu:319-334 quaternionToMatrix,
// 345-476 projectGaussiansWorldToScreen_kernel, 1411-1437 invert2x2).
// ---------------------------------------------------------------------------
// Contraction policy.  The reference's kernels are compiled by nvcc with its
// default --fmad=true: a multiply feeding an add becomes one FMA, and in a sum
// of two products the first product is fused: a*b + c*d = fma(a, b, c*d),
// a*b - c*d = fma(a, b, -(c*d)), a*b + c*d + e*f = fma(e, f, fma(a, b, c*d)),
// acc += a*b*c = fma(a*b, c, acc); the tile-centre depth of the keys,
// z + a*b + c*d, is fma(a, b, z) + c*d (oracle_emit_keys; matched against the
// keys of the reference's nvcc build).  Built with FVGS_ORACLE_NO_FMA every
// product and sum rounds on its own instead (what the reference's source
// gives compiled with contraction off; oracle/ref_host.cpp).
#ifndef FVGS_ORACLE_NO_FMA
inline float f_fma(float a, float b, float c) { return std::fmaf(a, b, c); }
#else
inline float f_fma(float a, float b, float c) { return a * b + c; }
#endif
inline float dot2(float a, float b, float c, float d) { return f_fma(a, b, c * d); }    // a*b + c*d
inline float diff2(float a, float b, float c, float d) { return f_fma(a, b, -(c * d)); }  // a*b - c*d
inline float dot3(float a, float b, float c, float d, float e, float f) { return f_fma(e, f, dot2(a, b, c, d)); }

// quaternionToMatrix: q read as (x,y,z,w) = (.x,.y,.z,.w); no normalisation.
inline void quat_to_R_f32(const float q[4], float R[3][3]) {
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    R[0][0] = f_fma(-2.f, dot2(y, y, z, z), 1.f);
    R[0][1] = 2.f * diff2(x, y, w, z);
    R[0][2] = 2.f * dot2(x, z, w, y);
    R[1][0] = 2.f * dot2(x, y, w, z);
    R[1][1] = f_fma(-2.f, dot2(x, x, z, z), 1.f);
    R[1][2] = 2.f * diff2(y, z, w, x);
    R[2][0] = 2.f * diff2(x, z, w, y);
    R[2][1] = 2.f * dot2(y, z, w, x);
    R[2][2] = f_fma(-2.f, dot2(x, x, y, y), 1.f);
}

struct Proj32 {
    bool visible;
    float u, v, z;
    float cxx, cyy, cxy;  // Sigma2D stored order (xx, yy, xy)
    float ixx, iyy, ixy;  // inverse, stored order (xx, yy, xy)
    float phx, phy;
};

// projectGaussiansWorldToScreen_kernel (src/GSCudaKernels.cu:345-476), every
// expression in the kernel's own order: the 3x3 products Sigma_cam and
// Sigma_2d as its 9-term accumulation loops (zero Jacobian entries included).
inline Proj32 project_one_f32(const float p[3], const float s[3], const float q[4],
                              const float cam_t[3], const float R[3][3],
                              const fvgs_intrinsics& K, int W, int H) {
    Proj32 o;
    std::memset(&o, 0, sizeof(o));
    const float d0 = p[0] - cam_t[0], d1 = p[1] - cam_t[1], d2 = p[2] - cam_t[2];
    // pos_cam = R^T (p - t)  (:372-378)
    const float pcx = dot3(R[0][0], d0, R[1][0], d1, R[2][0], d2);
    const float pcy = dot3(R[0][1], d0, R[1][1], d1, R[2][1], d2);
    const float pcz = dot3(R[0][2], d0, R[1][2], d1, R[2][2], d2);
    if (pcz <= 0.0f) return o;  // :381
    const float inv_z = 1.0f / pcz;
    const float u = f_fma(K.fx, pcx * inv_z, K.cx);
    const float v = f_fma(K.fy, pcy * inv_z, K.cy);
    if (u < 0.0f || u >= (float)W || v < 0.0f || v >= (float)H) return o;  // :391
    o.visible = true;
    o.u = u;
    o.v = v;
    o.z = pcz;
    // Sigma = M M^T, M = R_g diag(s)  (:404-420)
    float Rg[3][3];
    quat_to_R_f32(q, Rg);
    float M[3][3];
    for (int i = 0; i < 3; ++i) {
        M[i][0] = Rg[i][0] * s[0];
        M[i][1] = Rg[i][1] * s[1];
        M[i][2] = Rg[i][2] * s[2];
    }
    float S[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = i; j < 3; ++j) {
            S[i][j] = dot3(M[i][0], M[j][0], M[i][1], M[j][1], M[i][2], M[j][2]);
            S[j][i] = S[i][j];
        }
    // Sigma_cam[i][j] = sum_k sum_l R[k][i] Sigma[k][l] R[l][j], every entry (:423-433)
    float C[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            float acc = 0.0f;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) acc = f_fma(R[k][i] * S[k][l], R[l][j], acc);
            C[i][j] = acc;
        }
    // EWA: J = [fx/z 0 -fx x/z^2; 0 fy/z -fy y/z^2]  (:438-460)
    const float J[2][3] = {{K.fx * inv_z, 0.0f, (((-K.fx) * pcx) * inv_z) * inv_z},
                           {0.0f, K.fy * inv_z, (((-K.fy) * pcy) * inv_z) * inv_z}};
    float S2[2][2];
    for (int i = 0; i < 2; ++i)
        for (int j = i; j < 2; ++j) {
            float acc = 0.0f;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) acc = f_fma(J[i][k] * C[k][l], J[j][l], acc);
            S2[i][j] = acc;
            S2[j][i] = acc;
        }
    const float sxx = S2[0][0], syy = S2[1][1], sxy = S2[0][1];
    o.cxx = sxx;
    o.cyy = syy;
    o.cxy = sxy;
    // invert2x2 (:1411-1437): det == 0 -> identity.
    const float det = diff2(sxx, syy, sxy, sxy);
    if (det == 0.0f) {
        o.ixx = 1.0f;
        o.iyy = 1.0f;
        o.ixy = 0.0f;
    } else {
        const float inv_det = 1.0f / det;
        o.ixx = syy * inv_det;
        o.iyy = sxx * inv_det;
        o.ixy = (-sxy) * inv_det;
    }
    // p_hat = (x/z^2, y/z^2)  (:475)
    o.phx = (pcx * inv_z) * inv_z;
    o.phy = (pcy * inv_z) * inv_z;
    return o;
}

// countTilesPerGaussian_kernel / generateTileHashes_kernel bbox
// (src/GSCudaKernels.cu:565-590, 617-639).
struct Rect {
    int x0, y0, x1, y1;
};
inline Rect tile_rect_f32(float u, float v, float cxx, float cyy, int W, int H, int tw, int th,
                          int ntx, int nty, float radius_sigma) {
    const float rx = radius_sigma * std::sqrt(cxx);
    const float ry = radius_sigma * std::sqrt(cyy);
    const float bx0 = std::fmax(0.0f, u - rx);
    const float bx1 = std::fmin((float)(W - 1), u + rx);
    const float by0 = std::fmax(0.0f, v - ry);
    const float by1 = std::fmin((float)(H - 1), v + ry);
    Rect r;
    r.x0 = (int)(bx0 / (float)tw);
    r.x1 = (int)(bx1 / (float)tw);
    r.y0 = (int)(by0 / (float)th);
    r.y1 = (int)(by1 / (float)th);
    r.x0 = std::max(0, std::min(r.x0, ntx - 1));
    r.x1 = std::max(0, std::min(r.x1, ntx - 1));
    r.y0 = std::max(0, std::min(r.y0, nty - 1));
    r.y1 = std::max(0, std::min(r.y1, nty - 1));
    return r;
}

inline uint32_t f2u(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

// ---------------------------------------------------------------------------
// FP64 helpers
// ---------------------------------------------------------------------------
inline void quat_to_R_f64(const float qf[4], double R[3][3]) {
    const double x = qf[0], y = qf[1], z = qf[2], w = qf[3];
    R[0][0] = 1.0 - 2.0 * (y * y + z * z);
    R[0][1] = 2.0 * (x * y - w * z);
    R[0][2] = 2.0 * (x * z + w * y);
    R[1][0] = 2.0 * (x * y + w * z);
    R[1][1] = 1.0 - 2.0 * (x * x + z * z);
    R[1][2] = 2.0 * (y * z - w * x);
    R[2][0] = 2.0 * (x * z - w * y);
    R[2][1] = 2.0 * (y * z + w * x);
    R[2][2] = 1.0 - 2.0 * (x * x + y * y);
}

// Constants the reference compares against, as the float values it uses.
const double kInv255 = (double)(1.0f / 255.0f);
const double k099 = (double)0.99f;
const double k1em4 = (double)0.0001f;
const double k1em3 = (double)0.001f;

// Depth weight of the tracking residual: the reference's
// (|e| < thr ? 1 : thr / |e|) / z_obs (src/GSCudaKernels.cu:1120-1121,
// 1283-1284) with FVGS_Q_DEPTH_HUBER, else Tukey's biweight
// (1 - (e / thr)^2)^2 / z_obs, zero beyond thr.
inline double depth_w(double derr, double thr, double z_obs, bool huber) {
    const double ld = std::fabs(derr);
    double w;
    if (huber) {
        w = (ld < thr) ? 1.0 : thr / ld;
    } else {
        const double r = ld / thr, t = 1.0 - r * r;
        w = (ld < thr) ? t * t : 0.0;
    }
    return w / z_obs;
}

struct Rec {  // one Gaussian's 2D record as the blending kernels consume it
    double u, v, z, o, cx, cy, cz, phx, phy, r, g, b;
};

inline Rec load_rec(const float* rec12, uint32_t g) {
    const float* p = rec12 + (size_t)g * 12;
    Rec r;
    r.u = p[0]; r.v = p[1]; r.z = p[2]; r.o = p[3];
    r.cx = p[4]; r.cy = p[5]; r.cz = p[6]; r.phx = p[7];
    r.phy = p[8]; r.r = p[9]; r.g = p[10]; r.b = p[11];
    return r;
}

}  // namespace

extern "C" {

/*
 * Project N Gaussians (FP32, reference order).  Outputs in the reference's
 * buffer layout: uv[2N], cov2d[3N] (xx,yy,xy), inv2d[3N] stored order
 * (xx,yy,xy), depth[N], phat[2N], visible[N] (1 = written by the reference
 * kernel, 0 = culled slot, left as zeros here).
 */
int oracle_project(const float* pos, const float* scl, const float* rot, int n, const fvgs_pose* pose,
                   const fvgs_intrinsics* K, int W, int H, float* uv, float* cov2d, float* inv2d,
                   float* depth, float* phat, uint8_t* visible) {
    float R[3][3];
    quat_to_R_f32(pose->orientation, R);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        Proj32 p = project_one_f32(pos + 3 * (size_t)i, scl + 3 * (size_t)i, rot + 4 * (size_t)i,
                                   pose->position, R, *K, W, H);
        uv[2 * (size_t)i] = p.u;
        uv[2 * (size_t)i + 1] = p.v;
        cov2d[3 * (size_t)i] = p.cxx;
        cov2d[3 * (size_t)i + 1] = p.cyy;
        cov2d[3 * (size_t)i + 2] = p.cxy;
        inv2d[3 * (size_t)i] = p.ixx;
        inv2d[3 * (size_t)i + 1] = p.iyy;
        inv2d[3 * (size_t)i + 2] = p.ixy;
        depth[i] = p.z;
        phat[2 * (size_t)i] = p.phx;
        phat[2 * (size_t)i + 1] = p.phy;
        visible[i] = p.visible ? 1 : 0;
    }
    return 0;
}

/*
 * Tile counts (countTilesPerGaussian_kernel, src/GSCudaKernels.cu:549-593).
 * With FVGS_Q_CULLED_SLOTS clear, culled Gaussians get count 0.
 * rect[4N] = (x0, y0, x1, y1) tile rectangle (inclusive).
 */
int oracle_count(const float* uv, const float* cov2d, const uint8_t* visible, int n, int W, int H,
                 int tw, int th, float radius_sigma, uint32_t quirks, uint32_t* count,
                 int32_t* rect) {
    const int ntx = (W + tw - 1) / tw, nty = (H + th - 1) / th;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        Rect r = tile_rect_f32(uv[2 * (size_t)i], uv[2 * (size_t)i + 1], cov2d[3 * (size_t)i],
                               cov2d[3 * (size_t)i + 1], W, H, tw, th, ntx, nty, radius_sigma);
        uint32_t c = (uint32_t)((r.x1 - r.x0 + 1) * (r.y1 - r.y0 + 1));
        if (!visible[i] && !(quirks & FVGS_Q_CULLED_SLOTS)) c = 0;
        count[i] = c;
        rect[4 * (size_t)i] = r.x0;
        rect[4 * (size_t)i + 1] = r.y0;
        rect[4 * (size_t)i + 2] = r.x1;
        rect[4 * (size_t)i + 3] = r.y1;
    }
    return 0;
}

/*
 * Keys in generation order (exclusive scan of counts, then
 * generateTileHashes_kernel, src/GSCudaKernels.cu:596-667):
 * key = tile_id << 32 | bits(z + phx*dx + phy*dy), dx,dy = tile centre - uv,
 * the depth evaluated as the reference's nvcc build does: the first product
 * fused with z, the second rounded and added, fmaf(phx, dx, z) + phy*dy
 * (matched bit for bit against that build's keys; without FMA, the source's
 * one rounding per operation).  Row-major tile loop.
 * Returns the instance count, or -1 if it exceeds cap.
 */
int64_t oracle_emit_keys(const float* uv, const float* depth, const float* phat, const uint32_t* count,
                         const int32_t* rect, int n, int W, int tw, int th, int64_t cap,
                         uint64_t* keys, uint32_t* vals) {
    const int ntx = (W + tw - 1) / tw;
    std::vector<int64_t> off((size_t)n + 1);
    off[0] = 0;
    for (int i = 0; i < n; ++i) off[i + 1] = off[i] + count[i];
    const int64_t total = off[n];
    if (total > cap) return -1;
#pragma omp parallel for schedule(dynamic, 1024)
    for (int i = 0; i < n; ++i) {
        if (count[i] == 0) continue;
        int64_t w = off[i];
        const float u = uv[2 * (size_t)i], v = uv[2 * (size_t)i + 1], z = depth[i];
        const float phx = phat[2 * (size_t)i], phy = phat[2 * (size_t)i + 1];
        const int32_t* r = rect + 4 * (size_t)i;
        for (int ty = r[1]; ty <= r[3]; ++ty)
            for (int tx = r[0]; tx <= r[2]; ++tx) {
                const float tcx = ((float)tx + 0.5f) * (float)tw;
                const float tcy = ((float)ty + 0.5f) * (float)th;
                const float dx = tcx - u, dy = tcy - v;
                const float d = f_fma(phx, dx, z) + phy * dy;
                const uint32_t tile = (uint32_t)(ty * ntx + tx);
                keys[w] = ((uint64_t)tile << 32) | (uint64_t)f2u(d);
                vals[w] = (uint32_t)i;
                ++w;
            }
    }
    return total;
}

/*
 * Stable sort by the full 64-bit key (thrust::sort_by_key on uint64,
 * src/GSSlam.cu:624-628, a stable radix sort), then per-tile ranges
 * (computeIndicesRanges_kernel, src/GSCudaKernels.cu:669-707).
 * ranges[2T] zero-initialised first (src/GSSlam.cu:469-471).
 */
int oracle_sort_ranges(uint64_t* keys, uint32_t* vals, int64_t n_inst, int num_tiles, uint32_t quirks,
                       uint32_t* ranges) {
    std::vector<int64_t> perm((size_t)n_inst);
    for (int64_t i = 0; i < n_inst; ++i) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t b) { return keys[a] < keys[b]; });
    std::vector<uint64_t> k2((size_t)n_inst);
    std::vector<uint32_t> v2((size_t)n_inst);
    for (int64_t i = 0; i < n_inst; ++i) {
        k2[i] = keys[perm[i]];
        v2[i] = vals[perm[i]];
    }
    std::copy(k2.begin(), k2.end(), keys);
    std::copy(v2.begin(), v2.end(), vals);
    std::memset(ranges, 0, sizeof(uint32_t) * 2 * (size_t)num_tiles);
    int64_t limit = n_inst;
    if (quirks & FVGS_Q_RANGE_LAUNCH) {
        const int64_t launched = (int64_t)((num_tiles + 255) / 256) * 256;
        limit = std::min(limit, launched);
    }
    if (!(quirks & FVGS_Q_RANGE_LAUNCH)) {
        // intended: [first, last + 1) of every tile present
        for (int64_t idx = 0; idx < n_inst; ++idx) {
            const uint32_t t = (uint32_t)(keys[idx] >> 32);
            if (idx == 0 || (uint32_t)(keys[idx - 1] >> 32) != t) ranges[2 * (size_t)t] = (uint32_t)idx;
            if (idx == n_inst - 1 || (uint32_t)(keys[idx + 1] >> 32) != t)
                ranges[2 * (size_t)t + 1] = (uint32_t)(idx + 1);
        }
        return 0;
    }
    for (int64_t idx = 0; idx < limit; ++idx) {
        const uint32_t t = (uint32_t)(keys[idx] >> 32);
        if (idx == 0) {
            ranges[2 * (size_t)t] = 0;
            continue;  // the reference returns here, even when n_inst == 1
        }
        const uint32_t pt = (uint32_t)(keys[idx - 1] >> 32);
        if (pt != t) {
            ranges[2 * (size_t)pt + 1] = (uint32_t)idx;
            ranges[2 * (size_t)t] = (uint32_t)idx;
        }
        if (idx == n_inst - 1) ranges[2 * (size_t)t + 1] = (uint32_t)n_inst;
    }
    return 0;
}

/*
 * Build the 12-float blending record per Gaussian from the FP32 projection:
 * (u, v, z, opacity, c.x, c.y, c.z, phat.x, phat.y, r, g, b), with c the
 * inverse covariance in the order the blending kernels consume it.
 */
int oracle_make_records(const float* uv, const float* inv2d, const float* depth, const float* phat,
                        const float* colors, const float* opac, int n, uint32_t quirks, float* rec) {
    for (int i = 0; i < n; ++i) {
        float* r = rec + 12 * (size_t)i;
        r[0] = uv[2 * (size_t)i];
        r[1] = uv[2 * (size_t)i + 1];
        r[2] = depth[i];
        r[3] = opac[i];
        const float ixx = inv2d[3 * (size_t)i], iyy = inv2d[3 * (size_t)i + 1], ixy = inv2d[3 * (size_t)i + 2];
        r[4] = ixx;
        if (quirks & FVGS_Q_INVSIGMA_SWAP) {
            r[5] = iyy;
            r[6] = ixy;
        } else {
            r[5] = ixy;
            r[6] = iyy;
        }
        r[7] = phat[2 * (size_t)i];
        r[8] = phat[2 * (size_t)i + 1];
        r[9] = colors[3 * (size_t)i];
        r[10] = colors[3 * (size_t)i + 1];
        r[11] = colors[3 * (size_t)i + 2];
    }
    return 0;
}

/*
 * Fused tracking kernel getRgbdPoseJacobians (src/GSCudaKernels.cu:922-1392)
 * in FP64, one pixel at a time ("each pixel scans its tile list"), followed by
 * the host reduction of src/GSSlam.cu:2205-2226.
 *
 * Inputs: rec[12N] blending records, ranges[2T], indices (sorted values),
 * observed rgb/depth and Sobel gradients (dense row-major), pose, K.
 * Outputs: tile_out[27T] (Jtr[6], JtJ upper[21]) per tile; JtJ[36] symmetric
 * and Jtr[6] = -sum (camera frame, before the IMU extrinsic transform);
 * optional per-pixel images (colour incl. background, depth, final T,
 * n_contrib) of the forward blend -- pass null to skip.  tile_mask (T bytes,
 * nullable): only tiles with a non-zero byte are evaluated, the others get
 * zero partials.
 */
int oracle_track(const float* rec, const uint32_t* ranges, const uint32_t* indices, const float* obs_rgb,
                 const float* obs_depth, const float* gx, const float* gy, const fvgs_pose* pose,
                 const fvgs_intrinsics* Kf, const fvgs_params* P, int W, int H, double* tile_out,
                 double* JtJ, double* Jtr, double* img_color, double* img_depth, double* img_T,
                 uint32_t* img_nc, const uint8_t* tile_mask) {
    const int tw = P->tile_w, th = P->tile_h;
    const int ntx = (W + tw - 1) / tw, nty = (H + th - 1) / th, T = ntx * nty;
    double R[3][3];
    quat_to_R_f64(pose->orientation, R);
    const double fx = Kf->fx, fy = Kf->fy, cx = Kf->cx, cy = Kf->cy;
    const double bg[3] = {P->bg[0], P->bg[1], P->bg[2]};
    const double alpha_thresh = P->alpha_thresh, color_thresh = P->color_thresh,
                 depth_thresh = P->depth_thresh;
    const bool huber = (P->quirks & FVGS_Q_DEPTH_HUBER) != 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < T; ++t) {
        const int tx = t % ntx, ty = t / ntx;
        double acc[27];
        for (int k = 0; k < 27; ++k) acc[k] = 0.0;
        if (tile_mask && !tile_mask[t]) {  // not evaluated: zero partials, images untouched
            for (int k = 0; k < 27; ++k) tile_out[27 * (size_t)t + k] = 0.0;
            continue;
        }
        const uint32_t rs = ranges[2 * (size_t)t], re = ranges[2 * (size_t)t + 1];
        const int n_total = (int)(re - rs);
        for (int ly = 0; ly < th; ++ly)
            for (int lx = 0; lx < tw; ++lx) {
                const int x = tx * tw + lx, y = ty * th + ly;
                const bool in_bounds = (x < W && y < H);
                const size_t p = (size_t)y * W + x;
                double imgd = 0.0;
                if (in_bounds) imgd = obs_depth[p];
                bool inside = in_bounds && imgd > (double)0.1f;
                double col[3] = {0, 0, 0};
                double depth = 0.0, final_T = 1.0;
                uint32_t n_contrib = 0;
                if (n_total > 0) {
                    double Tr = 1.0;
                    uint32_t contributor = 0, last = 0;
                    bool done = !inside;
                    for (int i = 0; i < n_total && !done; ++i) {
                        contributor++;
                        const Rec g = load_rec(rec, indices[rs + i]);
                        const double dx = g.u - x, dy = g.v - y;
                        const double v = g.cx * dx * dx + 2.0 * g.cy * dx * dy + g.cz * dy * dy;
                        const double a = std::min(k099, g.o * std::exp(-0.5 * v));
                        if (a < kInv255 || v <= 0.0) continue;
                        const double test_T = Tr * (1.0 - a);
                        if (test_T < k1em4) {
                            done = true;
                            continue;
                        }
                        col[0] += g.r * a * Tr;
                        col[1] += g.g * a * Tr;
                        col[2] += g.b * a * Tr;
                        const double d = g.z + dx * g.phx + dy * g.phy;
                        if (Tr > 0.5 && test_T < 0.5) depth = d;
                        Tr = test_T;
                        last = contributor;
                    }
                    if (inside) {
                        final_T = Tr;
                        n_contrib = last;
                        col[0] += Tr * bg[0];
                        col[1] += Tr * bg[1];
                        col[2] += Tr * bg[2];
                    }
                }
                if (in_bounds) {
                    if (img_color) {
                        img_color[3 * p] = col[0];
                        img_color[3 * p + 1] = col[1];
                        img_color[3 * p + 2] = col[2];
                    }
                    if (img_depth) img_depth[p] = depth;
                    if (img_T) img_T[p] = final_T;
                    if (img_nc) img_nc[p] = n_contrib;
                }
                inside = inside && (final_T < alpha_thresh);
                if (!inside) continue;

                // ---- per-pixel term (src/GSCudaKernels.cu:1052-1173) ----
                const double e[3] = {col[0] - obs_rgb[3 * p], col[1] - obs_rgb[3 * p + 1],
                                     col[2] - obs_rgb[3 * p + 2]};
                const double depth_error = (imgd > (double)0.1f) ? (depth - imgd) : 0.0;
                const double closs = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                const double wc = (closs < color_thresh) ? 1.0 : color_thresh / closs;
                const double ray[3] = {(x - cx) / fx, (y - cy) / fy, 1.0};
                const double rc[9] = {0, -ray[2], ray[1], ray[2], 0, -ray[0], -ray[1], ray[0], 0};
                const double gX[3] = {gx[3 * p], gx[3 * p + 1], gx[3 * p + 2]};
                const double gY[3] = {gy[3 * p], gy[3 * p + 1], gy[3 * p + 2]};
                const double inv_imgd = 1.0 / imgd;
                double Jp[6];
                Jp[0] = fx * inv_imgd;
                Jp[1] = 0.0;
                Jp[2] = 0.0;
                Jp[3] = fy * inv_imgd;
                Jp[4] = -fx * ray[0] * inv_imgd;
                Jp[5] = -fy * ray[1] * inv_imgd;
                double Jc[9];
                for (int r = 0; r < 3; ++r)
                    for (int k = 0; k < 3; ++k) Jc[r * 3 + k] = Jp[2 * r] * gX[k] + Jp[2 * r + 1] * gY[k];
                double JJ[9];
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) {
                        double s = 0;
                        for (int k = 0; k < 3; ++k) s += Jc[r * 3 + k] * Jc[c * 3 + k];
                        JJ[r * 3 + c] = wc * s;
                    }
                double Jr[3];
                for (int r = 0; r < 3; ++r)
                    Jr[r] = -wc * (Jc[r * 3] * e[0] + Jc[r * 3 + 1] * e[1] + Jc[r * 3 + 2] * e[2]);
                {
                    const double wd = depth_w(depth_error, depth_thresh, imgd, huber);
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) JJ[r * 3 + c] += wd * ray[r] * ray[c];
                    for (int r = 0; r < 3; ++r) Jr[r] += wd * depth_error * ray[r];
                }
                auto accumulate = [&](const double JJm[9], const double Jrm[3], double dscale,
                                      const double rcm[9]) {
                    double Jpose[18];
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) {
                            Jpose[r * 3 + c] = R[r][c];
                            Jpose[9 + r * 3 + c] = dscale * rcm[r * 3 + c];
                        }
                    double tmp[18];
                    for (int r = 0; r < 6; ++r)
                        for (int c = 0; c < 3; ++c) {
                            double s = 0;
                            for (int k = 0; k < 3; ++k) s += Jpose[r * 3 + k] * JJm[k * 3 + c];
                            tmp[r * 3 + c] = s;
                        }
                    int idx = 0;
                    for (int r = 0; r < 6; ++r)
                        for (int c = r; c < 6; ++c) {
                            double s = 0;
                            for (int k = 0; k < 3; ++k) s += tmp[r * 3 + k] * Jpose[c * 3 + k];
                            acc[6 + idx] += s;
                            ++idx;
                        }
                    for (int r = 0; r < 6; ++r) {
                        double s = 0;
                        for (int k = 0; k < 3; ++k) s += Jpose[r * 3 + k] * Jrm[k];
                        acc[r] += s;
                    }
                };
                accumulate(JJ, Jr, imgd, rc);

                // ---- second pass over contributors (src/GSCudaKernels.cu:1175-1350) ----
                double prod_alpha = 1.0, Tm = 1.0;
                double accc[3] = {0, 0, 0};
                for (int i = 0; i < n_total && i < (int)n_contrib; ++i) {
                    const Rec g = load_rec(rec, indices[rs + i]);
                    const double dx = g.u - x, dy = g.v - y;
                    const double v = g.cx * dx * dx + 2.0 * g.cy * dx * dy + g.cz * dy * dy;
                    const double G = std::exp(-0.5 * v);
                    const double a = std::min(k099, g.o * G);
                    if (a < kInv255) continue;
                    const double d = g.z + dx * g.phx + dy * g.phy;
                    const double gc[3] = {g.r, g.g, g.b};
                    double da[3];
                    for (int k = 0; k < 3; ++k) {
                        da[k] = gc[k] * prod_alpha;
                        accc[k] += a * da[k];
                    }
                    const double inv1m = 1.0 / (1.0 - a);
                    for (int k = 0; k < 3; ++k) da[k] -= (col[k] - accc[k]) * inv1m;
                    const double dl0 = g.cx * dx + g.cy * dy, dl1 = g.cy * dx + g.cz * dy;
                    const double rg[3] = {(g.u - cx) / fx, (g.v - cy) / fy, 1.0};
                    const double rcg[9] = {0, -rg[2], rg[1], rg[2], 0, -rg[0], -rg[1], rg[0], 0};
                    const double inv_d = 1.0 / d;
                    const double Jt[6] = {fx * inv_d, 0.0, 0.0, fy * inv_d, -fx * rg[0] * inv_d,
                                          -fy * rg[1] * inv_d};
                    const double jt_dl[3] = {Jt[0] * dl0 + Jt[1] * dl1, Jt[2] * dl0 + Jt[3] * dl1,
                                             Jt[4] * dl0 + Jt[5] * dl1};
                    double Jcam[9];
                    for (int r = 0; r < 3; ++r)
                        for (int k = 0; k < 3; ++k) Jcam[r * 3 + k] = jt_dl[r] * a * da[k];
                    double JJg[9];
                    for (int r = 0; r < 3; ++r)
                        for (int c = 0; c < 3; ++c) {
                            double s = 0;
                            for (int k = 0; k < 3; ++k) s += Jcam[r * 3 + k] * Jcam[c * 3 + k];
                            JJg[r * 3 + c] = wc * s;
                        }
                    double Jrg[3];
                    for (int r = 0; r < 3; ++r)
                        Jrg[r] = -wc * (Jcam[r * 3] * e[0] + Jcam[r * 3 + 1] * e[1] + Jcam[r * 3 + 2] * e[2]);
                    prod_alpha *= (1.0 - a);
                    if (Tm > 0.5 && prod_alpha <= 0.5 && imgd > 0.5) {
                        Tm = prod_alpha;
                        const double wd = depth_w(depth_error, depth_thresh, imgd, huber);
                        for (int r = 0; r < 3; ++r)
                            for (int c = 0; c < 3; ++c) JJg[r * 3 + c] += wd * rg[r] * rg[c];
                        for (int r = 0; r < 3; ++r) Jrg[r] += wd * depth_error * rg[r];
                    }
                    accumulate(JJg, Jrg, d, rcg);
                    if (prod_alpha < k1em3) break;
                }
            }
        for (int k = 0; k < 27; ++k) tile_out[27 * (size_t)t + k] = acc[k];
    }
    // Host reduction (src/GSSlam.cu:2205-2226): sum tiles in order,
    // symmetric 6x6 from the upper triangle, Jtr negated.
    double tot[27];
    for (int k = 0; k < 27; ++k) tot[k] = 0.0;
    for (int t = 0; t < T; ++t)
        for (int k = 0; k < 27; ++k) tot[k] += tile_out[27 * (size_t)t + k];
    int idx = 0;
    for (int i = 0; i < 6; ++i) {
        for (int j = i; j < 6; ++j) {
            JtJ[i * 6 + j] = tot[6 + idx];
            JtJ[j * 6 + i] = tot[6 + idx];
            ++idx;
        }
        Jtr[i] = -tot[i];
    }
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Analytic pose Jacobian (the tracking kernel with FVGS_Q_POSE_JAC_APPROX
// clear).  The residuals are those of getRgbdPoseJacobians
// (src/GSCudaKernels.cu:979-1052: rendered colour minus observed colour with
// the colour weight, median depth minus observed depth with the depth
// weight, pixels with observed depth > 0.1 and final T < alpha_thresh), but
// the Jacobian is the exact derivative of the rendered colour and median depth
// with respect to the pose update of PoseLocalParameterization::Plus
// (src/PoseLocalParameterization.cpp:22-44): delta = (dp, dtheta) with
// t' = t + dp, q' = q (x) exp(dtheta).  With p_cam = R^T (p - t):
//   d p_cam / d dp = -R^T,   d p_cam / d dtheta = [p_cam]x,
//   d Sigma_cam / d dtheta_j = -[e_j]x Sigma_cam + Sigma_cam [e_j]x.
// Each contributor's screen mean (u, v), conic (the consumed slots a, b, c of
// v = a dx^2 + 2 b dx dy + c dy^2), depth z and p_hat move with the pose; the
// colour follows through alpha = o exp(-v/2) (zero where alpha is clamped at
// 0.99) and the depth through d = z + dx phat.x + dy phat.y of the Gaussian
// where T crosses 0.5.
// ---------------------------------------------------------------------------
namespace {

struct GeoD {  // derivatives of one Gaussian's screen quantities w.r.t. delta
    double du[6], dv[6], da[6], db[6], dc[6], dz[6], dphx[6], dphy[6];
};

// c3 = (x, y, z, Sxx, Sxy, Sxz, Syy, Syz, Szz): camera-frame mean and 3D
// covariance.  Tangent columns 0-2 are the translation, expressed in the
// frame given by Tr (rows of Tr are the columns of d p_cam / d dp up to sign:
// world frame Tr = R, camera frame Tr = I), 3-5 the rotation.
void gauss_derivs(const double* c3, const double Tr[3][3], double fx, double fy, bool swap, GeoD& o) {
    const double x = c3[0], y = c3[1], z = c3[2];
    const double S[3][3] = {{c3[3], c3[4], c3[5]}, {c3[4], c3[6], c3[7]}, {c3[5], c3[7], c3[8]}};
    const double iz = 1.0 / z, iz2 = iz * iz, iz3 = iz2 * iz;
    const double J0[3] = {fx * iz, 0.0, -fx * x * iz2};
    const double J1[3] = {0.0, fy * iz, -fy * y * iz2};
    double M0[3], M1[3];
    for (int i = 0; i < 3; ++i) {
        M0[i] = S[i][0] * J0[0] + S[i][1] * J0[1] + S[i][2] * J0[2];
        M1[i] = S[i][0] * J1[0] + S[i][1] * J1[1] + S[i][2] * J1[2];
    }
    const double s00 = J0[0] * M0[0] + J0[1] * M0[1] + J0[2] * M0[2];
    const double s01 = J0[0] * M1[0] + J0[1] * M1[1] + J0[2] * M1[2];
    const double s11 = J1[0] * M1[0] + J1[1] * M1[1] + J1[2] * M1[2];
    const double det = s00 * s11 - s01 * s01;
    const double q00 = s11 / det, q01 = -s01 / det, q11 = s00 / det;
    for (int k = 0; k < 6; ++k) {
        double dp[3];
        double dS[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        if (k < 3) {
            for (int i = 0; i < 3; ++i) dp[i] = -Tr[k][i];
        } else {
            const int j = k - 3;
            const double e[3] = {j == 0 ? 1.0 : 0.0, j == 1 ? 1.0 : 0.0, j == 2 ? 1.0 : 0.0};
            // p x e
            dp[0] = y * e[2] - z * e[1];
            dp[1] = z * e[0] - x * e[2];
            dp[2] = x * e[1] - y * e[0];
            const double E[3][3] = {{0, -e[2], e[1]}, {e[2], 0, -e[0]}, {-e[1], e[0], 0}};
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) {
                    double s = 0.0;
                    for (int m = 0; m < 3; ++m) s += -E[r][m] * S[m][c] + S[r][m] * E[m][c];
                    dS[r][c] = s;
                }
        }
        const double dJ0[3] = {-fx * iz2 * dp[2], 0.0, -fx * iz2 * dp[0] + 2.0 * fx * x * iz3 * dp[2]};
        const double dJ1[3] = {0.0, -fy * iz2 * dp[2], -fy * iz2 * dp[1] + 2.0 * fy * y * iz3 * dp[2]};
        double ds00 = 0, ds01 = 0, ds11 = 0;
        for (int i = 0; i < 3; ++i) {
            ds00 += 2.0 * dJ0[i] * M0[i];
            ds01 += dJ0[i] * M1[i] + dJ1[i] * M0[i];
            ds11 += 2.0 * dJ1[i] * M1[i];
        }
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) {
                ds00 += J0[r] * dS[r][c] * J0[c];
                ds01 += J0[r] * dS[r][c] * J1[c];
                ds11 += J1[r] * dS[r][c] * J1[c];
            }
        // d(Sigma^-1) = -Q dSigma Q
        const double dq00 = -(q00 * q00 * ds00 + 2.0 * q00 * q01 * ds01 + q01 * q01 * ds11);
        const double dq01 = -(q00 * q01 * ds00 + (q00 * q11 + q01 * q01) * ds01 + q01 * q11 * ds11);
        const double dq11 = -(q01 * q01 * ds00 + 2.0 * q01 * q11 * ds01 + q11 * q11 * ds11);
        o.du[k] = J0[0] * dp[0] + J0[1] * dp[1] + J0[2] * dp[2];
        o.dv[k] = J1[0] * dp[0] + J1[1] * dp[1] + J1[2] * dp[2];
        o.da[k] = dq00;
        o.db[k] = swap ? dq11 : dq01;
        o.dc[k] = swap ? dq01 : dq11;
        o.dz[k] = dp[2];
        o.dphx[k] = dp[0] * iz2 - 2.0 * x * iz3 * dp[2];
        o.dphy[k] = dp[1] * iz2 - 2.0 * y * iz3 * dp[2];
    }
}

// FP64 camera-frame mean and covariance of one Gaussian (the projection's
// formulas, src/GSCudaKernels.cu:366-433).
void cam3d_one(const float* p, const float* s, const float* q, const double t[3], const double R[3][3], double* o) {
    const double d[3] = {(double)p[0] - t[0], (double)p[1] - t[1], (double)p[2] - t[2]};
    double pc[3];
    for (int i = 0; i < 3; ++i) pc[i] = R[0][i] * d[0] + R[1][i] * d[1] + R[2][i] * d[2];
    double Rg[3][3];
    quat_to_R_f64(q, Rg);
    double M[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[i][j] = Rg[i][j] * (double)s[j];
    double Sg[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Sg[i][j] = M[i][0] * M[j][0] + M[i][1] * M[j][1] + M[i][2] * M[j][2];
    double C[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k)
                for (int l = 0; l < 3; ++l) acc += R[k][i] * Sg[k][l] * R[l][j];
            C[i][j] = acc;
        }
    o[0] = pc[0];
    o[1] = pc[1];
    o[2] = pc[2];
    o[3] = C[0][0];
    o[4] = C[0][1];
    o[5] = C[0][2];
    o[6] = C[1][1];
    o[7] = C[1][2];
    o[8] = C[2][2];
}

void quat_to_R_d(const double q[4], double R[3][3]) {
    const double x = q[0], y = q[1], z = q[2], w = q[3];
    R[0][0] = 1.0 - 2.0 * (y * y + z * z);
    R[0][1] = 2.0 * (x * y - w * z);
    R[0][2] = 2.0 * (x * z + w * y);
    R[1][0] = 2.0 * (x * y + w * z);
    R[1][1] = 1.0 - 2.0 * (x * x + z * z);
    R[1][2] = 2.0 * (y * z - w * x);
    R[2][0] = 2.0 * (x * z - w * y);
    R[2][1] = 2.0 * (y * z + w * x);
    R[2][2] = 1.0 - 2.0 * (x * x + y * y);
}

}  // namespace

extern "C" {

/*
 * FP64 camera-frame geometry of every Gaussian at a pose: cam3d[9N] =
 * (x, y, z, Sxx, Sxy, Sxz, Syy, Syz, Szz), the inputs of the analytic pose
 * Jacobian.
 */
int oracle_cam3d(const float* pos, const float* scl, const float* rot, int n, const fvgs_pose* pose,
                 double* cam3d) {
    double R[3][3];
    quat_to_R_f64(pose->orientation, R);
    const double t[3] = {pose->position[0], pose->position[1], pose->position[2]};
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i)
        cam3d_one(pos + 3 * (size_t)i, scl + 3 * (size_t)i, rot + 4 * (size_t)i, t, R, cam3d + 9 * (size_t)i);
    return 0;
}

/*
 * The tracking forward blend (src/GSCudaKernels.cu:979-1041) entirely in FP64
 * at an FP64 pose (t[3], q[4] (x, y, z, w)), over the given tile lists: the
 * projection's formulas in FP64 (a Gaussian that this projection culls is
 * skipped), the consumed conic as the quirk bits select.  Every pixel is
 * treated as having valid observed depth.  Outputs colour (incl. background)
 * and median depth per pixel; sig[3P] = (Gaussians blended, list position of
 * the median-depth Gaussian + 1 (0: none), n_contrib), which identifies the
 * piecewise-smooth branch a pixel is on.  For finite-difference checks of the
 * analytic Jacobian.
 */
int oracle_forward64(const float* pos, const float* scl, const float* rot, const float* col, const float* opa, int n,
                     const double* t, const double* q, const fvgs_intrinsics* K, const fvgs_params* P, int W, int H,
                     const uint32_t* ranges, const uint32_t* indices, double* out_color, double* out_depth,
                     uint32_t* sig) {
    double R[3][3];
    quat_to_R_d(q, R);
    const double fx = K->fx, fy = K->fy, cx = K->cx, cy = K->cy;
    const bool swap = (P->quirks & FVGS_Q_INVSIGMA_SWAP) != 0;
    struct G64 {
        bool ok;
        double u, v, z, a, b, c, phx, phy;
    };
    std::vector<G64> g(n > 0 ? n : 1);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        double c3[9];
        cam3d_one(pos + 3 * (size_t)i, scl + 3 * (size_t)i, rot + 4 * (size_t)i, t, R, c3);
        G64 o{};
        const double x = c3[0], y = c3[1], z = c3[2];
        if (z > 0.0) {
            const double iz = 1.0 / z;
            o.u = fx * x * iz + cx;
            o.v = fy * y * iz + cy;
            o.ok = !(o.u < 0.0 || o.u >= W || o.v < 0.0 || o.v >= H);
            const double J0[3] = {fx * iz, 0.0, -fx * x * iz * iz};
            const double J1[3] = {0.0, fy * iz, -fy * y * iz * iz};
            const double S[3][3] = {{c3[3], c3[4], c3[5]}, {c3[4], c3[6], c3[7]}, {c3[5], c3[7], c3[8]}};
            double s00 = 0, s01 = 0, s11 = 0;
            for (int r = 0; r < 3; ++r)
                for (int cc = 0; cc < 3; ++cc) {
                    s00 += J0[r] * S[r][cc] * J0[cc];
                    s01 += J0[r] * S[r][cc] * J1[cc];
                    s11 += J1[r] * S[r][cc] * J1[cc];
                }
            const double det = s00 * s11 - s01 * s01;
            const double q00 = s11 / det, q01 = -s01 / det, q11 = s00 / det;
            o.a = q00;
            o.b = swap ? q11 : q01;
            o.c = swap ? q01 : q11;
            o.z = z;
            o.phx = x * iz * iz;
            o.phy = y * iz * iz;
        }
        g[i] = o;
    }
    const int tw = P->tile_w, th = P->tile_h;
    const int ntx = (W + tw - 1) / tw, nty = (H + th - 1) / th, T = ntx * nty;
    const double bg[3] = {P->bg[0], P->bg[1], P->bg[2]};
#pragma omp parallel for schedule(dynamic, 1)
    for (int tt = 0; tt < T; ++tt) {
        const int tx = tt % ntx, ty = tt / ntx;
        const uint32_t rs = ranges[2 * (size_t)tt], re = ranges[2 * (size_t)tt + 1];
        for (int ly = 0; ly < th; ++ly)
            for (int lx = 0; lx < tw; ++lx) {
                const int x = tx * tw + lx, y = ty * th + ly;
                if (x >= W || y >= H) continue;
                const size_t p = (size_t)y * W + x;
                double c[3] = {0, 0, 0}, depth = 0.0, Tr = 1.0;
                uint32_t nbl = 0, med = 0, last = 0;
                for (uint32_t i = rs; i < re; ++i) {
                    const uint32_t gi = indices[i];
                    if (gi >= (uint32_t)n || !g[gi].ok) continue;
                    const G64& o = g[gi];
                    const uint32_t ord = i - rs + 1;
                    const double dx = o.u - x, dy = o.v - y;
                    const double v = o.a * dx * dx + 2.0 * o.b * dx * dy + o.c * dy * dy;
                    const double al = std::min(k099, (double)opa[gi] * std::exp(-0.5 * v));
                    if (al < kInv255 || v <= 0.0) continue;
                    const double test_T = Tr * (1.0 - al);
                    if (test_T < k1em4) break;
                    for (int k = 0; k < 3; ++k) c[k] += (double)col[3 * (size_t)gi + k] * al * Tr;
                    if (Tr > 0.5 && test_T < 0.5) {
                        depth = o.z + dx * o.phx + dy * o.phy;
                        med = ord;
                    }
                    Tr = test_T;
                    ++nbl;
                    last = ord;
                }
                for (int k = 0; k < 3; ++k) out_color[3 * p + k] = c[k] + Tr * bg[k];
                out_depth[p] = depth;
                sig[3 * p] = nbl;
                sig[3 * p + 1] = med;
                sig[3 * p + 2] = last;
            }
    }
    return 0;
}

/*
 * The tracking kernel with the analytic pose Jacobian, in FP64, one pixel at
 * a time: the forward blend of oracle_track (same records, lists and
 * thresholds), then for every valid pixel the colour Jacobian
 * J_C = sum_i dC/dalpha_i dalpha_i/dv_i dv_i/ddelta over the Gaussians the
 * forward blended, dC/dalpha_i = c_i T_i - (C - A_i) / (1 - alpha_i) (A_i the
 * colour accumulated up to and including i, C the final colour with the
 * background), and the depth Jacobian J_D of the median-depth Gaussian.  A
 * pixel adds wc J_C^T J_C + wd J_D^T J_D to JtJ and -(wc J_C^T e_c +
 * wd J_D^T e_d) to the tile's Jtr sum (the reference's per-tile sign;
 * src/GSSlam.cu:2225 negates it), with the reference's colour and depth
 * weights.  cam3d (oracle_cam3d at the same pose) supplies the geometry.
 * Outputs as oracle_track (world frame); optional per-pixel Jacobians
 * pix_jc[18P] (3 x 6 row-major) and pix_jd[6P].
 */
int oracle_track_intended(const float* rec, const double* cam3d, const uint32_t* ranges, const uint32_t* indices,
                          const float* obs_rgb, const float* obs_depth, const fvgs_pose* pose,
                          const fvgs_intrinsics* Kf, const fvgs_params* P, int W, int H, double* tile_out,
                          double* JtJ, double* Jtr, double* img_color, double* img_depth, double* img_T,
                          uint32_t* img_nc, double* pix_jc, double* pix_jd, const uint8_t* tile_mask) {
    const int tw = P->tile_w, th = P->tile_h;
    const int ntx = (W + tw - 1) / tw, nty = (H + th - 1) / th, T = ntx * nty;
    double R[3][3];
    quat_to_R_f64(pose->orientation, R);
    const double fx = Kf->fx, fy = Kf->fy;
    const bool swap = (P->quirks & FVGS_Q_INVSIGMA_SWAP) != 0;
    const double bg[3] = {P->bg[0], P->bg[1], P->bg[2]};
    const double alpha_thresh = P->alpha_thresh, color_thresh = P->color_thresh,
                 depth_thresh = P->depth_thresh;
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < T; ++t) {
        const int tx = t % ntx, ty = t / ntx;
        double acc[27];
        for (int k = 0; k < 27; ++k) acc[k] = 0.0;
        if (tile_mask && !tile_mask[t]) {  // not evaluated: zero partials, images untouched
            for (int k = 0; k < 27; ++k) tile_out[27 * (size_t)t + k] = 0.0;
            continue;
        }
        const uint32_t rs = ranges[2 * (size_t)t], re = ranges[2 * (size_t)t + 1];
        const int n_total = (int)(re - rs);
        std::vector<GeoD> dcache(n_total > 0 ? n_total : 1);
        std::vector<char> have(n_total > 0 ? n_total : 1, 0);
        for (int ly = 0; ly < th; ++ly)
            for (int lx = 0; lx < tw; ++lx) {
                const int x = tx * tw + lx, y = ty * th + ly;
                const bool in_bounds = (x < W && y < H);
                const size_t p = (size_t)y * W + x;
                double imgd = 0.0;
                if (in_bounds) imgd = obs_depth[p];
                bool inside = in_bounds && imgd > (double)0.1f;
                double col[3] = {0, 0, 0};
                double depth = 0.0, final_T = 1.0;
                uint32_t n_contrib = 0;
                if (n_total > 0) {
                    double Tr = 1.0;
                    uint32_t contributor = 0, last = 0;
                    bool done = !inside;
                    for (int i = 0; i < n_total && !done; ++i) {
                        contributor++;
                        const Rec g = load_rec(rec, indices[rs + i]);
                        const double dx = g.u - x, dy = g.v - y;
                        const double v = g.cx * dx * dx + 2.0 * g.cy * dx * dy + g.cz * dy * dy;
                        const double a = std::min(k099, g.o * std::exp(-0.5 * v));
                        if (a < kInv255 || v <= 0.0) continue;
                        const double test_T = Tr * (1.0 - a);
                        if (test_T < k1em4) {
                            done = true;
                            continue;
                        }
                        col[0] += g.r * a * Tr;
                        col[1] += g.g * a * Tr;
                        col[2] += g.b * a * Tr;
                        const double d = g.z + dx * g.phx + dy * g.phy;
                        if (Tr > 0.5 && test_T < 0.5) depth = d;
                        Tr = test_T;
                        last = contributor;
                    }
                    if (inside) {
                        final_T = Tr;
                        n_contrib = last;
                        col[0] += Tr * bg[0];
                        col[1] += Tr * bg[1];
                        col[2] += Tr * bg[2];
                    }
                }
                if (in_bounds) {
                    if (img_color) {
                        img_color[3 * p] = col[0];
                        img_color[3 * p + 1] = col[1];
                        img_color[3 * p + 2] = col[2];
                    }
                    if (img_depth) img_depth[p] = depth;
                    if (img_T) img_T[p] = final_T;
                    if (img_nc) img_nc[p] = n_contrib;
                    if (pix_jc)
                        for (int k = 0; k < 18; ++k) pix_jc[18 * p + k] = 0.0;
                    if (pix_jd)
                        for (int k = 0; k < 6; ++k) pix_jd[6 * p + k] = 0.0;
                }
                inside = inside && (final_T < alpha_thresh);
                if (!inside) continue;

                double JC[3][6], JD[6];
                for (int k = 0; k < 6; ++k) {
                    JC[0][k] = JC[1][k] = JC[2][k] = 0.0;
                    JD[k] = 0.0;
                }
                double prod = 1.0, rem[3] = {col[0], col[1], col[2]};
                for (int i = 0; i < n_total && i < (int)n_contrib; ++i) {
                    const uint32_t gi = indices[rs + i];
                    const Rec g = load_rec(rec, gi);
                    const double dx = g.u - x, dy = g.v - y;
                    const double v = g.cx * dx * dx + 2.0 * g.cy * dx * dy + g.cz * dy * dy;
                    const double raw = g.o * std::exp(-0.5 * v);
                    const double a = std::min(k099, raw);
                    if (a < kInv255 || v <= 0.0) continue;
                    if (!have[i]) {
                        gauss_derivs(cam3d + 9 * (size_t)gi, R, fx, fy, swap, dcache[i]);
                        have[i] = 1;
                    }
                    const GeoD& D = dcache[i];
                    const double gc[3] = {g.r, g.g, g.b};
                    double dCda[3];
                    for (int k = 0; k < 3; ++k) {
                        rem[k] -= gc[k] * a * prod;
                        dCda[k] = gc[k] * prod - rem[k] / (1.0 - a);
                    }
                    const double dadv = (raw > k099) ? 0.0 : -0.5 * a;
                    const double cu = 2.0 * (g.cx * dx + g.cy * dy), cv = 2.0 * (g.cy * dx + g.cz * dy);
                    const double ca = dx * dx, cb = 2.0 * dx * dy, cc = dy * dy;
                    for (int k = 0; k < 6; ++k) {
                        const double dvd = cu * D.du[k] + cv * D.dv[k] + ca * D.da[k] + cb * D.db[k] + cc * D.dc[k];
                        for (int c = 0; c < 3; ++c) JC[c][k] += dCda[c] * dadv * dvd;
                    }
                    const double np = prod * (1.0 - a);
                    if (prod > 0.5 && np < 0.5)
                        for (int k = 0; k < 6; ++k)
                            JD[k] = D.dz[k] + g.phx * D.du[k] + dx * D.dphx[k] + g.phy * D.dv[k] + dy * D.dphy[k];
                    prod = np;
                }
                const double e[3] = {col[0] - obs_rgb[3 * p], col[1] - obs_rgb[3 * p + 1],
                                     col[2] - obs_rgb[3 * p + 2]};
                const double derr = depth - imgd;
                const double closs = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
                const double wc = (closs < color_thresh) ? 1.0 : color_thresh / closs;
                const double wd = depth_w(derr, depth_thresh, imgd, (P->quirks & FVGS_Q_DEPTH_HUBER) != 0);
                int idx = 0;
                for (int i = 0; i < 6; ++i)
                    for (int j = i; j < 6; ++j) {
                        double s = wd * JD[i] * JD[j];
                        for (int c = 0; c < 3; ++c) s += wc * JC[c][i] * JC[c][j];
                        acc[6 + idx] += s;
                        ++idx;
                    }
                for (int i = 0; i < 6; ++i) {
                    double s = wd * JD[i] * derr;
                    for (int c = 0; c < 3; ++c) s += wc * JC[c][i] * e[c];
                    acc[i] -= s;
                }
                if (pix_jc)
                    for (int c = 0; c < 3; ++c)
                        for (int k = 0; k < 6; ++k) pix_jc[18 * p + 6 * c + k] = JC[c][k];
                if (pix_jd)
                    for (int k = 0; k < 6; ++k) pix_jd[6 * p + k] = JD[k];
            }
        for (int k = 0; k < 27; ++k) tile_out[27 * (size_t)t + k] = acc[k];
    }
    double tot[27];
    for (int k = 0; k < 27; ++k) tot[k] = 0.0;
    for (int t = 0; t < T; ++t)
        for (int k = 0; k < 27; ++k) tot[k] += tile_out[27 * (size_t)t + k];
    int idx = 0;
    for (int i = 0; i < 6; ++i) {
        for (int j = i; j < 6; ++j) {
            JtJ[i * 6 + j] = tot[6 + idx];
            JtJ[j * 6 + i] = tot[6 + idx];
            ++idx;
        }
        Jtr[i] = -tot[i];
    }
    return 0;
}

/*
 * Bucket bookkeeping of the mapping step: perTileBucketCount +
 * thrust::inclusive_scan (src/GSCudaKernels.cu:2074-2090, src/GSSlam.cu:1130-1147).
 * bucket_incl[T] = inclusive prefix of ceil(n_tile/32); returns the total.
 */
int64_t oracle_buckets(const uint32_t* ranges, int num_tiles, uint32_t* bucket_incl) {
    int64_t acc = 0;
    for (int t = 0; t < num_tiles; ++t) {
        const int n = (int)(ranges[2 * (size_t)t + 1] - ranges[2 * (size_t)t]);
        acc += (uint32_t)(n + 31) / 32u;
        bucket_incl[t] = (uint32_t)acc;
    }
    return acc;
}

/*
 * Mapping forward optimizeGaussiansForwardPass (src/GSCudaKernels.cu:2092-2263),
 * FP64.  Per pixel: final_T, n_contrib, colour (with background), depth,
 * colour error, observed depth (the reference stores it in depth_error).
 * Per bucket x pixel checkpoints sampled_T / sampled_ar (written only while
 * the pixel is still blending, as in the reference).  max_contrib per tile.
 * Buffers sampled_* hold num_buckets * tile_w*tile_h entries.
 */
int oracle_map_forward(const float* rec, const uint32_t* ranges, const uint32_t* indices,
                       const uint32_t* bucket_incl, const float* obs_rgb, const float* obs_depth,
                       const fvgs_params* P, int W, int H, double* final_T, uint32_t* n_contrib,
                       uint32_t* max_contrib, double* out_color, double* out_depth, double* color_err,
                       double* depth_obs, double* sampled_T, double* sampled_ar) {
    const int tw = P->tile_w, th = P->tile_h, BS = tw * th;
    const int ntx = (W + tw - 1) / tw, nty = (H + th - 1) / th, T = ntx * nty;
    const double bg[3] = {P->bg[0], P->bg[1], P->bg[2]};
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < T; ++t) {
        const int tx = t % ntx, ty = t / ntx;
        const uint32_t rs = ranges[2 * (size_t)t];
        const int n = (int)(ranges[2 * (size_t)t + 1] - rs);
        const uint32_t bucket_base = (t == 0) ? 0u : bucket_incl[t - 1];
        uint32_t maxc = 0;
        for (int tid = 0; tid < BS; ++tid) {
            const int x = tx * tw + tid % tw, y = ty * th + tid / tw;
            const bool inside = (x < W && y < H);
            bool done = !inside;
            double Tr = 1.0, col[3] = {0, 0, 0}, depth = 0.0;
            uint32_t contributor = 0, last = 0;
            for (int gi = 0; gi < n && !done; ++gi) {
                if (gi % 32 == 0) {
                    const size_t s = ((size_t)bucket_base + gi / 32) * BS + tid;
                    sampled_T[s] = Tr;
                    sampled_ar[3 * s] = col[0];
                    sampled_ar[3 * s + 1] = col[1];
                    sampled_ar[3 * s + 2] = col[2];
                }
                contributor++;
                const Rec g = load_rec(rec, indices[rs + gi]);
                const double dx = x - g.u, dy = y - g.v;
                const double v = g.cx * dx * dx + 2.0 * g.cy * dx * dy + g.cz * dy * dy;
                const double a = std::min(k099, g.o * std::exp(-0.5 * v));
                if (a < kInv255 || v <= 0.0) continue;
                const double Tpre = Tr;
                col[0] += Tr * a * g.r;
                col[1] += Tr * a * g.g;
                col[2] += Tr * a * g.b;
                const double test_T = Tr * (1.0 - a);
                if (Tpre > 0.5 && test_T <= 0.5) depth = g.z + g.phx * dx + g.phy * dy;
                Tr = test_T;
                last = contributor;
                if (test_T < k1em4) done = true;
            }
            if (inside) {
                const size_t p = (size_t)y * W + x;
                final_T[p] = Tr;
                n_contrib[p] = last;
                for (int k = 0; k < 3; ++k) col[k] += Tr * bg[k];
                for (int k = 0; k < 3; ++k) {
                    out_color[3 * p + k] = col[k];
                    color_err[3 * p + k] = col[k] - (double)obs_rgb[3 * p + k];
                }
                out_depth[p] = depth;
                depth_obs[p] = obs_depth[p];
            }
            maxc = std::max(maxc, last);
        }
        max_contrib[t] = maxc;
    }
    return 0;
}

/*
 * Mapping backward optimizeGaussiansPerGaussianPass
 * (src/GSCudaKernels.cu:2265-2502), FP64.  The warp's shuffle pipeline is
 * restated sequentially: for each bucket of 32 tile-list entries and each
 * pixel, the per-pixel state (T, accumulated colour) starts from the
 * forward checkpoint and flows through the bucket's Gaussians in order.
 * delta2d[13N] accumulates DeltaGaussian2D (GSCudaKernels.cuh:11-20):
 * meanImg.xy, invSigmaImg.xyz, color.xyz, depth, alpha, pHat.xy, n.
 */
int oracle_map_backward(const float* rec, const uint32_t* ranges, const uint32_t* indices,
                        const uint32_t* bucket_incl, const double* sampled_T, const double* sampled_ar,
                        const uint32_t* n_contrib, const uint32_t* max_contrib, const double* out_color,
                        const double* out_depth, const double* color_err, const double* depth_obs,
                        const fvgs_params* P, int W, int H, double* delta2d) {
    const int tw = P->tile_w, th = P->tile_h, BS = tw * th;
    const int ntx = (W + tw - 1) / tw, nty = (H + th - 1) / th, T = ntx * nty;
    const double w_depth = P->w_depth, w_dist = P->w_dist;
    const bool cap = (P->quirks & FVGS_Q_MAP_CAP256) != 0;
#pragma omp parallel for schedule(dynamic, 1)
    for (int t = 0; t < T; ++t) {
        const int tx = t % ntx, ty = t / ntx;
        const uint32_t rs = ranges[2 * (size_t)t];
        const uint32_t n = ranges[2 * (size_t)t + 1] - rs;
        const uint32_t bucket_base = (t == 0) ? 0u : bucket_incl[t - 1];
        const uint32_t nb = (n + 31) / 32;
        const uint32_t n_splat = cap ? std::min(n, 256u) : n;
        for (uint32_t b = 0; b < nb; ++b) {
            if (b * 32 >= max_contrib[t]) continue;
            const size_t gb = (size_t)bucket_base + b;
            double dl[32][13];
            std::memset(dl, 0, sizeof(dl));
            Rec gr[32];
            for (int k = 0; k < 32; ++k) {
                const uint32_t j = b * 32 + k;
                if (j < n_splat) gr[k] = load_rec(rec, indices[rs + j]);
            }
            if (b * 32 >= n_splat) continue;  // lane 0 invalid -> whole bucket idle
            for (int idx = 0; idx < BS; ++idx) {
                const int px = tx * tw + idx % tw, py = ty * th + idx / tw;
                if (px >= W || py >= H) continue;
                const size_t p = (size_t)py * W + px;
                double Tr = sampled_T[gb * BS + idx];
                double acc[3] = {sampled_ar[3 * (gb * BS + idx)], sampled_ar[3 * (gb * BS + idx) + 1],
                                 sampled_ar[3 * (gb * BS + idx) + 2]};
                const double color[3] = {out_color[3 * p], out_color[3 * p + 1], out_color[3 * p + 2]};
                const double depth = out_depth[p];
                const uint32_t lastc = n_contrib[p];
                const double ce[3] = {color_err[3 * p], color_err[3 * p + 1], color_err[3 * p + 2]};
                const double imgd = depth_obs[p];
                for (int k = 0; k < 32; ++k) {
                    const uint32_t j = b * 32 + k;
                    if (j >= n_splat) continue;
                    if (j >= lastc) continue;
                    const Rec& g = gr[k];
                    const double dx = g.u - px, dy = g.v - py;
                    const double v = g.cx * dx * dx + 2.0 * g.cy * dx * dy + g.cz * dy * dy;
                    const double G = std::exp(-0.5 * v);
                    const double a = std::min(k099, g.o * G);
                    if (a < kInv255) continue;
                    const double gc[3] = {g.r, g.g, g.b};
                    double da[3];
                    for (int c = 0; c < 3; ++c) {
                        da[c] = gc[c] * Tr;
                        acc[c] += da[c] * a;
                    }
                    const double inv1m = 1.0 / (1.0 - a);
                    for (int c = 0; c < 3; ++c) {
                        da[c] -= (color[c] - acc[c]) * inv1m;
                        da[c] *= -ce[c];
                    }
                    const double dla = da[0] + da[1] + da[2];
                    const double aG = a * dla;
                    double* D = dl[k];
                    D[12] += 1.0;
                    for (int c = 0; c < 3; ++c) D[5 + c] -= a * Tr * ce[c];
                    D[9] -= aG;
                    D[0] -= aG * (g.cx * dx + g.cy * dy);
                    D[1] -= aG * (g.cy * dx + g.cz * dy);
                    D[2] -= 0.5 * aG * dx * dx;
                    D[3] -= 0.5 * aG * dx * dy;
                    D[4] -= 0.5 * aG * dy * dy;
                    const double test_T = Tr * (1.0 - a);
                    if (Tr > 0.5 && test_T <= 0.5) {
                        const double derr = (imgd > (double)0.1f) ? (depth - imgd) : 0.0;
                        D[8] -= w_depth * derr;
                        D[0] -= w_depth * derr * g.phx;
                        D[1] -= w_depth * derr * g.phy;
                        D[10] -= w_depth * derr * dx;
                        D[11] -= w_depth * derr * dy;
                    }
                    const double di = g.z + dx * g.phx + dy * g.phy;
                    const double dd = di - depth;
                    const double dc = w_dist * a * Tr * dd;
                    D[8] -= dc;
                    D[0] -= dc * g.phx;
                    D[1] -= dc * g.phy;
                    D[10] -= dc * dx;
                    D[11] -= dc * dy;
                    Tr = test_T;
                }
            }
            for (int k = 0; k < 32; ++k) {
                const uint32_t j = b * 32 + k;
                if (j >= n_splat || dl[k][12] == 0.0) continue;
                const uint32_t gid = indices[rs + j];
                for (int f = 0; f < 13; ++f) {
#pragma omp atomic
                    delta2d[13 * (size_t)gid + f] += dl[k][f];
                }
            }
        }
    }
    return 0;
}

namespace {
struct Qd {
    double x, y, z, w;
};
// Eigen's Quaternion::_transformVector: uv = 2 vec x v; v + w uv + vec x uv.
inline void q_apply(const Qd& q, const double v[3], double o[3]) {
    double uv[3] = {q.y * v[2] - q.z * v[1], q.z * v[0] - q.x * v[2], q.x * v[1] - q.y * v[0]};
    for (int k = 0; k < 3; ++k) uv[k] += uv[k];
    const double c[3] = {q.y * uv[2] - q.z * uv[1], q.z * uv[0] - q.x * uv[2], q.x * uv[1] - q.y * uv[0]};
    for (int k = 0; k < 3; ++k) o[k] = v[k] + q.w * uv[k] + c[k];
}
inline Qd q_inverse(const Qd& q) {  // conjugate / squared norm
    const double n2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (n2 > 0) return Qd{-q.x / n2, -q.y / n2, -q.z / n2, q.w / n2};
    return Qd{0, 0, 0, 0};
}
inline void q_to_R(const Qd& q, double R[3][3]) {  // Eigen toRotationMatrix
    const double tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    R[0][0] = 1 - (tyy + tzz); R[0][1] = txy - twz; R[0][2] = txz + twy;
    R[1][0] = txy + twz; R[1][1] = 1 - (txx + tzz); R[1][2] = tyz - twx;
    R[2][0] = txz - twy; R[2][1] = tyz + twx; R[2][2] = 1 - (txx + tyy);
}
inline void mm3(const double A[3][3], const double B[3][3], double C[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}
inline void inv3(const double A[3][3], double I[3][3]) {
    const double c00 = A[1][1] * A[2][2] - A[1][2] * A[2][1];
    const double c01 = A[1][2] * A[2][0] - A[1][0] * A[2][2];
    const double c02 = A[1][0] * A[2][1] - A[1][1] * A[2][0];
    const double det = A[0][0] * c00 + A[0][1] * c01 + A[0][2] * c02;
    const double id = 1.0 / det;
    I[0][0] = c00 * id;
    I[1][0] = c01 * id;
    I[2][0] = c02 * id;
    I[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id;
    I[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id;
    I[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id;
    I[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
    I[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
    I[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
}
}  // namespace

/*
 * computeDeltaGaussians3D_kernel (src/GSCudaKernels.cu:2504-2720), FP64.
 * delta3d[14N] = position.xyz, scale.xyz, orientation.xyz, color.xyz, alpha, n.
 * Gaussians with n == 0 get all zeros.
 */
int oracle_delta3d(const float* pos, const float* scl, const float* rot, const double* delta2d, int ng,
                   const fvgs_pose* pose, const fvgs_intrinsics* K, float lambda_iso, double* delta3d) {
    const double fx = K->fx, fy = K->fy;
    const Qd qcw{pose->orientation[0], pose->orientation[1], pose->orientation[2], pose->orientation[3]};
    const Qd qcw_inv = q_inverse(qcw);
    double Rcw[3][3];
    q_to_R(qcw_inv, Rcw);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ng; ++i) {
        const double* d2 = delta2d + 13 * (size_t)i;
        double* o = delta3d + 14 * (size_t)i;
        for (int k = 0; k < 14; ++k) o[k] = 0.0;
        const double n = d2[12];
        if (n == 0.0) continue;
        o[13] = n;
        const double eta_n = 1.0 / (5.0 + n);
        for (int c = 0; c < 3; ++c) o[9 + c] = d2[5 + c] * eta_n;
        o[12] = d2[9] * eta_n;
        const double dw[3] = {pos[3 * (size_t)i] - (double)pose->position[0],
                              pos[3 * (size_t)i + 1] - (double)pose->position[1],
                              pos[3 * (size_t)i + 2] - (double)pose->position[2]};
        double mc[3];
        q_apply(qcw_inv, dw, mc);
        const Qd qg{rot[4 * (size_t)i], rot[4 * (size_t)i + 1], rot[4 * (size_t)i + 2], rot[4 * (size_t)i + 3]};
        const double s[3] = {scl[3 * (size_t)i], scl[3 * (size_t)i + 1], scl[3 * (size_t)i + 2]};
        const double z = mc[2];
        const double J[3][3] = {{fx / z, 0.0, -fx * mc[0] / (z * z)}, {0.0, fy / z, -fy * mc[1] / (z * z)},
                                {0.0, 0.0, 1.0}};
        double Rg[3][3];
        q_to_R(qg, Rg);
        double Tm[3][3], RS[3][3], M[3][3], Sp[3][3], Spi[3][3];
        mm3(J, Rcw, Tm);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) RS[r][c] = Rg[r][c] * s[c];
        mm3(Tm, RS, M);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) Sp[r][c] = M[r][0] * M[c][0] + M[r][1] * M[c][1] + M[r][2] * M[c][2];
        inv3(Sp, Spi);
        const double dmu2[3] = {d2[0], d2[1], 0.0};
        double tmp[3];
        for (int r = 0; r < 3; ++r)
            tmp[r] = J[0][r] * dmu2[0] + J[1][r] * dmu2[1] + J[2][r] * dmu2[2];
        const double dz = d2[8];
        tmp[0] += dz * (mc[0] / z);
        tmp[1] += dz * (mc[1] / z);
        tmp[2] += dz * 1.0;
        double dmu3[3];
        q_apply(qcw, tmp, dmu3);
        const double dph[2] = {d2[10], d2[11]};
        const double n2 = mc[0] * mc[0] + mc[1] * mc[1] + mc[2] * mc[2];
        const double nm = std::sqrt(n2);
        const double in3 = 1.0 / (n2 * nm);
        const double dpdm[3] = {-mc[0] * mc[2] * in3, -mc[1] * mc[2] * in3,
                                (mc[0] * mc[0] + mc[1] * mc[1]) * in3};
        const double fac = (Spi[2][0] * dph[0] + Spi[2][1] * dph[1]) / Spi[2][2];
        {
            const double v[3] = {dpdm[0] * fac, dpdm[1] * fac, dpdm[2] * fac};
            double w[3];
            q_apply(qcw, v, w);
            for (int k = 0; k < 3; ++k) dmu3[k] += w[k];
        }
        const double sxx = Sp[0][0] + (double)0.001f, sxy = Sp[1][0], syy = Sp[1][1] + (double)0.001f;
        const double den = sxx * syy - sxy * sxy;
        const double d2i = 1.0 / ((den * den) + (double)0.0000001f);
        const double Li[3] = {d2[2], d2[3], d2[4]};
        const double dSxx = d2i * (-syy * syy * Li[0] + 2 * sxy * syy * Li[1] + (den - sxx * syy) * Li[2]);
        const double dSyy = d2i * (-sxx * sxx * Li[2] + 2 * sxx * sxy * Li[1] + (den - sxx * syy) * Li[0]);
        const double dSxy = d2i * 2 * (sxy * syy * Li[0] - (den + 2 * sxy * sxy) * Li[1] + sxx * sxy * Li[2]);
        double S3[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) S3[r][c] = RS[r][0] * RS[c][0] + RS[r][1] * RS[c][1] + RS[r][2] * RS[c][2];
        auto dotrow = [&](const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
        double dT[2][3];
        for (int j = 0; j < 3; ++j) {
            dT[0][j] = 2 * dotrow(Tm[0], S3[j]) * dSxx + dotrow(Tm[1], S3[j]) * dSxy;
            dT[1][j] = 2 * dotrow(Tm[1], S3[j]) * dSyy + dotrow(Tm[0], S3[j]) * dSxy;
        }
        const double zt = z / nm;
        const double a_ = 0.5 * zt * dph[0] / Spi[2][2];
        const double b_ = 0.5 * zt * dph[1] / Spi[2][2];
        const double c_ = -zt * (dph[0] * Spi[2][0] + dph[1] * Spi[2][1]) / (Spi[2][2] * Spi[2][2]);
        const double dLSi[3][3] = {{0, 0, a_}, {0, 0, b_}, {a_, b_, c_}};
        double t1[3][3], dSp[3][3];
        mm3(Spi, dLSi, t1);
        mm3(t1, Spi, dSp);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) dSp[r][c] = -dSp[r][c];
        double TS[3][3], ST[3][3];
        mm3(Tm, S3, TS);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) ST[r][c] = S3[r][0] * Tm[c][0] + S3[r][1] * Tm[c][1] + S3[r][2] * Tm[c][2];
        for (int a = 0; a < 2; ++a)
            for (int j = 0; j < 3; ++j) {
                double s1 = 0, s2 = 0;
                for (int k = 0; k < 3; ++k) {
                    s1 += TS[k][j] * dSp[k][a];
                    s2 += ST[j][k] * dSp[a][k];
                }
                dT[a][j] += s1 + s2;
            }
        const double dJ00 = Rcw[0][0] * dT[0][0] + Rcw[0][1] * dT[0][1] + Rcw[0][2] * dT[0][2];
        const double dJ02 = Rcw[2][0] * dT[0][0] + Rcw[2][1] * dT[0][1] + Rcw[2][2] * dT[0][2];
        const double dJ11 = Rcw[1][0] * dT[1][0] + Rcw[1][1] * dT[1][1] + Rcw[1][2] * dT[1][2];
        const double dJ12 = Rcw[2][0] * dT[1][0] + Rcw[2][1] * dT[1][1] + Rcw[2][2] * dT[1][2];
        const double iz = 1.0 / z, iz2 = iz * iz, iz3 = iz2 * iz;
        const double dmc[3] = {-fx * iz2 * dJ02, -fy * iz2 * dJ12,
                               -fx * iz2 * dJ00 - fy * iz2 * dJ11 + (2 * fx * mc[0]) * iz3 * dJ02 +
                                   (2 * fy * mc[1]) * iz3 * dJ12};
        {
            double w[3];
            q_apply(qcw, dmc, w);
            for (int k = 0; k < 3; ++k) dmu3[k] += w[k];
        }
        for (int k = 0; k < 3; ++k) o[k] = eta_n * dmu3[k];
        double dS3[3][3];
        dS3[0][0] = Tm[0][0] * Tm[0][0] * dSxx + Tm[0][0] * Tm[1][0] * dSxy + Tm[1][0] * Tm[1][0] * dSyy;
        dS3[1][1] = Tm[0][1] * Tm[0][1] * dSxx + Tm[0][1] * Tm[1][1] * dSxy + Tm[1][1] * Tm[1][1] * dSyy;
        dS3[2][2] = Tm[0][2] * Tm[0][2] * dSxx + Tm[0][2] * Tm[1][2] * dSxy + Tm[1][2] * Tm[1][2] * dSyy;
        dS3[1][0] = dS3[0][1] = Tm[0][0] * Tm[0][1] * dSxx +
                                0.5 * (Tm[0][0] * Tm[1][1] + Tm[0][1] * Tm[1][0]) * dSxy + Tm[1][0] * Tm[1][1] * dSyy;
        dS3[2][0] = dS3[0][2] = Tm[0][0] * Tm[0][2] * dSxx +
                                0.5 * (Tm[0][0] * Tm[1][2] + Tm[0][2] * Tm[1][0]) * dSxy + Tm[1][0] * Tm[1][2] * dSyy;
        dS3[2][1] = dS3[1][2] = Tm[0][2] * Tm[0][1] * dSxx +
                                0.5 * (Tm[0][1] * Tm[1][2] + Tm[0][2] * Tm[1][1]) * dSxy + Tm[1][1] * Tm[1][2] * dSyy;
        {
            double TtD[3][3];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) TtD[r][c] = Tm[0][r] * dSp[0][c] + Tm[1][r] * dSp[1][c] + Tm[2][r] * dSp[2][c];
            double add[3][3];
            mm3(TtD, Tm, add);
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c) dS3[r][c] += add[r][c];
        }
        double dM[3][3];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) dM[r][c] = 2.0 * (RS[0][r] * dS3[0][c] + RS[1][r] * dS3[1][c] + RS[2][r] * dS3[2][c]);
        double dLds[3];
        for (int k = 0; k < 3; ++k) dLds[k] = Rg[0][k] * dM[k][0] + Rg[1][k] * dM[k][1] + Rg[2][k] * dM[k][2];
        const double ms = (s[0] + s[1] + s[2]) / 3.0;
        const double dl[3] = {s[0] - ms, s[1] - ms, s[2] - ms};
        const double li = (double)lambda_iso * (1.0 / 3.0);
        dLds[0] -= li * (2 * dl[0] - dl[1] - dl[2]);
        dLds[1] -= li * (-dl[0] + 2 * dl[1] - dl[2]);
        dLds[2] -= li * (-dl[0] - dl[1] + 2 * dl[2]);
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) dM[r][c] *= s[r];
        double th_[3] = {0, 0, 0};
        for (int r = 0; r < 3; ++r) {
            const double* a = Rg[r];
            const double b[3] = {dM[0][r], dM[1][r], dM[2][r]};
            th_[0] += a[1] * b[2] - a[2] * b[1];
            th_[1] += a[2] * b[0] - a[0] * b[2];
            th_[2] += a[0] * b[1] - a[1] * b[0];
        }
        for (int k = 0; k < 3; ++k) {
            o[6 + k] = -eta_n * th_[k];
            o[3 + k] = eta_n * dLds[k];
        }
    }
    return 0;
}

/*
 * updateGaussiansParametersAdam_kernel (src/GSCudaKernels.cu:2779-2882), FP64.
 * params in/out as doubles: pos[3N], scl[3N], rot[4N] (x,y,z,w), col[3N],
 * opa[N]; adam[27N] = AdamStateGaussian3D (GSCudaKernels.cuh:32-45):
 * m_pos, v_pos, m_scale, v_scale, m_rot, v_rot, m_col, v_col (3 each),
 * m_alpha, v_alpha, k.
 */
int oracle_adam(double* pos, double* scl, double* rot, double* col, double* opa, double* adam,
                const double* delta3d, int ng, float eta, const fvgs_params* P) {
    const double b1 = P->adam_beta1, b2 = P->adam_beta2, eps = P->adam_eps;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < ng; ++i) {
        const double* d = delta3d + 14 * (size_t)i;
        if (d[13] == 0.0) continue;
        double* A = adam + 27 * (size_t)i;
        A[26] += 1.0;
        const double a1 = 1.0 - b1, a2 = 1.0 - b2;
        const double b1t = 1.0 / (1.0 - std::pow(b1, A[26]));
        const double b2t = 1.0 / (1.0 - std::pow(b2, A[26]));
        auto step = [&](double& m, double& v, double g) {
            m = a1 * g + b1 * m;
            v = a2 * g * g + b2 * v;
            return (double)eta * (b1t * m) / std::sqrt(b2t * v + eps);
        };
        for (int k = 0; k < 3; ++k) pos[3 * (size_t)i + k] += step(A[k], A[3 + k], d[k]);
        double dq[3];
        for (int k = 0; k < 3; ++k) dq[k] = step(A[12 + k], A[15 + k], d[6 + k]);
        {
            double* q = rot + 4 * (size_t)i;
            const double ax = q[0], ay = q[1], az = q[2], aw = q[3];
            const double bx = 0.5 * dq[0], by = 0.5 * dq[1], bz = 0.5 * dq[2], bw = 1.0;
            double nx = aw * bx + bw * ax + (ay * bz - az * by);
            double ny = aw * by + bw * ay + (az * bx - ax * bz);
            double nz = aw * bz + bw * az + (ax * by - ay * bx);
            double nw = aw * bw - (ax * bx + ay * by + az * bz);
            const double nn = std::sqrt(nx * nx + ny * ny + nz * nz + nw * nw);
            if (nn > 0) {
                nx /= nn; ny /= nn; nz /= nn; nw /= nn;
            }
            q[0] = nx; q[1] = ny; q[2] = nz; q[3] = nw;
        }
        for (int k = 0; k < 3; ++k) scl[3 * (size_t)i + k] += step(A[6 + k], A[9 + k], d[3 + k]);
        for (int k = 0; k < 3; ++k) col[3 * (size_t)i + k] += step(A[18 + k], A[21 + k], d[9 + k]);
        const double da = step(A[24], A[25], d[12]);
        double a = opa[i];
        const double as = std::log(a / (1.0 - a)) + da / (a - a * a);
        a = std::max((double)0.01f, std::min((double)0.99f, 1.0 / (1.0 + std::exp(-as))));
        opa[i] = a;
        for (int k = 0; k < 3; ++k) {
            scl[3 * (size_t)i + k] = std::max((double)0.001f, scl[3 * (size_t)i + k]);
            col[3 * (size_t)i + k] = std::min(1.0, std::max(0.0, col[3 * (size_t)i + k]));
        }
    }
    return 0;
}

/*
 * Render-form forward pass forwardPassTileKernel (src/GSCudaKernels.cu:710-859)
 * in FP64, one pixel at a time over its tile's whole sorted list: the inverse
 * of Sigma2D in its true (xx, xy, yy) layout (the kernel inverts Sigma2D
 * itself, 817, with invert2x2, 1411-1437 -- the FP32 values the projection
 * stores, inv2d (xx, yy, xy)), w = opacity * exp(-0.5 (ixx dx^2 + iyy dy^2 +
 * 2 ixy dx dy)) with d = pixel - mean, colour += (1 - A) w c, A += (1 - A) w,
 * no alpha clamp or 1/255 threshold, stop once A >= 0.99, median depth
 * z + phat . d at the first 0.5 crossing of 1 - A (1e10 if none), no
 * background.  color[3P], depth[P].
 */
int oracle_render_view(const float* uv, const float* inv2d, const float* depth, const float* phat,
                       const float* colors, const float* opac, const uint32_t* ranges, const uint32_t* indices,
                       int W, int H, int tw, int th, double* color, double* out_depth) {
    const int ntx = (W + tw - 1) / tw;
#pragma omp parallel for schedule(dynamic, 16)
    for (int p = 0; p < W * H; ++p) {
        const int x = p % W, y = p / W;
        const int tile = (y / th) * ntx + (x / tw);
        const uint32_t r0 = ranges[2 * (size_t)tile], r1 = ranges[2 * (size_t)tile + 1];
        double c[3] = {0.0, 0.0, 0.0};
        double A = 0.0, d = 1e10;
        bool has_depth = false;
        for (uint32_t k = r0; k < r1; ++k) {
            const uint32_t g = indices[k];
            const double dx = (double)x - uv[2 * (size_t)g], dy = (double)y - uv[2 * (size_t)g + 1];
            const double ixx = inv2d[3 * (size_t)g], iyy = inv2d[3 * (size_t)g + 1], ixy = inv2d[3 * (size_t)g + 2];
            const double w = (double)opac[g] * std::exp(-0.5 * (ixx * dx * dx + iyy * dy * dy + 2.0 * ixy * dx * dy));
            const double Tb = 1.0 - A;
            for (int ch = 0; ch < 3; ++ch) c[ch] += Tb * w * colors[3 * (size_t)g + ch];
            A += Tb * w;
            const double Ta = 1.0 - A;
            if (!has_depth && Tb > 0.5 && Ta <= 0.5) {
                d = (double)depth[g] + (double)phat[2 * (size_t)g] * dx + (double)phat[2 * (size_t)g + 1] * dy;
                has_depth = true;
            }
            if (A >= 0.99) break;
        }
        for (int ch = 0; ch < 3; ++ch) color[3 * (size_t)p + ch] = c[ch];
        out_depth[p] = d;
    }
    return 0;
}

/*
 * Frame preprocessing of GSSlam::initAndCopyImgs (src/GSSlam.cu:1913-1969):
 * one cv::pyrDown step (5-tap binomial [1 4 6 4 1]/16 in each direction,
 * reflect-101 borders, output ((W+1)/2, (H+1)/2)).  8-bit images: integer
 * sums, (sum + 128) >> 8; float images: the same weights in float, rows first
 * then columns, times 1/256.  c channels, dense row-major.
 */
static inline int reflect101(int i, int n) {
    if (n == 1) return 0;
    while (i < 0 || i >= n) i = (i < 0) ? -i : 2 * n - 2 - i;
    return i;
}

int oracle_pyrdown_u8(const uint8_t* src, int W, int H, int c, uint8_t* dst) {
    const int W2 = (W + 1) / 2, H2 = (H + 1) / 2;
    const int wts[5] = {1, 4, 6, 4, 1};
    std::vector<int> row((size_t)H * W2 * c);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W2; ++x)
            for (int ch = 0; ch < c; ++ch) {
                int s = 0;
                for (int k = -2; k <= 2; ++k) s += wts[k + 2] * src[((size_t)y * W + reflect101(2 * x + k, W)) * c + ch];
                row[((size_t)y * W2 + x) * c + ch] = s;
            }
    for (int y = 0; y < H2; ++y)
        for (int x = 0; x < W2; ++x)
            for (int ch = 0; ch < c; ++ch) {
                int s = 0;
                for (int k = -2; k <= 2; ++k) s += wts[k + 2] * row[((size_t)reflect101(2 * y + k, H) * W2 + x) * c + ch];
                dst[((size_t)y * W2 + x) * c + ch] = (uint8_t)((s + 128) >> 8);
            }
    return 0;
}

int oracle_pyrdown_f32(const float* src, int W, int H, int c, float* dst) {
    const int W2 = (W + 1) / 2, H2 = (H + 1) / 2;
    const float wts[5] = {1.f, 4.f, 6.f, 4.f, 1.f};
    std::vector<float> row((size_t)H * W2 * c);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W2; ++x)
            for (int ch = 0; ch < c; ++ch) {
                float s = 0.f;
                for (int k = -2; k <= 2; ++k) s += wts[k + 2] * src[((size_t)y * W + reflect101(2 * x + k, W)) * c + ch];
                row[((size_t)y * W2 + x) * c + ch] = s;
            }
    for (int y = 0; y < H2; ++y)
        for (int x = 0; x < W2; ++x)
            for (int ch = 0; ch < c; ++ch) {
                float s = 0.f;
                for (int k = -2; k <= 2; ++k) s += wts[k + 2] * row[((size_t)reflect101(2 * y + k, H) * W2 + x) * c + ch];
                dst[((size_t)y * W2 + x) * c + ch] = s * (1.0f / 256.0f);
            }
    return 0;
}


/*
 * Map maintenance (src/GSCudaKernels.cu:1455-1739, drivers src/GSSlam.cu:
 * 1467-1904).  rec[12N] are the blending records of oracle_make_records
 * (u, v, z, opacity, c.x, c.y, c.z, phat.x, phat.y, r, g, b), c the inverse
 * 2D covariance in the order the reference's kernels consume the stored
 * inverse.
 *
 * computeGaussiansVisibility_kernel (1455-1537): every pixel inside the image
 * walks the first min(n, cap) Gaussians of its tile list (cap <= 0: all), in
 * order: d = mean - pixel, q = c.x dx^2 + 2 c.y dx dy + c.z dy^2,
 * alpha = min(0.99, opacity exp(-q/2)); alpha < 1/255 skips the Gaussian;
 * otherwise the Gaussian is visible and T *= 1 - alpha; the pixel stops once
 * T < 0.5.  FP64.  vis[i] is set to 1 for visible Gaussians (not cleared).
 */
int oracle_visibility(const float* rec, const uint32_t* ranges, const uint32_t* indices, int n_gauss, int W, int H,
                      int tw, int th, int cap, uint8_t* vis) {
    const int ntx = (W + tw - 1) / tw;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const int tile = (y / th) * ntx + (x / tw);
            const uint32_t r0 = ranges[2 * (size_t)tile], r1 = ranges[2 * (size_t)tile + 1];
            uint32_t n = r1 > r0 ? r1 - r0 : 0;
            if (cap > 0 && n > (uint32_t)cap) n = (uint32_t)cap;
            double T = 1.0;
            for (uint32_t k = 0; k < n; ++k) {
                const uint32_t g = indices[r0 + k];
                if ((int)g >= n_gauss) continue;
                const float* r = rec + 12 * (size_t)g;
                const double dx = (double)r[0] - x, dy = (double)r[1] - y;
                const double q = r[4] * dx * dx + 2.0 * r[5] * dx * dy + r[6] * dy * dy;
                const double alpha = std::min(0.99, (double)r[3] * std::exp(-0.5 * q));
                if (alpha < 1.0 / 255.0) continue;
                vis[g] = 1;
                T *= 1.0 - alpha;
                if (T < 0.5) break;
            }
        }
    return 0;
}

/*
 * computeOutliers_kernel (1620-1715): for every pixel inside the image and
 * every Gaussian of its tile list: d = pixel - mean, rendered depth
 * z + phat . d, q = c.x dx^2 + c.z dy^2 + 2 c.y dx dy (evalGaussian2D,
 * 1401-1409, called with the stored inverse's x, z, y components),
 * alpha = opacity exp(-q/2); alpha < 1/255 or rendered depth <= 0 skips;
 * total_alpha += alpha, and outlier_prob += alpha where the observed depth is
 * > 0.1 and the rendered depth < 0.8 x observed.  No alpha clamp and no
 * early stop.  FP64 arithmetic, with each alpha rounded to FP32 (the
 * reference's float: with the stored-layout inverse the quadratic form can be
 * indefinite, and exp(-q/2) then overflows to inf as in FP32); FP64 sums,
 * accumulated into the outputs (not cleared).
 */
int oracle_outlier_scores(const float* rec, const uint32_t* ranges, const uint32_t* indices, int n_gauss,
                          const float* obs_depth, int W, int H, int tw, int th, double* total_alpha,
                          double* outlier_prob) {
    const int ntx = (W + tw - 1) / tw;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const int tile = (y / th) * ntx + (x / tw);
            const uint32_t r0 = ranges[2 * (size_t)tile], r1 = ranges[2 * (size_t)tile + 1];
            const double d_obs = obs_depth[(size_t)y * W + x];
            for (uint32_t k = r0; k < r1; ++k) {
                const uint32_t g = indices[k];
                if ((int)g >= n_gauss) continue;
                const float* r = rec + 12 * (size_t)g;
                const double dx = x - (double)r[0], dy = y - (double)r[1];
                const double dr = (double)r[2] + (double)r[7] * dx + (double)r[8] * dy;
                const double q = r[4] * dx * dx + r[6] * dy * dy + 2.0 * r[5] * dx * dy;
                const double alpha = (double)(float)((double)r[3] * std::exp(-0.5 * q));
                if (alpha < 1.0 / 255.0 || dr <= 0.0) continue;
                total_alpha[g] += alpha;
                if (d_obs > 0.1 && dr < 0.8 * d_obs) outlier_prob[g] += alpha;
            }
        }
    return 0;
}

/*
 * removeOutliers_kernel (1717-1739) on the FP32 accumulators of the reference
 * (the sums rounded to float): state 0xff where total_alpha > 1 and
 * outlier_prob / total_alpha > threshold in FP32 (an infinite total gives a
 * share of 0 or NaN: kept), else 0.  Returns the number marked.
 */
int oracle_outlier_states(const double* total_alpha, const double* outlier_prob, int n, float threshold,
                          uint8_t* states) {
    int marked = 0;
    for (int i = 0; i < n; ++i) {
        const float ta = (float)total_alpha[i], op = (float)outlier_prob[i];
        const bool rm = ta > 1.0f && op / ta > threshold;
        states[i] = rm ? 0xff : 0;
        marked += rm;
    }
    return marked;
}

/*
 * pruneGaussians_kernel (1566-1618), in FP32 as the reference: state 0xff
 * where opacity < alpha_threshold, else where (s_x + s_y + s_z - s_max -
 * s_min) / s_max < scale_ratio_threshold or s_max < min_scale.  Returns the
 * number marked.
 */
int oracle_prune_states(const float* scales, const float* opac, int n, float alpha_threshold,
                        float scale_ratio_threshold, float min_scale, uint8_t* states) {
    int marked = 0;
    for (int i = 0; i < n; ++i) {
        bool rm;
        if (opac[i] < alpha_threshold) {
            rm = true;
        } else {
            const float sx = scales[3 * (size_t)i], sy = scales[3 * (size_t)i + 1], sz = scales[3 * (size_t)i + 2];
            const float smax = std::fmax(sx, std::fmax(sy, sz));
            const float smin = std::fmin(sx, std::fmin(sy, sz));
            const float smed = sx + sy + sz - smax - smin;
            rm = smed / smax < scale_ratio_threshold || smax < min_scale;
        }
        states[i] = rm ? 0xff : 0;
        marked += rm;
    }
    return marked;
}


/*
 * Seeding Gaussians from an RGB-D frame: GSSlam::initializeGaussiansFromRgbd
 * (src/GSSlam.cu:271-407) with computeNormalsFromDepth_kernel and
 * initGaussiansFromRgbd_kernel (src/GSCudaKernels.cu:87-315), and
 * GSSlam::densify (src/GSSlam.cu:1351-1465) with computeDensityMask_kernel and
 * densifyGaussians_kernel (src/GSCudaKernels.cu:1741-2066).
 *
 * FP32 in the reference's operation order (-ffp-contract=off): every product,
 * sum, quotient and square root rounded once, as the CUDA kernels do with
 * explicit intrinsics, so the seeds are bit-identical.  The quaternion helpers
 * of src/GSCudaKernels.cu:20-84 read and write float4 as (w, x, y, z): the
 * camera orientation is taken raw in that order and the seeds' orientations
 * are written in it.  The colour image is 8-bit, 3 bytes per pixel in the
 * reference's (b, g, r) order.  The reference hands out seed slots with an
 * atomic counter (unspecified order); here seeds are written in row-major
 * order of their sample cell, the first ones up to the capacity.
 */
struct V3 {
    float x, y, z;
};
static V3 v3_cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static float v3_norm(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
// rotateByQuaternion: q = (w, x, y, z) raw, t = 2 (qv x v), v + w t + qv x t
static V3 quat_rotate(const float* q, V3 v) {
    const V3 qv = {q[1], q[2], q[3]};
    const V3 c = v3_cross(qv, v);
    const V3 t = {2.0f * c.x, 2.0f * c.y, 2.0f * c.z};
    const V3 c2 = v3_cross(qv, t);
    return {v.x + q[0] * t.x + c2.x, v.y + q[0] * t.y + c2.y, v.z + q[0] * t.z + c2.z};
}
static void quat_mul(const float* a, const float* b, float* out) {
    const float aw = a[0], ax = a[1], ay = a[2], az = a[3];
    const float bw = b[0], bx = b[1], by = b[2], bz = b[3];
    out[0] = aw * bw - ax * bx - ay * by - az * bz;
    out[1] = aw * bx + ax * bw + ay * bz - az * by;
    out[2] = aw * by - ax * bz + ay * bw + az * bx;
    out[3] = aw * bz + ax * by - ay * bx + az * bw;
}
static V3 v3_normalize8(V3 v) {
    const float n = v3_norm(v);
    if (n > 1e-8f) {
        const float inv = 1.0f / n;
        return {v.x * inv, v.y * inv, v.z * inv};
    }
    return {0.0f, 0.0f, 0.0f};
}
static void quat_from_two(V3 from, V3 to, float* q) {
    const V3 u = v3_normalize8(from), v = v3_normalize8(to);
    const float dot = u.x * v.x + u.y * v.y + u.z * v.z;
    if (dot < -0.999999f) {
        const V3 axis = (std::fabs(u.x) < 0.1f) ? V3{1.0f, 0.0f, 0.0f} : V3{0.0f, 1.0f, 0.0f};
        const V3 o = v3_normalize8(v3_cross(u, axis));
        q[0] = 0.0f, q[1] = o.x, q[2] = o.y, q[3] = o.z;
        return;
    }
    const V3 c = v3_cross(u, v);
    float r[4] = {1.0f + dot, c.x, c.y, c.z};
    const float n = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3]);
    if (n > 1e-8f) {
        const float inv = 1.0f / n;
        for (int k = 0; k < 4; ++k) r[k] *= inv;
    } else {
        r[0] = 1.0f, r[1] = r[2] = r[3] = 0.0f;
    }
    for (int k = 0; k < 4; ++k) q[k] = r[k];
}
// computeNormalsFromDepth_kernel for pixel (u, v)
static V3 depth_normal(const float* depth, int W, int H, int u, int v) {
    V3 n = {0.0f, 0.0f, 1.0f};
    if (u > 0 && u < W - 1 && v > 0 && v < H - 1) {
        const float zc = depth[(size_t)v * W + u], zl = depth[(size_t)v * W + u - 1], zr = depth[(size_t)v * W + u + 1];
        const float zu = depth[(size_t)(v - 1) * W + u], zd = depth[(size_t)(v + 1) * W + u];
        if (zc > 0.01f && zl > 0.01f && zr > 0.01f && zu > 0.01f && zd > 0.01f) {
            const float dzx = (zr - zl) / 2.0f, dzy = (zd - zu) / 2.0f;
            n = v3_cross(V3{1.0f, 0.0f, dzx}, V3{0.0f, 1.0f, dzy});
            const float nn = v3_norm(n);
            if (nn > 1e-6f) n = {n.x / nn, n.y / nn, n.z / nn};
            if (n.z < 0.0f) n = {-n.x, -n.y, -n.z};
        }
    }
    return n;
}

/*
 * mode 0 (init): one seed per sample pixel (sx * sample, sy * sample) with
 * depth z > 0 (finite): position t + R (((u - cx) z / fx, (v - cy) z / fy, z)),
 * scale init_scale, orientation turning +z onto the normal (camera normal
 * from the depth map, rotated to the world), colour (r, g, b) / 255, opacity
 * init_opacity.
 * mode 1 (densify): with sample > 1, one seed per sample cell holding at
 * least sample^2 / 2 pixels with mask > 0 and depth > 0 (mean pixel, depth
 * and colour; scale (s, s, 0.1 s), s = z sample / f; orientation the camera
 * orientation; opacity 1); with sample = 1, one seed per such pixel (s with a
 * factor 0.8).  mask: W x H floats.
 * Writes at most max_out seeds; returns how many were written.
 */
int oracle_seed(int mode, const uint8_t* bgr, const float* depth, const float* mask, int W, int H, int sample,
                const fvgs_intrinsics* K, const float* pose_t, const float* pose_q, float init_scale,
                float init_opacity, int max_out, float* pos, float* scl, float* rot, float* col, float* opa) {
    const int sw = (W + sample - 1) / sample, sh = (H + sample - 1) / sample;
    const float fx = K->fx, fy = K->fy, cx = K->cx, cy = K->cy;
    int count = 0;
    auto emit = [&](V3 pw, V3 sc, const float* q, V3 c, float o) {
        if (count >= max_out) return;
        const size_t i = (size_t)count++;
        pos[3 * i] = pw.x, pos[3 * i + 1] = pw.y, pos[3 * i + 2] = pw.z;
        scl[3 * i] = sc.x, scl[3 * i + 1] = sc.y, scl[3 * i + 2] = sc.z;
        for (int k = 0; k < 4; ++k) rot[4 * i + k] = q[k];
        col[3 * i] = c.x, col[3 * i + 1] = c.y, col[3 * i + 2] = c.z;
        opa[i] = o;
    };
    auto to_world = [&](V3 pc) {
        const V3 r = quat_rotate(pose_q, pc);
        return V3{pose_t[0] + r.x, pose_t[1] + r.y, pose_t[2] + r.z};
    };
    auto rgb_at = [&](int u, int v) {
        const uint8_t* p = bgr + ((size_t)v * W + u) * 3;
        return V3{(float)p[2] / 255.0f, (float)p[1] / 255.0f, (float)p[0] / 255.0f};
    };
    const V3 zaxis = {0.0f, 0.0f, 1.0f};
    if (mode == 0) {
        for (int sy = 0; sy < sh; ++sy)
            for (int sx = 0; sx < sw; ++sx) {
                const int u = sx * sample, v = sy * sample;
                const float z = depth[(size_t)v * W + u];
                if (!(z > 0.0f) || std::isinf(z) || std::isnan(z)) continue;
                V3 n = depth_normal(depth, W, H, u, v);
                const float nl = v3_norm(n);
                if (nl < 1e-6f) n = zaxis;
                else n = {n.x / nl, n.y / nl, n.z / nl};
                const V3 pc = {((float)u - cx) * z / fx, ((float)v - cy) * z / fy, z};
                V3 nw = quat_rotate(pose_q, n);
                const float nwl = v3_norm(nw);
                if (nwl > 1e-6f) nw = {nw.x / nwl, nw.y / nwl, nw.z / nwl};
                const V3 axis0 = v3_cross(zaxis, nw);
                const float al = v3_norm(axis0);
                const float ac = zaxis.x * nw.x + zaxis.y * nw.y + zaxis.z * nw.z;
                float q[4];
                if (al < 1e-6f) {
                    if (ac > 0.0f) q[0] = 1.0f, q[1] = 0.0f, q[2] = 0.0f, q[3] = 0.0f;
                    else q[0] = 0.0f, q[1] = 1.0f, q[2] = 0.0f, q[3] = 0.0f;
                } else {
                    const V3 ax = {axis0.x / al, axis0.y / al, axis0.z / al};
                    const float hs = std::sqrt(std::fmax(0.0f, (1.0f - ac) / 2.0f));
                    const float hc = std::sqrt(std::fmax(0.0f, (1.0f + ac) / 2.0f));
                    q[0] = hc, q[1] = hs * ax.x, q[2] = hs * ax.y, q[3] = hs * ax.z;
                }
                emit(to_world(pc), V3{init_scale, init_scale, init_scale}, q, rgb_at(u, v), init_opacity);
            }
        return count;
    }
    float q_cam[4];
    quat_from_two(zaxis, zaxis, q_cam);  // normal (0, 0, 1): the reference passes no normal map
    float q[4];
    quat_mul(pose_q, q_cam, q);
    if (sample > 1) {
        for (int sy = 0; sy < sh; ++sy)
            for (int sx = 0; sx < sw; ++sx) {
                const int u0 = sx * sample, v0 = sy * sample;
                V3 ip = {0.0f, 0.0f, 0.0f}, ca = {0.0f, 0.0f, 0.0f};
                int n = 0;
                for (int u = u0; u < u0 + sample && u < W; ++u)
                    for (int v = v0; v < v0 + sample && v < H; ++v) {
                        if (!(mask[(size_t)v * W + u] > 0.0f)) continue;
                        const float d = depth[(size_t)v * W + u];
                        if (!(d > 0.0f)) continue;
                        const V3 c = rgb_at(u, v);
                        ip = {ip.x + (float)u, ip.y + (float)v, ip.z + d};
                        ca = {ca.x + c.x, ca.y + c.y, ca.z + c.z};
                        ++n;
                    }
                if ((uint32_t)n < (((uint32_t)sample * (uint32_t)sample) >> 1)) continue;
                const float inv_n = 1.0f / (float)n;
                ip = {ip.x * inv_n, ip.y * inv_n, ip.z * inv_n};
                ca = {ca.x * inv_n, ca.y * inv_n, ca.z * inv_n};
                const V3 pc = {ip.z * (ip.x - cx) / fx, ip.z * (ip.y - cy) / fy, ip.z};
                const float sx_ = ip.z * (float)sample / fx, sy_ = ip.z * (float)sample / fy;
                const float s2 = 0.5f * (sx_ + sy_);
                emit(to_world(pc), V3{s2, s2, 0.1f * s2}, q, ca, 1.0f);
            }
        return count;
    }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            if (!(mask[(size_t)y * W + x] > 0.0f)) continue;
            const float d = depth[(size_t)y * W + x];
            if (!(d > 0.0f)) continue;
            const V3 pc = {d * ((float)x - cx) / fx, d * ((float)y - cy) / fy, d};
            const float sx_ = 0.8f * d * (float)sample / fx, sy_ = 0.8f * d * (float)sample / fy;
            const float s2 = 0.5f * (sx_ + sy_);
            emit(to_world(pc), V3{s2, s2, 0.1f * s2}, q, rgb_at(x, y), 1.0f);
        }
    return count;
}

/*
 * computeDensityMask_kernel (src/GSCudaKernels.cu:1741-1857) over a binned
 * view, FP64: every pixel with observed depth >= 0.5 walks its tile list
 * (d = mean - pixel, q = c.x dx^2 + 2 c.y dx dy + c.z dy^2, alpha =
 * min(0.99, opacity exp(-q/2)), alpha < 1/255 skipped, P *= 1 - alpha, the
 * depth z + phat . d where P first falls below 0.5, stop once P < 1e-4).
 * mask = P where depth > 0.5 and P > 0.5; 1 where depth > 0.5, P <= 0.5 and
 * the rendered depth exceeds the observed one by more than 0.2 x observed;
 * else 0.
 */
int oracle_density_mask(const float* rec, const uint32_t* ranges, const uint32_t* indices, int n_gauss,
                        const float* obs_depth, int W, int H, int tw, int th, double* mask) {
    const int ntx = (W + tw - 1) / tw;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const int tile = (y / th) * ntx + (x / tw);
            const uint32_t r0 = ranges[2 * (size_t)tile], r1 = ranges[2 * (size_t)tile + 1];
            const double d_obs = obs_depth[(size_t)y * W + x];
            double P = 1.0, T = 1.0, dr = 0.0;
            if (!(d_obs < 0.5)) {
                for (uint32_t k = r0; k < r1; ++k) {
                    const uint32_t g = indices[k];
                    if ((int)g >= n_gauss) continue;
                    const float* r = rec + 12 * (size_t)g;
                    const double dx = (double)r[0] - x, dy = (double)r[1] - y;
                    const double q = r[4] * dx * dx + 2.0 * r[5] * dx * dy + r[6] * dy * dy;
                    const double alpha = std::min(0.99, (double)r[3] * std::exp(-0.5 * q));
                    if (alpha < 1.0 / 255.0) continue;
                    P *= 1.0 - alpha;
                    if (T > 0.5 && P < 0.5) {
                        T = P;
                        dr = (double)r[2] + (double)r[7] * dx + (double)r[8] * dy;
                    }
                    if (P < 0.0001) break;
                }
            }
            double val = 0.0;
            if (d_obs > 0.5) {
                if (P > 0.5) val = P;
                else if (d_obs < dr && dr - d_obs > 0.2 * d_obs) val = 1.0;
            }
            mask[(size_t)y * W + x] = val;
        }
    return 0;
}

}  // extern "C"
