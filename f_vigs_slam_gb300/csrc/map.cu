// map.cu -- mapping step (forward with checkpoints, per-Gaussian backward,
// 2D->3D chain rule and Adam) for sm_103a.
//
// Reference: GSSlam::optimizeGaussiansKeyframe (src/GSSlam.cu:1083-1320) with
// perTileBucketCount (src/GSCudaKernels.cu:2074-2090),
// optimizeGaussiansForwardPass (2092-2263), optimizeGaussiansPerGaussianPass
// (2265-2502), computeDeltaGaussians3D_kernel (2504-2720) and
// updateGaussiansParametersAdam_kernel (2722-2882).
//
// GPU structure:
//  * forward: one CTA per 16x16 tile, Gaussian records staged in shared memory;
//    checkpoints (T, accumulated colour) as one float4 per (bucket, pixel).
//    With MAP_CAP256 only buckets 0..7 can receive gradients, so only those are
//    checkpointed (tile*8 + b), and no bucket scan is needed.
//  * backward: one CTA per tile; the tile's per-pixel forward results are
//    staged once in shared memory and every warp runs the reference's
//    lane-per-Gaussian pipeline over the 256 pixels, shuffling only the
//    evolving state (T and the accumulated colour: 4 values, not 13);
//  * 2D->3D and Adam are fused: the 3D deltas never go to memory.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

constexpr int kMPix = 256;
constexpr int kMBatch = 256;
constexpr int kCapBuckets = 8;
constexpr float kMInv255 = 1.0f / 255.0f;

template <bool CAP>
__global__ void __launch_bounds__(kMPix) map_forward_kernel(MapArgs a) {
    pdl_begin();
    __shared__ float4 s0[kMBatch];
    __shared__ float4 s1[kMBatch];
    __shared__ float4 s2[kMBatch];
    __shared__ uint32_t s_max;
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int tid = threadIdx.x;
    const int x = tx * 16 + (tid & 15), y = ty * 16 + (tid >> 4);
    const bool inside = (x < a.W && y < a.H);
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    const int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    const uint32_t base_slot = CAP ? (uint32_t)tile * kCapBuckets : a.bucket_base[tile];
    const float xf = (float)x, yf = (float)y;
    if (tid == 0) s_max = 0;
    float T = 1.f, cr = 0.f, cg = 0.f, cb = 0.f, depth = 0.f;
    uint32_t contributor = 0, last = 0;
    bool done = !inside;
    for (int base = 0; base < n; base += kMBatch) {
        if (__syncthreads_and(done)) break;
        const int li = base + tid;
        if (li < n) {
            const uint32_t g = a.indices[range.x + li];
            const bool ok = g < a.n_gauss;  // zero opacity otherwise: never blends
            float4 r0 = ok ? a.rec0[g] : make_float4(0.f, 0.f, 0.f, 0.f);
            r0.w = log2_opacity(r0.w);  // staged as log2(opacity) for gauss_alpha
            s0[tid] = r0;
            s1[tid] = ok ? a.rec1[g] : make_float4(0.f, 0.f, 0.f, 0.f);
            s2[tid] = ok ? a.rec2[g] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        if (!done) {
            const int cnt = min(kMBatch, n - base);
            for (int j = 0; j < cnt; ++j) {
                const int gi = base + j;
                if ((gi & 31) == 0 && (!CAP || gi < 32 * kCapBuckets))
                    a.sampled[(size_t)(base_slot + gi / 32) * kMPix + tid] = make_float4(T, cr, cg, cb);
                ++contributor;
                const float4 r0 = s0[j];
                const float4 r1 = s1[j];
                const float dx = xf - r0.x, dy = yf - r0.y;
                float dl0, dl1;
                const float v = conic_form(r1.x, r1.y, r1.z, dx, dy, dl0, dl1);
                const float alpha = gauss_alpha(r0.w, v);
                if (alpha < kMInv255 || v <= 0.0f) continue;
                const float4 r2 = s2[j];
                cr += T * alpha * r2.y;
                cg += T * alpha * r2.z;
                cb += T * alpha * r2.w;
                const float test_T = T * (1.0f - alpha);
                if (T > 0.5f && test_T <= 0.5f) depth = r0.z + r1.w * dx + r2.x * dy;
                T = test_T;
                last = contributor;
                if (test_T < 0.0001f) {
                    done = true;
                    break;
                }
            }
        }
    }
    if (inside) {
        const size_t p = (size_t)y * a.W + x;
        a.final_T[p] = T;
        a.n_contrib[p] = last;
        cr += T * a.bg[0];
        cg += T * a.bg[1];
        cb += T * a.bg[2];
        a.color[3 * p] = cr;
        a.color[3 * p + 1] = cg;
        a.color[3 * p + 2] = cb;
        a.depth[p] = depth;
        a.color_err[3 * p] = cr - a.obs_rgb[3 * p];
        a.color_err[3 * p + 1] = cg - a.obs_rgb[3 * p + 1];
        a.color_err[3 * p + 2] = cb - a.obs_rgb[3 * p + 2];
    }
    __syncthreads();
    if (last) atomicMax(&s_max, last);
    __syncthreads();
    if (tid == 0) a.max_contrib[tile] = s_max;
}

template <bool CAP>
__global__ void __launch_bounds__(kMPix, 4) map_backward_kernel(MapArgs a) {
    pdl_begin();
    __shared__ float4 s_pc[kMPix];  // final colour (incl. background), median depth
    __shared__ float4 s_pe[kMPix];  // colour error, observed depth
    __shared__ uint32_t s_nc[kMPix];
    __shared__ uint16_t s_act[kMPix / 32][kMPix];  // per warp: the pixels its bucket can reach
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    const uint32_t n = range.y > range.x ? range.y - range.x : 0u;
    const uint32_t maxc = a.max_contrib[tile];
    uint32_t nb = (n + 31) / 32;
    if (CAP) nb = min(nb, (uint32_t)kCapBuckets);
    if (nb == 0 || maxc == 0) return;
    {
        const int px = tx * 16 + (tid & 15), py = ty * 16 + (tid >> 4);
        if (px < a.W && py < a.H) {
            const size_t p = (size_t)py * a.W + px;
            s_pc[tid] = make_float4(a.color[3 * p], a.color[3 * p + 1], a.color[3 * p + 2], a.depth[p]);
            s_pe[tid] = make_float4(a.color_err[3 * p], a.color_err[3 * p + 1], a.color_err[3 * p + 2],
                                    a.obs_depth[p]);
            s_nc[tid] = a.n_contrib[p];
        } else {
            s_nc[tid] = 0;  // out-of-image pixels are never processed
        }
    }
    __syncthreads();
    const uint32_t base_slot = CAP ? (uint32_t)tile * kCapBuckets : a.bucket_base[tile];
    const float w_depth = a.w_depth, w_dist = a.w_dist;
    for (uint32_t b = warp; b < nb; b += kMPix / 32) {
        if (b * 32 >= maxc) break;
        const uint32_t j = b * 32 + lane;
        bool valid_splat = j < n && (!CAP || j < 32u * kCapBuckets);
        float4 r0 = make_float4(0, 0, 0, 0), r1 = r0, r2 = r0;
        uint32_t gid = 0;
        if (valid_splat) {
            gid = a.indices[range.x + j];
            valid_splat = gid < a.n_gauss;
        }
        if (valid_splat) {
            r0 = a.rec0[gid];
            r1 = a.rec1[gid];
            r2 = a.rec2[gid];
        }
        const float lo2 = log2_opacity(r0.w);  // the forward pass's alpha from log2(opacity)
        float dmx = 0.f, dmy = 0.f, dix = 0.f, diy = 0.f, diz = 0.f, dcr = 0.f, dcg = 0.f, dcb = 0.f;
        float dz = 0.f, dal = 0.f, dpx = 0.f, dpy = 0.f;
        uint32_t dn = 0;
        float T = 0.f, a0 = 0.f, a1 = 0.f, a2 = 0.f;
        const float4* samp = a.sampled + (size_t)(base_slot + b) * kMPix;
        // Only pixels whose contributor count exceeds the bucket's first list
        // position can receive anything from it; the pipeline walks those, in
        // pixel order (each starts from its own checkpoint, so skipping the
        // others changes no sum).
        int n_act = 0;
        for (int c = 0; c < kMPix; c += 32) {
            const bool act = s_nc[c + lane] > b * 32;
            const unsigned m = __ballot_sync(kFullMask, act);
            if (act) s_act[warp][n_act + __popc(m & lanemask_lt())] = (uint16_t)(c + lane);
            n_act += __popc(m);
        }
        __syncwarp();
        for (int i = 0; i < n_act + 31; ++i) {
            T = __shfl_up_sync(kFullMask, T, 1);
            a0 = __shfl_up_sync(kFullMask, a0, 1);
            a1 = __shfl_up_sync(kFullMask, a1, 1);
            a2 = __shfl_up_sync(kFullMask, a2, 1);
            const int pos = i - lane;
            if (!valid_splat || pos < 0 || pos >= n_act) continue;
            const int idx = s_act[warp][pos];
            const uint32_t nc = s_nc[idx];
            if (lane == 0 && nc != 0) {
                const float4 sv = samp[idx];
                T = sv.x;
                a0 = sv.y;
                a1 = sv.z;
                a2 = sv.w;
            }
            if (j >= nc) continue;
            const float pxf = (float)(tx * 16 + (idx & 15)), pyf = (float)(ty * 16 + (idx >> 4));
            const float dx = r0.x - pxf, dy = r0.y - pyf;
            float dl0, dl1;  // the forward pass's conic form ((dx, dy) negated: same value)
            const float v = conic_form(r1.x, r1.y, r1.z, dx, dy, dl0, dl1);
            const float alpha = gauss_alpha(lo2, v);
            if (alpha < kMInv255) continue;
            const float4 pc = s_pc[idx];
            const float4 pe = s_pe[idx];
            float d0 = r2.y * T, d1 = r2.z * T, d2 = r2.w * T;
            a0 += d0 * alpha;
            a1 += d1 * alpha;
            a2 += d2 * alpha;
            const float inv1m = rcp_approx(1.0f - alpha);
            d0 = (d0 - (pc.x - a0) * inv1m) * -pe.x;
            d1 = (d1 - (pc.y - a1) * inv1m) * -pe.y;
            d2 = (d2 - (pc.z - a2) * inv1m) * -pe.z;
            const float aG = alpha * (d0 + d1 + d2);
            ++dn;
            const float aT = alpha * T;
            dcr -= aT * pe.x;
            dcg -= aT * pe.y;
            dcb -= aT * pe.z;
            dal -= aG;
            dmx -= aG * dl0;
            dmy -= aG * dl1;
            const float haG = 0.5f * aG;
            dix -= haG * dx * dx;
            diy -= haG * dx * dy;
            diz -= haG * dy * dy;
            const float test_T = T * (1.0f - alpha);
            const float phx = r1.w, phy = r2.x;
            if (T > 0.5f && test_T <= 0.5f) {
                const float derr = (pe.w > 0.1f) ? (pc.w - pe.w) : 0.0f;
                const float wde = w_depth * derr;
                dz -= wde;
                dmx -= wde * phx;
                dmy -= wde * phy;
                dpx -= wde * dx;
                dpy -= wde * dy;
            }
            const float di = r0.z + dx * phx + dy * phy;
            const float dc = w_dist * alpha * T * (di - pc.w);
            dz -= dc;
            dmx -= dc * phx;
            dmy -= dc * phy;
            dpx -= dc * dx;
            dpy -= dc * dy;
            T = test_T;
        }
        if (valid_splat && dn > 0) {
            float* D = a.delta2d + (size_t)gid * 16;
            atomicAdd(D + 0, dmx);
            atomicAdd(D + 1, dmy);
            atomicAdd(D + 2, dix);
            atomicAdd(D + 3, diy);
            atomicAdd(D + 4, diz);
            atomicAdd(D + 5, dcr);
            atomicAdd(D + 6, dcg);
            atomicAdd(D + 7, dcb);
            atomicAdd(D + 8, dz);
            atomicAdd(D + 9, dal);
            atomicAdd(D + 10, dpx);
            atomicAdd(D + 11, dpy);
            atomicAdd(reinterpret_cast<uint32_t*>(D + 12), dn);
        }
    }
}

// ----------------------- 2D -> 3D chain rule + Adam ------------------------
struct Q4 {
    float x, y, z, w;
};
// Eigen's quaternion-vector product: uv = 2 vec x v; v + w uv + vec x uv.
__device__ __forceinline__ float3 qapply(const Q4& q, float3 v) {
    float3 uv = make_float3(q.y * v.z - q.z * v.y, q.z * v.x - q.x * v.z, q.x * v.y - q.y * v.x);
    uv.x += uv.x;
    uv.y += uv.y;
    uv.z += uv.z;
    const float3 c = make_float3(q.y * uv.z - q.z * uv.y, q.z * uv.x - q.x * uv.z, q.x * uv.y - q.y * uv.x);
    return make_float3(v.x + q.w * uv.x + c.x, v.y + q.w * uv.y + c.y, v.z + q.w * uv.z + c.z);
}
__device__ __forceinline__ void qmat(const Q4& q, float R[3][3]) {
    const float tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
    const float twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const float txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const float tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    R[0][0] = 1 - (tyy + tzz); R[0][1] = txy - twz; R[0][2] = txz + twy;
    R[1][0] = txy + twz; R[1][1] = 1 - (txx + tzz); R[1][2] = tyz - twx;
    R[2][0] = txz - twy; R[2][1] = tyz + twx; R[2][2] = 1 - (txx + tyy);
}
__device__ __forceinline__ void mm3(const float A[3][3], const float B[3][3], float C[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}

__device__ __forceinline__ float adam_step(float& m, float& v, float g, float eta, float a1, float b1, float b1t,
                                           float a2, float b2, float b2t, float eps) {
    m = a1 * g + b1 * m;
    v = a2 * g * g + b2 * v;
    return eta * (b1t * m) * rsqrtf(b2t * v + eps);
}

__global__ void __launch_bounds__(256) map_update_kernel(MapUpdateArgs a, const DevStatus* st) {
    pdl_begin();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < a.n_cst && a.cst) a.cst[i].valid = 0;
    if (i >= a.n) return;
    // An instance overflow leaves the binning incomplete; the host re-runs the
    // step with larger buffers, so the parameters must stay untouched.
    if (st->flags & kErrOverflow) return;
    const float4* D4 = reinterpret_cast<const float4*>(a.delta2d + (size_t)i * 16);
    // the contributor count first: most of a large map has no gradient, and
    // then only this one sector of the record is read
    const float4 q3 = D4[3];
    const uint32_t nn = __float_as_uint(q3.x);
    if (nn == 0) {
        if (a.dbg_delta3d)
            for (int k = 0; k < 16; ++k) a.dbg_delta3d[(size_t)i * 16 + k] = 0.f;
        return;
    }
    const float4 q0 = D4[0], q1 = D4[1], q2 = D4[2];
    const float d_mean[2] = {q0.x, q0.y};
    const float d_inv[3] = {q0.z, q0.w, q1.x};
    const float d_col[3] = {q1.y, q1.z, q1.w};
    const float d_depth = q2.x, d_alpha = q2.y;
    const float d_ph[2] = {q2.z, q2.w};
    const float eta_n = 1.0f / (5.0f + (float)nn);
    const float fx = a.K.fx, fy = a.K.fy;
    const DevPose* P = a.pose;
    const Q4 qcw{P->q[0], P->q[1], P->q[2], P->q[3]};
    const float n2q = qcw.x * qcw.x + qcw.y * qcw.y + qcw.z * qcw.z + qcw.w * qcw.w;
    const Q4 qinv = (n2q > 0.f) ? Q4{-qcw.x / n2q, -qcw.y / n2q, -qcw.z / n2q, qcw.w / n2q} : Q4{0, 0, 0, 0};
    float Rcw[3][3];
    qmat(qinv, Rcw);
    const float4 pw = a.pos[i];
    const float4 sw = a.scale[i];
    const float4 rw = a.rot[i];
    float4 cw = a.col[i];
    const float3 mc = qapply(qinv, make_float3(pw.x - P->t[0], pw.y - P->t[1], pw.z - P->t[2]));
    const float z = mc.z;
    const float J[3][3] = {{fx / z, 0.f, -fx * mc.x / (z * z)}, {0.f, fy / z, -fy * mc.y / (z * z)}, {0.f, 0.f, 1.f}};
    const Q4 qg{rw.x, rw.y, rw.z, rw.w};
    float Rg[3][3];
    qmat(qg, Rg);
    const float s[3] = {sw.x, sw.y, sw.z};
    float Tm[3][3], RS[3][3], M[3][3], Sp[3][3];
    mm3(J, Rcw, Tm);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) RS[r][c] = Rg[r][c] * s[c];
    mm3(Tm, RS, M);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Sp[r][c] = M[r][0] * M[c][0] + M[r][1] * M[c][1] + M[r][2] * M[c][2];
    // 3x3 inverse by cofactors
    float Spi[3][3];
    {
        const float c00 = Sp[1][1] * Sp[2][2] - Sp[1][2] * Sp[2][1];
        const float c01 = Sp[1][2] * Sp[2][0] - Sp[1][0] * Sp[2][2];
        const float c02 = Sp[1][0] * Sp[2][1] - Sp[1][1] * Sp[2][0];
        const float id = 1.0f / (Sp[0][0] * c00 + Sp[0][1] * c01 + Sp[0][2] * c02);
        Spi[0][0] = c00 * id;
        Spi[1][0] = c01 * id;
        Spi[2][0] = c02 * id;
        Spi[0][1] = (Sp[0][2] * Sp[2][1] - Sp[0][1] * Sp[2][2]) * id;
        Spi[1][1] = (Sp[0][0] * Sp[2][2] - Sp[0][2] * Sp[2][0]) * id;
        Spi[2][1] = (Sp[0][1] * Sp[2][0] - Sp[0][0] * Sp[2][1]) * id;
        Spi[0][2] = (Sp[0][1] * Sp[1][2] - Sp[0][2] * Sp[1][1]) * id;
        Spi[1][2] = (Sp[0][2] * Sp[1][0] - Sp[0][0] * Sp[1][2]) * id;
        Spi[2][2] = (Sp[0][0] * Sp[1][1] - Sp[0][1] * Sp[1][0]) * id;
    }
    float3 tmp;
    tmp.x = J[0][0] * d_mean[0] + J[1][0] * d_mean[1] + d_depth * (mc.x / z);
    tmp.y = J[0][1] * d_mean[0] + J[1][1] * d_mean[1] + d_depth * (mc.y / z);
    tmp.z = J[0][2] * d_mean[0] + J[1][2] * d_mean[1] + d_depth;
    float3 dmu3 = qapply(qcw, tmp);
    const float n2 = mc.x * mc.x + mc.y * mc.y + mc.z * mc.z;
    const float nm = sqrtf(n2);
    const float in3 = 1.0f / (n2 * nm);
    {
        const float fac = (Spi[2][0] * d_ph[0] + Spi[2][1] * d_ph[1]) / Spi[2][2];
        const float3 w = qapply(qcw, make_float3(-mc.x * mc.z * in3 * fac, -mc.y * mc.z * in3 * fac,
                                                 (mc.x * mc.x + mc.y * mc.y) * in3 * fac));
        dmu3.x += w.x;
        dmu3.y += w.y;
        dmu3.z += w.z;
    }
    const float sxx = Sp[0][0] + 0.001f, sxy = Sp[1][0], syy = Sp[1][1] + 0.001f;
    const float den = sxx * syy - sxy * sxy;
    const float d2i = 1.0f / ((den * den) + 0.0000001f);
    const float dSxx = d2i * (-syy * syy * d_inv[0] + 2 * sxy * syy * d_inv[1] + (den - sxx * syy) * d_inv[2]);
    const float dSyy = d2i * (-sxx * sxx * d_inv[2] + 2 * sxx * sxy * d_inv[1] + (den - sxx * syy) * d_inv[0]);
    const float dSxy = d2i * 2 * (sxy * syy * d_inv[0] - (den + 2 * sxy * sxy) * d_inv[1] + sxx * sxy * d_inv[2]);
    float S3[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) S3[r][c] = RS[r][0] * RS[c][0] + RS[r][1] * RS[c][1] + RS[r][2] * RS[c][2];
    float dT[2][3];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        const float t0 = Tm[0][0] * S3[jj][0] + Tm[0][1] * S3[jj][1] + Tm[0][2] * S3[jj][2];
        const float t1 = Tm[1][0] * S3[jj][0] + Tm[1][1] * S3[jj][1] + Tm[1][2] * S3[jj][2];
        dT[0][jj] = 2 * t0 * dSxx + t1 * dSxy;
        dT[1][jj] = 2 * t1 * dSyy + t0 * dSxy;
    }
    const float zt = z / nm;
    const float av = 0.5f * zt * d_ph[0] / Spi[2][2];
    const float bv = 0.5f * zt * d_ph[1] / Spi[2][2];
    const float cv = -zt * (d_ph[0] * Spi[2][0] + d_ph[1] * Spi[2][1]) / (Spi[2][2] * Spi[2][2]);
    const float dLSi[3][3] = {{0.f, 0.f, av}, {0.f, 0.f, bv}, {av, bv, cv}};
    float t1m[3][3], dSp[3][3];
    mm3(Spi, dLSi, t1m);
    mm3(t1m, Spi, dSp);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) dSp[r][c] = -dSp[r][c];
    float TS[3][3];
    mm3(Tm, S3, TS);
#pragma unroll
    for (int aa = 0; aa < 2; ++aa)
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
            float s1 = 0.f, s2 = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                s1 += TS[k][jj] * dSp[k][aa];
                // (S3 T^T)[jj][k] = S3 row jj . T row k
                s2 += (S3[jj][0] * Tm[k][0] + S3[jj][1] * Tm[k][1] + S3[jj][2] * Tm[k][2]) * dSp[aa][k];
            }
            dT[aa][jj] += s1 + s2;
        }
    const float dJ00 = Rcw[0][0] * dT[0][0] + Rcw[0][1] * dT[0][1] + Rcw[0][2] * dT[0][2];
    const float dJ02 = Rcw[2][0] * dT[0][0] + Rcw[2][1] * dT[0][1] + Rcw[2][2] * dT[0][2];
    const float dJ11 = Rcw[1][0] * dT[1][0] + Rcw[1][1] * dT[1][1] + Rcw[1][2] * dT[1][2];
    const float dJ12 = Rcw[2][0] * dT[1][0] + Rcw[2][1] * dT[1][1] + Rcw[2][2] * dT[1][2];
    const float iz = 1.0f / z, iz2 = iz * iz, iz3 = iz2 * iz;
    {
        const float3 w = qapply(qcw, make_float3(-fx * iz2 * dJ02, -fy * iz2 * dJ12,
                                                 -fx * iz2 * dJ00 - fy * iz2 * dJ11 + (2 * fx * mc.x) * iz3 * dJ02 +
                                                     (2 * fy * mc.y) * iz3 * dJ12));
        dmu3.x += w.x;
        dmu3.y += w.y;
        dmu3.z += w.z;
    }
    float dS3[3][3];
    dS3[0][0] = Tm[0][0] * Tm[0][0] * dSxx + Tm[0][0] * Tm[1][0] * dSxy + Tm[1][0] * Tm[1][0] * dSyy;
    dS3[1][1] = Tm[0][1] * Tm[0][1] * dSxx + Tm[0][1] * Tm[1][1] * dSxy + Tm[1][1] * Tm[1][1] * dSyy;
    dS3[2][2] = Tm[0][2] * Tm[0][2] * dSxx + Tm[0][2] * Tm[1][2] * dSxy + Tm[1][2] * Tm[1][2] * dSyy;
    dS3[1][0] = dS3[0][1] = Tm[0][0] * Tm[0][1] * dSxx + 0.5f * (Tm[0][0] * Tm[1][1] + Tm[0][1] * Tm[1][0]) * dSxy +
                            Tm[1][0] * Tm[1][1] * dSyy;
    dS3[2][0] = dS3[0][2] = Tm[0][0] * Tm[0][2] * dSxx + 0.5f * (Tm[0][0] * Tm[1][2] + Tm[0][2] * Tm[1][0]) * dSxy +
                            Tm[1][0] * Tm[1][2] * dSyy;
    dS3[2][1] = dS3[1][2] = Tm[0][2] * Tm[0][1] * dSxx + 0.5f * (Tm[0][1] * Tm[1][2] + Tm[0][2] * Tm[1][1]) * dSxy +
                            Tm[1][1] * Tm[1][2] * dSyy;
    {
        float TtD[3][3], add[3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) TtD[r][c] = Tm[0][r] * dSp[0][c] + Tm[1][r] * dSp[1][c] + Tm[2][r] * dSp[2][c];
        mm3(TtD, Tm, add);
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) dS3[r][c] += add[r][c];
    }
    float dM[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) dM[r][c] = 2.0f * (RS[0][r] * dS3[0][c] + RS[1][r] * dS3[1][c] + RS[2][r] * dS3[2][c]);
    float dLds[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) dLds[k] = Rg[0][k] * dM[k][0] + Rg[1][k] * dM[k][1] + Rg[2][k] * dM[k][2];
    {
        const float ms = (s[0] + s[1] + s[2]) / 3.f;
        const float l0 = s[0] - ms, l1 = s[1] - ms, l2 = s[2] - ms;
        const float li = a.lambda_iso * (1.f / 3.f);
        dLds[0] -= li * (2.f * l0 - l1 - l2);
        dLds[1] -= li * (-l0 + 2.f * l1 - l2);
        dLds[2] -= li * (-l0 - l1 + 2.f * l2);
    }
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) dM[r][c] *= s[r];
    float th0 = 0.f, th1 = 0.f, th2 = 0.f;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float b0 = dM[0][r], b1 = dM[1][r], b2 = dM[2][r];
        th0 += Rg[r][1] * b2 - Rg[r][2] * b1;
        th1 += Rg[r][2] * b0 - Rg[r][0] * b2;
        th2 += Rg[r][0] * b1 - Rg[r][1] * b0;
    }
    float d3[14];
    d3[0] = eta_n * dmu3.x;
    d3[1] = eta_n * dmu3.y;
    d3[2] = eta_n * dmu3.z;
    d3[3] = eta_n * dLds[0];
    d3[4] = eta_n * dLds[1];
    d3[5] = eta_n * dLds[2];
    d3[6] = -eta_n * th0;
    d3[7] = -eta_n * th1;
    d3[8] = -eta_n * th2;
    d3[9] = d_col[0] * eta_n;
    d3[10] = d_col[1] * eta_n;
    d3[11] = d_col[2] * eta_n;
    d3[12] = d_alpha * eta_n;
    d3[13] = (float)nn;
    if (a.dbg_delta3d) {
        for (int k = 0; k < 14; ++k) a.dbg_delta3d[(size_t)i * 16 + k] = d3[k];
        a.dbg_delta3d[(size_t)i * 16 + 14] = 0.f;
        a.dbg_delta3d[(size_t)i * 16 + 15] = 0.f;
    }

    // --------------------------------- Adam ---------------------------------
    // state planes (float4 per Gaussian): 0 m_pos,1 v_pos,2 m_scl,3 v_scl,
    // 4 m_rot,5 v_rot,6 m_col,7 v_col,8 (m_alpha, v_alpha, k, -)
    float4* S = a.adam;
    const size_t NN = (size_t)a.cap;
    float4 mp = S[0 * NN + i], vp = S[1 * NN + i], ms = S[2 * NN + i], vs = S[3 * NN + i];
    float4 mr = S[4 * NN + i], vr = S[5 * NN + i], mcl = S[6 * NN + i], vcl = S[7 * NN + i];
    float4 mal = S[8 * NN + i];
    mal.z += 1.f;
    const float b1 = a.beta1, b2 = a.beta2, eps = a.eps, eta = a.eta;
    const float a1 = 1.f - b1, a2 = 1.f - b2;
    const float b1t = 1.0f / (1.f - powf(b1, mal.z));
    const float b2t = 1.0f / (1.f - powf(b2, mal.z));
    float4 np = pw;
    np.x += adam_step(mp.x, vp.x, d3[0], eta, a1, b1, b1t, a2, b2, b2t, eps);
    np.y += adam_step(mp.y, vp.y, d3[1], eta, a1, b1, b1t, a2, b2, b2t, eps);
    np.z += adam_step(mp.z, vp.z, d3[2], eta, a1, b1, b1t, a2, b2, b2t, eps);
    const float dq0 = adam_step(mr.x, vr.x, d3[6], eta, a1, b1, b1t, a2, b2, b2t, eps);
    const float dq1 = adam_step(mr.y, vr.y, d3[7], eta, a1, b1, b1t, a2, b2, b2t, eps);
    const float dq2 = adam_step(mr.z, vr.z, d3[8], eta, a1, b1, b1t, a2, b2, b2t, eps);
    float4 nr;
    {
        const float bx = 0.5f * dq0, by = 0.5f * dq1, bz = 0.5f * dq2;
        float x = rw.w * bx + rw.x + (rw.y * bz - rw.z * by);
        float y = rw.w * by + rw.y + (rw.z * bx - rw.x * bz);
        float zq = rw.w * bz + rw.z + (rw.x * by - rw.y * bx);
        float w = rw.w - (rw.x * bx + rw.y * by + rw.z * bz);
        const float nq = sqrtf(x * x + y * y + zq * zq + w * w);
        if (nq > 0.f) {
            const float inq = 1.0f / nq;
            x *= inq;
            y *= inq;
            zq *= inq;
            w *= inq;
        }
        nr = make_float4(x, y, zq, w);
    }
    float4 ns = sw;
    ns.x += adam_step(ms.x, vs.x, d3[3], eta, a1, b1, b1t, a2, b2, b2t, eps);
    ns.y += adam_step(ms.y, vs.y, d3[4], eta, a1, b1, b1t, a2, b2, b2t, eps);
    ns.z += adam_step(ms.z, vs.z, d3[5], eta, a1, b1, b1t, a2, b2, b2t, eps);
    cw.x += adam_step(mcl.x, vcl.x, d3[9], eta, a1, b1, b1t, a2, b2, b2t, eps);
    cw.y += adam_step(mcl.y, vcl.y, d3[10], eta, a1, b1, b1t, a2, b2, b2t, eps);
    cw.z += adam_step(mcl.z, vcl.z, d3[11], eta, a1, b1, b1t, a2, b2, b2t, eps);
    const float dalpha = adam_step(mal.x, mal.y, d3[12], eta, a1, b1, b1t, a2, b2, b2t, eps);
    {
        const float al = cw.w;
        const float as = logf(al / (1.f - al)) + dalpha / (al - al * al);
        cw.w = fmaxf(0.01f, fminf(0.99f, 1.f / (1.f + expf(-as))));
    }
    ns.x = fmaxf(0.001f, ns.x);
    ns.y = fmaxf(0.001f, ns.y);
    ns.z = fmaxf(0.001f, ns.z);
    cw.x = fminf(1.f, fmaxf(0.f, cw.x));
    cw.y = fminf(1.f, fmaxf(0.f, cw.y));
    cw.z = fminf(1.f, fmaxf(0.f, cw.z));
    a.pos[i] = np;
    a.scale[i] = ns;
    a.rot[i] = nr;
    a.col[i] = cw;
    if (a.attr_sr) {
        a.attr_sr[i] = pack_sr(ns, nr);
        a.attr_c[i] = pack_c(cw);
    }
    S[0 * NN + i] = mp;
    S[1 * NN + i] = vp;
    S[2 * NN + i] = ms;
    S[3 * NN + i] = vs;
    S[4 * NN + i] = mr;
    S[5 * NN + i] = vr;
    S[6 * NN + i] = mcl;
    S[7 * NN + i] = vcl;
    S[8 * NN + i] = mal;
}

// Exclusive scan of per-tile bucket counts ceil(n_t/32) (one CTA).
__global__ void __launch_bounds__(1024) bucket_scan_kernel(const uint2* ranges, int T, uint32_t* bucket_base,
                                                           uint32_t* total) {
    pdl_begin();
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int base = 0; base < T; base += 1024) {
        const int t = base + threadIdx.x;
        uint32_t c = 0;
        if (t < T) c = (ranges[t].y - ranges[t].x + 31) / 32;
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_w[w] = incl;
        __syncthreads();
        if (w == 0) {
            const uint32_t v = s_w[lane];
            uint32_t vi = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(kFullMask, vi, o);
                if (lane >= o) vi += y;
            }
            s_w[lane] = vi - v;
        }
        __syncthreads();
        const uint32_t carry = s_carry;
        if (t < T) bucket_base[t] = carry + s_w[w] + incl - c;
        __syncthreads();
        if (threadIdx.x == 1023) s_carry = carry + s_w[w] + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = s_carry;
}

cudaError_t launch_map_forward(const MapArgs& a, bool cap, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (cap) return launch_chained(map_forward_kernel<true>, dim3(T), dim3(kMPix), 0, s, a);
    return launch_chained(map_forward_kernel<false>, dim3(T), dim3(kMPix), 0, s, a);
}

cudaError_t launch_map_backward(const MapArgs& a, bool cap, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (cap) return launch_chained(map_backward_kernel<true>, dim3(T), dim3(kMPix), 0, s, a);
    return launch_chained(map_backward_kernel<false>, dim3(T), dim3(kMPix), 0, s, a);
}

cudaError_t launch_bucket_scan(const uint2* ranges, int T, uint32_t* bucket_base, uint32_t* total, cudaStream_t s) {
    return launch_chained(bucket_scan_kernel, dim3(1), dim3(1024), 0, s, ranges, T, bucket_base, total);
}

cudaError_t launch_map_update(const MapUpdateArgs& a, const DevStatus* st, cudaStream_t s) {
    if (a.n <= 0) return cudaSuccess;
    return launch_chained(map_update_kernel, dim3((a.n + 255) / 256), dim3(256), 0, s, a, st);
}

int map_cap_buckets() { return kCapBuckets; }

__global__ void pack_reduced_kernel(const float4* __restrict__ scale, const float4* __restrict__ rot,
                                    const float4* __restrict__ col, uint32_t n, uint4* __restrict__ sr,
                                    uint2* __restrict__ c) {
    pdl_begin();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    sr[i] = pack_sr(scale[i], rot[i]);
    c[i] = pack_c(col[i]);
}

cudaError_t launch_pack_reduced(const float4* scale, const float4* rot, const float4* col, uint32_t n, uint4* sr,
                                uint2* c, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    return launch_chained(pack_reduced_kernel, dim3((n + 255) / 256), dim3(256), 0, s, scale, rot, col, n, sr, c);
}

}  // namespace fvgs
