// maintenance.cu -- map maintenance kernels for sm_103a: visibility and
// covisibility, outlier scores, prune marking, and stable compaction of the
// Gaussian planes.
//
// Reference: computeGaussiansVisibility_kernel, computeGaussiansCovisibility_
// kernel, pruneGaussians_kernel, computeOutliers_kernel and removeOutliers_
// kernel (src/GSCudaKernels.cu:1455-1739), driven by GSSlam::removeOutliers,
// GSSlam::prune and GSSlam::computeCovisibilityRatio (src/GSSlam.cu:1467-1904), which
// remove the marked Gaussians with thrust::sort_by_key on the 0 / 0xff states
// (survivors first, in order) and shrink the Gaussian count.
//
// Every blending kernel here reads the packed records of the binning (rec0 =
// u, v, z, opacity; rec1 = c.x, c.y, c.z, phat.x; rec2 = phat.y, rgb), where
// c is the inverse 2D covariance in the order the reference's tracking
// kernels consume it (c.y as the xy term, c.z as the yy term).  The
// reference's visibility and outlier kernels read the stored inverse the same
// way, so the same record serves both.
//
// Layout choices:
//  * visibility: one CTA per 16x16 tile, one thread per pixel, as the
//    reference (a pixel's transmittance depends on the Gaussians before it);
//    a Gaussian's flag is written once per tile, from a shared hit mask,
//    instead of once per pixel;
//  * outlier scores: the reference adds every (pixel, Gaussian) contribution
//    with two global atomics.  Here a thread takes one Gaussian of the tile
//    list, sums its contributions over the tile's pixels in a fixed order and
//    adds the tile's totals with one atomic per accumulator: the same sums,
//    one global update per (tile, Gaussian);
//  * compaction: mark (state + survivors per block) -> one-CTA scan of the
//    block counts -> scatter into the session's second set of planes, after
//    which the host swaps the plane pointers.  The source planes are never
//    written, so an aborted pass leaves the map as it was.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

constexpr int kMPix = 256;  // 16 x 16 pixels per tile

__global__ void __launch_bounds__(kMPix) visibility_kernel(VisArgs a) {
    pdl_begin();
    // alpha = min(0.99, o exp(-q/2)) as one ex2.approx of log2(o) + the
    // conic pre-scaled by -log2(e)/2 (the tracking kernels' weight)
    __shared__ float4 sA[kMPix];  // u, v, log2(opacity), c'.x
    __shared__ float2 sB[kMPix];  // 2 c'.y, c'.z
    __shared__ int sHit[kMPix];
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int tid = threadIdx.x;
    const int x = tx * 16 + (tid & 15), y = ty * 16 + (tid >> 4);
    const bool inside = x < a.W && y < a.H;
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    if (a.cap > 0) n = min(n, a.cap);
    const float px = (float)x, py = (float)y;
    float T = 1.f;
    bool done = !inside;
    for (int base = 0; base < n; base += kMPix) {
        if (__syncthreads_and(done)) break;
        const int li = base + tid;
        uint32_t g = 0xffffffffu;
        if (li < n) {
            g = a.indices[range.x + li];
            float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0;
            if (g < a.n_gauss) {
                r0 = a.rec0[g];
                r1 = a.rec1[g];
            }
            constexpr float kNegHalfLog2e = -0.72134752044448170368f;
            sA[tid] = make_float4(r0.x, r0.y, log2_opacity(r0.w), kNegHalfLog2e * r1.x);
            sB[tid] = make_float2(2.0f * kNegHalfLog2e * r1.y, kNegHalfLog2e * r1.z);
        }
        sHit[tid] = 0;
        __syncthreads();
        const int cnt = min(kMPix, n - base);
        for (int j = 0; j < cnt && !done; ++j) {
            const float4 gA = sA[j];
            const float2 gB = sB[j];
            const float dx = gA.x - px, dy = gA.y - py;
            const float t = __fmaf_rn(dx, __fmaf_rn(gA.w, dx, __fmul_rn(gB.x, dy)),
                                      __fmaf_rn(__fmul_rn(gB.y, dy), dy, gA.z));
            float w;
            asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(w) : "f"(t));
            const float alpha = fminf(0.99f, w);
            if (alpha < 1.0f / 255.0f) continue;
            sHit[j] = 1;
            T *= 1.0f - alpha;
            if (T < 0.5f) done = true;
        }
        __syncthreads();
        if (li < n && g < a.n_gauss && sHit[tid]) a.vis[g] = 1;
    }
}

__global__ void __launch_bounds__(kMPix) outliers_kernel(OutlierArgs a) {
    pdl_begin();
    __shared__ float sD[kMPix];  // per pixel: 0.8 x observed depth where it is > 0.1, else -inf
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int x0 = tx * 16, y0 = ty * 16;
    const int tid = threadIdx.x;
    {
        const int x = x0 + (tid & 15), y = y0 + (tid >> 4);
        const float d_obs = (x < a.W && y < a.H) ? a.obs_depth[(size_t)y * a.W + x] : 0.f;
        // a pair counts as an outlier where d_obs > 0.1 and dr < 0.8 d_obs: one compare per pair
        sD[tid] = d_obs > 0.1f ? 0.8f * d_obs : -INFINITY;
    }
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    const int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    const int w = min(16, a.W - x0), h = min(16, a.H - y0);
    __syncthreads();
    // One thread per Gaussian of the tile list, over all pixels of the tile
    // in row-major order (every lane of a warp reads the same pixel's depth:
    // a shared-memory broadcast); its sums go out with one atomic each.
    for (int li = tid; li < n; li += kMPix) {
        const uint32_t g = a.indices[range.x + li];
        if (g >= a.n_gauss) continue;
        const float4 r0 = a.rec0[g], r1 = a.rec1[g];
        const float phy = a.rec2[g].x;
        const float lo2 = log2_opacity(r0.w);  // alpha = o exp(-q/2) = 2^(log2 o - q log2(e) / 2)
        float ta = 0.f, to = 0.f;
        for (int yy = 0; yy < h; ++yy) {
            const float dy = (float)(y0 + yy) - r0.y;
            const float q_row = r1.z * dy * dy, b_row = 2.0f * r1.y * dy;
            const float dr_row = r0.z + phy * dy;
            float pxf = (float)x0;  // the pixel's x as a float, stepped exactly (integers < 2^24)
#pragma unroll 4
            for (int xx = 0; xx < w; ++xx, pxf += 1.0f) {
                const float dx = pxf - r0.x;
                const float q = (r1.x * dx + b_row) * dx + q_row;
                const float alpha = gauss_weight(lo2, q);
                const float dr = dr_row + r1.w * dx;
                if (alpha < 1.0f / 255.0f || dr <= 0.0f) continue;
                ta += alpha;
                if (dr < sD[yy * 16 + xx]) to += alpha;
            }
        }
        if (ta != 0.f) atomicAdd(a.total_alpha + g, ta);
        if (to != 0.f) atomicAdd(a.outlier_prob + g, to);
    }
}

template <int MODE>
__global__ void __launch_bounds__(kCompactBlock) mark_kernel(MarkArgs a) {
    pdl_begin();
    const uint32_t i = blockIdx.x * kCompactBlock + threadIdx.x;
    bool remove = false;
    if (i < a.n) {
        if (MODE == kMarkPrune) {
            const float alpha = a.col[i].w;
            const float4 sc = a.scale[i];
            if (alpha < a.alpha_thr) {
                remove = true;
            } else {
                const float smax = fmaxf(sc.x, fmaxf(sc.y, sc.z));
                const float smin = fminf(sc.x, fminf(sc.y, sc.z));
                const float smed = __fsub_rn(__fsub_rn(__fadd_rn(__fadd_rn(sc.x, sc.y), sc.z), smax), smin);
                remove = __fdiv_rn(smed, smax) < a.ratio_thr || smax < a.min_scale;
            }
        } else {
            const float tot = a.total_alpha[i];
            remove = tot > 1.0f && __fdiv_rn(a.outlier_prob[i], tot) > a.threshold;
        }
        a.states[i] = remove ? 0xff : 0;
    }
    const int keep = __syncthreads_count(i < a.n && !remove);
    if (threadIdx.x == 0) a.block_keep[blockIdx.x] = (uint32_t)keep;
}

// Exclusive scan of the per-block survivor counts (one CTA); counters[0] =
// survivors, counters[1] = removed.
__global__ void __launch_bounds__(1024) compact_scan_kernel(const uint32_t* __restrict__ block_keep, int nb,
                                                            uint32_t n, uint32_t* __restrict__ block_base,
                                                            uint32_t* __restrict__ counters) {
    pdl_begin();
    __shared__ uint32_t warp_sum[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t carry = 0;
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nb ? block_keep[i] : 0u;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) warp_sum[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t ws = warp_sum[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += t;
            }
            warp_sum[lane] = ws;  // inclusive over warps
        }
        __syncthreads();
        const uint32_t before = warp > 0 ? warp_sum[warp - 1] : 0u;
        if (i < nb) block_base[i] = carry + before + incl - v;
        carry += warp_sum[31];
        __syncthreads();  // warp_sum is rewritten by the next round
    }
    if (threadIdx.x == 0) {
        counters[0] = carry;
        counters[1] = n - carry;
    }
}

__global__ void __launch_bounds__(kCompactBlock) compact_scatter_kernel(CompactArgs a) {
    pdl_begin();
    if (a.counters[1] == 0) return;  // nothing removed: the host keeps the current planes
    __shared__ uint32_t wk[kCompactBlock / 32], wr[kCompactBlock / 32];
    const uint32_t i = blockIdx.x * kCompactBlock + threadIdx.x;
    const bool valid = i < a.n;
    const bool keep = valid && a.states[i] == 0;
    const unsigned bk = __ballot_sync(0xffffffffu, keep), brm = __ballot_sync(0xffffffffu, valid && !keep);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        wk[warp] = __popc(bk);
        wr[warp] = __popc(brm);
    }
    __syncthreads();
    if (!valid) return;
    uint32_t k_before = 0, r_before = 0;
    for (int w = 0; w < warp; ++w) {
        k_before += wk[w];
        r_before += wr[w];
    }
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t base_keep = a.block_base[blockIdx.x];
    // every block before this one is full, so the removed items before it are
    // its start minus the survivors before it; they follow all survivors
    const uint32_t base_rem = a.counters[0] + (blockIdx.x * (uint32_t)kCompactBlock - base_keep);
    const uint32_t dst = keep ? base_keep + k_before + __popc(bk & lt) : base_rem + r_before + __popc(brm & lt);
    a.pos_out[dst] = a.pos[i];
    a.scale_out[dst] = a.scale[i];
    a.rot_out[dst] = a.rot[i];
    a.col_out[dst] = a.col[i];
    if (a.adam) {
        const size_t cap = a.cap;
#pragma unroll
        for (int p = 0; p < 9; ++p) a.adam_out[p * cap + dst] = a.adam[p * cap + i];
    }
}

// Counts over two visibility masks: counters[0] += |a & b|, counters[1] += |a | b|.
__global__ void __launch_bounds__(256) covis_count_kernel(const uint8_t* __restrict__ va, const uint8_t* __restrict__ vb,
                                                          uint32_t n, uint32_t* __restrict__ counters) {
    pdl_begin();
    uint32_t inter = 0, uni = 0;
    const uint32_t n16 = n / 16;
    const uint4* a4 = reinterpret_cast<const uint4*>(va);
    const uint4* b4 = reinterpret_cast<const uint4*>(vb);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n16; k += stride) {
        const uint4 x = a4[k], y = b4[k];
        const uint32_t xa[4] = {x.x, x.y, x.z, x.w}, ya[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const uint32_t p = (xa[c] >> (8 * b)) & 0xffu, q = (ya[c] >> (8 * b)) & 0xffu;
                inter += (p & q) != 0u;
                uni += (p | q) != 0u;
            }
        }
    }
    for (uint32_t k = n16 * 16 + blockIdx.x * blockDim.x + threadIdx.x; k < n; k += stride) {
        inter += (va[k] & vb[k]) != 0;
        uni += (va[k] | vb[k]) != 0;
    }
    inter = __reduce_add_sync(0xffffffffu, inter);
    uni = __reduce_add_sync(0xffffffffu, uni);
    if ((threadIdx.x & 31) == 0 && (inter | uni)) {
        atomicAdd(counters, inter);
        atomicAdd(counters + 1, uni);
    }
}

cudaError_t launch_visibility(const VisArgs& a, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    return launch_chained(visibility_kernel, dim3(T), dim3(kMPix), 0, s, a);
}

cudaError_t launch_outliers(const OutlierArgs& a, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    return launch_chained(outliers_kernel, dim3(T), dim3(kMPix), 0, s, a);
}

static unsigned compact_blocks(uint32_t n) { return (n + kCompactBlock - 1) / kCompactBlock; }

cudaError_t launch_mark(MarkMode mode, const MarkArgs& a, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    const dim3 grid(compact_blocks(a.n));
    return mode == kMarkPrune ? launch_chained(mark_kernel<kMarkPrune>, grid, dim3(kCompactBlock), 0, s, a)
                              : launch_chained(mark_kernel<kMarkOutliers>, grid, dim3(kCompactBlock), 0, s, a);
}

cudaError_t launch_compact_scan(const uint32_t* block_keep, uint32_t n, uint32_t* block_base, uint32_t* counters,
                                cudaStream_t s) {
    return launch_chained(compact_scan_kernel, dim3(1), dim3(1024), 0, s, block_keep, (int)compact_blocks(n), n,
                          block_base, counters);
}

cudaError_t launch_compact_scatter(const CompactArgs& a, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    return launch_chained(compact_scatter_kernel, dim3(compact_blocks(a.n)), dim3(kCompactBlock), 0, s, a);
}

cudaError_t launch_covis_count(const uint8_t* va, const uint8_t* vb, uint32_t n, uint32_t* counters,
                               cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const unsigned want = (n / 16 + 255) / 256 + 1;
    const unsigned grid = want < 4u * 152u ? want : 4u * 152u;
    return launch_chained(covis_count_kernel, dim3(grid), dim3(256), 0, s, va, vb, n, counters);
}

}  // namespace fvgs
