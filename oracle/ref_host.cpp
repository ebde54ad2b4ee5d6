/*
 * ref_host.cpp -- the reference's own binning kernels (taken verbatim from
 * src/GSCudaKernels.cu into oracle/_ref/ref_binning_kernels.inc by
 * oracle/ref_build.py) run on the CPU, one emulated CUDA thread at a time,
 * in the order GSSlam::prepareRasterization launches them
 * (src/GSSlam.cu:408-646).
 *
 * TEST INFRASTRUCTURE ONLY: it pins the CPU restatement (oracle/fvgs_oracle.cpp)
 * to the reference's source.  Compiled with floating-point contraction off,
 * so it is compared with the restatement built the same way.
 *
 * Glue that the reference takes from Thrust is restated here:
 * thrust::exclusive_scan (an exact integer scan) and thrust::sort_by_key on
 * the 64-bit keys (a stable sort).  The kernels' CUDA built-ins are given
 * host definitions: the launch coordinates, max / min with CUDA's float
 * semantics (fmaxf / fminf), __float_as_uint.
 */
#include <cuda_runtime.h>  // vector types and make_* (host-usable)

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "CudaMathOperations.cuh"

namespace refhost {

dim3 blockIdx, threadIdx, blockDim, gridDim;

inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }
inline int max(int a, int b) { return a > b ? a : b; }
inline int min(int a, int b) { return a < b ? a : b; }
inline uint32_t __float_as_uint(float f) {
    uint32_t u;
    std::memcpy(&u, &f, sizeof(u));
    return u;
}

// The layouts of include/f_vigs_slam/RepresentationClasses.hpp:100-122.
struct IntrinsicParameters {
    float2 f, c;
};
struct CameraPose {
    float3 position;
    float4 orientation;
};

constexpr int kTile = 16;
#define TILE_SIZE 16
#include "ref_binning_kernels.inc"
#undef TILE_SIZE

// Run kernel body `k` for every thread of a 1-D launch of `blocks` x 256.
template <typename F>
void launch(int blocks, F&& k) {
    blockDim = dim3(256, 1, 1);
    gridDim = dim3((unsigned)blocks, 1, 1);
    for (int b = 0; b < blocks; ++b)
        for (int t = 0; t < 256; ++t) {
            blockIdx = dim3((unsigned)b, 0, 0);
            threadIdx = dim3((unsigned)t, 0, 0);
            k();
        }
}

}  // namespace refhost

extern "C" {

/*
 * The reference's binning of n Gaussians (positions[3n], scales[3n],
 * orientations[4n] raw float4) for the camera pose (t[3], q[4] raw float4)
 * and intrinsics K = (fx, fy, cx, cy), W x H, 16 x 16 tiles, radius 3 sigma.
 * Outputs: uv[2n], cov2d[3n], inv2d[3n], depth[n], phat[2n] (culled
 * Gaussians keep the zeros the buffers start with), counts[n]; the sorted
 * keys and values (at most cap; *n_inst receives the total), ranges[2T]
 * and bucket counts[T].  range_mode 0 launches the range kernel as the
 * reference does (ceil(T / 256) blocks of 256 threads); 1 with one thread
 * per instance.  Returns 0, or 1 when the instances exceed cap.
 */
int ref_binning_host(const float* pos, const float* scl, const float* rot, int n, const float* cam_t,
                     const float* cam_q, const float* K4, int W, int H, int range_mode, float* uv, float* cov2d,
                     float* inv2d, float* depth, float* phat, uint32_t* counts, uint64_t* keys, uint32_t* vals,
                     uint64_t cap, uint32_t* ranges, uint32_t* buckets, uint64_t* n_inst) {
    using namespace refhost;
    CameraPose pose;
    pose.position = make_float3(cam_t[0], cam_t[1], cam_t[2]);
    pose.orientation = make_float4(cam_q[0], cam_q[1], cam_q[2], cam_q[3]);
    IntrinsicParameters K;
    K.f = make_float2(K4[0], K4[1]);
    K.c = make_float2(K4[2], K4[3]);
    const int ntx = (W + kTile - 1) / kTile, nty = (H + kTile - 1) / kTile;
    const int T = ntx * nty;
    std::vector<float3> p3(n), s3(n), cov(n), inv(n);
    std::vector<float4> q4(n);
    std::vector<float2> uv2(n), ph2(n);
    for (int i = 0; i < n; ++i) {
        p3[i] = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        s3[i] = make_float3(scl[3 * i], scl[3 * i + 1], scl[3 * i + 2]);
        q4[i] = make_float4(rot[4 * i], rot[4 * i + 1], rot[4 * i + 2], rot[4 * i + 3]);
        uv2[i] = make_float2(0.f, 0.f);
        ph2[i] = make_float2(0.f, 0.f);
        cov[i] = make_float3(0.f, 0.f, 0.f);
        inv[i] = make_float3(0.f, 0.f, 0.f);
    }
    std::vector<float> dep(n, 0.f);
    std::vector<uint32_t> cnt(n, 0u), off(n, 0u);
    const int blocks = (n + 255) / 256;
    launch(blocks, [&] {
        projectGaussiansWorldToScreen_kernel(uv2.data(), cov.data(), inv.data(), dep.data(), ph2.data(), p3.data(),
                                             s3.data(), q4.data(), pose, K, W, H, n);
    });
    launch(blocks, [&] {
        countTilesPerGaussian_kernel(cnt.data(), uv2.data(), cov.data(), W, H, n, ntx, nty, 3.0f);
    });
    uint64_t total = 0;
    for (int i = 0; i < n; ++i) {  // thrust::exclusive_scan (u32, as the reference's offsets)
        off[i] = (uint32_t)total;
        total += cnt[i];
    }
    *n_inst = total;
    for (int i = 0; i < n; ++i) {
        uv[2 * i] = uv2[i].x;
        uv[2 * i + 1] = uv2[i].y;
        cov2d[3 * i] = cov[i].x;
        cov2d[3 * i + 1] = cov[i].y;
        cov2d[3 * i + 2] = cov[i].z;
        inv2d[3 * i] = inv[i].x;
        inv2d[3 * i + 1] = inv[i].y;
        inv2d[3 * i + 2] = inv[i].z;
        depth[i] = dep[i];
        phat[2 * i] = ph2[i].x;
        phat[2 * i + 1] = ph2[i].y;
        counts[i] = cnt[i];
    }
    if (total > cap) return 1;
    std::vector<uint64_t> h(total);
    std::vector<uint32_t> g(total);
    launch(blocks, [&] {
        generateTileHashes_kernel(h.data(), g.data(), off.data(), uv2.data(), cov.data(), dep.data(), ph2.data(), W,
                                  H, n, ntx, nty, 3.0f);
    });
    // thrust::sort_by_key on the 64-bit keys: stable
    std::vector<uint64_t> order(total);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](uint64_t a, uint64_t b) { return h[a] < h[b]; });
    std::vector<uint64_t> hs(total);
    for (uint64_t k = 0; k < total; ++k) {
        hs[k] = h[order[k]];
        keys[k] = hs[k];
        vals[k] = g[order[k]];
    }
    std::vector<uint2> rg(T, make_uint2(0u, 0u));
    const int rblocks = range_mode == 0 ? (T + 255) / 256 : (int)((total + 255) / 256);
    launch(rblocks, [&] { computeIndicesRanges_kernel(rg.data(), hs.data(), (uint32_t)total, T); });
    std::vector<uint32_t> bc(T, 0u);
    launch((T + 255) / 256, [&] { perTileBucketCount(bc.data(), rg.data(), T); });
    for (int t = 0; t < T; ++t) {
        ranges[2 * t] = rg[t].x;
        ranges[2 * t + 1] = rg[t].y;
        buckets[t] = bc[t];
    }
    return 0;
}

}  // extern "C"
