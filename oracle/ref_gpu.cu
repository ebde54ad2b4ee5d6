/*
 * ref_gpu.cu -- the reference's own binning kernels (taken verbatim from
 * src/GSCudaKernels.cu into oracle/_ref/ref_binning_kernels.inc by
 * oracle/ref_build.py), compiled by nvcc with the reference's flags and
 * launched on the GPU as GSSlam::prepareRasterization launches them
 * (src/GSSlam.cu:408-646): grids of 256-thread blocks over the Gaussians,
 * the range kernel over ceil(T / 256) blocks.
 *
 * TEST INFRASTRUCTURE ONLY: its outputs are the reference's own binning, the
 * ground truth the library's keys, indices and ranges are compared with.
 * Thrust's exclusive scan and stable key sort are done on the host (exact
 * integer scan; stable sort by the 64-bit key).  Every kernel here checks its
 * thread index against its element count; buffers are sized to those counts.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <vector>

#include "CudaMathOperations.cuh"

namespace refgpu {

// The layouts of include/f_vigs_slam/RepresentationClasses.hpp:100-122.
struct IntrinsicParameters {
    float2 f, c;
};
struct CameraPose {
    float3 position;
    float4 orientation;
};

#define TILE_SIZE 16
#include "ref_binning_kernels.inc"
#undef TILE_SIZE

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    bool alloc(size_t count) {
        n = count ? count : 1;
        return cudaMalloc(&p, sizeof(T) * n) == cudaSuccess && cudaMemset(p, 0, sizeof(T) * n) == cudaSuccess;
    }
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace refgpu

extern "C" {

/*
 * As ref_binning_host (oracle/ref_host.cpp), on the GPU.  Returns 0, 1 when
 * the instances exceed cap, -1 on a CUDA error.
 */
int ref_binning_gpu(const float* pos, const float* scl, const float* rot, int n, const float* cam_t,
                    const float* cam_q, const float* K4, int W, int H, int range_mode, float* uv, float* cov2d,
                    float* inv2d, float* depth, float* phat, uint32_t* counts, uint64_t* keys, uint32_t* vals,
                    uint64_t cap, uint32_t* ranges, uint32_t* buckets, uint64_t* n_inst) {
    using namespace refgpu;
    CameraPose pose;
    pose.position = make_float3(cam_t[0], cam_t[1], cam_t[2]);
    pose.orientation = make_float4(cam_q[0], cam_q[1], cam_q[2], cam_q[3]);
    IntrinsicParameters K;
    K.f = make_float2(K4[0], K4[1]);
    K.c = make_float2(K4[2], K4[3]);
    const int ntx = (W + 15) / 16, nty = (H + 15) / 16, T = ntx * nty;
    std::vector<float3> p3(n), s3(n);
    std::vector<float4> q4(n);
    for (int i = 0; i < n; ++i) {
        p3[i] = make_float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        s3[i] = make_float3(scl[3 * i], scl[3 * i + 1], scl[3 * i + 2]);
        q4[i] = make_float4(rot[4 * i], rot[4 * i + 1], rot[4 * i + 2], rot[4 * i + 3]);
    }
    DevBuf<float3> d_p3, d_s3, d_cov, d_inv;
    DevBuf<float4> d_q4;
    DevBuf<float2> d_uv, d_ph;
    DevBuf<float> d_dep;
    DevBuf<uint32_t> d_cnt, d_off;
    if (!d_p3.alloc(n) || !d_s3.alloc(n) || !d_cov.alloc(n) || !d_inv.alloc(n) || !d_q4.alloc(n) || !d_uv.alloc(n) ||
        !d_ph.alloc(n) || !d_dep.alloc(n) || !d_cnt.alloc(n) || !d_off.alloc(n))
        return -1;
    if (cudaMemcpy(d_p3.p, p3.data(), sizeof(float3) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d_s3.p, s3.data(), sizeof(float3) * n, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d_q4.p, q4.data(), sizeof(float4) * n, cudaMemcpyHostToDevice) != cudaSuccess)
        return -1;
    const dim3 block(256), grid((n + 255) / 256);
    if (n > 0) {
        projectGaussiansWorldToScreen_kernel<<<grid, block>>>(d_uv.p, d_cov.p, d_inv.p, d_dep.p, d_ph.p, d_p3.p,
                                                              d_s3.p, d_q4.p, pose, K, W, H, n);
        countTilesPerGaussian_kernel<<<grid, block>>>(d_cnt.p, d_uv.p, d_cov.p, W, H, n, ntx, nty, 3.0f);
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    std::vector<float2> uv2(n), ph2(n);
    std::vector<float3> cov(n), inv(n);
    std::vector<float> dep(n);
    std::vector<uint32_t> cnt(n), off(n);
    if (cudaMemcpy(uv2.data(), d_uv.p, sizeof(float2) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(ph2.data(), d_ph.p, sizeof(float2) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cov.data(), d_cov.p, sizeof(float3) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(inv.data(), d_inv.p, sizeof(float3) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(dep.data(), d_dep.p, sizeof(float) * n, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(cnt.data(), d_cnt.p, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    uint64_t total = 0;
    for (int i = 0; i < n; ++i) {  // thrust::exclusive_scan
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
    if (total > 0xffffffffull) return 1;
    DevBuf<uint64_t> d_h;
    DevBuf<uint32_t> d_g;
    DevBuf<uint2> d_rg;
    DevBuf<uint32_t> d_bc;
    if (!d_h.alloc(total) || !d_g.alloc(total) || !d_rg.alloc(T) || !d_bc.alloc(T)) return -1;
    if (cudaMemcpy(d_off.p, off.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice) != cudaSuccess) return -1;
    if (n > 0)
        generateTileHashes_kernel<<<grid, block>>>(d_h.p, d_g.p, d_off.p, d_uv.p, d_cov.p, d_dep.p, d_ph.p, W, H, n,
                                                   ntx, nty, 3.0f);
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    std::vector<uint64_t> h(total);
    std::vector<uint32_t> g(total);
    if (cudaMemcpy(h.data(), d_h.p, sizeof(uint64_t) * total, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(g.data(), d_g.p, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
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
    if (total && cudaMemcpy(d_h.p, hs.data(), sizeof(uint64_t) * total, cudaMemcpyHostToDevice) != cudaSuccess)
        return -1;
    const unsigned rblocks = range_mode == 0 ? (unsigned)((T + 255) / 256) : (unsigned)((total + 255) / 256);
    if (rblocks) computeIndicesRanges_kernel<<<rblocks, block>>>(d_rg.p, d_h.p, (uint32_t)total, T);
    perTileBucketCount<<<(T + 255) / 256, block>>>(d_bc.p, d_rg.p, T);
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    std::vector<uint2> rg(T);
    std::vector<uint32_t> bc(T);
    if (cudaMemcpy(rg.data(), d_rg.p, sizeof(uint2) * T, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(bc.data(), d_bc.p, sizeof(uint32_t) * T, cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    for (int t = 0; t < T; ++t) {
        ranges[2 * t] = rg[t].x;
        ranges[2 * t + 1] = rg[t].y;
        buckets[t] = bc[t];
    }
    return 0;
}

}  // extern "C"
