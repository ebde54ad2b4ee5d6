// preprocess.cu -- frame preprocessing on the GPU for sm_103a.
//
// Reference: GSSlam::initAndCopyImgs (src/GSSlam.cu:1913-1969), which runs on
// the host for every frame: an image pyramid by cv::pyrDown (8-bit colour,
// float depth; uint16 millimetre depth is first scaled by 0.001), then per
// level the colour as float / 255 and its 3x3 Sobel derivatives
// (cv::Sobel(.., CV_32F, 1, 0, 3) and (0, 1, 3)), uploaded as the tracking
// inputs.  Here the camera frame is copied to the device once and every level
// is produced there, one launch per level (chained by programmatic dependent
// launch): level 0 stages its 8-bit tile and Sobel halo in shared memory;
// every coarser level stages the finer level's 8-bit window under its pixels
// and halo, filters its own 8-bit colour there (stored for the next level),
// and takes the Sobel from shared memory.
//  * pyrDown: 5-tap binomial [1 4 6 4 1]/16 in x and y, reflect-101 borders,
//    output ((W + 1) / 2, (H + 1) / 2); 8-bit images in integers with
//    (sum + 128) >> 8, float images as row sums then column sums, times 1/256,
//    in that order;
//  * colour: c * (1/255), and once more (1/255) for the observed image when
//    the caller reproduces computeRgbdPoseJacobians' second scaling
//    (src/GSSlam.cu:2158);
//  * Sobel: ((p[y-1][x+1] - p[y-1][x-1]) + 2 (p[y][x+1] - p[y][x-1])) +
//    (p[y+1][x+1] - p[y+1][x-1]) and its transpose, reflect-101 borders.
// Every operation is an explicitly rounded FP32 op, so the results match the
// CPU restatement bit for bit.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

__device__ __forceinline__ int reflect101(int i, int n) {
    if (n == 1) return 0;
    // at most two reflections for the 2-pixel reach of these filters
    if (i < 0) i = -i;
    if (i >= n) i = 2 * n - 2 - i;
    if (i < 0) i = -i;
    return i;
}

constexpr int kTW = 32, kTH = 8;              // output pixels of one CTA, one per thread
constexpr int kHW = kTW + 2, kHH = kTH + 2;    // with the Sobel halo
constexpr int kSW = 2 * kTW + 7, kSH = 2 * kTH + 7;  // finer-level window of a pyrDown CTA

__device__ __forceinline__ float u8f(uint8_t v) { return __fmul_rn((float)v, 1.0f / 255.0f); }

// Colour (/255, and /255 again for the observed image with double_scale) and
// its Sobel derivatives at tile cell (hx, hy) of a (kHH x kHW x 3) 8-bit
// tile whose cells around it are the reflect-101 neighbours.
__device__ __forceinline__ void color_sobel_at(const uint8_t (*t)[kHW * 3], int hx, int hy, int double_scale,
                                               size_t p, float* __restrict__ rgb, float* __restrict__ gx,
                                               float* __restrict__ gy) {
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const int xm = 3 * (hx - 1) + ch, xc = 3 * hx + ch, xp = 3 * (hx + 1) + ch;
        const float f = u8f(t[hy][xc]);
        rgb[3 * p + ch] = double_scale ? __fmul_rn(f, 1.0f / 255.0f) : f;
        const float a = __fsub_rn(u8f(t[hy - 1][xp]), u8f(t[hy - 1][xm]));
        const float b = __fsub_rn(u8f(t[hy][xp]), u8f(t[hy][xm]));
        const float c = __fsub_rn(u8f(t[hy + 1][xp]), u8f(t[hy + 1][xm]));
        gx[3 * p + ch] = __fadd_rn(__fadd_rn(a, __fmul_rn(2.0f, b)), c);
        const float d = __fsub_rn(u8f(t[hy + 1][xm]), u8f(t[hy - 1][xm]));
        const float e = __fsub_rn(u8f(t[hy + 1][xc]), u8f(t[hy - 1][xc]));
        const float f2 = __fsub_rn(u8f(t[hy + 1][xp]), u8f(t[hy - 1][xp]));
        gy[3 * p + ch] = __fadd_rn(__fadd_rn(d, __fmul_rn(2.0f, e)), f2);
    }
}

// Level 0: the camera frame's 8-bit tile with its halo staged in shared
// memory (reflect-101), then per pixel the depth in metres and the colour /
// Sobel outputs.
__global__ void __launch_bounds__(kTW * kTH) prep_level0_kernel(const uint8_t* __restrict__ img,
                                                                const void* __restrict__ raw_depth, int u16_mm,
                                                                int W, int H, int double_scale,
                                                                float* __restrict__ rgb, float* __restrict__ gx,
                                                                float* __restrict__ gy, float* __restrict__ depth) {
    pdl_begin();
    __shared__ uint8_t t[kHH][kHW * 3];
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    for (int i = threadIdx.x; i < kHH * kHW; i += kTW * kTH) {
        const int hy = i / kHW, hx = i - hy * kHW;
        // cells past the image's far edge are not read; clamp them in range
        const int xs = reflect101(min(x0 + hx - 1, W), W), ys = reflect101(min(y0 + hy - 1, H), H);
        const uint8_t* q = img + ((size_t)ys * W + xs) * 3;
        t[hy][3 * hx] = q[0];
        t[hy][3 * hx + 1] = q[1];
        t[hy][3 * hx + 2] = q[2];
    }
    __syncthreads();
    const int lx = threadIdx.x % kTW, ly = threadIdx.x / kTW;
    const int x = x0 + lx, y = y0 + ly;
    if (x >= W || y >= H) return;
    const size_t p = (size_t)y * W + x;
    depth[p] = u16_mm ? __fmul_rn((float)static_cast<const uint16_t*>(raw_depth)[p], 0.001f)
                      : static_cast<const float*>(raw_depth)[p];
    color_sobel_at(t, lx + 1, ly + 1, double_scale, p, rgb, gx, gy);
}

// One pyrDown level and its outputs.  The CTA's window of the finer 8-bit
// level (the 5-tap footprint of its pixels and of their Sobel halo, read
// through reflect-101) is staged in shared memory; the level's 8-bit colour
// is filtered there (separably, exact in integers) for the pixels and the
// halo (halo cells at the level's own reflect-101 positions), stored for the
// next level, and fed to the Sobel; the depth is filtered per pixel from the
// finer level's depth.
__global__ void __launch_bounds__(kTW * kTH) prep_level_kernel(const uint8_t* __restrict__ prev,
                                                               const float* __restrict__ prev_depth, int Wp, int Hp,
                                                               int double_scale, uint8_t* __restrict__ cur,
                                                               float* __restrict__ rgb, float* __restrict__ gx,
                                                               float* __restrict__ gy, float* __restrict__ depth) {
    pdl_begin();
    __shared__ uint8_t sp[kSH][kSW * 3];
    __shared__ uint16_t hs[kSH][kHW * 3];
    __shared__ uint8_t t[kHH][kHW * 3];
    const int W = (Wp + 1) / 2, H = (Hp + 1) / 2;
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    // the window starts at the first tap of level pixel x0 - 1
    const int cx0 = 2 * x0 - 4, cy0 = 2 * y0 - 4;
    for (int i = threadIdx.x; i < kSH * kSW; i += kTW * kTH) {
        const int sy = i / kSW, sx = i - sy * kSW;
        // taps of the level's pixels and halo lie in [-2, Wp + 1]; clamp the
        // window's unused cells into that range before reflecting
        const int xs = reflect101(max(-2, min(cx0 + sx, Wp + 1)), Wp);
        const int ys = reflect101(max(-2, min(cy0 + sy, Hp + 1)), Hp);
        const uint8_t* q = prev + ((size_t)ys * Wp + xs) * 3;
        sp[sy][3 * sx] = q[0];
        sp[sy][3 * sx + 1] = q[1];
        sp[sy][3 * sx + 2] = q[2];
    }
    __syncthreads();
    // separable filter, exact in integers: horizontal 5-tap sums (at most
    // 16 * 255) of every window row at every level column of the pixels and
    // halo, then the vertical sums of those
    const int wts[5] = {1, 4, 6, 4, 1};
    for (int i = threadIdx.x; i < kSH * kHW; i += kTW * kTH) {
        const int r = i / kHW, hx = i - r * kHW;
        const int bx = 2 * reflect101(min(x0 + hx - 1, W), W) - 2 - cx0;  // first tap in the window
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            int h = 0;
#pragma unroll
            for (int kx = 0; kx < 5; ++kx) h += wts[kx] * sp[r][3 * (bx + kx) + ch];
            hs[r][3 * hx + ch] = (uint16_t)h;
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kHH * kHW; i += kTW * kTH) {
        const int hy = i / kHW, hx = i - hy * kHW;
        const int by = 2 * reflect101(min(y0 + hy - 1, H), H) - 2 - cy0;
        const bool own = hx >= 1 && hx <= kTW && hy >= 1 && hy <= kTH && x0 + hx - 1 < W && y0 + hy - 1 < H;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            int v = 0;
#pragma unroll
            for (int ky = 0; ky < 5; ++ky) v += wts[ky] * hs[by + ky][3 * hx + ch];
            const uint8_t u = (uint8_t)((v + 128) >> 8);
            t[hy][3 * hx + ch] = u;
            if (own) cur[((size_t)(y0 + hy - 1) * W + (x0 + hx - 1)) * 3 + ch] = u;
        }
    }
    __syncthreads();
    const int lx = threadIdx.x % kTW, ly = threadIdx.x / kTW;
    const int x = x0 + lx, y = y0 + ly;
    if (x >= W || y >= H) return;
    const size_t p = (size_t)y * W + x;
    // depth: row sums then column sums, times 1/256, each op rounded
    const float fw[5] = {1.f, 4.f, 6.f, 4.f, 1.f};
    int xs[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xs[k] = reflect101(2 * x + k - 2, Wp);
    float s = 0.f;
#pragma unroll
    for (int ky = 0; ky < 5; ++ky) {
        const float* row = prev_depth + (size_t)reflect101(2 * y + ky - 2, Hp) * Wp;
        float r = 0.f;
#pragma unroll
        for (int kx = 0; kx < 5; ++kx) r = __fadd_rn(r, __fmul_rn(fw[kx], row[xs[kx]]));
        s = __fadd_rn(s, __fmul_rn(fw[ky], r));
    }
    depth[p] = __fmul_rn(s, 1.0f / 256.0f);
    color_sobel_at(t, lx + 1, ly + 1, double_scale, p, rgb, gx, gy);
}

cudaError_t launch_prep_level0(const uint8_t* img, const void* raw_depth, int u16_mm, int W, int H, int double_scale,
                               float* rgb, float* gx, float* gy, float* depth, cudaStream_t s) {
    if (W <= 0 || H <= 0) return cudaSuccess;
    return launch_chained(prep_level0_kernel, dim3((W + kTW - 1) / kTW, (H + kTH - 1) / kTH), dim3(kTW * kTH), 0,
                          s, img, raw_depth, u16_mm, W, H, double_scale, rgb, gx, gy, depth);
}

cudaError_t launch_prep_level(const uint8_t* prev, const float* prev_depth, int Wp, int Hp, int double_scale,
                              uint8_t* cur, float* rgb, float* gx, float* gy, float* depth, cudaStream_t s) {
    const int W = (Wp + 1) / 2, H = (Hp + 1) / 2;
    if (Wp <= 0 || Hp <= 0) return cudaSuccess;
    return launch_chained(prep_level_kernel, dim3((W + kTW - 1) / kTW, (H + kTH - 1) / kTH), dim3(kTW * kTH), 0, s,
                          prev, prev_depth, Wp, Hp, double_scale, cur, rgb, gx, gy, depth);
}

}  // namespace fvgs
