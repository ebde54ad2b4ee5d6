// preprocess.cu -- frame preprocessing on the GPU for sm_103a.
//
// Reference: GSSlam::initAndCopyImgs (src/GSSlam.cu:1913-1969), which runs on
// the host for every frame: an image pyramid by cv::pyrDown (8-bit colour,
// float depth; uint16 millimetre depth is first scaled by 0.001), then per
// level the colour as float / 255 and its 3x3 Sobel derivatives
// (cv::Sobel(.., CV_32F, 1, 0, 3) and (0, 1, 3)), uploaded as the tracking
// inputs.  Here the camera frame is copied to the device once and every level
// is produced there:
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

__global__ void pyrdown_u8_kernel(const uint8_t* __restrict__ src, int W, int H, int c, uint8_t* __restrict__ dst) {
    const int W2 = (W + 1) / 2, H2 = (H + 1) / 2;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W2 || y >= H2) return;
    const int wts[5] = {1, 4, 6, 4, 1};
    int xs[5], ys[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        xs[k] = reflect101(2 * x + k - 2, W);
        ys[k] = reflect101(2 * y + k - 2, H);
    }
    for (int ch = 0; ch < c; ++ch) {
        int s = 0;
#pragma unroll
        for (int ky = 0; ky < 5; ++ky) {
            int r = 0;
#pragma unroll
            for (int kx = 0; kx < 5; ++kx) r += wts[kx] * src[((size_t)ys[ky] * W + xs[kx]) * c + ch];
            s += wts[ky] * r;
        }
        dst[((size_t)y * W2 + x) * c + ch] = (uint8_t)((s + 128) >> 8);
    }
}

__global__ void pyrdown_f32_kernel(const float* __restrict__ src, int W, int H, float* __restrict__ dst) {
    const int W2 = (W + 1) / 2, H2 = (H + 1) / 2;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W2 || y >= H2) return;
    const float wts[5] = {1.f, 4.f, 6.f, 4.f, 1.f};
    int xs[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) xs[k] = reflect101(2 * x + k - 2, W);
    float s = 0.f;
#pragma unroll
    for (int ky = 0; ky < 5; ++ky) {
        const float* row = src + (size_t)reflect101(2 * y + ky - 2, H) * W;
        float r = 0.f;
#pragma unroll
        for (int kx = 0; kx < 5; ++kx) r = __fadd_rn(r, __fmul_rn(wts[kx], row[xs[kx]]));
        s = __fadd_rn(s, __fmul_rn(wts[ky], r));
    }
    dst[(size_t)y * W2 + x] = __fmul_rn(s, 1.0f / 256.0f);
}

// Depth of the camera frame in metres: float as is, or uint16 millimetres.
__global__ void depth_in_kernel(const void* __restrict__ src, int u16_mm, size_t n, float* __restrict__ dst) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst[i] = u16_mm ? __fmul_rn((float)static_cast<const uint16_t*>(src)[i], 0.001f)
                    : static_cast<const float*>(src)[i];
}

__device__ __forceinline__ float u8f(const uint8_t* img, int W, int x, int y, int ch) {
    return __fmul_rn((float)img[((size_t)y * W + x) * 3 + ch], 1.0f / 255.0f);
}

// Colour to float (/255, and /255 again for the observed image with
// double_scale) and its Sobel derivatives, one pixel per thread.
__global__ void color_sobel_kernel(const uint8_t* __restrict__ img, int W, int H, int double_scale,
                                   float* __restrict__ rgb, float* __restrict__ gx, float* __restrict__ gy) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const int xm = reflect101(x - 1, W), xp = reflect101(x + 1, W);
    const int ym = reflect101(y - 1, H), yp = reflect101(y + 1, H);
    const size_t p = (size_t)y * W + x;
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float f = u8f(img, W, x, y, ch);
        rgb[3 * p + ch] = double_scale ? __fmul_rn(f, 1.0f / 255.0f) : f;
        const float a = __fsub_rn(u8f(img, W, xp, ym, ch), u8f(img, W, xm, ym, ch));
        const float b = __fsub_rn(u8f(img, W, xp, y, ch), u8f(img, W, xm, y, ch));
        const float c = __fsub_rn(u8f(img, W, xp, yp, ch), u8f(img, W, xm, yp, ch));
        gx[3 * p + ch] = __fadd_rn(__fadd_rn(a, __fmul_rn(2.0f, b)), c);
        const float d = __fsub_rn(u8f(img, W, xm, yp, ch), u8f(img, W, xm, ym, ch));
        const float e = __fsub_rn(u8f(img, W, x, yp, ch), u8f(img, W, x, ym, ch));
        const float f2 = __fsub_rn(u8f(img, W, xp, yp, ch), u8f(img, W, xp, ym, ch));
        gy[3 * p + ch] = __fadd_rn(__fadd_rn(d, __fmul_rn(2.0f, e)), f2);
    }
}

static dim3 grid2(int W, int H) { return dim3((W + 31) / 32, (H + 7) / 8); }

cudaError_t launch_pyrdown_u8(const uint8_t* src, int W, int H, int c, uint8_t* dst, cudaStream_t s) {
    pyrdown_u8_kernel<<<grid2((W + 1) / 2, (H + 1) / 2), dim3(32, 8), 0, s>>>(src, W, H, c, dst);
    return cudaGetLastError();
}

cudaError_t launch_pyrdown_f32(const float* src, int W, int H, float* dst, cudaStream_t s) {
    pyrdown_f32_kernel<<<grid2((W + 1) / 2, (H + 1) / 2), dim3(32, 8), 0, s>>>(src, W, H, dst);
    return cudaGetLastError();
}

cudaError_t launch_depth_in(const void* src, int u16_mm, size_t n, float* dst, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    depth_in_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, u16_mm, n, dst);
    return cudaGetLastError();
}

cudaError_t launch_color_sobel(const uint8_t* img, int W, int H, int double_scale, float* rgb, float* gx, float* gy,
                               cudaStream_t s) {
    color_sobel_kernel<<<grid2(W, H), dim3(32, 8), 0, s>>>(img, W, H, double_scale, rgb, gx, gy);
    return cudaGetLastError();
}

}  // namespace fvgs
