// render.cu -- render-form forward pass (the viewer's image) for sm_103a.
//
// Reference: forwardPassTileKernel (src/GSCudaKernels.cu:710-859) launched by
// GSSlam::rasterize / renderView (src/GSSlam.cu:648-799).  Its semantics
// differ from the tracking kernel's forward blend:
//  * the inverse 2D covariance is taken in its true (xx, xy, yy) layout (the
//    kernel inverts Sigma2D itself, 817, so the stored-layout swap of the
//    tracking kernels does not apply);
//  * every Gaussian of the tile list blends with w = opacity *
//    exp(-0.5 (ixx dx^2 + iyy dy^2 + 2 ixy dx dy)), d = pixel - mean: no 0.99
//    clamp, no 1/255 threshold, no v <= 0 skip (a negative opacity blends a
//    negative weight, as there);
//  * colour += (1 - A) w c, A += (1 - A) w; a pixel stops once A >= 0.99
//    (the transmittance 1 - A is carried here as T <- T (1 - w), the same
//    quantity without the cancellation of 1 - A near A = 0.99);
//  * median depth z + phat . d at the first crossing of 1 - A through 0.5,
//    1e10 where there is none; no background colour.
// The reference writes its float3 colour into an 8-bit, 3-channel image (an
// overrun); here the image is a float RGB buffer, with an optional 8-bit copy
// (round(255 c), saturated).
#include <type_traits>

#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

constexpr int kRPix = 256;  // 16 x 16 pixels per tile

// w = o exp(-q/2) as 2^t with t = log2|o| + c'xx dx^2 + 2 c'xy dx dy +
// c'yy dy^2, the inverse covariance pre-scaled by -log2(e)/2 once per staged
// Gaussian: five FP32 ops and the PTX ex2.approx per pair (the tracking
// kernels' weight, without their thresholds).  The exponent's FP32 rounding
// adds about 1.4e-7 |t| relative error to w, so under 3e-6 wherever
// w > 2^-20.  Opacity zero gives w = 0, NaN gives NaN, as o exp(..) does; a
// batch holding a negative opacity takes the loop that applies its sign.
constexpr float kNegHalfLog2e = -0.72134752044448170368f;

__global__ void __launch_bounds__(kRPix) render_view_kernel(RenderArgs a) {
    pdl_begin();
    __shared__ float4 sA[kRPix];  // u, v, log2|opacity|, z
    __shared__ float4 sB[kRPix];  // c'xx, 2 c'xy, c'yy, phat.x
    __shared__ float4 sC[kRPix];  // phat.y, r, g, b
    __shared__ float sS[kRPix];   // sign of the opacity (read only by batches with a negative one)
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int tid = threadIdx.x;
    const int x = tx * 16 + (tid & 15), y = ty * 16 + (tid >> 4);
    const bool inside = x < a.W && y < a.H;
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    const int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    const bool swap = (a.quirks & FVGS_Q_INVSIGMA_SWAP) != 0;
    const float px = (float)x, py = (float)y;
    float cr = 0.f, cg = 0.f, cb = 0.f, T = 1.f, depth = 1e10f;
    bool has_depth = false, done = !inside;

    // one pair; NEG: the weight takes the sign of the Gaussian's opacity
    auto blend = [&](int j, auto neg_tag) {
        constexpr bool NEG = decltype(neg_tag)::value;
        const float4 gA = sA[j];
        const float4 gB = sB[j];
        const float dx = px - gA.x, dy = py - gA.y;
        const float t = __fmaf_rn(dx, __fmaf_rn(gB.x, dx, __fmul_rn(gB.y, dy)),
                                  __fmaf_rn(__fmul_rn(gB.z, dy), dy, gA.z));
        float w;
        asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(w) : "f"(t));
        if (NEG) w *= sS[j];
        const float Tb = T;
        const float Tw = Tb * w;
        const float4 gC = sC[j];
        cr += Tw * gC.y;
        cg += Tw * gC.z;
        cb += Tw * gC.w;
        T = Tb * (1.0f - w);  // 1 - A of the reference, without the cancellation
        if (!has_depth && Tb > 0.5f && T <= 0.5f) {
            depth = gA.w + gB.w * dx + gC.x * dy;
            has_depth = true;
        }
        if (T <= 0.01f) done = true;  // A >= 0.99
    };

    for (int base = 0; base < n; base += kRPix) {
        if (__syncthreads_and(done)) break;
        const int li = base + tid;
        bool neg = false;
        if (li < n) {
            const uint32_t g = a.indices[range.x + li];
            float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0;
            if (g < a.n_gauss) {
                r0 = a.rec0[g];
                r1 = a.rec1[g];
                r2 = a.rec2[g];
            }
            // the packed record holds the inverse in the tracking kernels'
            // consumed order; undo the swap for the true layout
            const float ixy = swap ? r1.z : r1.y, iyy = swap ? r1.y : r1.z;
            neg = r0.w < 0.f;
            sA[tid] = make_float4(r0.x, r0.y, log2f(fabsf(r0.w)), r0.z);
            sB[tid] = make_float4(kNegHalfLog2e * r1.x, 2.0f * kNegHalfLog2e * ixy, kNegHalfLog2e * iyy, r1.w);
            sC[tid] = r2;
            sS[tid] = neg ? -1.0f : 1.0f;
        }
        const bool any_neg = __syncthreads_or(neg);
        const int cnt = min(kRPix, n - base);
        if (!any_neg) {
            for (int j = 0; j < cnt && !done; ++j) blend(j, std::false_type{});
        } else {
            for (int j = 0; j < cnt && !done; ++j) blend(j, std::true_type{});
        }
    }
    if (!inside) return;
    const size_t p = (size_t)y * a.W + x;
    a.out_rgb[3 * p] = cr;
    a.out_rgb[3 * p + 1] = cg;
    a.out_rgb[3 * p + 2] = cb;
    a.out_depth[p] = depth;
    if (a.out_rgb8) {
        a.out_rgb8[3 * p] = (uint8_t)__float2int_rn(__saturatef(cr) * 255.0f);
        a.out_rgb8[3 * p + 1] = (uint8_t)__float2int_rn(__saturatef(cg) * 255.0f);
        a.out_rgb8[3 * p + 2] = (uint8_t)__float2int_rn(__saturatef(cb) * 255.0f);
    }
}

cudaError_t launch_render_view(const RenderArgs& a, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    return launch_chained(render_view_kernel, dim3(T), dim3(kRPix), 0, s, a);
}

}  // namespace fvgs
