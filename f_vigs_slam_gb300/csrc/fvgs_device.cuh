// fvgs_device.cuh -- device-side layouts and helpers shared by the sm_103a
// kernels of the fvgs library.
//
// HBM layout (one session):
//   Gaussians, SoA of 16-byte vectors (read with 128-bit loads):
//     g_pos[N]   float4 (x, y, z, 0)
//     g_scale[N] float4 (sx, sy, sz, 0)
//     g_rot[N]   float4 (x, y, z, w)      raw quaternion as the reference reads it
//     g_col[N]   float4 (r, g, b, opacity)
//   Blending record, 48 B per Gaussian (three float4 planes):
//     rec0 = (u, v, z, opacity)
//     rec1 = (c.x, c.y, c.z, phat.x)      c = inverse 2D covariance in the order
//     rec2 = (phat.y, r, g, b)             the blending kernels consume it
//   Reduced-precision attributes (precision form; the float4 planes stay the
//   master copy that mapping updates):
//     g_sr[N]    uint4 scale bf16 x3, rotation bf16 x4 (raw order), 2 B spare
//     g_c[N]     uint2 colour and opacity fp16 x4
//   Binning record, 32 B per Gaussian: (rect x0|y0<<16, x1|y1<<16, count,
//     phat.y bits, u, v, z, phat.x).
//   Instances: u64 key = tile << 32 | float bits of the tile-centre depth,
//     u32 value = Gaussian index; two ping-pong buffers for the radix sort.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/fvgs_types.h"

namespace fvgs {

constexpr uint32_t kFullMask = 0xffffffffu;

// Device-side status word bits (session->status[0]); host reads after a step.
constexpr uint32_t kErrOverflow = 1u << 0;  // instance capacity exceeded
constexpr uint32_t kErrTimeout = 1u << 1;   // bounded wait gave up
constexpr uint32_t kErrBounds = 1u << 2;    // index check failed (debug builds)

// Status block layout in device memory (u32 words).
struct DevStatus {
    uint32_t flags;         // kErr* bits
    uint32_t n_instances;   // total instances of the last binning (may exceed capacity)
    uint32_t n_instances_clamped;  // min(total, capacity): the number sorted
    uint32_t mode;          // last binning: kBinFull or kBinIncremental
    uint32_t n_enter;       // last binning: instances new to their tile since the binning before
    uint32_t n_changed;     // last binning: Gaussians with such instances
    uint32_t pad[2];
};

// Binning modes.  Full: every instance is scattered into its tile bucket and
// each bucket is sorted.  Incremental (a previous binning of the same Gaussians
// on the same tile grid exists): each tile keeps the members of its previous
// sorted list that are still inside their Gaussian's new tile rectangle, in
// their previous order, and appends only the instances that entered it; the
// adaptive per-tile sort then has little left to do.  Both give identical
// results.
constexpr uint32_t kBinFull = 0;
constexpr uint32_t kBinIncremental = 1;

// Pose state kept on the device so a whole tracking frame runs without the host.
struct DevPose {
    float t[3];
    float q[4];     // (x, y, z, w) as the kernels read it
    float pad;
    double td[3];   // master copy of the GN iterate
    double qd[4];
};

// quaternionToMatrix (src/GSCudaKernels.cu:319-334) with the fixed FP32
// operation order shared with the CPU restatement (bit-exact keys).
__device__ __forceinline__ void quat_to_R(const float q[4], float R[3][3]) {
    const float x = q[0], y = q[1], z = q[2], w = q[3];
    R[0][0] = __fmaf_rn(-2.f, __fmaf_rn(y, y, __fmul_rn(z, z)), 1.f);
    R[0][1] = __fmul_rn(2.f, __fmaf_rn(x, y, -__fmul_rn(w, z)));
    R[0][2] = __fmul_rn(2.f, __fmaf_rn(x, z, __fmul_rn(w, y)));
    R[1][0] = __fmul_rn(2.f, __fmaf_rn(x, y, __fmul_rn(w, z)));
    R[1][1] = __fmaf_rn(-2.f, __fmaf_rn(x, x, __fmul_rn(z, z)), 1.f);
    R[1][2] = __fmul_rn(2.f, __fmaf_rn(y, z, -__fmul_rn(w, x)));
    R[2][0] = __fmul_rn(2.f, __fmaf_rn(x, z, -__fmul_rn(w, y)));
    R[2][1] = __fmul_rn(2.f, __fmaf_rn(y, z, __fmul_rn(w, x)));
    R[2][2] = __fmaf_rn(-2.f, __fmaf_rn(x, x, __fmul_rn(y, y)), 1.f);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Tile-rectangle record of the binning (bin0): x0 | y0 << 16, x1 | y1 << 16
// (inclusive), instance count (0: no instances), phat.y bits.
__device__ __forceinline__ bool rect_contains(uint4 b0, int tx, int ty) {
    return b0.z != 0u && tx >= (int)(b0.x & 0xffffu) && tx <= (int)(b0.y & 0xffffu) && ty >= (int)(b0.x >> 16) &&
           ty <= (int)(b0.y >> 16);
}

// Tiles of rectangle R1 = [x0..x1] x [y0..y1] outside R0 (has_prev: R0 =
// [px0..px1] x [py0..py1]), as at most four rectangles around their
// intersection I in a fixed order: rows above I, rows below I (full width),
// columns left of I, columns right of I (rows of I).  entering_count gives
// their number, entering_tile the local-th of them.
struct EnterSplit {
    int x0, y0, x1, y1;      // R1
    int ix0, iy0, ix1, iy1;  // I (when overlapping)
    bool whole;              // no overlap: every tile of R1 enters
};
__device__ __forceinline__ EnterSplit enter_split(int x0, int y0, int x1, int y1, bool has_prev, int px0, int py0,
                                                  int px1, int py1) {
    EnterSplit e;
    e.x0 = x0;
    e.y0 = y0;
    e.x1 = x1;
    e.y1 = y1;
    e.ix0 = max(x0, px0);
    e.ix1 = min(x1, px1);
    e.iy0 = max(y0, py0);
    e.iy1 = min(y1, py1);
    e.whole = !has_prev || e.ix0 > e.ix1 || e.iy0 > e.iy1;
    return e;
}
__device__ __forceinline__ uint32_t entering_count(const EnterSplit& e) {
    const uint32_t all = (uint32_t)((e.x1 - e.x0 + 1) * (e.y1 - e.y0 + 1));
    return e.whole ? all : all - (uint32_t)((e.ix1 - e.ix0 + 1) * (e.iy1 - e.iy0 + 1));
}
__device__ __forceinline__ void entering_tile(const EnterSplit& e, uint32_t local, int& tx, int& ty) {
    const int w = e.x1 - e.x0 + 1;
    if (e.whole) {
        tx = e.x0 + (int)(local % (uint32_t)w);
        ty = e.y0 + (int)(local / (uint32_t)w);
        return;
    }
    const uint32_t top = (uint32_t)((e.iy0 - e.y0) * w);
    if (local < top) {
        tx = e.x0 + (int)(local % (uint32_t)w);
        ty = e.y0 + (int)(local / (uint32_t)w);
        return;
    }
    local -= top;
    const uint32_t bottom = (uint32_t)((e.y1 - e.iy1) * w);
    if (local < bottom) {
        tx = e.x0 + (int)(local % (uint32_t)w);
        ty = e.iy1 + 1 + (int)(local / (uint32_t)w);
        return;
    }
    local -= bottom;
    const int wl = e.ix0 - e.x0, h = e.iy1 - e.iy0 + 1;
    if (local < (uint32_t)(wl * h)) {
        tx = e.x0 + (int)(local % (uint32_t)wl);
        ty = e.iy0 + (int)(local / (uint32_t)wl);
        return;
    }
    local -= (uint32_t)(wl * h);
    const int wr = e.x1 - e.ix1;
    tx = e.ix1 + 1 + (int)(local % (uint32_t)wr);
    ty = e.iy0 + (int)(local / (uint32_t)wr);
}

// Depth of a Gaussian at the centre of tile (tx, ty) -- the sort key of the
// reference's generateTileHashes_kernel (src/GSCudaKernels.cu:596-667),
// z + pHat.x * dx + pHat.y * dy with d = tile centre - projected mean, as the
// reference's nvcc build evaluates it: the first product fused with z, the
// second rounded and added, fmaf(phx, dx, z) + phy * dy (matched bit for bit
// against keys of that build).
__device__ __forceinline__ float tile_depth(int tx, int ty, int tw, int th, float u, float v, float z, float phx,
                                            uint32_t phy_bits) {
    const float tcx = __fmul_rn(__fadd_rn((float)tx, 0.5f), (float)tw);
    const float tcy = __fmul_rn(__fadd_rn((float)ty, 0.5f), (float)th);
    const float dx = __fsub_rn(tcx, u);
    const float dy = __fsub_rn(tcy, v);
    return __fadd_rn(__fmaf_rn(phx, dx, z), __fmul_rn(__uint_as_float(phy_bits), dy));
}

// Programmatic dependent launch.  Kernels of the binning / tracking / mapping
// chains are launched with programmatic stream serialisation: each lets the
// next kernel be scheduled once all of its own CTAs have started, and waits
// (in hardware, until its predecessor grid has completed and its memory is
// visible) before touching any data.  Outside such a launch both are no-ops.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// A Gaussian of opacity o yields alpha = min(0.99, o exp(-v/2)) < 1/255
// (with or without the clamp) exactly when v > 2 ln(255 o).  The bound
// returned is that value plus a margin far above the rounding of expf and of
// the product, so pairs beyond it are rejected without evaluating the
// exponential, with the same outcome.
__device__ __forceinline__ float reject_bound(float o) {
    if (!(o > 0.0f)) return -INFINITY;
    const float b = 2.0f * logf(255.0f * o);
    return b + 1e-3f + 1e-4f * fabsf(b);
}

// The conic's quadratic form v = a dx^2 + 2 b dx dy + c dy^2, evaluated as
// dx * dl0 + dy * dl1 with dl0 = a dx + b dy, dl1 = b dx + c dy: the
// gradient terms the backward passes need come for free.  A pass that
// re-derives another pass's per-pixel accept / reject decisions uses the same
// expression (the tracking passes, the mapping forward and backward).
__device__ __forceinline__ float conic_form(float a, float b, float c, float dx, float dy, float& dl0, float& dl1) {
    dl0 = __fmaf_rn(a, dx, __fmul_rn(b, dy));
    dl1 = __fmaf_rn(b, dx, __fmul_rn(c, dy));
    return __fmaf_rn(dx, dl0, __fmul_rn(dy, dl1));
}

// alpha = min(0.99, o exp(-v / 2)) from log2(o), computed once per Gaussian:
// o exp(-v/2) = 2^(log2 o - v log2(e) / 2), one FMA and the PTX ex2.approx
// (about 2 ulp; the FP32 rounding of the exponent adds under 7e-7 relative
// where alpha >= 1/255).  A pass that re-derives another pass's alphas uses
// it too (the tracking passes; the mapping forward and backward).
// log2 of an opacity for gauss_weight / gauss_alpha.  A non-positive (or
// NaN) opacity maps to -inf, i.e. weight 0: such a Gaussian never reaches
// alpha 1/255, as o exp(-v/2) <= 0 never does.
__device__ __forceinline__ float log2_opacity(float o) { return log2f(fmaxf(o, 0.0f)); }

__device__ __forceinline__ float gauss_weight(float log2_o, float v) {
    float e;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(e) : "f"(__fmaf_rn(v, -0.72134752044448170368f, log2_o)));
    return e;
}
__device__ __forceinline__ float gauss_alpha(float log2_o, float v) { return fminf(0.99f, gauss_weight(log2_o, v)); }

// PTX rcp.approx.f32 (at most one ulp from 1/x; subnormals kept).
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Reduced-precision attribute words (round to nearest even).
__device__ __forceinline__ uint32_t bf16_bits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bf16_val(uint32_t b) { return __bfloat162float(__ushort_as_bfloat16((unsigned short)b)); }
__device__ __forceinline__ uint32_t f16_bits(float x) { return __half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ float f16_val(uint32_t b) { return __half2float(__ushort_as_half((unsigned short)b)); }
__device__ __forceinline__ uint4 pack_sr(float4 s, float4 q) {
    return make_uint4(bf16_bits(s.x) | (bf16_bits(s.y) << 16), bf16_bits(s.z) | (bf16_bits(q.x) << 16),
                      bf16_bits(q.y) | (bf16_bits(q.z) << 16), bf16_bits(q.w));
}
__device__ __forceinline__ uint2 pack_c(float4 c) {
    return make_uint2(f16_bits(c.x) | (f16_bits(c.y) << 16), f16_bits(c.z) | (f16_bits(c.w) << 16));
}
__device__ __forceinline__ void unpack_sr(uint4 w, float4& s, float4& q) {
    s = make_float4(bf16_val(w.x & 0xffffu), bf16_val(w.x >> 16), bf16_val(w.y & 0xffffu), 0.f);
    q = make_float4(bf16_val(w.y >> 16), bf16_val(w.z & 0xffffu), bf16_val(w.z >> 16), bf16_val(w.w & 0xffffu));
}
__device__ __forceinline__ float4 unpack_c(uint2 w) {
    return make_float4(f16_val(w.x & 0xffffu), f16_val(w.x >> 16), f16_val(w.y & 0xffffu), f16_val(w.y >> 16));
}

// Bounded spin budget for device-side waits; on expiry a kernel records
// kErrTimeout and carries on with a safe value instead of hanging.
constexpr uint32_t kSpinLimit = 1u << 24;

}  // namespace fvgs
