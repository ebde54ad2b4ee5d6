// seed.cu -- Gaussians seeded from an RGB-D frame on sm_103a: the first map
// (RGB-D initialisation) and densification where the map misses the frame.
//
// Reference: GSSlam::initializeGaussiansFromRgbd (src/GSSlam.cu:271-407) with
// computeNormalsFromDepth_kernel + initGaussiansFromRgbd_kernel
// (src/GSCudaKernels.cu:87-315), and GSSlam::densify (src/GSSlam.cu:1351-1465)
// with computeDensityMask_kernel + densifyGaussians_kernel
// (src/GSCudaKernels.cu:1741-2066).
//
// Seeds come from a grid of sample cells (one pixel each for the
// initialisation).  The reference reserves each seed's slot with an atomic
// counter, so its order is whatever the hardware makes it; here a seed's slot
// is its rank among the seeding cells in row-major order: count (per-block
// seed counts) -> scan (the compaction scan) -> emit (each cell recomputes its
// seed and writes it at that rank, if below the capacity).  The outcome is one
// of the reference's possible outcomes, and it is deterministic.
//
// Arithmetic: FP32 in the reference's operation order, every product, sum,
// quotient and square root an explicitly rounded intrinsic (no contraction),
// so the seeds match the CPU restatement bit for bit.  The reference's
// quaternion helpers (src/GSCudaKernels.cu:20-84) read and write float4 as
// (w, x, y, z): the camera orientation is taken raw in that order and the
// seeds' orientations are written in it.  The per-pixel normal of the
// initialisation is computed inline from the five depth values it needs.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

namespace {

struct V3 {
    float x, y, z;
};

__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ V3 cross(V3 a, V3 b) {
    return {sub(mul(a.y, b.z), mul(a.z, b.y)), sub(mul(a.z, b.x), mul(a.x, b.z)), sub(mul(a.x, b.y), mul(a.y, b.x))};
}
__device__ __forceinline__ float norm3(V3 a) { return __fsqrt_rn(add(add(mul(a.x, a.x), mul(a.y, a.y)), mul(a.z, a.z))); }

// rotateByQuaternion: q = (w, x, y, z), t = 2 (qv x v), v + w t + qv x t
__device__ __forceinline__ V3 quat_rotate(float4 q, V3 v) {
    const V3 qv = {q.y, q.z, q.w};
    const V3 c = cross(qv, v);
    const V3 t = {mul(2.0f, c.x), mul(2.0f, c.y), mul(2.0f, c.z)};
    const V3 c2 = cross(qv, t);
    return {add(add(v.x, mul(q.x, t.x)), c2.x), add(add(v.y, mul(q.x, t.y)), c2.y), add(add(v.z, mul(q.x, t.z)), c2.z)};
}

__device__ __forceinline__ float4 quat_mul(float4 a, float4 b) {
    const float aw = a.x, ax = a.y, ay = a.z, az = a.w;
    const float bw = b.x, bx = b.y, by = b.z, bz = b.w;
    float4 o;
    o.x = sub(sub(sub(mul(aw, bw), mul(ax, bx)), mul(ay, by)), mul(az, bz));
    o.y = sub(add(add(mul(aw, bx), mul(ax, bw)), mul(ay, bz)), mul(az, by));
    o.z = add(add(sub(mul(aw, by), mul(ax, bz)), mul(ay, bw)), mul(az, bx));
    o.w = add(sub(add(mul(aw, bz), mul(ax, by)), mul(ay, bx)), mul(az, bw));
    return o;
}

__device__ __forceinline__ V3 normalize8(V3 v) {
    const float n = norm3(v);
    if (n > 1e-8f) {
        const float inv = dv(1.0f, n);
        return {mul(v.x, inv), mul(v.y, inv), mul(v.z, inv)};
    }
    return {0.0f, 0.0f, 0.0f};
}

__device__ __forceinline__ float4 quat_from_two(V3 from, V3 to) {
    const V3 u = normalize8(from), v = normalize8(to);
    const float dot = add(add(mul(u.x, v.x), mul(u.y, v.y)), mul(u.z, v.z));
    if (dot < -0.999999f) {
        const V3 axis = (fabsf(u.x) < 0.1f) ? V3{1.0f, 0.0f, 0.0f} : V3{0.0f, 1.0f, 0.0f};
        const V3 o = normalize8(cross(u, axis));
        return make_float4(0.0f, o.x, o.y, o.z);
    }
    const V3 c = cross(u, v);
    float4 q = make_float4(add(1.0f, dot), c.x, c.y, c.z);
    const float n = __fsqrt_rn(add(add(add(mul(q.x, q.x), mul(q.y, q.y)), mul(q.z, q.z)), mul(q.w, q.w)));
    if (n > 1e-8f) {
        const float inv = dv(1.0f, n);
        q = make_float4(mul(q.x, inv), mul(q.y, inv), mul(q.z, inv), mul(q.w, inv));
    } else {
        q = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    }
    return q;
}

// computeNormalsFromDepth_kernel for pixel (u, v)
__device__ __forceinline__ V3 depth_normal(const float* __restrict__ d, int W, int H, int u, int v) {
    V3 n = {0.0f, 0.0f, 1.0f};
    if (u > 0 && u < W - 1 && v > 0 && v < H - 1) {
        const size_t p = (size_t)v * W + u;
        const float zc = d[p], zl = d[p - 1], zr = d[p + 1], zu = d[p - W], zd = d[p + W];
        if (zc > 0.01f && zl > 0.01f && zr > 0.01f && zu > 0.01f && zd > 0.01f) {
            const float dzx = dv(sub(zr, zl), 2.0f), dzy = dv(sub(zd, zu), 2.0f);
            n = cross(V3{1.0f, 0.0f, dzx}, V3{0.0f, 1.0f, dzy});
            const float nn = norm3(n);
            if (nn > 1e-6f) n = {dv(n.x, nn), dv(n.y, nn), dv(n.z, nn)};
            if (n.z < 0.0f) n = {-n.x, -n.y, -n.z};
        }
    }
    return n;
}

__device__ __forceinline__ V3 rgb_at(const uint8_t* __restrict__ bgr, int W, int u, int v) {
    const uint8_t* p = bgr + ((size_t)v * W + u) * 3;
    return {dv((float)p[2], 255.0f), dv((float)p[1], 255.0f), dv((float)p[0], 255.0f)};
}

struct Seed {
    V3 pos, scale;
    float4 rot;
    V3 col;
    float opacity;
};

// One sample cell: whether it seeds a Gaussian, and (when `full`) the seed.
template <int MODE>
__device__ __forceinline__ bool seed_cell(const SeedArgs& a, int cell, bool full, Seed& out) {
    const int sx = cell % a.ncx, sy = cell / a.ncx;
    const float fx = a.K.fx, fy = a.K.fy, cx = a.K.cx, cy = a.K.cy;
    if (MODE == kSeedInit) {
        const int u = sx * a.sample, v = sy * a.sample;
        const float z = a.depth[(size_t)v * a.W + u];
        if (!(z > 0.0f) || isinf(z)) return false;
        if (!full) return true;
        V3 n = depth_normal(a.depth, a.W, a.H, u, v);
        const float nl = norm3(n);
        if (nl < 1e-6f) n = {0.0f, 0.0f, 1.0f};
        else n = {dv(n.x, nl), dv(n.y, nl), dv(n.z, nl)};
        const V3 pc = {dv(mul(sub((float)u, cx), z), fx), dv(mul(sub((float)v, cy), z), fy), z};
        const V3 r = quat_rotate(a.pose_q, pc);
        out.pos = {add(a.pose_t.x, r.x), add(a.pose_t.y, r.y), add(a.pose_t.z, r.z)};
        V3 nw = quat_rotate(a.pose_q, n);
        const float nwl = norm3(nw);
        if (nwl > 1e-6f) nw = {dv(nw.x, nwl), dv(nw.y, nwl), dv(nw.z, nwl)};
        const V3 zaxis = {0.0f, 0.0f, 1.0f};
        const V3 axis = cross(zaxis, nw);
        const float al = norm3(axis);
        const float ac = add(add(mul(zaxis.x, nw.x), mul(zaxis.y, nw.y)), mul(zaxis.z, nw.z));
        if (al < 1e-6f) {
            out.rot = ac > 0.0f ? make_float4(1.0f, 0.0f, 0.0f, 0.0f) : make_float4(0.0f, 1.0f, 0.0f, 0.0f);
        } else {
            const V3 ax = {dv(axis.x, al), dv(axis.y, al), dv(axis.z, al)};
            const float hs = __fsqrt_rn(fmaxf(0.0f, dv(sub(1.0f, ac), 2.0f)));
            const float hc = __fsqrt_rn(fmaxf(0.0f, dv(add(1.0f, ac), 2.0f)));
            out.rot = make_float4(hc, mul(hs, ax.x), mul(hs, ax.y), mul(hs, ax.z));
        }
        out.scale = {a.init_scale, a.init_scale, a.init_scale};
        out.col = rgb_at(a.bgr, a.W, u, v);
        out.opacity = a.init_opacity;
        return true;
    }
    // densify: the reference passes no normal map, so the seed's orientation
    // is the camera's, composed with the rotation from +z onto +z
    const float4 q = quat_mul(a.pose_q, quat_from_two(V3{0.0f, 0.0f, 1.0f}, V3{0.0f, 0.0f, 1.0f}));
    if (a.sample > 1) {
        const int u0 = sx * a.sample, v0 = sy * a.sample;
        V3 ip = {0.0f, 0.0f, 0.0f}, ca = {0.0f, 0.0f, 0.0f};
        int n = 0;
        for (int u = u0; u < u0 + a.sample && u < a.W; ++u)
            for (int v = v0; v < v0 + a.sample && v < a.H; ++v) {
                const size_t p = (size_t)v * a.W + u;
                if (!(a.mask[p] > 0.0f)) continue;
                const float d = a.depth[p];
                if (!(d > 0.0f)) continue;
                ++n;
                if (!full) continue;
                const V3 c = rgb_at(a.bgr, a.W, u, v);
                ip = {add(ip.x, (float)u), add(ip.y, (float)v), add(ip.z, d)};
                ca = {add(ca.x, c.x), add(ca.y, c.y), add(ca.z, c.z)};
            }
        if ((uint32_t)n < (((uint32_t)a.sample * (uint32_t)a.sample) >> 1)) return false;
        if (!full) return true;
        const float inv_n = dv(1.0f, (float)n);
        ip = {mul(ip.x, inv_n), mul(ip.y, inv_n), mul(ip.z, inv_n)};
        ca = {mul(ca.x, inv_n), mul(ca.y, inv_n), mul(ca.z, inv_n)};
        const V3 pc = {dv(mul(ip.z, sub(ip.x, cx)), fx), dv(mul(ip.z, sub(ip.y, cy)), fy), ip.z};
        const V3 r = quat_rotate(a.pose_q, pc);
        out.pos = {add(a.pose_t.x, r.x), add(a.pose_t.y, r.y), add(a.pose_t.z, r.z)};
        const float s = mul(0.5f, add(dv(mul(ip.z, (float)a.sample), fx), dv(mul(ip.z, (float)a.sample), fy)));
        out.scale = {s, s, mul(0.1f, s)};
        out.rot = q;
        out.col = ca;
        out.opacity = 1.0f;
        return true;
    }
    const size_t p = (size_t)sy * a.W + sx;
    if (!(a.mask[p] > 0.0f)) return false;
    const float d = a.depth[p];
    if (!(d > 0.0f)) return false;
    if (!full) return true;
    const V3 pc = {dv(mul(d, sub((float)sx, cx)), fx), dv(mul(d, sub((float)sy, cy)), fy), d};
    const V3 r = quat_rotate(a.pose_q, pc);
    out.pos = {add(a.pose_t.x, r.x), add(a.pose_t.y, r.y), add(a.pose_t.z, r.z)};
    const float d8 = mul(0.8f, d);
    const float s = mul(0.5f, add(dv(mul(d8, (float)a.sample), fx), dv(mul(d8, (float)a.sample), fy)));
    out.scale = {s, s, mul(0.1f, s)};
    out.rot = q;
    out.col = rgb_at(a.bgr, a.W, sx, sy);
    out.opacity = 1.0f;
    return true;
}

}  // namespace

template <int MODE>
__global__ void __launch_bounds__(kCompactBlock) seed_count_kernel(SeedArgs a) {
    pdl_begin();
    const int cell = blockIdx.x * kCompactBlock + threadIdx.x;
    Seed unused;
    const bool seeds = cell < a.ncx * a.ncy && seed_cell<MODE>(a, cell, false, unused);
    const int k = __syncthreads_count(seeds);
    if (threadIdx.x == 0) a.block_keep[blockIdx.x] = (uint32_t)k;
}

template <int MODE>
__global__ void __launch_bounds__(kCompactBlock) seed_emit_kernel(SeedArgs a) {
    pdl_begin();
    __shared__ uint32_t wsum[kCompactBlock / 32];
    const int cell = blockIdx.x * kCompactBlock + threadIdx.x;
    Seed sd;
    const bool seeds = cell < a.ncx * a.ncy && seed_cell<MODE>(a, cell, true, sd);
    const unsigned bal = __ballot_sync(0xffffffffu, seeds);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wsum[warp] = __popc(bal);
    __syncthreads();
    if (!seeds) return;
    uint32_t before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    const uint64_t dst = (uint64_t)a.n0 + a.block_base[blockIdx.x] + before + __popc(bal & ((1u << lane) - 1u));
    if (dst >= a.cap) return;
    a.pos[dst] = make_float4(sd.pos.x, sd.pos.y, sd.pos.z, 0.f);
    a.scale[dst] = make_float4(sd.scale.x, sd.scale.y, sd.scale.z, 0.f);
    a.rot[dst] = sd.rot;
    a.col[dst] = make_float4(sd.col.x, sd.col.y, sd.col.z, sd.opacity);
    if (a.adam) {
#pragma unroll
        for (int p = 0; p < 9; ++p) a.adam[(size_t)p * a.cap + dst] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
}

// computeDensityMask_kernel: one CTA per 16x16 tile, one thread per pixel.
__global__ void __launch_bounds__(256) density_mask_kernel(DensityArgs a) {
    pdl_begin();
    __shared__ float4 sA[256];  // u, v, opacity, c.x
    __shared__ float4 sB[256];  // c.y, c.z, z, phat.x
    __shared__ float sC[256];   // phat.y
    const int tile = blockIdx.x;
    const int tx = tile % a.ntx, ty = tile / a.ntx;
    const int tid = threadIdx.x;
    const int x = tx * 16 + (tid & 15), y = ty * 16 + (tid >> 4);
    const bool inside = x < a.W && y < a.H;
    const float d_obs = inside ? a.obs_depth[(size_t)y * a.W + x] : 0.f;
    uint2 range = a.ranges[tile];
    range.y = min(range.y, a.n_list);
    const int n = range.y > range.x ? (int)(range.y - range.x) : 0;
    const float px = (float)x, py = (float)y;
    float P = 1.f, T = 1.f, dr = 0.f;
    bool done = !inside || d_obs < 0.5f;
    for (int base = 0; base < n; base += 256) {
        if (__syncthreads_and(done)) break;
        const int li = base + tid;
        if (li < n) {
            const uint32_t g = a.indices[range.x + li];
            float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = r0, r2 = r0;
            if (g < a.n_gauss) {
                r0 = a.rec0[g];
                r1 = a.rec1[g];
                r2 = a.rec2[g];
            }
            sA[tid] = make_float4(r0.x, r0.y, r0.w, r1.x);
            sB[tid] = make_float4(r1.y, r1.z, r0.z, r1.w);
            sC[tid] = r2.x;
        }
        __syncthreads();
        const int cnt = min(256, n - base);
        for (int j = 0; j < cnt && !done; ++j) {
            const float4 gA = sA[j];
            const float4 gB = sB[j];
            const float dx = gA.x - px, dy = gA.y - py;
            const float v = gA.w * dx * dx + 2.0f * gB.x * dx * dy + gB.y * dy * dy;
            const float alpha = fminf(0.99f, gA.z * expf(-0.5f * v));
            if (alpha < 1.0f / 255.0f) continue;
            P *= 1.0f - alpha;
            if (T > 0.5f && P < 0.5f) {
                T = P;
                dr = gB.z + gB.w * dx + sC[j] * dy;
            }
            if (P < 0.0001f) done = true;
        }
    }
    if (!inside) return;
    float val = 0.f;
    if (d_obs > 0.5f) {
        if (P > 0.5f) val = P;
        else if (d_obs < dr && dr - d_obs > 0.2f * d_obs) val = 1.0f;
    }
    a.mask[(size_t)y * a.W + x] = val;
}

cudaError_t launch_seed_count(SeedMode mode, const SeedArgs& a, cudaStream_t s) {
    const int cells = a.ncx * a.ncy;
    if (cells <= 0) return cudaSuccess;
    const dim3 grid((cells + kCompactBlock - 1) / kCompactBlock);
    return mode == kSeedInit ? launch_chained(seed_count_kernel<kSeedInit>, grid, dim3(kCompactBlock), 0, s, a)
                             : launch_chained(seed_count_kernel<kSeedDensify>, grid, dim3(kCompactBlock), 0, s, a);
}

cudaError_t launch_seed_emit(SeedMode mode, const SeedArgs& a, cudaStream_t s) {
    const int cells = a.ncx * a.ncy;
    if (cells <= 0) return cudaSuccess;
    const dim3 grid((cells + kCompactBlock - 1) / kCompactBlock);
    return mode == kSeedInit ? launch_chained(seed_emit_kernel<kSeedInit>, grid, dim3(kCompactBlock), 0, s, a)
                             : launch_chained(seed_emit_kernel<kSeedDensify>, grid, dim3(kCompactBlock), 0, s, a);
}

cudaError_t launch_density_mask(const DensityArgs& a, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    return launch_chained(density_mask_kernel, dim3(T), dim3(256), 0, s, a);
}

}  // namespace fvgs
