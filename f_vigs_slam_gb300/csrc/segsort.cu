// segsort.cu -- per-tile sort of tile-bucketed instances for sm_103a.
//
// The reference sorts all (tile << 32 | depth bits) keys with a stable 64-bit
// radix sort (thrust::sort_by_key, src/GSSlam.cu:624-628).  A Gaussian has at
// most one instance per tile and instances are generated in Gaussian-index
// order, so inside a tile that stable order is exactly the order of the
// unique composite key (depth bits << 32 | Gaussian index).  Instances are
// therefore collected per tile and each tile is sorted on its own:
//  * full mode: the tile bucket was filled by the scatter (any order);
//  * incremental mode: the tile's previous sorted list, minus the members
//    that left the tile, with keys recomputed for the new pose, followed by
//    the entering instances -- nearly sorted;
//  * up to 4096 instances: one CTA, in shared memory -- every thread sorts 16
//    keys in registers with a bitonic network, then merge-path rounds double
//    the sorted runs.  Runs already in order (the common case for nearly
//    sorted input) are recognised by one comparison and left alone;
//  * larger tiles (rare: huge splats, culled slots piled into tile 0) are
//    listed by the first kernel and sorted by a second one: chunks of 4096 in
//    shared memory, then merge-path passes through global memory.
// The output is the sorted Gaussian indices; the reference-format keys are
// rebuilt on request (make_keys_kernel) since the blending kernels only read
// ranges and indices.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

constexpr int kSegThreads = 256;
constexpr int kSegItems = 16;
constexpr int kSegCap = kSegThreads * kSegItems;  // 4096
constexpr int kSmallItems = 8;                     // lists of up to 2048 keys
constexpr uint64_t kKeyInf = ~0ull;

__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }  // one pad word per 16 keys

// Sort ITEMS keys in registers (bitonic network, ascending).
template <int ITEMS>
__device__ __forceinline__ void sort_items(uint64_t (&k)[ITEMS]) {
#pragma unroll
    for (int sz = 2; sz <= ITEMS; sz <<= 1)
#pragma unroll
        for (int j = sz >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < ITEMS; ++i) {
                const int l = i ^ j;
                if (l > i) {
                    const bool up = (i & sz) == 0;
                    const uint64_t a = k[i], b = k[l];
                    if ((a > b) == up) {
                        k[i] = b;
                        k[l] = a;
                    }
                }
            }
}

// One merge-path round over runs of length L of s[0..m) (m a multiple of
// ITEMS): thread t produces outputs [ITEMS t, ITEMS (t + 1)) of the pair of runs
// containing them.
// Returns false when the pair is already in order (nothing to write).  Both
// run heads are re-read from shared memory each step (register-held heads
// measured slower: more registers, fewer resident CTAs).
template <int ITEMS>
__device__ __forceinline__ bool merge_round(const uint64_t* s, int t, int m, int L, uint64_t (&k)[ITEMS]) {
    const int per_pair = (2 * L) / ITEMS;
    const int ps = (t / per_pair) * 2 * L;
    const int d = (t % per_pair) * ITEMS;
    const int la = min(L, m - ps);
    const int lb = min(L, max(0, m - ps - L));
    if (lb == 0 || s[spad(ps + la - 1)] <= s[spad(ps + la)]) return false;
    int lo = max(0, d - lb), hi = min(d, la);
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s[spad(ps + mid)] <= s[spad(ps + la + d - 1 - mid)])
            lo = mid + 1;
        else
            hi = mid;
    }
    int ai = lo, bj = d - lo;
#pragma unroll
    for (int r = 0; r < ITEMS; ++r) {
        const uint64_t a = ai < la ? s[spad(ps + ai)] : kKeyInf;
        const uint64_t b = bj < lb ? s[spad(ps + la + bj)] : kKeyInf;
        const bool ta = a <= b;
        k[r] = ta ? a : b;
        ai += ta ? 1 : 0;
        bj += ta ? 0 : 1;
    }
    return true;
}

// Sort s[0..m) (padded layout, m a multiple of ITEMS, <= 256 ITEMS) in shared
// memory with the CTA.  Threads >= m/ITEMS only take part in the barriers.
// Lists of up to 2048 keys use ITEMS = 8, so every thread of the CTA sorts
// and merges instead of at most half of them.  While a merged pair spans at
// most one warp's 32 ITEMS keys the round touches only that warp's slice, so
// it synchronises the warp, not the CTA.
template <int ITEMS = kSegItems>
__device__ void block_merge_sort(uint64_t* s, int m) {
    const int t = threadIdx.x;
    const int active = m / ITEMS;
    uint64_t k[ITEMS];
    if (t < active) {
#pragma unroll
        for (int j = 0; j < ITEMS; ++j) k[j] = s[spad(t * ITEMS + j)];
        bool sorted = true;
#pragma unroll
        for (int j = 0; j + 1 < ITEMS; ++j) sorted = sorted && k[j] <= k[j + 1];
        if (!sorted) {
            sort_items(k);
#pragma unroll
            for (int j = 0; j < ITEMS; ++j) s[spad(t * ITEMS + j)] = k[j];
        }
    }
    __syncthreads();
    const bool desc = t + 1 < active && s[spad(t * ITEMS + ITEMS - 1)] > s[spad((t + 1) * ITEMS)];
    if (!__syncthreads_or(desc)) return;  // every run boundary already in order
    constexpr int kWarpSpan = 32 * ITEMS;
    for (int L = ITEMS; L < m; L <<= 1) {
        const bool warp_local = 2 * L <= kWarpSpan;
        bool wrote = false;
        if (t < active) wrote = merge_round(s, t, m, L, k);
        if (warp_local)
            __syncwarp();
        else
            __syncthreads();
        if (wrote) {
#pragma unroll
            for (int r = 0; r < ITEMS; ++r) s[spad(t * ITEMS + r)] = k[r];
        }
        if (4 * L <= kWarpSpan)
            __syncwarp();
        else
            __syncthreads();
    }
    __syncthreads();
}

__device__ __forceinline__ void write_sorted(uint64_t key, uint32_t dst, uint32_t* vals) {
    vals[dst] = (uint32_t)key;
}

// Incremental mode: collect tile `tile`'s instances into dst (shared memory in
// the padded layout, or global memory) -- first the members of the previous
// sorted list whose Gaussian's new rectangle still holds the tile, in their
// previous order, with the key for the new projection; then the entering
// instances.  Returns the number collected (the tile's count when consistent);
// writes stop at n_cap.
constexpr int kGatherItems = 4;
template <bool SMEM>
__device__ int gather_tile(uint64_t* dst, uint32_t tile, int n_cap, const SegSortIncr& inc, uint32_t* s_wsum,
                           int* n_kept) {
    const int tx = (int)(tile % (uint32_t)inc.ntx), ty = (int)(tile / (uint32_t)inc.ntx);
    uint2 ro = inc.ranges_prev[tile];
    ro.y = (uint32_t)min((uint64_t)ro.y, inc.capacity);
    const int n_old = ro.y > ro.x ? (int)(ro.y - ro.x) : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int kept = 0;
    for (int c0 = 0; c0 < n_old; c0 += kSegThreads * kGatherItems) {
        const int i0 = c0 + threadIdx.x * kGatherItems;  // blocked: keeps the previous order
        uint32_t gid[kGatherItems];
        uint64_t key[kGatherItems];
        bool keep[kGatherItems];
#pragma unroll
        for (int j = 0; j < kGatherItems; ++j) gid[j] = i0 + j < n_old ? inc.vals_prev[ro.x + i0 + j] : 0xffffffffu;
        uint4 b0[kGatherItems];
        float4 b1[kGatherItems];
#pragma unroll
        for (int j = 0; j < kGatherItems; ++j) {
            // both halves of the 32-byte record at once: one dependent step
            b0[j] = make_uint4(0, 0, 0, 0);
            b1[j] = make_float4(0, 0, 0, 0);
            if (gid[j] < inc.n_gauss) {
                b0[j] = inc.bins[gid[j]].r;
                b1[j] = inc.bins[gid[j]].p;
            }
        }
        int cnt = 0;
#pragma unroll
        for (int j = 0; j < kGatherItems; ++j) {
            keep[j] = gid[j] < inc.n_gauss && rect_contains(b0[j], tx, ty);
            const float d = tile_depth(tx, ty, inc.tw, inc.th, b1[j].x, b1[j].y, b1[j].z, b1[j].w, b0[j].w);
            key[j] = ((uint64_t)__float_as_uint(d) << 32) | gid[j];
            cnt += keep[j] ? 1 : 0;
        }
        // CTA exclusive scan of the per-thread counts
        uint32_t incl = (uint32_t)cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) s_wsum[w] = incl;
        __syncthreads();
        uint32_t before = 0, total = 0;
#pragma unroll
        for (int q = 0; q < kSegThreads / 32; ++q) {
            const uint32_t v = s_wsum[q];
            before += q < w ? v : 0u;
            total += v;
        }
        int pos = kept + (int)(before + incl) - cnt;
#pragma unroll
        for (int j = 0; j < kGatherItems; ++j) {
            if (keep[j]) {
                if (pos < n_cap) dst[SMEM ? spad(pos) : pos] = key[j];
                ++pos;
            }
        }
        kept += (int)total;
        __syncthreads();
    }
    const uint2 re = inc.enter_ranges[tile];
    const int ne = (int)(re.y - re.x);
    for (int i = threadIdx.x; i < ne; i += kSegThreads) {
        const int pos = kept + i;
        if (pos < n_cap) dst[SMEM ? spad(pos) : pos] = inc.enter_keys[re.x + i];
    }
    *n_kept = kept;
    return kept + ne;
}

// Nearly sorted survivors: bounded odd-even transposition passes over
// s[0..ns).  Returns true (uniformly) once a pass of each parity found nothing
// to swap, false when the pass budget ran out first.
constexpr int kFixMaxPasses = 24;
constexpr int kFixMaxDescents = 64;
constexpr int kMaxEntering = 32;
__device__ bool odd_even_fix(uint64_t* s, int ns) {
    int quiet = 0;
    for (int pass = 0; pass < kFixMaxPasses; ++pass) {
        bool swapped = false;
        for (int i = 2 * (int)threadIdx.x + (pass & 1); i + 1 < ns; i += 2 * kSegThreads) {
            const uint64_t a = s[spad(i)], b = s[spad(i + 1)];
            if (a > b) {
                s[spad(i)] = b;
                s[spad(i + 1)] = a;
                swapped = true;
            }
        }
        if (__syncthreads_or(swapped))
            quiet = 0;
        else if (++quiet == 2)
            return true;
    }
    return false;
}

// Number of keys of the sorted s[base..base+len) below key (keys are unique).
__device__ __forceinline__ int rank_in(const uint64_t* s, int base, int len, uint64_t key) {
    int lo = 0, hi = len;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (s[spad(base + mid)] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(kSegThreads) segsort_kernel(uint64_t* comp, const uint2* __restrict__ ranges,
                                                              uint32_t* vals, SegSortWork w, DevStatus* st,
                                                              SegSortIncr inc) {
    pdl_begin();
    __shared__ uint64_t s[kSegCap + kSegCap / 16];
    __shared__ uint32_t s_wsum[kSegThreads / 32];
    __shared__ int s_desc;
    if (st->flags & kErrOverflow) return;
    const bool incr = st->mode == kBinIncremental;
    const uint32_t tile = blockIdx.x;
    const uint2 r = ranges[tile];
    const int n = (int)(r.y - r.x);
    if (n <= 0) return;
    if (n > kSegCap) {
        if (incr) {
            int kept;
            const int got = gather_tile<false>(comp + r.x, tile, n, inc, s_wsum, &kept);
            if (got != n && threadIdx.x == 0) atomicOr(&st->flags, kErrBounds);
        }
        if (threadIdx.x == 0) w.large_list[atomicAdd(&w.large_ctrl[0], 1u)] = tile;
        return;
    }
    const int m = (n + kSegItems - 1) / kSegItems * kSegItems;
    if (incr) {
        int kept;
        const int got = gather_tile<true>(s, tile, n, inc, s_wsum, &kept);
        if (got != n && threadIdx.x == 0) atomicOr(&st->flags, kErrBounds);
        const int ns = min(kept, n), ne = n - ns;
        if (threadIdx.x == 0) s_desc = 0;
        __syncthreads();
        int desc = 0;
        for (int i = threadIdx.x; i + 1 < ns; i += kSegThreads) desc += s[spad(i)] > s[spad(i + 1)] ? 1 : 0;
        if (desc) atomicAdd(&s_desc, desc);
        __syncthreads();
        const int n_desc = s_desc;
        bool fixed = ne <= kMaxEntering && n_desc <= kFixMaxDescents;
        if (fixed && n_desc > 0) fixed = odd_even_fix(s, ns);
        if (fixed) {
            // survivors sorted: rank the few entering keys among themselves,
            // then every key goes straight to its merged position
            if (ne > 1 && threadIdx.x < 32) {
                const int j = threadIdx.x;
                const uint64_t key = j < ne ? s[spad(ns + j)] : kKeyInf;
                int rank = 0;
                for (int q = 0; q < ne; ++q) rank += s[spad(ns + q)] < key ? 1 : 0;
                __syncwarp();
                if (j < ne) s[spad(ns + rank)] = key;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < ns; i += kSegThreads) {
                const uint64_t key = s[spad(i)];
                const int before = ne ? rank_in(s, ns, ne, key) : 0;
                write_sorted(key, r.x + i + before, vals);
            }
            for (int j = threadIdx.x; j < ne; j += kSegThreads) {
                const uint64_t key = s[spad(ns + j)];
                write_sorted(key, r.x + j + rank_in(s, 0, ns, key), vals);
            }
            return;
        }
        if (threadIdx.x < m - n) s[spad(n + threadIdx.x)] = kKeyInf;
    } else {
        for (int i = threadIdx.x; i < m; i += kSegThreads) s[spad(i)] = i < n ? comp[r.x + i] : kKeyInf;
    }
    __syncthreads();
    if (m <= kSegThreads * kSmallItems)
        block_merge_sort<kSmallItems>(s, (n + kSmallItems - 1) / kSmallItems * kSmallItems);
    else
        block_merge_sort<kSegItems>(s, m);
    for (int i = threadIdx.x; i < n; i += kSegThreads) write_sorted(s[spad(i)], r.x + i, vals);
}

// Large buckets: persistent CTAs take listed tiles; each sorts 4096-key
// chunks in shared memory into tmp, then merges runs through global memory
// (every thread merges kSegItems outputs after its own merge-path search).
__global__ void __launch_bounds__(kSegThreads) segsort_large_kernel(uint64_t* comp, uint64_t* tmp,
                                                                    const uint2* __restrict__ ranges, uint32_t* vals,
                                                                    SegSortWork w, const DevStatus* st) {
    pdl_begin();
    __shared__ uint64_t s[kSegCap + kSegCap / 16];
    __shared__ uint32_t s_idx;
    if (st->flags & kErrOverflow) return;
    for (;;) {
        if (threadIdx.x == 0) s_idx = atomicAdd(&w.large_ctrl[1], 1u);
        __syncthreads();
        const uint32_t idx = s_idx;
        __syncthreads();
        if (idx >= w.large_ctrl[0]) return;
        const uint32_t tile = w.large_list[idx];
        const uint2 r = ranges[tile];
        const int n = (int)(r.y - r.x);
        uint64_t* src = tmp + r.x;
        uint64_t* dst = comp + r.x;
        // sorted chunks of 4096 into src
        for (int c0 = 0; c0 < n; c0 += kSegCap) {
            const int cn = min(kSegCap, n - c0);
            for (int i = threadIdx.x; i < kSegCap; i += kSegThreads) s[spad(i)] = i < cn ? comp[r.x + c0 + i] : kKeyInf;
            __syncthreads();
            block_merge_sort(s, kSegCap);
            for (int i = threadIdx.x; i < cn; i += kSegThreads) src[c0 + i] = s[spad(i)];
            __syncthreads();
        }
        // merge passes src -> dst, runs of L doubling
        for (int L = kSegCap; L < n; L <<= 1) {
            for (int o = threadIdx.x * kSegItems; o < n; o += kSegThreads * kSegItems) {
                const int ps = (o / (2 * L)) * 2 * L;
                const int d = o - ps;
                const int la = min(L, n - ps);
                const int lb = max(0, min(L, n - ps - L));
                const uint64_t* A = src + ps;
                const uint64_t* B = src + ps + la;
                int lo = max(0, d - lb), hi = min(d, la);
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (A[mid] <= B[d - 1 - mid])
                        lo = mid + 1;
                    else
                        hi = mid;
                }
                int ai = lo, bj = d - lo;
                const int outn = min(kSegItems, la + lb - d);
                for (int q = 0; q < outn; ++q) {
                    const uint64_t a = ai < la ? A[ai] : kKeyInf;
                    const uint64_t b = bj < lb ? B[bj] : kKeyInf;
                    const bool ta = a <= b;
                    dst[ps + d + q] = ta ? a : b;
                    ai += ta ? 1 : 0;
                    bj += ta ? 0 : 1;
                }
            }
            __syncthreads();
            uint64_t* tsw = src;
            src = dst;
            dst = tsw;
        }
        for (int i = threadIdx.x; i < n; i += kSegThreads) write_sorted(src[i], r.x + i, vals);
        __syncthreads();
    }
}

cudaError_t launch_segsort(uint64_t* comp, uint64_t* tmp, const uint2* ranges, int num_tiles, uint32_t* vals,
                           SegSortWork w, const DevStatus* st, int large_grid, const SegSortIncr& inc,
                           cudaStream_t s) {
    if (num_tiles <= 0) return cudaSuccess;
    // the list counters were zeroed by the tile-offsets kernel of this binning
    cudaError_t e = launch_chained(segsort_kernel, dim3(num_tiles), dim3(kSegThreads), 0, s, comp, ranges, vals, w,
                                   const_cast<DevStatus*>(st), inc);
    if (e != cudaSuccess) return e;
    return launch_chained(segsort_large_kernel, dim3(large_grid), dim3(kSegThreads), 0, s, comp, tmp, ranges, vals, w,
                          st);
}

// One CTA per tile: key = tile << 32 | bits of the tile-centre depth of the
// Gaussian at each sorted position.
__global__ void __launch_bounds__(256) make_keys_kernel(const BinRec* __restrict__ bins,
                                                        const uint2* __restrict__ ranges,
                                                        const uint32_t* __restrict__ vals, uint32_t n_gauss, int ntx,
                                                        int tw, int th, const DevStatus* st, uint64_t* keys) {
    pdl_begin();
    if (st->flags & kErrOverflow) return;
    const uint32_t tile = blockIdx.x;
    const uint2 r = ranges[tile];
    const int tx = (int)(tile % (uint32_t)ntx), ty = (int)(tile / (uint32_t)ntx);
    for (uint32_t i = r.x + threadIdx.x; i < r.y; i += blockDim.x) {
        const uint32_t g = vals[i];
        if (g >= n_gauss) continue;
        const BinRec b = bins[g];
        const float d = tile_depth(tx, ty, tw, th, b.p.x, b.p.y, b.p.z, b.p.w, b.r.w);
        keys[i] = ((uint64_t)tile << 32) | __float_as_uint(d);
    }
}

cudaError_t launch_make_keys(const BinRec* bins, const uint2* ranges, const uint32_t* vals, uint32_t n_gauss,
                             int num_tiles, int ntx, int tw, int th, const DevStatus* st, uint64_t* keys,
                             cudaStream_t s) {
    if (num_tiles <= 0) return cudaSuccess;
    return launch_chained(make_keys_kernel, dim3(num_tiles), dim3(256), 0, s, bins, ranges, vals, n_gauss, ntx, tw,
                          th, st, keys);
}

}  // namespace fvgs
