// sort.cu -- stable LSD radix sort of (u64 key, u32 value) pairs for sm_103a.
//
// Replaces thrust::sort_by_key on the 64-bit tile|depth keys
// (src/GSSlam.cu:624-628), which is a stable radix sort.  Only the key bits
// that can be non-zero are sorted: 32 depth bits plus ceil(log2(tiles)) tile
// bits, so 640x480 and 1280x720 frames take 6 digit passes instead of 8.
//
// Structure: one histogram kernel computes the digit counts of every pass in
// a single read of the keys; then one "onesweep" kernel per pass ranks a
// 4096-item tile (512 threads x 8 items) in shared memory -- a warp finds the
// lanes sharing its digit with 8 ballots, and only the group's leader bumps
// the warp's shared counter, so ranks are stable within the tile -- obtains
// the tile's global digit offsets by decoupled look-back that polls 8
// predecessor tiles per round trip, and scatters through shared memory so
// that runs of equal digits are written contiguously.
//
// The CTAs are persistent (grid = resident capacity) and take tiles from an
// atomic counter, so every tile a CTA waits on is owned by a running CTA.
// Look-back status words are 64-bit (epoch | flag | count): a new epoch per
// pass makes stale words invisible without clearing the array.  Every wait is
// bounded; on expiry the kernel records kErrTimeout, and destination indices
// are range-checked so a failed wait cannot write out of bounds.
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace fvgs {

constexpr int kSortThreads = 512;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;  // 4096
constexpr int kRadix = 256;
constexpr int kMaxPasses = 8;
constexpr int kLookWindow = 8;
constexpr size_t kSortSmemBytes = (size_t)kSortTile * (sizeof(uint64_t) + sizeof(uint32_t));

constexpr uint64_t kFlagAgg = 1ull << 32;
constexpr uint64_t kFlagInc = 2ull << 32;

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Exclusive scan of one value per thread over the first 256 threads of the
// block (all threads must call it).
__device__ __forceinline__ uint32_t block_excl_scan256(uint32_t x, uint32_t* s_warp) {
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    uint32_t incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(kFullMask, incl, o);
        if (l >= o) incl += y;
    }
    if (l == 31 && w < 8) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t v = (l < 8) ? s_warp[l] : 0u;
        uint32_t vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(kFullMask, vi, o);
            if (l >= o) vi += y;
        }
        if (l < 8) s_warp[l] = vi - v;
    }
    __syncthreads();
    const uint32_t r = (w < 8) ? s_warp[w] + incl - x : 0u;
    __syncthreads();
    return r;
}

// Digit histograms of every pass in one read of the keys.  Each warp counts
// into its own shared histograms, so atomics only conflict among the lanes of
// one instruction.
constexpr int kHistThreads = 256;
__global__ void __launch_bounds__(kHistThreads) radix_hist_kernel(const uint64_t* __restrict__ keys,
                                                                  const DevStatus* st, int n_passes,
                                                                  uint32_t* __restrict__ hist) {
    extern __shared__ uint32_t sh[];  // [warps][n_passes][256]
    const int nw = kHistThreads / 32, w = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < nw * n_passes * kRadix; i += kHistThreads) sh[i] = 0;
    __syncthreads();
    uint32_t* mine = sh + (size_t)w * n_passes * kRadix;
    const uint32_t n = st->n_instances_clamped;
    const uint32_t n2 = n / 2;
    const ulonglong2* k2 = reinterpret_cast<const ulonglong2*>(keys);
    for (uint32_t i = blockIdx.x * kHistThreads + threadIdx.x; i < n2; i += gridDim.x * kHistThreads) {
        const ulonglong2 kk = k2[i];
        for (int p = 0; p < n_passes; ++p) {
            atomicAdd(&mine[p * kRadix + ((uint32_t)(kk.x >> (8 * p)) & 0xffu)], 1u);
            atomicAdd(&mine[p * kRadix + ((uint32_t)(kk.y >> (8 * p)) & 0xffu)], 1u);
        }
    }
    if ((n & 1u) && blockIdx.x == 0 && threadIdx.x == 0) {
        const uint64_t k = keys[n - 1];
        for (int p = 0; p < n_passes; ++p) atomicAdd(&mine[p * kRadix + ((uint32_t)(k >> (8 * p)) & 0xffu)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_passes * kRadix; i += kHistThreads) {
        uint32_t c = 0;
        for (int ww = 0; ww < nw; ++ww) c += sh[(size_t)ww * n_passes * kRadix + i];
        if (c) atomicAdd(&hist[i], c);
    }
}

__global__ void __launch_bounds__(kSortThreads, 2)
    radix_onesweep_kernel(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
                          uint64_t* __restrict__ kout, uint32_t* __restrict__ vout, const DevStatus* st,
                          const uint32_t* __restrict__ hist, uint64_t* lookback, uint32_t* tile_counter,
                          int shift, uint32_t epoch, uint32_t* err_flags) {
    extern __shared__ __align__(16) uint8_t smem_raw[];
    uint64_t* s_keys = reinterpret_cast<uint64_t*>(smem_raw);
    uint32_t* s_vals = reinterpret_cast<uint32_t*>(s_keys + kSortTile);
    __shared__ uint32_t s_whist[kSortWarps][kRadix];
    __shared__ uint32_t s_gbase[kRadix];
    __shared__ uint32_t s_prefix[kRadix];
    __shared__ uint32_t s_lexcl[kRadix];
    __shared__ uint32_t s_scan[8];
    __shared__ uint32_t s_tile;

    const uint32_t n = st->n_instances_clamped;
    const uint32_t n_tiles = (n + kSortTile - 1) / kSortTile;
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const uint64_t ep = (uint64_t)epoch << 34;
    const bool digit_thread = tid < kRadix;

    {
        const uint32_t g = block_excl_scan256(digit_thread ? hist[tid] : 0u, s_scan);
        if (digit_thread) s_gbase[tid] = g;
    }

    for (;;) {
        if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
        for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads) (&s_whist[0][0])[i] = 0;
        __syncthreads();
        const uint32_t tile = s_tile;
        if (tile >= n_tiles) break;

        // ---- rank: warp-striped items, ballot multisplit, leader atomics ----
        const uint32_t base = tile * kSortTile + w * (32 * kSortItems);
        uint64_t k[kSortItems];
        uint32_t v[kSortItems];
        uint32_t rank[kSortItems];
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            const uint32_t idx = base + j * 32 + lane;
            const bool valid = idx < n;
            k[j] = valid ? kin[idx] : 0ull;
            v[j] = valid ? vin[idx] : 0u;
        }
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            const uint32_t idx = base + j * 32 + lane;
            const bool valid = idx < n;
            const uint32_t dig = (uint32_t)(k[j] >> shift) & 0xffu;
            uint32_t peers = __ballot_sync(kFullMask, valid);
#pragma unroll
            for (int b = 0; b < 8; ++b) {
                const bool bit = (dig >> b) & 1u;
                const uint32_t vote = __ballot_sync(kFullMask, bit);
                peers &= bit ? vote : ~vote;
            }
            const int leader = __ffs(peers) - 1;
            uint32_t b0 = 0;
            if (valid && lane == leader) b0 = atomicAdd(&s_whist[w][dig], (uint32_t)__popc(peers));
            b0 = __shfl_sync(kFullMask, b0, valid ? leader : lane);
            rank[j] = b0 + __popc(peers & lt);
        }
        __syncthreads();
        // ---- per digit: exclusive offsets across warps, tile count ----
        uint32_t cta_cnt = 0;
        if (digit_thread) {
#pragma unroll
            for (int ww = 0; ww < kSortWarps; ++ww) {
                const uint32_t c = s_whist[ww][tid];
                s_whist[ww][tid] = cta_cnt;
                cta_cnt += c;
            }
            // ---- decoupled look-back, kLookWindow predecessors per poll ----
            uint64_t* lb = lookback + (size_t)tile * kRadix + tid;
            uint32_t prefix = 0;
            if (tile == 0) {
                st_relaxed(lb, ep | kFlagInc | cta_cnt);
            } else {
                st_relaxed(lb, ep | kFlagAgg | cta_cnt);
                int t = (int)tile - 1;
                uint32_t spins = 0;
                bool found = false;
                while (!found && t >= 0) {
                    uint64_t wv[kLookWindow];
#pragma unroll
                    for (int i = 0; i < kLookWindow; ++i)
                        wv[i] = (t - i >= 0) ? ld_relaxed(lookback + (size_t)(t - i) * kRadix + tid) : 0ull;
                    int consumed = 0;
#pragma unroll
                    for (int i = 0; i < kLookWindow; ++i) {
                        if (found || consumed != i || t - i < 0) continue;
                        const uint64_t x = wv[i];
                        if ((x >> 34) == (uint64_t)epoch && (x & (3ull << 32))) {
                            prefix += (uint32_t)x;
                            consumed = i + 1;
                            if (x & kFlagInc) found = true;
                        }
                    }
                    t -= consumed;
                    if (consumed == 0 && ++spins > kSpinLimit) {
                        atomicOr(err_flags, kErrTimeout);
                        break;
                    }
                }
                st_relaxed(lb, ep | kFlagInc | (prefix + cta_cnt));
            }
            s_prefix[tid] = prefix;
        }
        {
            const uint32_t e = block_excl_scan256(cta_cnt, s_scan);
            if (digit_thread) s_lexcl[tid] = e;
        }
        __syncthreads();
        // ---- scatter into shared memory at the tile-local sorted position ----
#pragma unroll
        for (int j = 0; j < kSortItems; ++j) {
            const uint32_t idx = base + j * 32 + lane;
            if (idx < n) {
                const uint32_t dig = (uint32_t)(k[j] >> shift) & 0xffu;
                const uint32_t pos = s_lexcl[dig] + s_whist[w][dig] + rank[j];
                s_keys[pos] = k[j];
                s_vals[pos] = v[j];
            }
        }
        __syncthreads();
        // ---- coalesced write-out: runs of equal digits are contiguous ----
        const uint32_t tile_n = min((uint32_t)kSortTile, n - tile * kSortTile);
        for (uint32_t i = tid; i < tile_n; i += kSortThreads) {
            const uint64_t kk = s_keys[i];
            const uint32_t dig = (uint32_t)(kk >> shift) & 0xffu;
            const uint32_t dst = s_gbase[dig] + s_prefix[dig] + (i - s_lexcl[dig]);
            if (dst < n) {
                kout[dst] = kk;
                vout[dst] = s_vals[i];
            }
        }
        __syncthreads();
    }
}

int sort_num_passes(int key_bits) {
    const int p = (key_bits + 7) / 8;
    return p + (p & 1);
}

size_t sort_lookback_words(uint64_t max_items) {
    return (size_t)((max_items + kSortTile - 1) / kSortTile + 1) * kRadix;
}

size_t sort_ctrl_words() { return (size_t)kMaxPasses * kRadix + kMaxPasses; }

cudaError_t sort_init(SortWorkspace* ws, int device) {
    cudaError_t e = cudaFuncSetAttribute(radix_onesweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kSortSmemBytes);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(radix_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(sizeof(uint32_t) * (kHistThreads / 32) * kMaxPasses * kRadix));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, radix_onesweep_kernel, kSortThreads,
                                                      kSortSmemBytes);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) return e;
    ws->persistent_ctas = (per_sm > 0 ? per_sm : 1) * sms;
    ws->num_sms = sms;
    if (ws->epoch == 0) ws->epoch = 1;
    return cudaSuccess;
}

cudaError_t launch_radix_sort(uint64_t* keys, uint32_t* vals, const DevStatus* st, int key_bits,
                              SortWorkspace* ws, uint32_t* err_flags, cudaStream_t s) {
    const int passes = sort_num_passes(key_bits);
    if (passes > kMaxPasses) return cudaErrorInvalidValue;
    // Epochs are 30-bit; on wrap the look-back array is cleared once.
    if (ws->epoch + (uint32_t)passes >= (1u << 30)) {
        cudaError_t e = cudaMemsetAsync(ws->lookback, 0, sizeof(uint64_t) * sort_lookback_words(ws->max_items), s);
        if (e != cudaSuccess) return e;
        ws->epoch = 1;
    }
    cudaError_t e = cudaMemsetAsync(ws->ctrl, 0, sizeof(uint32_t) * sort_ctrl_words(), s);
    if (e != cudaSuccess) return e;
    radix_hist_kernel<<<ws->num_sms * 2, kHistThreads, sizeof(uint32_t) * (kHistThreads / 32) * passes * kRadix, s>>>(
        keys, st, passes, ws->ctrl);
    uint64_t* kin = keys;
    uint32_t* vin = vals;
    uint64_t* kout = ws->keys_alt;
    uint32_t* vout = ws->vals_alt;
    for (int p = 0; p < passes; ++p) {
        radix_onesweep_kernel<<<ws->persistent_ctas, kSortThreads, kSortSmemBytes, s>>>(
            kin, vin, kout, vout, st, ws->ctrl + p * kRadix, ws->lookback, ws->ctrl + kMaxPasses * kRadix + p,
            8 * p, ws->epoch + (uint32_t)p, err_flags);
        uint64_t* tk = kin;
        kin = kout;
        kout = tk;
        uint32_t* tv = vin;
        vin = vout;
        vout = tv;
    }
    ws->epoch += (uint32_t)passes;
    return cudaGetLastError();
}

}  // namespace fvgs
