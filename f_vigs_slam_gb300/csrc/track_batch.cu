// track_batch.cu -- the persistent tracking kernel of the batching form: the
// tiles of many sessions (each with its own map, frame size and pose) in one
// launch, each CTA taking tile after tile from a shared work counter.
//
// Per tile it runs the same body as the per-frame kernel (track_tile.cuh:
// forward blend, pose Jacobian, the tile's J^T J / J^T r partials written to
// the session's tile buffer), so a session's partials are bit-identical to
// those of its own per-frame launch with the same tile shape.  The reference
// renders and differentiates one frame per launch (getRgbdPoseJacobians,
// src/GSCudaKernels.cu:922-1392, launched by GSSlam::computeRgbdPoseJacobians,
// src/GSSlam.cu:2179-2202); batching sessions is this library's form.
#include <mutex>

#include "track_tile.cuh"

namespace fvgs {

template <int TW, int TH, int BATCH, bool ANALYTIC, int MIN_CTAS>
__global__ void __launch_bounds__(TW * TH, MIN_CTAS)
    track_batch_kernel(const TrackJob* __restrict__ jobs, const uint32_t* __restrict__ begin, int n_jobs,
                       uint32_t total, uint32_t* counters) {
    pdl_begin();
    constexpr int NT = TW * TH;
    constexpr int kWords = (int)(sizeof(TrackArgs) / 4);
    static_assert(sizeof(TrackArgs) % 4 == 0, "job arguments are copied as 32-bit words");
    extern __shared__ __align__(128) unsigned char s_dyn[];
    __shared__ TrackArgs s_args;
    __shared__ int s_job, s_tile;
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0) {
            const uint32_t item = atomicAdd(&counters[0], 1u);
            int job = -1, tile = 0;
            if (item < total) {
                // the last job whose range starts at or before the item
                int lo = 0, hi = n_jobs - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (begin[mid] <= item)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                job = lo;
                tile = (int)(item - begin[lo]);
            }
            s_job = job;
            s_tile = tile;
        }
        __syncthreads();
        const int job = s_job;
        if (job < 0) break;
        if (job != cur) {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&jobs[job].a);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&s_args);
            for (int k = threadIdx.x; k < kWords; k += NT) dst[k] = src[k];
            __syncthreads();
            cur = job;
        }
        track_tile_body<TW, TH, false, false, false, BATCH, ANALYTIC>(s_args, RecMaps{}, s_tile, s_dyn);
        __syncthreads();  // the tile's shared state is consumed before the next item is taken
    }
    // Every CTA that leaves has drawn an item past the end; the last one to
    // leave resets the counters for the next launch (no other CTA touches
    // them again).
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&counters[1], 1u) == gridDim.x - 1) {
            atomicExch(&counters[0], 0u);
            atomicExch(&counters[1], 0u);
        }
    }
}

namespace {

using BatchKernel = void (*)(const TrackJob*, const uint32_t*, int, uint32_t, uint32_t*);

struct BatchPick {
    BatchKernel fn = nullptr;
    int threads = 0;
    size_t smem = 0;
};

// Register budget: 64 per thread for the reference Jacobian, 80 for the
// analytic one (its single fused pass holds the colour-Jacobian sums).
template <int TW, int TH, int BATCH, bool ANALYTIC>
BatchPick bpick() {
    return {track_batch_kernel<TW, TH, BATCH, ANALYTIC, (ANALYTIC ? 768 : 1024) / (TW * TH)>, TW * TH,
            body_smem_bytes<TW, TH, BATCH, ANALYTIC, false>()};
}

template <int TW, int TH, bool ANALYTIC>
BatchPick bpick_batch(int batch) {
    if (batch == 128) return bpick<TW, TH, 128, ANALYTIC>();
    if (batch == 512) return bpick<TW, TH, 512, ANALYTIC>();
    return bpick<TW, TH, 256, ANALYTIC>();
}

BatchPick pick_batch(int tw, int th, bool analytic, int variant) {
    const int batch = track_variant_batch(variant);
    if (tw == 16 && th == 16) return analytic ? bpick_batch<16, 16, true>(batch) : bpick_batch<16, 16, false>(batch);
    if (tw == 8 && th == 8) return analytic ? bpick_batch<8, 8, true>(batch) : bpick_batch<8, 8, false>(batch);
    if (tw == 32 && th == 8) return analytic ? bpick_batch<32, 8, true>(batch) : bpick_batch<32, 8, false>(batch);
    return {};
}

// Resident CTAs per SM of each instantiation (the persistent grid's size),
// computed once.
struct OccEntry {
    BatchKernel fn;
    int blocks;
};
std::mutex g_occ_mutex;
OccEntry g_occ[64];
int g_occ_n = 0;

int resident_blocks(const BatchPick& k) {
    std::lock_guard<std::mutex> lock(g_occ_mutex);
    for (int i = 0; i < g_occ_n; ++i)
        if (g_occ[i].fn == k.fn) return g_occ[i].blocks;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k.fn, k.threads, k.smem) != cudaSuccess || n < 1) {
        cudaGetLastError();
        n = 1;
    }
    if (g_occ_n < 64) g_occ[g_occ_n++] = {k.fn, n};
    return n;
}

}  // namespace

cudaError_t track_batch_configure_device() {
    const int shapes[3][2] = {{16, 16}, {8, 8}, {32, 8}};
    const int variants[3] = {0, 3, 4};  // batches of 256, 128, 512
    for (auto& sh : shapes)
        for (int analytic = 0; analytic < 2; ++analytic)
            for (int v : variants) {
                const BatchPick k = pick_batch(sh[0], sh[1], analytic != 0, v);
                const cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k.fn),
                                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)k.smem);
                if (e != cudaSuccess) return e;
            }
    return cudaSuccess;
}

cudaError_t launch_track_batch(const TrackJob* jobs, const uint32_t* begin, int n_jobs, uint32_t total_tiles,
                               int tile_w, int tile_h, bool analytic, int variant, uint32_t* counters, int num_sms,
                               cudaStream_t s) {
    if (n_jobs <= 0 || total_tiles == 0) return cudaSuccess;
    const BatchPick k = pick_batch(tile_w, tile_h, analytic, variant);
    if (!k.fn || !jobs || !begin || !counters) return cudaErrorInvalidValue;
    const uint32_t slots = (uint32_t)num_sms * (uint32_t)resident_blocks(k);
    const uint32_t grid = total_tiles < slots ? total_tiles : slots;
    return launch_chained(k.fn, dim3(grid), dim3(k.threads), k.smem, s, jobs, begin, n_jobs, total_tiles, counters);
}

}  // namespace fvgs
