// noalloc.cu -- an allocation-free entry point for the RGB-D pose Jacobian.
//
// Some callers cannot call cudaMalloc: a tracking thread embedded in a host
// application that owns the GPU's memory budget (its allocator is the only one
// allowed to reserve device memory), or a real-time loop whose latency budget
// forbids the implicit synchronisation of cudaMalloc / cudaFree.  They already
// hold the screen-space buffers of a binned frame (the reference's layout) and
// the observed images, and only need JtJ / Jtr back.
//
// fvgs_rgbd_pose_jacobians_noalloc serves them.  Its only scratch -- the
// per-tile partial sums, the reduced 6x6 system and the pose the kernels read
// -- lives in the file-scope array g_noalloc_scratch below, sized for at most
// FVGS_NOALLOC_MAX_TILES 16x16 tiles.  Every GPU that loads this library holds
// that array (about 1.8 MB) until the process exits.
//
// Rules of use:
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (with that device current) and caches it per device
//    ordinal, so only the device's primary context (the one the CUDA runtime
//    uses) is supported.
//  * The call waits for its stream and copies the result to the caller's
//    (possibly pageable) memory, so it cannot be called while the stream is
//    being captured into a CUDA graph.
//  * All calls share the array and it keeps the last call's contents.  Every
//    word a call reads is first written by the same call (all tile partials of
//    the frame, the pose, the reduced system), so nothing needs clearing.
//  * Calls whose work overlaps on the GPU race on the array: issue them on one
//    stream, or synchronise between them.
//  * No cudaMalloc, cudaFree or allocating library routine is called.
#include <cstring>
#include <mutex>

#include "../../include/fvgs.h"
#include "fvgs_device.cuh"
#include "fvgs_launch.h"

namespace {

using fvgs::DevPose;

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t kOffTiles = 0;
constexpr size_t kTilesBytes = align256((size_t)FVGS_NOALLOC_MAX_TILES * FVGS_POSEDATA_FLOATS * sizeof(float));
constexpr size_t kOffOut = kOffTiles + kTilesBytes;
constexpr size_t kOutBytes = align256(48 * sizeof(double));
constexpr size_t kOffPose = kOffOut + kOutBytes;
constexpr size_t kScratchBytes = kOffPose + align256(sizeof(DevPose));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (resolved once).
int scratch_for_current_device(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return FVGS_E_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return FVGS_E_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return FVGS_OK;
}

__global__ void noalloc_set_pose_kernel(DevPose* dst, fvgs_pose p) {
    fvgs::pdl_begin();
    for (int k = 0; k < 3; ++k) {
        dst->t[k] = p.position[k];
        dst->td[k] = (double)p.position[k];
    }
    for (int k = 0; k < 4; ++k) {
        dst->q[k] = p.orientation[k];
        dst->qd[k] = (double)p.orientation[k];
    }
}

}  // namespace

// A failed CUDA call: clear the error the runtime keeps, so the caller's next
// CUDA check does not report it against another operation.
int cuda_failed() {
    cudaGetLastError();
    return FVGS_E_CUDA;
}

extern "C" int fvgs_rgbd_pose_jacobians_noalloc(
    const uint32_t* ranges, const uint32_t* indices, const float* positions_2d, const float* depths,
    const float* inv_covariances_2d, const float* p_hats, const float* colors, const float* opacities,
    const float* grad_x, const float* grad_y, const float* observed_rgb, const float* observed_depth,
    const fvgs_pose* pose, const fvgs_intrinsics* K, const fvgs_params* params, int width, int height,
    uint32_t n_gaussians, uint32_t n_instances, double* JtJ, double* Jtr, void* cuda_stream) {
    if (!ranges || !indices || !positions_2d || !depths || !inv_covariances_2d || !p_hats || !colors ||
        !opacities || !grad_x || !grad_y || !observed_rgb || !observed_depth || !pose || !K || !JtJ || !Jtr)
        return FVGS_E_INVALID;
    fvgs_params P;
    if (params) P = *params;
    else fvgs_params_default(&P);
    if (P.tile_w != 16 || P.tile_h != 16 || width <= 0 || height <= 0) return FVGS_E_INVALID;
    const long long ntx = (width + 15) / 16, nty = (height + 15) / 16;
    if (ntx * nty > FVGS_NOALLOC_MAX_TILES) return FVGS_E_CAPACITY;  // frame larger than the static scratch
    unsigned char* base = nullptr;
    const int rc = scratch_for_current_device(&base);
    if (rc != FVGS_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    float* tiles = reinterpret_cast<float*>(base + kOffTiles);
    double* out = reinterpret_cast<double*>(base + kOffOut);
    DevPose* dpose = reinterpret_cast<DevPose*>(base + kOffPose);

    noalloc_set_pose_kernel<<<1, 1, 0, s>>>(dpose, *pose);
    if (cudaGetLastError() != cudaSuccess) return cuda_failed();
    fvgs::TrackArgs ta;
    std::memset(&ta, 0, sizeof(ta));
    ta.ranges = reinterpret_cast<const uint2*>(ranges);
    ta.indices = indices;
    // list entries at or past n_instances and indices at or above n_gaussians
    // are skipped, as for the library's own buffers; 0 = not checked
    ta.n_list = n_instances ? n_instances : 0xffffffffu;
    ta.n_gauss = n_gaussians ? n_gaussians : 0xffffffffu;
    ta.obs_rgb = observed_rgb;
    ta.obs_depth = observed_depth;
    ta.gx = grad_x;
    ta.gy = grad_y;
    ta.pose = dpose;
    ta.K = *K;
    ta.W = width;
    ta.H = height;
    ta.ntx = (int)ntx;
    ta.nty = (int)nty;
    ta.bg[0] = P.bg[0];
    ta.bg[1] = P.bg[1];
    ta.bg[2] = P.bg[2];
    ta.alpha_thresh = P.alpha_thresh;
    ta.color_thresh = P.color_thresh;
    ta.depth_thresh = P.depth_thresh;
    ta.tile_out = tiles;
    ta.ref_uv = positions_2d;
    ta.ref_depth = depths;
    ta.ref_inv = inv_covariances_2d;
    ta.ref_phat = p_hats;
    ta.ref_col = colors;
    ta.ref_opa = opacities;
    // the reference's buffers hold no camera-frame geometry: always the
    // reference's approximate Jacobian
    ta.quirks = P.quirks | FVGS_Q_POSE_JAC_APPROX;
    ta.variant = 0;
    if (fvgs::launch_track_ref_layout(ta, s) != cudaSuccess) return cuda_failed();
    if (fvgs::launch_track_reduce(tiles, (int)(ntx * nty), 1, dpose, out, s) != cudaSuccess) return cuda_failed();
    if (cudaMemcpyAsync(JtJ, out, sizeof(double) * 36, cudaMemcpyDefault, s) != cudaSuccess ||
        cudaMemcpyAsync(Jtr, out + 36, sizeof(double) * 6, cudaMemcpyDefault, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return cuda_failed();
    return FVGS_OK;
}
