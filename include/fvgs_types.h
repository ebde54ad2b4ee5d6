/*
 * fvgs_types.h -- plain C types shared by the fvgs C-ABI (include/fvgs.h) and
 * every component that talks to it.
 *
 * Conventions (all follow the reference kernels, jcevasco2003/f_vigs_slam):
 *  - Gaussian parameters are the reference's `Gaussians` SoA
 *    (include/f_vigs_slam/RepresentationClasses.hpp:53-99): positions float3,
 *    scales float3, orientations float4, colors float3, opacities float.
 *  - Quaternions are passed as the raw float4 the kernels read, i.e. the
 *    component order (x, y, z, w) that quaternionToMatrix uses
 *    (src/GSCudaKernels.cu:319-334), for both Gaussians and camera poses.
 *  - Camera pose: world->camera transform is p_cam = R(q)^T (p_world - t)
 *    (src/GSCudaKernels.cu:372-378).
 *  - Images are dense row-major, no pitch: rgb/grad are float3 per pixel,
 *    depth is one float per pixel (src/GSSlam.cu:2179-2202).
 */
#ifndef FVGS_TYPES_H
#define FVGS_TYPES_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum fvgs_status {
    FVGS_OK = 0,
    FVGS_E_INVALID = -1,   /* bad argument (null pointer, size out of range) */
    FVGS_E_NOMEM = -2,     /* device or pinned-host allocation failed */
    FVGS_E_CUDA = -3,      /* a CUDA runtime call or kernel launch failed */
    FVGS_E_CAPACITY = -4,  /* a fixed-capacity buffer would overflow */
    FVGS_E_TIMEOUT = -5,   /* a bounded device-side wait gave up */
    FVGS_E_STATE = -6,     /* call made in the wrong state (e.g. no frame set) */
    FVGS_E_ADMISSION = -7  /* serving layer: request or session not admitted */
} fvgs_status;

/*
 * Reference-behaviour switches.  Each bit reproduces one documented quirk of
 * the reference kernels; clearing it selects the evidently intended
 * behaviour.  GPU kernels and the CPU restatement honour the same bits.
 *
 *  CULLED_SLOTS  projectGaussiansWorldToScreen_kernel returns without writing
 *                for culled Gaussians (src/GSCudaKernels.cu:381,391) while the
 *                count/hash kernels still bin every Gaussian.  With the bit
 *                set, culled slots behave as zero records (uv=0, cov=0, z=0):
 *                one instance with key 0 in tile 0.  Clear: culled Gaussians
 *                emit no instances.
 *  RANGE_LAUNCH  computeIndicesRanges_kernel is launched with ceil(T/256)*256
 *                threads but indexes instances (src/GSSlam.cu:633-640), so only
 *                boundaries among the first 256*ceil(T/256) sorted instances
 *                are recorded.  Clear: ranges over all instances.
 *  INVSIGMA_SWAP inverse 2D covariance is stored (xx, yy, xy)
 *                (src/GSCudaKernels.cu:469) but read as (xx, xy, yy) by the
 *                blending kernels (src/GSCudaKernels.cu:1007,1197,2204,2419).
 *                Set: v = ixx dx^2 + 2 iyy dx dy + ixy dy^2 (reference).
 *                Clear: the true quadratic form.
 *  MAP_CAP256    optimizeGaussiansPerGaussianPass only gives gradients to the
 *                first 256 Gaussians of each tile (src/GSCudaKernels.cu:2329).
 *  VIS_CAP256    computeGaussiansVisibility_kernel only considers the first
 *                256 Gaussians of each tile (src/GSCudaKernels.cu:1476).
 *  ADAM_STAY     removeOutliers / prune reorder the five parameter arrays but
 *                not adam_states_ (src/GSSlam.cu:1536-1548,1668-1680), so a
 *                surviving Gaussian that moves down inherits the optimiser
 *                moments of the one that held its new index.  Clear: the
 *                moments move with their Gaussian.
 *  POSE_WXYZ     (host mirror, include/f_vigs_slam) GSSlam builds the camera
 *                orientation as make_float4(w, x, y, z) (src/GSSlam.cu:2121)
 *                for kernels that read (x, y, z, w).  Clear: (x, y, z, w).
 *  COLOR_RESCALE (host mirror) computeRgbdPoseJacobians scales the [0, 1]
 *                colour pyramid by 1/255 once more (src/GSSlam.cu:2158).
 *                Clear: the pyramid colour as is.
 *  POSE_JAC_APPROX getRgbdPoseJacobians' approximate pose Jacobian
 *                (src/GSCudaKernels.cu:1043-1350): a per-pixel term from the
 *                observed image's Sobel gradients at the observed depth plus,
 *                per contributing Gaussian, the derivative through its screen
 *                mean taken at the cancelling per-pixel depth
 *                z + dx phat.x + dy phat.y.  Clear: the analytic derivative of
 *                the rendered colour and median depth with respect to the pose
 *                update, through every blended Gaussian's screen mean, conic
 *                and depth (the gradient images are then not read).
 *  DEPTH_HUBER   the tracking depth weight (|e| < 0.2 ? 1 : 0.2 / |e|) / z_obs
 *                (src/GSCudaKernels.cu:1120-1121, 1283-1284; 0.2 is
 *                depth_thresh).  Clear: Tukey's biweight
 *                (1 - (e / depth_thresh)^2)^2 / z_obs, zero beyond
 *                depth_thresh: a median depth jumps between the layers of a
 *                map at occlusion edges, and those residuals would otherwise
 *                pull the pose.
 */
#define FVGS_Q_CULLED_SLOTS  0x1u
#define FVGS_Q_RANGE_LAUNCH  0x2u
#define FVGS_Q_INVSIGMA_SWAP 0x4u
#define FVGS_Q_MAP_CAP256    0x8u
#define FVGS_Q_VIS_CAP256    0x10u
#define FVGS_Q_ADAM_STAY     0x20u
#define FVGS_Q_POSE_WXYZ     0x40u
#define FVGS_Q_COLOR_RESCALE 0x80u
#define FVGS_Q_POSE_JAC_APPROX 0x100u
#define FVGS_Q_DEPTH_HUBER   0x200u
/* Default: the reference's arithmetic (swap, caps, optimiser state left in
 * place, the host's pose order and colour rescale, the approximate pose
 * Jacobian and its depth weight) with the two launch/slot defects that make its outputs
 * degenerate (NaN tile 0, empty ranges) off. */
#define FVGS_QUIRKS_DEFAULT                                                                          \
    (FVGS_Q_INVSIGMA_SWAP | FVGS_Q_MAP_CAP256 | FVGS_Q_VIS_CAP256 | FVGS_Q_ADAM_STAY | FVGS_Q_POSE_WXYZ | \
     FVGS_Q_COLOR_RESCALE | FVGS_Q_POSE_JAC_APPROX | FVGS_Q_DEPTH_HUBER)
/* Every reference behaviour off: the intended semantics, and the analytic
 * pose Jacobian with which Gauss-Newton tracking converges. */
#define FVGS_QUIRKS_INTENDED 0u

typedef struct fvgs_pose {
    float position[3];     /* camera centre in world frame */
    float orientation[4];  /* raw float4 (x, y, z, w) as the kernels read it */
} fvgs_pose;

typedef struct fvgs_intrinsics {
    float fx, fy, cx, cy;  /* IntrinsicParameters{f, c} (RepresentationClasses.hpp:101-105) */
} fvgs_intrinsics;

/*
 * Tunables and hard-coded constants of the reference, in one POD.
 * Defaults (fvgs_params_default) are the reference's values:
 *  tile 16x16 (src/GSCudaKernels.cu:6), radius 3 sigma (src/GSSlam.cu:540),
 *  bg black, thresholds 0.2/0.1/0.2 (src/GSSlam.cu:2175-2177),
 *  w_depth 1, w_dist 0.1, lambda_iso 0.01 (src/GSSlam.cu:1241-1250),
 *  Adam 0.9/0.999/1e-8 (src/GSSlam.cu:1282-1284).
 */
typedef struct fvgs_params {
    int32_t tile_w;
    int32_t tile_h;
    float radius_sigma;
    float bg[3];
    float alpha_thresh;
    float color_thresh;
    float depth_thresh;
    float w_depth;
    float w_dist;
    float lambda_iso;
    float adam_beta1;
    float adam_beta2;
    float adam_eps;
    uint32_t quirks;
    /* pseudo-factor eigenvalue floor used by RgbdPoseCost (src/RgbdPoseCost.cu:57) */
    double eig_eps;
} fvgs_params;

/* Per-tile record of the tracking reduction, PoseOptimizationRgbdData
 * (RepresentationClasses.hpp:249-274): Jtr[6] then the 21 upper-triangular
 * JtJ entries, row-major with i <= j. */
#define FVGS_POSEDATA_FLOATS 27

#ifdef __cplusplus
}
#endif
#endif /* FVGS_TYPES_H */
