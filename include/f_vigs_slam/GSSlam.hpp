/*
 * f_vigs_slam/GSSlam.hpp -- C++ mirror of the reference's GSSlam for the
 * Gaussian-splatting hot path (include/f_vigs_slam/GSSlam.cuh:27-175 of
 * jcevasco2003/f_vigs_slam), built on the fvgs C-ABI (include/fvgs.h).
 *
 * Same member names and argument meanings as the reference for the calls
 * that reach the GPU path: setIntrinsics, setImuToCamExtrinsics,
 * initAndCopyImgs, initializeGaussiansFromRgbd, prepareRasterization,
 * renderView, computeRgbdPoseJacobians, optimizeGaussiansKeyframe,
 * removeOutliers, computeCovisibilityRatio, addKeyframe, prune, densify,
 * getGaussiansCount, getGaussianData.  Differences, all forced by working
 * without OpenCV, Eigen and Ceres:
 *  - images are raw host buffers (8-bit colour, 3 bytes per pixel in the
 *    camera's (b, g, r) order; depth float metres or uint16 millimetres)
 *    instead of cv::Mat;
 *  - Eigen arguments are templates (any vector with operator[] and any
 *    quaternion with x(), y(), z(), w(); any 6x6 matrix with operator()(i, j)
 *    and 6-vector with operator[]) so Eigen callers compile unchanged, and
 *    each has a plain-array overload;
 *  - the constructor takes the capacity and the largest frame (the
 *    reference grows its buffers on demand);
 *  - the full SLAM loop (compute, the Ceres problem, the IMU) stays with the
 *    caller; setCurrentPose gives removeOutliers / addKeyframe /
 *    computeCovisibilityRatio the pose the reference keeps in current_pose_.
 * Errors: the reference prints and returns; here every member returns as the
 * reference does and keeps the library status in lastStatus() (0 = ok);
 * computeRgbdPoseJacobians also returns false on failure.
 *
 * Reference behaviours of the host code, selected by fvgs_params.quirks:
 * FVGS_Q_POSE_WXYZ builds the camera orientation as make_float4(w, x, y, z)
 * (src/GSSlam.cu:2121) for kernels that read (x, y, z, w);
 * FVGS_Q_COLOR_RESCALE scales the [0, 1] colour pyramid by 1/255 once more
 * for tracking (src/GSSlam.cu:2158).
 */
#ifndef F_VIGS_SLAM_GSSLAM_HPP
#define F_VIGS_SLAM_GSSLAM_HPP

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "../fvgs.h"
#include "../fvgs_estimator.h"
#include "RepresentationClasses.hpp"

namespace f_vigs_slam {

class GSSlam {
public:
    explicit GSSlam(uint32_t max_gaussians = 1u << 20, int max_width = 1280, int max_height = 720,
                    const fvgs_params* params = nullptr, int device = 0) {
        if (params) params_ = *params;
        else fvgs_params_default(&params_);
        status_ = fvgs_session_create(&params_, device, max_gaussians, max_width, max_height, &s_);
        max_Gaussians = max_gaussians;
    }
    ~GSSlam() {
        if (s_) fvgs_session_destroy(s_);
    }
    GSSlam(const GSSlam&) = delete;
    GSSlam& operator=(const GSSlam&) = delete;

    // ---- configuration (GSSlam.cuh:31-42)
    void setIntrinsics(const IntrinsicParameters& params) {
        intrinsics_ = params;
        intrinsics_set_ = true;
    }
    void setGaussInitSizePx(int size_px) { gauss_init_size_px_ = std::max(1, size_px); }
    void setGaussInitScale(float scale) { gauss_init_scale_ = std::max(1e-5f, scale); }
    template <class V3, class Q, class = std::enable_if_t<std::is_class<Q>::value>>
    void setImuToCamExtrinsics(const V3& t_imu_cam, const Q& q_imu_cam) {
        const double t[3] = {t_imu_cam[0], t_imu_cam[1], t_imu_cam[2]};
        const double q[4] = {q_imu_cam.x(), q_imu_cam.y(), q_imu_cam.z(), q_imu_cam.w()};
        setImuToCamExtrinsics(t, q);
    }
    void setImuToCamExtrinsics(const double t_imu_cam[3], const double q_imu_cam_xyzw[4]) {
        std::memcpy(t_imu_cam_, t_imu_cam, sizeof(t_imu_cam_));
        std::memcpy(q_imu_cam_, q_imu_cam_xyzw, sizeof(q_imu_cam_));
    }
    void setEtaGaussian(float eta) { eta_gaussian_ = std::max(1e-5f, eta); }
    void setCurrentPose(const CameraPose& pose) { current_pose_ = pose; }
    const CameraPose& getCurrentPose() const { return current_pose_; }

    // ---- map (GSSlam.cuh:44-59)
    bool hasGaussians() const { return n_Gaussians > 0; }
    uint32_t getGaussiansCount() const { return n_Gaussians; }
    /* The whole map in the reference's Gaussians SoA layout (fvgs_upload_gaussians). */
    void setGaussians(const float* positions, const float* scales, const float* orientations, const float* colors,
                      const float* opacities, uint32_t n) {
        if (!ok()) return;
        status_ = fvgs_upload_gaussians(s_, positions, scales, orientations, colors, opacities, n);
        if (status_ == FVGS_OK) n_Gaussians = n;
    }
    uint32_t getGaussianData(std::vector<float3>& positions, std::vector<float3>& colors) {
        positions.clear();
        colors.clear();
        if (!ok() || n_Gaussians == 0) return 0;
        const size_t n = n_Gaussians;
        std::vector<float> pos(3 * n), scl(3 * n), rot(4 * n), col(3 * n), opa(n);
        status_ = fvgs_download_gaussians(s_, pos.data(), scl.data(), rot.data(), col.data(), opa.data(),
                                          n_Gaussians);
        if (status_ != FVGS_OK) return 0;
        positions.resize(n);
        colors.resize(n);
        for (size_t i = 0; i < n; ++i) {
            positions[i] = float3{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
            colors[i] = float3{col[3 * i], col[3 * i + 1], col[3 * i + 2]};
        }
        return n_Gaussians;
    }
    /* initializeGaussiansFromRgbd (src/GSSlam.cu:271-407): depth as float
     * metres, or uint16 scaled by 0.001 (depth_u16_mm). */
    void initializeGaussiansFromRgbd(const uint8_t* bgr, const void* depth, int width, int height,
                                     const CameraPose& camera_pose, bool depth_u16_mm = false) {
        if (!ok() || !intrinsics_set_ || !bgr || !depth) return;
        status_ = fvgs_preprocess_frame(s_, bgr, depth, depth_u16_mm ? 1 : 0, width, height, 1, 0);
        loaded_ = Loaded::Other;
        if (status_ != FVGS_OK) return;
        uint32_t n = 0;
        const fvgs_pose p = to_fvgs(camera_pose);
        const fvgs_intrinsics K = to_fvgs(intrinsics_);
        status_ = fvgs_init_gaussians(s_, &p, &K, gauss_init_size_px_, gauss_init_scale_, gauss_init_opacity_, &n);
        if (status_ == FVGS_OK) n_Gaussians = n;
        current_pose_ = camera_pose;
    }

    // ---- frames (GSSlam::initAndCopyImgs, src/GSSlam.cu:1913-1969)
    void initAndCopyImgs(const uint8_t* bgr, const void* depth, int width, int height, bool depth_u16_mm = false) {
        if (!bgr || !depth) return;
        frame_w_ = width;
        frame_h_ = height;
        frame_bgr_.assign(bgr, bgr + (size_t)3 * width * height);
        const size_t db = (size_t)width * height * (depth_u16_mm ? sizeof(uint16_t) : sizeof(float));
        frame_depth_.assign(static_cast<const uint8_t*>(depth), static_cast<const uint8_t*>(depth) + db);
        frame_u16_ = depth_u16_mm;
        loaded_ = Loaded::None;
        load_frame(Loaded::Tracking);
    }

    // ---- rasterization (GSSlam.cuh:66-78)
    void prepareRasterization(const CameraPose& camera_pose, const IntrinsicParameters& intrinsics, int width,
                              int height) {
        if (!ok()) return;
        const fvgs_pose p = to_fvgs(camera_pose);
        const fvgs_intrinsics K = to_fvgs(intrinsics);
        uint32_t n = 0;
        status_ = fvgs_project_bin(s_, &p, &K, width, height, &n);
        last_nb_instances_ = status_ == FVGS_OK ? n : 0;
    }
    /* renderView into caller buffers: float rgb [3 W H], depth [W H], optional 8-bit rgb. */
    bool renderView(const CameraPose& camera_pose, const IntrinsicParameters& intrinsics, int width, int height,
                    float* rendered_rgb, float* rendered_depth, uint8_t* rendered_rgb8 = nullptr) {
        if (!ok()) return false;
        const fvgs_pose p = to_fvgs(camera_pose);
        const fvgs_intrinsics K = to_fvgs(intrinsics);
        status_ = fvgs_render_view(s_, &p, &K, width, height, rendered_rgb, rendered_depth, rendered_rgb8);
        return status_ == FVGS_OK;
    }

    // ---- tracking (GSSlam::computeRgbdPoseJacobians, src/GSSlam.cu:2103-2243)
    template <class M6, class V6, class V3, class Q,
              class = std::enable_if_t<std::is_class<M6>::value && std::is_class<Q>::value>>
    void computeRgbdPoseJacobians(M6& JtJ, V6& Jtr, int level, const V3& P_imu, const Q& Q_imu) {
        const double P[3] = {P_imu[0], P_imu[1], P_imu[2]};
        const double q[4] = {Q_imu.x(), Q_imu.y(), Q_imu.z(), Q_imu.w()};
        double H[36], g[6];
        computeRgbdPoseJacobians(H, g, level, P, q);
        for (int i = 0; i < 6; ++i) {
            Jtr[i] = g[i];
            for (int j = 0; j < 6; ++j) JtJ(i, j) = H[6 * i + j];
        }
    }
    /* IMU pose (P_imu, Q_imu as x, y, z, w) -> camera pose through the
     * extrinsics, binning + Jacobian kernel + reduction on the pyramid level,
     * then the J_cam_imu transform; JtJ row-major.  False (and zeros) on a
     * library error. */
    bool computeRgbdPoseJacobians(double JtJ[36], double Jtr[6], int level, const double P_imu[3],
                                  const double Q_imu[4]) {
        for (int i = 0; i < 36; ++i) JtJ[i] = 0.0;
        for (int i = 0; i < 6; ++i) Jtr[i] = 0.0;
        if (!ok()) return false;
        CameraPose cam;
        imu_to_camera(P_imu, Q_imu, cam);
        const int pyr_level = std::min(level, nb_pyr_levels_ - 1);
        IntrinsicParameters li = intrinsics_;
        const float scale = 1.0f / (float)(1 << pyr_level);
        li.f.x *= scale;
        li.f.y *= scale;
        li.c.x *= scale;
        li.c.y *= scale;
        if (n_Gaussians == 0) return true;
        load_frame(Loaded::Tracking);
        if (status_ != FVGS_OK) return false;
        const fvgs_pose p = to_fvgs(cam);
        const fvgs_intrinsics K = to_fvgs(li);
        double H[36], gc[6];
        status_ = fvgs_track_jacobian(s_, &p, &K, pyr_level, H, gc);
        if (status_ != FVGS_OK) return false;
        status_ = fvgs_jacobian_cam_to_imu(H, gc, q_imu_cam_, t_imu_cam_, Q_imu, JtJ, Jtr);
        return status_ == FVGS_OK;
    }

    // ---- mapping (GSSlam::optimizeGaussiansKeyframe, src/GSSlam.cu:1083-1320)
    void optimizeGaussiansKeyframe(const KeyframeData& keyframe, float eta = 0.002f) {
        if (!ok() || n_Gaussians == 0 || keyframe.color_img.empty() || keyframe.depth_img.empty()) return;
        if (!load_keyframe(keyframe)) return;
        const fvgs_pose p = to_fvgs(keyframe.getPose());
        const fvgs_intrinsics K = to_fvgs(keyframe.getIntrinsics());
        status_ = fvgs_map_step(s_, &p, &K, 0, eta);
    }

    // ---- map maintenance (src/GSSlam.cu:1322-1904)
    void addKeyframe() {
        KeyframeData kf;
        kf.setPose(current_pose_);
        kf.intrinsics = intrinsics_;
        kf.width = frame_w_;
        kf.height = frame_h_;
        kf.color_img = frame_bgr_;
        kf.depth_img = frame_depth_metres();
        kf.keyframe_id = (uint32_t)keyframes_.size();
        keyframes_.push_back(kf);
        current_keyframe_idx_ = (int)keyframes_.size() - 1;
    }
    float computeCovisibilityRatio() {
        if (!ok() || n_Gaussians == 0 || keyframes_.empty() || frame_w_ == 0) return 1.0f;
        size_t idx = (size_t)current_keyframe_idx_;
        if (current_keyframe_idx_ < 0 || idx >= keyframes_.size()) idx = keyframes_.size() - 1;
        const KeyframeData& kf = keyframes_[idx];
        const fvgs_pose pa = to_fvgs(kf.getPose()), pb = to_fvgs(current_pose_);
        const fvgs_intrinsics Ka = to_fvgs(kf.getIntrinsics()), Kb = to_fvgs(intrinsics_);
        float ratio = 0.0f;
        status_ = fvgs_covisibility(s_, &pa, &Ka, kf.getWidth(), kf.getHeight(), &pb, &Kb, frame_w_, frame_h_,
                                    nullptr, nullptr, &ratio);
        return status_ == FVGS_OK ? ratio : 0.0f;
    }
    void removeOutliers() {
        if (!ok() || n_Gaussians == 0 || frame_w_ == 0) return;
        load_frame(Loaded::Tracking);
        if (status_ != FVGS_OK) return;
        const fvgs_pose p = to_fvgs(current_pose_);
        const fvgs_intrinsics K = to_fvgs(intrinsics_);
        uint32_t removed = 0;
        status_ = fvgs_remove_outliers(s_, &p, &K, 0, 0.6f, 1, &removed);
        if (status_ == FVGS_OK) n_Gaussians -= removed;
    }
    void prune() {
        if (!ok() || n_Gaussians == 0) return;
        uint32_t removed = 0;
        status_ = fvgs_prune(s_, 0.05f, 0.05f, 0.005f, 1, &removed);
        if (status_ == FVGS_OK) n_Gaussians -= removed;
    }
    void densify(const KeyframeData& keyframe) {
        if (!ok() || n_Gaussians == 0 || keyframe.color_img.empty() || keyframe.depth_img.empty()) return;
        if (!load_keyframe(keyframe)) return;
        const fvgs_pose p = to_fvgs(keyframe.getPose());
        const fvgs_intrinsics K = to_fvgs(keyframe.getIntrinsics());
        uint32_t added = 0;
        status_ = fvgs_densify(s_, &p, &K, gauss_init_size_px_, nullptr, &added);
        if (status_ == FVGS_OK) n_Gaussians += added;
    }
    const std::vector<KeyframeData>& keyframes() const { return keyframes_; }

    // ---- additions of this interface (status, session, diagnostics)
    int lastStatus() const { return status_; }
    fvgs_session* session() { return s_; }
    uint32_t lastInstanceCount() const { return last_nb_instances_; }
    /* The camera pose computeRgbdPoseJacobians builds from an IMU pose (x, y, z, w). */
    void imu_to_camera(const double P_imu[3], const double Q_imu[4], CameraPose& cam) const {
        // P_cam = P_imu + Q_imu t_imu_cam, Q_cam = Q_imu q_imu_cam (src/GSSlam.cu:2113-2121)
        const double qx = Q_imu[0], qy = Q_imu[1], qz = Q_imu[2], qw = Q_imu[3];
        const double* t = t_imu_cam_;
        double u[3] = {qy * t[2] - qz * t[1], qz * t[0] - qx * t[2], qx * t[1] - qy * t[0]};
        for (double& c : u) c += c;
        const double r[3] = {t[0] + qw * u[0] + (qy * u[2] - qz * u[1]), t[1] + qw * u[1] + (qz * u[0] - qx * u[2]),
                             t[2] + qw * u[2] + (qx * u[1] - qy * u[0])};
        const double* b = q_imu_cam_;
        const double cw = qw * b[3] - qx * b[0] - qy * b[1] - qz * b[2];
        const double cx = qw * b[0] + qx * b[3] + qy * b[2] - qz * b[1];
        const double cy = qw * b[1] + qy * b[3] + qz * b[0] - qx * b[2];
        const double cz = qw * b[2] + qz * b[3] + qx * b[1] - qy * b[0];
        cam.position = float3{(float)(P_imu[0] + r[0]), (float)(P_imu[1] + r[1]), (float)(P_imu[2] + r[2])};
        if (params_.quirks & FVGS_Q_POSE_WXYZ)
            cam.orientation = float4{(float)cw, (float)cx, (float)cy, (float)cz};
        else
            cam.orientation = float4{(float)cx, (float)cy, (float)cz, (float)cw};
    }

private:
    enum class Loaded { None, Tracking, Other };

    bool ok() const { return s_ != nullptr; }
    // The float4 goes to the kernels as it is (the reference passes it raw).
    static fvgs_pose to_fvgs(const CameraPose& c) {
        fvgs_pose p;
        p.position[0] = c.position.x;
        p.position[1] = c.position.y;
        p.position[2] = c.position.z;
        p.orientation[0] = c.orientation.x;
        p.orientation[1] = c.orientation.y;
        p.orientation[2] = c.orientation.z;
        p.orientation[3] = c.orientation.w;
        return p;
    }
    static fvgs_intrinsics to_fvgs(const IntrinsicParameters& k) { return fvgs_intrinsics{k.f.x, k.f.y, k.c.x, k.c.y}; }
    std::vector<float> frame_depth_metres() const {
        const size_t px = (size_t)frame_w_ * frame_h_;
        std::vector<float> d(px);
        if (frame_u16_) {
            const uint16_t* src = reinterpret_cast<const uint16_t*>(frame_depth_.data());
            for (size_t i = 0; i < px; ++i) d[i] = (float)src[i] * 0.001f;
        } else if (frame_depth_.size() >= px * sizeof(float)) {
            std::memcpy(d.data(), frame_depth_.data(), px * sizeof(float));
        }
        return d;
    }
    // The current frame's pyramid on the device, with the tracking colour
    // scaling (the second /255 with FVGS_Q_COLOR_RESCALE).
    void load_frame(Loaded want) {
        if (loaded_ == want || frame_w_ == 0) return;
        status_ = fvgs_preprocess_frame(s_, frame_bgr_.data(), frame_depth_.data(), frame_u16_ ? 1 : 0, frame_w_,
                                        frame_h_, nb_pyr_levels_, (params_.quirks & FVGS_Q_COLOR_RESCALE) ? 1 : 0);
        loaded_ = status_ == FVGS_OK ? want : Loaded::None;
    }
    // A keyframe's images as level 0 (colour scaled once, as its float copy of
    // pyr_color_[0] is in the reference).
    bool load_keyframe(const KeyframeData& kf) {
        status_ = fvgs_preprocess_frame(s_, kf.color_img.data(), kf.depth_img.data(), 0, kf.getWidth(),
                                        kf.getHeight(), 1, 0);
        loaded_ = Loaded::Other;
        return status_ == FVGS_OK;
    }

    fvgs_session* s_ = nullptr;
    fvgs_params params_{};
    int status_ = FVGS_OK;
    uint32_t n_Gaussians = 0, max_Gaussians = 0, last_nb_instances_ = 0;
    IntrinsicParameters intrinsics_{};
    bool intrinsics_set_ = false;
    int gauss_init_size_px_ = 10;
    float gauss_init_scale_ = 2.0f;
    float gauss_init_opacity_ = 0.8f;
    float eta_gaussian_ = 0.002f;
    int nb_pyr_levels_ = 3;
    double t_imu_cam_[3] = {0.0, 0.0, 0.0};
    double q_imu_cam_[4] = {0.0, 0.0, 0.0, 1.0};
    CameraPose current_pose_;
    std::vector<uint8_t> frame_bgr_, frame_depth_;
    int frame_w_ = 0, frame_h_ = 0;
    bool frame_u16_ = false;
    Loaded loaded_ = Loaded::None;
    std::vector<KeyframeData> keyframes_;
    int current_keyframe_idx_ = 0;
};

}  // namespace f_vigs_slam

#endif
