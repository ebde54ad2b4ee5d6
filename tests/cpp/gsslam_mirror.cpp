// Drives the C++ mirror of GSSlam / RgbdPoseCostFunction (include/f_vigs_slam)
// the way the reference's Ceres problem does: a map and a camera frame in,
// an IMU pose, Evaluate().  Reads its inputs from a binary file written by
// tests/test_gsslam_mirror.py and writes the results to another.
//
// input : int32 n, W, H, level; float32 positions[3n] scales[3n]
//         orientations[4n] colors[3n] opacities[n]; uint8 bgr[3WH];
//         float32 depth[WH]; float32 fx fy cx cy; float64 t_imu_cam[3]
//         q_imu_cam[4] (x,y,z,w) imu_pose[7] (p, q x,y,z,w)
// output: int32 status; float32 camera position[3] orientation[4] (raw);
//         float64 JtJ[36] Jtr[6] (IMU frame); int32 evaluate_ok;
//         float64 residuals[6] jacobian[42]; uint32 n_gaussians;
//         then the map maintenance at the camera pose: int32 status after
//         each of removeOutliers, computeCovisibilityRatio, prune, densify,
//         optimizeGaussiansKeyframe, renderView; uint32 count after
//         removeOutliers, prune, densify; float32 covisibility ratio
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <f_vigs_slam/RgbdPoseCost.hpp>

template <class T>
static bool rd(FILE* f, T* p, size_t n) { return fread(p, sizeof(T), n, f) == n; }
template <class T>
static void wr(FILE* f, const T* p, size_t n) { fwrite(p, sizeof(T), n, f); }

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* in = fopen(argv[1], "rb");
    if (!in) return 2;
    int32_t hdr[4];
    if (!rd(in, hdr, 4)) return 3;
    const int n = hdr[0], W = hdr[1], H = hdr[2], level = hdr[3];
    std::vector<float> pos(3 * (size_t)n), scl(3 * (size_t)n), rot(4 * (size_t)n), col(3 * (size_t)n), opa(n);
    std::vector<uint8_t> bgr(3 * (size_t)W * H);
    std::vector<float> depth((size_t)W * H);
    float K[4];
    double t_ic[3], q_ic[4], imu[7];
    if (!rd(in, pos.data(), pos.size()) || !rd(in, scl.data(), scl.size()) || !rd(in, rot.data(), rot.size()) ||
        !rd(in, col.data(), col.size()) || !rd(in, opa.data(), opa.size()) || !rd(in, bgr.data(), bgr.size()) ||
        !rd(in, depth.data(), depth.size()) || !rd(in, K, 4) || !rd(in, t_ic, 3) || !rd(in, q_ic, 4) ||
        !rd(in, imu, 7))
        return 3;
    fclose(in);

    f_vigs_slam::GSSlam slam((uint32_t)n, W, H);
    f_vigs_slam::IntrinsicParameters intr;
    intr.f = float2{K[0], K[1]};
    intr.c = float2{K[2], K[3]};
    slam.setIntrinsics(intr);
    slam.setImuToCamExtrinsics(t_ic, q_ic);
    slam.setGaussians(pos.data(), scl.data(), rot.data(), col.data(), opa.data(), (uint32_t)n);
    slam.initAndCopyImgs(bgr.data(), depth.data(), W, H);

    f_vigs_slam::CameraPose cam;
    slam.imu_to_camera(imu, imu + 3, cam);
    double JtJ[36], Jtr[6];
    const bool jac_ok = slam.computeRgbdPoseJacobians(JtJ, Jtr, level, imu, imu + 3);

    f_vigs_slam::RgbdPoseCostFunction cost(&slam);
    cost.update(level);
    const double* params[1] = {imu};
    double residuals[6] = {}, jac[42] = {};
    double* jacs[1] = {jac};
    const ceres::CostFunction& cf = cost;
    const int32_t eval_ok = cf.Evaluate(params, residuals, jacs) ? 1 : 0;

    FILE* out = fopen(argv[2], "wb");
    if (!out) return 2;
    const int32_t status = jac_ok ? slam.lastStatus() : (slam.lastStatus() ? slam.lastStatus() : -100);
    wr(out, &status, 1);
    const float cp[7] = {cam.position.x, cam.position.y, cam.position.z, cam.orientation.x, cam.orientation.y,
                         cam.orientation.z, cam.orientation.w};
    wr(out, cp, 7);
    wr(out, JtJ, 36);
    wr(out, Jtr, 6);
    wr(out, &eval_ok, 1);
    wr(out, residuals, 6);
    wr(out, jac, 42);
    const uint32_t count = slam.getGaussiansCount();
    wr(out, &count, 1);

    // map maintenance as the reference's loop runs it after tracking
    slam.setCurrentPose(cam);
    slam.addKeyframe();
    int32_t st[6];
    uint32_t counts[3];
    slam.removeOutliers();
    st[0] = slam.lastStatus();
    counts[0] = slam.getGaussiansCount();
    const float ratio = slam.computeCovisibilityRatio();
    st[1] = slam.lastStatus();
    slam.prune();
    st[2] = slam.lastStatus();
    counts[1] = slam.getGaussiansCount();
    slam.densify(slam.keyframes()[0]);
    st[3] = slam.lastStatus();
    counts[2] = slam.getGaussiansCount();
    slam.optimizeGaussiansKeyframe(slam.keyframes()[0]);
    st[4] = slam.lastStatus();
    std::vector<float> img_rgb(3 * (size_t)W * H), img_d((size_t)W * H);
    slam.renderView(cam, intr, W, H, img_rgb.data(), img_d.data());
    st[5] = slam.lastStatus();
    wr(out, st, 6);
    wr(out, counts, 3);
    wr(out, &ratio, 1);
    fclose(out);
    printf("gsslam mirror: status %d evaluate %d gaussians %u\n", status, eval_ok, count);
    return 0;
}
