/*
 * f_vigs_slam/RgbdPoseCost.hpp -- C++ mirror of the reference's Ceres cost
 * function for the RGB-D pose term (include/f_vigs_slam/RgbdPoseCost.hpp:38-89,
 * src/RgbdPoseCost.cu:10-108 of jcevasco2003/f_vigs_slam) on the fvgs C-ABI.
 *
 * Same interface: constructed on a non-owning GSSlam*, update(level) selects
 * the pyramid level, Evaluate(parameters, residuals, jacobians) with
 * parameters[0] = the IMU pose [x, y, z, qx, qy, qz, qw], 6 residuals and an
 * optional 6 x 7 row-major Jacobian.  Evaluate asks GSSlam for the IMU-frame
 * JtJ / Jtr, turns them into the eigen-regularised pseudo factor (eigenvalues
 * above 1e-4 kept: r* = sqrt(1/l) U^T Jtr, J* = sqrt(l) U^T) and writes J*
 * into the first six columns (the seventh, the quaternion's over-
 * parameterisation, is zero).  The one difference from the reference, which
 * always returns true: Evaluate returns false when the library reports an
 * error, which Ceres treats as an unsuccessful step.
 */
#ifndef F_VIGS_SLAM_RGBD_POSE_COST_HPP
#define F_VIGS_SLAM_RGBD_POSE_COST_HPP

#include "GSSlam.hpp"
#include "ceres_compat.hpp"

namespace f_vigs_slam {

class RgbdPoseCostFunction : public ceres::SizedCostFunction<6, 7> {
public:
    explicit RgbdPoseCostFunction(GSSlam* gs_slam) : gs_slam_(gs_slam), level_(0) {}
    ~RgbdPoseCostFunction() override = default;

    void update(int level) { level_ = level; }

    bool Evaluate(double const* const* parameters, double* residuals, double** jacobians) const override {
        return const_cast<RgbdPoseCostFunction*>(this)->EvaluateNonConst(parameters, residuals, jacobians);
    }

    bool EvaluateNonConst(double const* const* parameters, double* residuals, double** jacobians) {
        if (!gs_slam_ || !parameters || !parameters[0] || !residuals) return false;
        const double* x = parameters[0];
        double JtJ[36], Jtr[6];
        if (!gs_slam_->computeRgbdPoseJacobians(JtJ, Jtr, level_, x, x + 3)) return false;
        double r_star[6], J_star[36];
        if (fvgs_pseudo_factor(JtJ, Jtr, 1e-4, r_star, J_star) != FVGS_OK) return false;
        for (int i = 0; i < 6; ++i) residuals[i] = r_star[i];
        if (jacobians && jacobians[0]) {
            double* J = jacobians[0];
            for (int i = 0; i < 6; ++i) {
                for (int j = 0; j < 6; ++j) J[7 * i + j] = J_star[6 * i + j];
                J[7 * i + 6] = 0.0;
            }
        }
        return true;
    }

private:
    GSSlam* gs_slam_;
    int level_;
};

}  // namespace f_vigs_slam

#endif
