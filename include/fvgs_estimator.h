/*
 * fvgs_estimator.h -- host FP64 estimator glue of the fvgs library: what the
 * reference's Ceres-based visual-inertial solve does around the GPU pose
 * Jacobian, as plain C calls (no Eigen, no Ceres).  Everything here runs on
 * the host in FP64: the GPU path returns the 6x6 system and these small dense
 * solves consume it.
 *
 * Conventions: matrices row-major; quaternions (x, y, z, w) (the coefficient
 * order of the reference's 7-double pose blocks p.xyz, q.xyzw); a speed-bias
 * block is v.xyz, ba.xyz, bg.xyz.
 */
#ifndef FVGS_ESTIMATOR_H
#define FVGS_ESTIMATOR_H

#include "fvgs_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/*
 * The IMU-frame system from the camera-frame one (GSSlam::computeRgbdPoseJacobians,
 * src/GSSlam.cu:2233-2243): J = [[I, -R_imu [t_imu_cam]x], [0, R_imu_cam^T]],
 * JtJ_imu = J^T JtJ_cam J, Jtr_imu = J^T Jtr_cam.  Outputs may alias nothing.
 */
int fvgs_jacobian_cam_to_imu(const double JtJ_cam[36], const double Jtr_cam[6], const double q_imu_cam[4],
                             const double t_imu_cam[3], const double q_imu[4], double JtJ_imu[36],
                             double Jtr_imu[6]);

/*
 * The eigen-regularised pseudo factor of RgbdPoseCostFunction::Evaluate
 * (src/RgbdPoseCost.cu:57-106): with JtJ = U diag(l) U^T (eigenvalues
 * ascending) and l kept where l > eps (1e-4 in the reference), J* = sqrt(l) U^T
 * (6x6) and r* = sqrt(1/l) U^T Jtr, so J*^T J* and J*^T r* reproduce the kept
 * part of the system.  Eigenvector signs are arbitrary, as in the reference.
 */
int fvgs_pseudo_factor(const double JtJ[36], const double Jtr[6], double eps, double r_star[6], double J_star[36]);

/*
 * IMU preintegration between two keyframes (Preintegration,
 * src/Preintegration.cpp:12-193): midpoint integration of the IMU samples
 * with first-order propagation of the 15x15 bias Jacobian and covariance
 * (noise densities acc_n, gyr_n, random walks acc_w, gyr_w).  The first
 * sample and the linearisation biases are given at creation.
 */
typedef struct fvgs_preint fvgs_preint;
int fvgs_preint_create(const double acc0[3], const double gyr0[3], const double ba[3], const double bg[3],
                       double acc_n, double gyr_n, double acc_w, double gyr_w, fvgs_preint** out);
int fvgs_preint_destroy(fvgs_preint* p);
int fvgs_preint_add(fvgs_preint* p, double dt, const double acc[3], const double gyr[3]);
/* Re-integrate every stored sample about new linearisation biases. */
int fvgs_preint_repropagate(fvgs_preint* p, const double ba[3], const double bg[3]);
/* Increments, integrated time, 15x15 Jacobian and covariance; any pointer may be null. */
int fvgs_preint_state(const fvgs_preint* p, double delta_p[3], double delta_q[4], double delta_v[3],
                      double* sum_dt, double jacobian[225], double covariance[225]);
/* Unweighted 15-dim residual (position, rotation vector part, velocity, bias
 * differences) with first-order bias correction (Preintegration::evaluate). */
int fvgs_preint_evaluate(const fvgs_preint* p, const double pose_i[7], const double speedbias_i[9],
                         const double pose_j[7], const double speedbias_j[9], double residual[15]);
/* State at j predicted from state i (Preintegration::predict). */
int fvgs_preint_predict(const fvgs_preint* p, const double pose_i[7], const double v_i[3], double pose_j[7],
                        double v_j[3]);

/*
 * The 15-dim IMU factor (ImuCostFunction::Evaluate, src/ImuCostFunction.cpp:
 * 88-215): repropagates when the bias estimate moved past 0.10 (accelerometer)
 * or 0.01 (gyroscope), whitens the residual with the upper Cholesky factor of
 * the inverse covariance, and fills the Jacobians with respect to pose_i
 * (15x7), speedbias_i (15x9), pose_j (15x7), speedbias_j (15x9); any Jacobian
 * pointer may be null.  FVGS_E_STATE if the covariance is not invertible
 * (e.g. no sample integrated yet).
 */
int fvgs_imu_factor(fvgs_preint* p, const double pose_i[7], const double speedbias_i[9], const double pose_j[7],
                    const double speedbias_j[9], double residual[15], double J_pose_i[105], double J_sb_i[135],
                    double J_pose_j[105], double J_sb_j[135]);

/*
 * Marginalization prior (MarginalizationInfo::marginalize,
 * src/MarginalizationFactor.cpp:278-360): A ((m+n) x (m+n)) and b of the
 * linearised factors, the first m (local) dimensions to be marginalised.
 * With eigenvalue-thresholded pseudo-inverses (threshold eps, 1e-8 in the
 * reference): A* = Arr - Arm Amm^+ Amr, b* = brr - Arm Amm^+ bmm, then
 * J = sqrt(S) V^T (n x n) and r = sqrt(S^-1) V^T b* from A* = V S V^T.
 */
int fvgs_marginalize(const double* A, const double* b, int m, int n, double eps, double* J, double* r);
/*
 * Prior residual r + J dx and its Jacobians (MarginalizationFactor::Evaluate,
 * src/MarginalizationFactor.cpp:398-470) for n_blocks kept parameter blocks:
 * block k has global size block_size[k] (7: a pose, whose local difference is
 * (p - p0, 2 vec(q0^-1 q), sign-flipped when its w < 0)), its local offset
 * block_idx[k] in [0, n), current value x[k] and linearisation point x0[k].
 * jacobians (may be null, or hold nulls) receive n x block_size[k] row-major
 * blocks whose last column is zero for poses.
 */
int fvgs_marginal_prior_evaluate(const double* J, const double* r, int n, int n_blocks, const int* block_size,
                                 const int* block_idx, const double* const* x, const double* const* x0,
                                 double* residual, double* const* jacobians);

/*
 * One Gauss-Newton step of the visual-inertial problem the reference gives
 * Ceres (GSSlam constructor, src/GSSlam.cu:150-185; optimizeWithCeres,
 * src/GSSlam.cu:2246-2290): the RGB-D pseudo factor on pose_j (from the
 * IMU-frame JtJ / Jtr of fvgs_jacobian_cam_to_imu, eigenvalues above eps
 * kept), the IMU factor between states i and j, and, when prior_J is given,
 * the marginalization prior on state i (prior_J 15x15, prior_r 15, its
 * linearisation point prior_x0 = pose 7 + speed-bias 9).  Without a prior
 * state i is held fixed and the normal equations are the 15-dim ones of
 * state j; with it both states move (30 dims: pose_i, speedbias_i, pose_j,
 * speedbias_j in local coordinates).  The system is solved in FP64
 * (Cholesky; an eigen-thresholded pseudo-inverse if it is not positive
 * definite) and the step applied as PoseLocalParameterization::Plus
 * (src/PoseLocalParameterization.cpp:22-44: p + dp, (q (x) [dtheta/2, 1])
 * normalised) and additively for the speed-bias blocks.  cost (may be null)
 * receives 0.5 (|r*|^2 + |r_imu|^2 + |r_prior|^2) before the step; delta (may
 * be null) the 30 local increments (zeros for a fixed state i).
 */
int fvgs_vi_step(fvgs_preint* p, const double JtJ_imu[36], const double Jtr_imu[6], double eps,
                 const double* prior_J, const double* prior_r, const double* prior_x0, double pose_i[7],
                 double speedbias_i[9], double pose_j[7], double speedbias_j[9], double* cost, double delta[30]);
/*
 * The prior the next frame starts from (the marginalization at the end of a
 * tracked frame, src/GSSlam.cu:958-973 with MarginalizationInfo): every
 * factor of fvgs_vi_step linearised at the given states, state i (15 local
 * dims) marginalised by fvgs_marginalize (threshold 1e-8): new_J 15x15,
 * new_r 15 on state j, new_x0 = (pose_j, speedbias_j).  The outputs may
 * alias the prior inputs: those are read before any output is written.
 */
int fvgs_vi_marginalize(fvgs_preint* p, const double JtJ_imu[36], const double Jtr_imu[6], double eps,
                        const double* prior_J, const double* prior_r, const double* prior_x0,
                        const double pose_i[7], const double speedbias_i[9], const double pose_j[7],
                        const double speedbias_j[9], double new_J[225], double new_r[15], double new_x0[16]);

#ifdef __cplusplus
}
#endif
#endif /* FVGS_ESTIMATOR_H */
