// estimator.cpp -- host FP64 estimator glue around the GPU pose Jacobian:
// the camera-to-IMU transform of JtJ / Jtr, the eigen-regularised pseudo
// factor of RgbdPoseCost, IMU preintegration with its 15-dim factor, and the
// Schur complement of the marginalization prior.
//
// References (jcevasco2003/f_vigs_slam):
//   GSSlam::computeRgbdPoseJacobians, src/GSSlam.cu:2233-2243 (J_cam_imu)
//   RgbdPoseCostFunction::Evaluate, src/RgbdPoseCost.cu:57-106 (pseudo factor)
//   Preintegration, src/Preintegration.cpp:12-193 (midpoint preintegration,
//     first-order bias correction; gravity (0, 0, 9.81))
//   ImuCostFunction::Evaluate, src/ImuCostFunction.cpp:88-215 (15-dim IMU
//     factor; its Jacobians use gravity (0, 0, 9.8), include/f_vigs_slam/
//     ImuCostFunction.hpp:19)
//   MarginalizationInfo::marginalize / MarginalizationFactor::Evaluate,
//     src/MarginalizationFactor.cpp:278-360,398-470 (eigen-thresholded Schur
//     complement, prior residual with the quaternion local difference)
//   the Ceres problem of GSSlam (src/GSSlam.cu:150-185, 2246-2290) and the
//     end-of-frame marginalization (958-973), as Gauss-Newton steps over the
//     15 / 30 local dimensions of the two states
//
// All of it stays FP64 on the host: these are the small dense solves the GPU
// path hands its 6x6 system to.  Quaternions are (x, y, z, w) arrays, the
// coefficient order of the reference's parameter blocks; the quaternion
// arithmetic follows the formulas the reference's Eigen calls evaluate
// (rotation of a vector by v + w t + q x t with t = 2 q x v, rotation matrix
// from the unit-quaternion formula), applied as written even where the
// reference applies them to a not-yet-normalised quaternion.  The symmetric
// eigendecompositions use the cyclic Jacobi method; eigenvalues ascend, as
// Eigen's SelfAdjointEigenSolver returns them.
#include <array>
#include <cmath>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

#include "../../include/fvgs_estimator.h"

namespace {

using V3 = std::array<double, 3>;

struct Quat {
    double x, y, z, w;
};

Quat qmul(const Quat& a, const Quat& b) {
    return {a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
            a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}
Quat qinv(const Quat& q) {
    const double n2 = q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w;
    if (n2 > 0.0) return {-q.x / n2, -q.y / n2, -q.z / n2, q.w / n2};
    return {0.0, 0.0, 0.0, 0.0};
}
Quat qnormalized(const Quat& q) {
    const double n = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (n > 0.0) return {q.x / n, q.y / n, q.z / n, q.w / n};
    return q;
}
V3 cross(const V3& a, const V3& b) {
    return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
// q * v as the reference's quaternion-vector product evaluates it
V3 qrot(const Quat& q, const V3& v) {
    const V3 qv = {q.x, q.y, q.z};
    V3 t = cross(qv, v);
    t = {2.0 * t[0], 2.0 * t[1], 2.0 * t[2]};
    const V3 c = cross(qv, t);
    return {v[0] + q.w * t[0] + c[0], v[1] + q.w * t[1] + c[1], v[2] + q.w * t[2] + c[2]};
}
// rotation matrix of a quaternion (unit-quaternion formula), row-major
void qmat(const Quat& q, double R[9]) {
    const double tx = 2.0 * q.x, ty = 2.0 * q.y, tz = 2.0 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    R[0] = 1.0 - (tyy + tzz), R[1] = txy - twz, R[2] = txz + twy;
    R[3] = txy + twz, R[4] = 1.0 - (txx + tzz), R[5] = tyz - twx;
    R[6] = txz - twy, R[7] = tyz + twx, R[8] = 1.0 - (txx + tyy);
}
void skew(const V3& v, double S[9]) {
    S[0] = 0.0, S[1] = -v[2], S[2] = v[1];
    S[3] = v[2], S[4] = 0.0, S[5] = -v[0];
    S[6] = -v[1], S[7] = v[0], S[8] = 0.0;
}

// Dense row-major helpers: C (r x c) = A (r x k) * B (k x c)
void matmul(const double* A, const double* B, double* C, int r, int k, int c) {
    for (int i = 0; i < r; ++i)
        for (int j = 0; j < c; ++j) {
            double s = 0.0;
            for (int t = 0; t < k; ++t) s += A[i * k + t] * B[t * c + j];
            C[i * c + j] = s;
        }
}
// C = A * B^T
void matmul_bt(const double* A, const double* B, double* C, int r, int k, int c) {
    for (int i = 0; i < r; ++i)
        for (int j = 0; j < c; ++j) {
            double s = 0.0;
            for (int t = 0; t < k; ++t) s += A[i * k + t] * B[j * k + t];
            C[i * c + j] = s;
        }
}
// 3x3 block (br, bc) of a row-major matrix with ld columns
void set_block(double* M, int ld, int br, int bc, const double B[9], double scale = 1.0) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) M[(br + i) * ld + bc + j] = scale * B[i * 3 + j];
}
void get_block(const double* M, int ld, int br, int bc, double B[9]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[i * 3 + j] = M[(br + i) * ld + bc + j];
}
void m3mul(const double* A, const double* B, double* C) { matmul(A, B, C, 3, 3, 3); }
V3 m3v(const double* A, const V3& v) {
    return {A[0] * v[0] + A[1] * v[1] + A[2] * v[2], A[3] * v[0] + A[4] * v[1] + A[5] * v[2],
            A[6] * v[0] + A[7] * v[1] + A[8] * v[2]};
}
void m3t(const double* A, double* T) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[j * 3 + i] = A[i * 3 + j];
}

// Symmetric eigendecomposition A = V diag(w) V^T by cyclic Jacobi rotations
// (Golub & Van Loan, Matrix Computations, 8.5).  A (n x n, row-major) is
// symmetrised first; w ascending, V's columns the eigenvectors.
void sym_eig(const double* A_in, int n, double* w, double* V) {
    std::vector<double> A(A_in, A_in + (size_t)n * n);
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) {
            const double s = 0.5 * (A[i * n + j] + A[j * n + i]);
            A[i * n + j] = A[j * n + i] = s;
        }
    for (int i = 0; i < n * n; ++i) V[i] = 0.0;
    for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i) {
            diag += A[i * n + i] * A[i * n + i];
            for (int j = i + 1; j < n; ++j) off += A[i * n + j] * A[i * n + j];
        }
        if (off <= 1e-30 * diag || off == 0.0) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (apq == 0.0) continue;
                const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // A <- A J
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^T A
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {  // V <- V J
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    // ascending order
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    for (int i = 1; i < n; ++i)
        for (int j = i; j > 0 && A[idx[j] * n + idx[j]] < A[idx[j - 1] * n + idx[j - 1]]; --j) std::swap(idx[j], idx[j - 1]);
    std::vector<double> Vs((size_t)n * n);
    for (int c = 0; c < n; ++c) {
        w[c] = A[idx[c] * n + idx[c]];
        for (int r = 0; r < n; ++r) Vs[r * n + c] = V[r * n + idx[c]];
    }
    std::memcpy(V, Vs.data(), sizeof(double) * n * n);
}

// J = sqrt(S) V^T and r = sqrt(S^-1) V^T g with S the eigenvalues above eps
// (zero below): the factor whose J^T J and J^T r reproduce the thresholded
// system.
void eig_factor(const double* A, const double* g, int n, double eps, double* J, double* r) {
    std::vector<double> w(n), V((size_t)n * n);
    sym_eig(A, n, w.data(), V.data());
    for (int i = 0; i < n; ++i) {
        const bool keep = w[i] > eps;
        const double s = keep ? std::sqrt(w[i]) : 0.0;
        const double si = keep ? std::sqrt(1.0 / w[i]) : 0.0;
        double proj = 0.0;
        for (int k = 0; k < n; ++k) {
            J[i * n + k] = s * V[k * n + i];
            proj += V[k * n + i] * g[k];
        }
        r[i] = si * proj;
    }
}

const V3 kGravityPreint = {0.0, 0.0, 9.81};
const V3 kGravityFactor = {0.0, 0.0, 9.8};

}  // namespace

struct fvgs_preint {
    V3 acc0, gyr0;            // last sample
    V3 lin_acc, lin_gyr;      // first sample (repropagation restarts here)
    V3 ba, bg;                // linearisation biases
    V3 dp, dv;
    Quat dq;
    double sum_dt = 0.0;
    double jac[225];          // 15 x 15
    double cov[225];
    double noise[324];        // 18 x 18
    std::vector<double> dt_buf;
    std::vector<V3> acc_buf, gyr_buf;

    void reset() {
        dp = {0.0, 0.0, 0.0};
        dv = {0.0, 0.0, 0.0};
        dq = {0.0, 0.0, 0.0, 1.0};
        sum_dt = 0.0;
        for (int i = 0; i < 225; ++i) jac[i] = (i % 16 == 0) ? 1.0 : 0.0;
        std::memset(cov, 0, sizeof(cov));
    }

    // one midpoint step (Preintegration::propagate, src/Preintegration.cpp:72-147)
    void propagate(double dt, const V3& acc1, const V3& gyr1) {
        const Quat prev_dq = dq;
        const V3 a0b = {acc0[0] - ba[0], acc0[1] - ba[1], acc0[2] - ba[2]};
        const V3 un_acc_0 = qrot(dq, a0b);
        const V3 un_gyr = {0.5 * (gyr0[0] + gyr1[0]) - bg[0], 0.5 * (gyr0[1] + gyr1[1]) - bg[1],
                           0.5 * (gyr0[2] + gyr1[2]) - bg[2]};
        dq = qmul(dq, Quat{un_gyr[0] * dt * 0.5, un_gyr[1] * dt * 0.5, un_gyr[2] * dt * 0.5, 1.0});
        const V3 a1b = {acc1[0] - ba[0], acc1[1] - ba[1], acc1[2] - ba[2]};
        const V3 un_acc_1 = qrot(dq, a1b);
        V3 un_acc;
        for (int k = 0; k < 3; ++k) un_acc[k] = 0.5 * (un_acc_0[k] + un_acc_1[k]);
        for (int k = 0; k < 3; ++k) {
            dp[k] = dp[k] + dv[k] * dt + 0.5 * un_acc[k] * dt * dt;
            dv[k] = dv[k] + un_acc[k] * dt;
        }
        double Rw[9], Ra0[9], Ra1[9], Rk[9], Rp[9];
        skew(un_gyr, Rw);
        skew(a0b, Ra0);
        skew(a1b, Ra1);
        qmat(dq, Rk);
        qmat(prev_dq, Rp);
        double ImW[9];  // I - [w]x dt
        for (int i = 0; i < 9; ++i) ImW[i] = ((i % 4 == 0) ? 1.0 : 0.0) - Rw[i] * dt;
        double RkRa1[9], RkRa1ImW[9], RpRa0[9], RkRa0[9], Rsum[9];
        m3mul(Rk, Ra1, RkRa1);
        m3mul(RkRa1, ImW, RkRa1ImW);
        m3mul(Rp, Ra0, RpRa0);
        m3mul(Rk, Ra0, RkRa0);
        for (int i = 0; i < 9; ++i) Rsum[i] = Rp[i] + Rk[i];
        const double dt2 = dt * dt;
        static const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        double F[225] = {};
        set_block(F, 15, 0, 0, I3);
        double b03[9];
        for (int i = 0; i < 9; ++i) b03[i] = -0.25 * RkRa0[i] * dt2 + -0.25 * RkRa1ImW[i] * dt2;
        set_block(F, 15, 0, 3, b03);
        set_block(F, 15, 0, 6, I3, dt);
        set_block(F, 15, 0, 9, Rsum, -0.25 * dt2);
        set_block(F, 15, 0, 12, RkRa1, -0.25 * dt2 * -dt);
        set_block(F, 15, 3, 3, ImW);
        set_block(F, 15, 3, 12, I3, -1.0 * dt);
        double b63[9];
        for (int i = 0; i < 9; ++i) b63[i] = -0.5 * RpRa0[i] * dt + -0.5 * RkRa1ImW[i] * dt;
        set_block(F, 15, 6, 3, b63);
        set_block(F, 15, 6, 6, I3);
        set_block(F, 15, 6, 9, Rsum, -0.5 * dt);
        set_block(F, 15, 6, 12, RkRa1, -0.5 * dt * -dt);
        set_block(F, 15, 9, 9, I3);
        set_block(F, 15, 12, 12, I3);
        double V[270] = {};  // 15 x 18
        auto setv = [&](int br, int bc, const double* B, double s) {
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) V[(br + i) * 18 + bc + j] = s * B[i * 3 + j];
        };
        setv(0, 0, Rp, 0.25 * dt2);
        setv(0, 3, RkRa1, -0.25 * dt2 * 0.5 * dt);
        setv(0, 6, Rk, 0.25 * dt2);
        setv(0, 9, RkRa1, -0.25 * dt2 * 0.5 * dt);
        setv(3, 3, I3, 0.5 * dt);
        setv(3, 9, I3, 0.5 * dt);
        setv(6, 0, Rp, 0.5 * dt);
        setv(6, 3, RkRa1, -0.5 * dt * 0.5 * dt);
        setv(6, 6, Rk, 0.5 * dt);
        setv(6, 9, RkRa1, -0.5 * dt * 0.5 * dt);
        setv(9, 12, I3, dt);
        setv(12, 15, I3, dt);
        double nj[225], FC[225], FCFt[225], VN[270], VNVt[225];
        matmul(F, jac, nj, 15, 15, 15);
        std::memcpy(jac, nj, sizeof(jac));
        matmul(F, cov, FC, 15, 15, 15);
        matmul_bt(FC, F, FCFt, 15, 15, 15);
        matmul(V, noise, VN, 15, 18, 18);
        matmul_bt(VN, V, VNVt, 15, 18, 15);
        for (int i = 0; i < 225; ++i) cov[i] = FCFt[i] + VNVt[i];
        dq = qnormalized(dq);
        sum_dt += dt;
        acc0 = acc1;
        gyr0 = gyr1;
    }
};

namespace {

V3 v3(const double* p) { return {p[0], p[1], p[2]}; }
Quat q4(const double* p) { return {p[0], p[1], p[2], p[3]}; }

// first-order bias-corrected increments (Preintegration::evaluate)
void corrected(const fvgs_preint* P, const V3& Bai, const V3& Bgi, Quat& cdq, V3& cdv, V3& cdp) {
    double dp_dba[9], dp_dbg[9], dq_dbg[9], dv_dba[9], dv_dbg[9];
    get_block(P->jac, 15, 0, 9, dp_dba);
    get_block(P->jac, 15, 0, 12, dp_dbg);
    get_block(P->jac, 15, 3, 12, dq_dbg);
    get_block(P->jac, 15, 6, 9, dv_dba);
    get_block(P->jac, 15, 6, 12, dv_dbg);
    const V3 dba = {Bai[0] - P->ba[0], Bai[1] - P->ba[1], Bai[2] - P->ba[2]};
    const V3 dbg = {Bgi[0] - P->bg[0], Bgi[1] - P->bg[1], Bgi[2] - P->bg[2]};
    const V3 th = m3v(dq_dbg, dbg);
    cdq = qmul(P->dq, Quat{th[0] / 2.0, th[1] / 2.0, th[2] / 2.0, 1.0});
    const V3 a = m3v(dv_dba, dba), b = m3v(dv_dbg, dbg), c = m3v(dp_dba, dba), d = m3v(dp_dbg, dbg);
    for (int k = 0; k < 3; ++k) {
        cdv[k] = P->dv[k] + a[k] + b[k];
        cdp[k] = P->dp[k] + c[k] + d[k];
    }
}

void residual15(const fvgs_preint* P, const double* pose_i, const double* sb_i, const double* pose_j,
                const double* sb_j, double r[15]) {
    const V3 Pi = v3(pose_i), Vi = v3(sb_i), Bai = v3(sb_i + 3), Bgi = v3(sb_i + 6);
    const V3 Pj = v3(pose_j), Vj = v3(sb_j), Baj = v3(sb_j + 3), Bgj = v3(sb_j + 6);
    const Quat Qi = q4(pose_i + 3), Qj = q4(pose_j + 3);
    Quat cdq;
    V3 cdv, cdp;
    corrected(P, Bai, Bgi, cdq, cdv, cdp);
    const Quat Qii = qinv(Qi);
    const double T = P->sum_dt;
    const V3 G = kGravityPreint;
    V3 a, b;
    for (int k = 0; k < 3; ++k) {
        a[k] = 0.5 * G[k] * T * T + Pj[k] - Pi[k] - Vi[k] * T;
        b[k] = G[k] * T + Vj[k] - Vi[k];
    }
    const V3 ra = qrot(Qii, a), rb = qrot(Qii, b);
    const Quat e = qmul(qinv(cdq), qmul(Qii, Qj));
    for (int k = 0; k < 3; ++k) {
        r[k] = ra[k] - cdp[k];
        r[6 + k] = rb[k] - cdv[k];
        r[9 + k] = Baj[k] - Bai[k];
        r[12 + k] = Bgj[k] - Bgi[k];
    }
    r[3] = e.x, r[4] = e.y, r[5] = e.z;
}

// Qleft / Qright of the reference (4x4 on (w, x, y, z)); their lower-right 3x3
void qleft_br(const Quat& q, double B[9]) {
    const double w = q.w, x = q.x, y = q.y, z = q.z;
    const double M[16] = {w, -x, -y, -z, x, w, -z, y, y, z, w, -x, z, -y, x, w};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[i * 3 + j] = M[(i + 1) * 4 + j + 1];
}
void qleft_qright_br(const Quat& a, const Quat& b, double B[9]) {
    const double w = a.w, x = a.x, y = a.y, z = a.z;
    const double L[16] = {w, -x, -y, -z, x, w, -z, y, y, z, w, -x, z, -y, x, w};
    const double w2 = b.w, x2 = b.x, y2 = b.y, z2 = b.z;
    const double R[16] = {w2, -x2, -y2, -z2, x2, w2, z2, -y2, y2, -z2, w2, x2, z2, y2, -x2, w2};
    double M[16];
    matmul(L, R, M, 4, 4, 4);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) B[i * 3 + j] = M[(i + 1) * 4 + j + 1];
}

// 15x15 upper Cholesky factor L^T of the information (covariance^-1), as
// LLT(cov.inverse()).matrixL().transpose().
bool sqrt_information(const double* cov, double* S) {
    const int n = 15;
    // inverse of the covariance by Gauss-Jordan with partial pivoting
    double A[225], I[225];
    std::memcpy(A, cov, sizeof(A));
    for (int i = 0; i < 225; ++i) I[i] = (i % 16 == 0) ? 1.0 : 0.0;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
        if (A[p * n + c] == 0.0) return false;
        if (p != c)
            for (int k = 0; k < n; ++k) {
                std::swap(A[c * n + k], A[p * n + k]);
                std::swap(I[c * n + k], I[p * n + k]);
            }
        const double d = A[c * n + c];
        for (int k = 0; k < n; ++k) {
            A[c * n + k] /= d;
            I[c * n + k] /= d;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = A[r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                A[r * n + k] -= f * A[c * n + k];
                I[r * n + k] -= f * I[c * n + k];
            }
        }
    }
    // Cholesky of the information from its lower triangle: L L^T
    double L[225] = {};
    for (int i = 0; i < n; ++i)
        for (int j = 0; j <= i; ++j) {
            double s = I[i * n + j];
            for (int k = 0; k < j; ++k) s -= L[i * n + k] * L[j * n + k];
            if (i == j) {
                if (!(s > 0.0)) return false;
                L[i * n + i] = std::sqrt(s);
            } else {
                L[i * n + j] = s / L[j * n + j];
            }
        }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) S[i * n + j] = L[j * n + i];
    return true;
}

}  // namespace

extern "C" {

int fvgs_jacobian_cam_to_imu(const double JtJ_cam[36], const double Jtr_cam[6], const double q_imu_cam[4],
                             const double t_imu_cam[3], const double q_imu[4], double JtJ_imu[36],
                             double Jtr_imu[6]) {
    if (!JtJ_cam || !Jtr_cam || !q_imu_cam || !t_imu_cam || !q_imu || !JtJ_imu || !Jtr_imu) return FVGS_E_INVALID;
    double R_ic[9], R_i[9], Pskew[9], RP[9];
    qmat(q4(q_imu_cam), R_ic);
    qmat(q4(q_imu), R_i);
    skew(v3(t_imu_cam), Pskew);
    m3mul(R_i, Pskew, RP);
    double J[36] = {};
    for (int i = 0; i < 3; ++i) {
        J[i * 6 + i] = 1.0;
        for (int j = 0; j < 3; ++j) {
            J[i * 6 + 3 + j] = -RP[i * 3 + j];
            J[(3 + i) * 6 + 3 + j] = R_ic[j * 3 + i];  // R_imu_cam^T
        }
    }
    double Jt[36], JtH[36], out[36];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) Jt[i * 6 + j] = J[j * 6 + i];
    matmul(Jt, JtJ_cam, JtH, 6, 6, 6);
    matmul(JtH, J, out, 6, 6, 6);
    double g[6];
    matmul(Jt, Jtr_cam, g, 6, 6, 1);
    std::memcpy(JtJ_imu, out, sizeof(out));
    std::memcpy(Jtr_imu, g, sizeof(g));
    return FVGS_OK;
}

int fvgs_pseudo_factor(const double JtJ[36], const double Jtr[6], double eps, double r_star[6],
                       double J_star[36]) {
    if (!JtJ || !Jtr || !r_star || !J_star) return FVGS_E_INVALID;
    eig_factor(JtJ, Jtr, 6, eps, J_star, r_star);
    return FVGS_OK;
}

int fvgs_preint_create(const double acc0[3], const double gyr0[3], const double ba[3], const double bg[3],
                       double acc_n, double gyr_n, double acc_w, double gyr_w, fvgs_preint** out) {
    if (!acc0 || !gyr0 || !ba || !bg || !out) return FVGS_E_INVALID;
    fvgs_preint* P = new (std::nothrow) fvgs_preint();
    if (!P) return FVGS_E_NOMEM;
    P->acc0 = P->lin_acc = v3(acc0);
    P->gyr0 = P->lin_gyr = v3(gyr0);
    P->ba = v3(ba);
    P->bg = v3(bg);
    P->reset();
    std::memset(P->noise, 0, sizeof(P->noise));
    const double d[6] = {acc_n * acc_n, gyr_n * gyr_n, acc_n * acc_n, gyr_n * gyr_n, acc_w * acc_w, gyr_w * gyr_w};
    for (int b = 0; b < 6; ++b)
        for (int k = 0; k < 3; ++k) P->noise[(3 * b + k) * 18 + 3 * b + k] = d[b];
    *out = P;
    return FVGS_OK;
}

int fvgs_preint_destroy(fvgs_preint* P) {
    if (!P) return FVGS_E_INVALID;
    delete P;
    return FVGS_OK;
}

int fvgs_preint_add(fvgs_preint* P, double dt, const double acc[3], const double gyr[3]) {
    if (!P || !acc || !gyr || !(dt >= 0.0)) return FVGS_E_INVALID;
    P->dt_buf.push_back(dt);
    P->acc_buf.push_back(v3(acc));
    P->gyr_buf.push_back(v3(gyr));
    P->propagate(dt, v3(acc), v3(gyr));
    return FVGS_OK;
}

int fvgs_preint_repropagate(fvgs_preint* P, const double ba[3], const double bg[3]) {
    if (!P || !ba || !bg) return FVGS_E_INVALID;
    P->acc0 = P->lin_acc;
    P->gyr0 = P->lin_gyr;
    P->ba = v3(ba);
    P->bg = v3(bg);
    P->reset();
    for (size_t i = 0; i < P->dt_buf.size(); ++i) P->propagate(P->dt_buf[i], P->acc_buf[i], P->gyr_buf[i]);
    return FVGS_OK;
}

int fvgs_preint_state(const fvgs_preint* P, double delta_p[3], double delta_q[4], double delta_v[3],
                      double* sum_dt, double jacobian[225], double covariance[225]) {
    if (!P) return FVGS_E_INVALID;
    if (delta_p) std::memcpy(delta_p, P->dp.data(), sizeof(double) * 3);
    if (delta_v) std::memcpy(delta_v, P->dv.data(), sizeof(double) * 3);
    if (delta_q) delta_q[0] = P->dq.x, delta_q[1] = P->dq.y, delta_q[2] = P->dq.z, delta_q[3] = P->dq.w;
    if (sum_dt) *sum_dt = P->sum_dt;
    if (jacobian) std::memcpy(jacobian, P->jac, sizeof(P->jac));
    if (covariance) std::memcpy(covariance, P->cov, sizeof(P->cov));
    return FVGS_OK;
}

int fvgs_preint_evaluate(const fvgs_preint* P, const double pose_i[7], const double speedbias_i[9],
                         const double pose_j[7], const double speedbias_j[9], double residual[15]) {
    if (!P || !pose_i || !speedbias_i || !pose_j || !speedbias_j || !residual) return FVGS_E_INVALID;
    residual15(P, pose_i, speedbias_i, pose_j, speedbias_j, residual);
    return FVGS_OK;
}

int fvgs_preint_predict(const fvgs_preint* P, const double pose_i[7], const double v_i[3], double pose_j[7],
                        double v_j[3]) {
    if (!P || !pose_i || !v_i || !pose_j || !v_j) return FVGS_E_INVALID;
    const Quat Qi = q4(pose_i + 3);
    const Quat Qj = qmul(Qi, P->dq);
    double R[9];
    qmat(Qi, R);
    const V3 Rdv = m3v(R, P->dv), Rdp = m3v(R, P->dp);
    const double T = P->sum_dt;
    const V3 G = kGravityPreint;
    for (int k = 0; k < 3; ++k) {
        v_j[k] = v_i[k] - G[k] * T + Rdv[k];
        pose_j[k] = pose_i[k] + v_i[k] * T - 0.5 * G[k] * T * T + Rdp[k];
    }
    pose_j[3] = Qj.x, pose_j[4] = Qj.y, pose_j[5] = Qj.z, pose_j[6] = Qj.w;
    return FVGS_OK;
}

int fvgs_imu_factor(fvgs_preint* P, const double pose_i[7], const double speedbias_i[9], const double pose_j[7],
                    const double speedbias_j[9], double residual[15], double J_pose_i[105], double J_sb_i[135],
                    double J_pose_j[105], double J_sb_j[135]) {
    if (!P || !pose_i || !speedbias_i || !pose_j || !speedbias_j || !residual) return FVGS_E_INVALID;
    const V3 Bai = v3(speedbias_i + 3), Bgi = v3(speedbias_i + 6);
    auto norm3 = [](const V3& a, const V3& b) {
        return std::sqrt((a[0] - b[0]) * (a[0] - b[0]) + (a[1] - b[1]) * (a[1] - b[1]) + (a[2] - b[2]) * (a[2] - b[2]));
    };
    if (norm3(Bai, P->ba) > 0.10 || norm3(Bgi, P->bg) > 0.01) fvgs_preint_repropagate(P, Bai.data(), Bgi.data());
    double r[15];
    residual15(P, pose_i, speedbias_i, pose_j, speedbias_j, r);
    double S[225];
    if (!sqrt_information(P->cov, S)) return FVGS_E_STATE;
    matmul(S, r, residual, 15, 15, 1);
    if (!J_pose_i && !J_sb_i && !J_pose_j && !J_sb_j) return FVGS_OK;

    const V3 Pi = v3(pose_i), Vi = v3(speedbias_i), Pj = v3(pose_j), Vj = v3(speedbias_j);
    const Quat Qi = q4(pose_i + 3), Qj = q4(pose_j + 3), Qii = qinv(Qi);
    const double T = P->sum_dt;
    const V3 G = kGravityFactor;
    double dp_dba[9], dp_dbg[9], dq_dbg[9], dv_dba[9], dv_dbg[9], Rii[9];
    get_block(P->jac, 15, 0, 9, dp_dba);
    get_block(P->jac, 15, 0, 12, dp_dbg);
    get_block(P->jac, 15, 3, 12, dq_dbg);
    get_block(P->jac, 15, 6, 9, dv_dba);
    get_block(P->jac, 15, 6, 12, dv_dbg);
    qmat(Qii, Rii);
    const V3 dbg = {Bgi[0] - P->bg[0], Bgi[1] - P->bg[1], Bgi[2] - P->bg[2]};
    const V3 th = m3v(dq_dbg, dbg);
    const Quat cdq = qmul(P->dq, Quat{0.5 * th[0], 0.5 * th[1], 0.5 * th[2], 1.0});
    static const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    auto finish = [&](double* Jraw, int cols, double* out) {
        double tmp[15 * 9];
        matmul(S, Jraw, tmp, 15, 15, cols);
        std::memcpy(out, tmp, sizeof(double) * 15 * cols);
    };
    if (J_pose_i) {
        double J[105] = {};
        set_block(J, 7, 0, 0, Rii, -1.0);
        V3 a;
        for (int k = 0; k < 3; ++k) a[k] = 0.5 * G[k] * T * T + Pj[k] - Pi[k] - Vi[k] * T;
        double B[9];
        skew(qrot(Qii, a), B);
        set_block(J, 7, 0, 3, B);
        qleft_qright_br(qmul(qinv(Qj), Qi), cdq, B);
        set_block(J, 7, 3, 3, B, -1.0);
        V3 b;
        for (int k = 0; k < 3; ++k) b[k] = G[k] * T + Vj[k] - Vi[k];
        skew(qrot(Qii, b), B);
        set_block(J, 7, 6, 3, B);
        finish(J, 7, J_pose_i);
    }
    if (J_sb_i) {
        double J[135] = {};
        set_block(J, 9, 0, 0, Rii, -T);
        set_block(J, 9, 0, 3, dp_dba, -1.0);
        set_block(J, 9, 0, 6, dp_dbg, -1.0);
        double L[9], Ld[9];
        qleft_br(qmul(qmul(qinv(Qj), Qi), P->dq), L);
        m3mul(L, dq_dbg, Ld);
        set_block(J, 9, 3, 6, Ld, -1.0);
        set_block(J, 9, 6, 0, Rii, -1.0);
        set_block(J, 9, 6, 3, dv_dba, -1.0);
        set_block(J, 9, 6, 6, dv_dbg, -1.0);
        set_block(J, 9, 9, 3, I3, -1.0);
        set_block(J, 9, 12, 6, I3, -1.0);
        finish(J, 9, J_sb_i);
    }
    if (J_pose_j) {
        double J[105] = {};
        set_block(J, 7, 0, 0, Rii);
        double B[9];
        qleft_br(qmul(qmul(qinv(cdq), Qii), Qj), B);
        set_block(J, 7, 3, 3, B);
        finish(J, 7, J_pose_j);
    }
    if (J_sb_j) {
        double J[135] = {};
        set_block(J, 9, 6, 0, Rii);
        set_block(J, 9, 9, 3, I3);
        set_block(J, 9, 12, 6, I3);
        finish(J, 9, J_sb_j);
    }
    return FVGS_OK;
}

int fvgs_marginalize(const double* A, const double* b, int m, int n, double eps, double* J, double* r) {
    if (!A || !b || !J || !r || m <= 0 || n <= 0) return FVGS_E_INVALID;
    const int N = m + n;
    std::vector<double> Amm((size_t)m * m), w(m), V((size_t)m * m), Ainv((size_t)m * m);
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) Amm[i * m + j] = 0.5 * (A[i * N + j] + A[j * N + i]);
    sym_eig(Amm.data(), m, w.data(), V.data());
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            double s = 0.0;
            for (int k = 0; k < m; ++k)
                if (w[k] > eps) s += V[i * m + k] * (1.0 / w[k]) * V[j * m + k];
            Ainv[i * m + j] = s;
        }
    // A* = Arr - Arm Amm^+ Amr, b* = brr - Arm Amm^+ bmm
    std::vector<double> ArmAinv((size_t)n * m), As((size_t)n * n), bs(n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < m; ++j) {
            double s = 0.0;
            for (int k = 0; k < m; ++k) s += A[(m + i) * N + k] * Ainv[k * m + j];
            ArmAinv[i * m + j] = s;
        }
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            double s = 0.0;
            for (int k = 0; k < m; ++k) s += ArmAinv[i * m + k] * A[k * N + m + j];
            As[i * n + j] = A[(m + i) * N + m + j] - s;
        }
        double s = 0.0;
        for (int k = 0; k < m; ++k) s += ArmAinv[i * m + k] * b[k];
        bs[i] = b[m + i] - s;
    }
    eig_factor(As.data(), bs.data(), n, eps, J, r);
    return FVGS_OK;
}

int fvgs_marginal_prior_evaluate(const double* J, const double* r, int n, int n_blocks, const int* block_size,
                                 const int* block_idx, const double* const* x, const double* const* x0,
                                 double* residual, double* const* jacobians) {
    if (!J || !r || n <= 0 || n_blocks < 0 || (n_blocks && (!block_size || !block_idx || !x || !x0)) || !residual)
        return FVGS_E_INVALID;
    std::vector<double> dx(n, 0.0);
    for (int i = 0; i < n_blocks; ++i) {
        const int size = block_size[i], idx = block_idx[i];
        const int local = size == 7 ? 6 : size;
        if (idx < 0 || idx + local > n) return FVGS_E_INVALID;
        if (size != 7) {
            for (int k = 0; k < size; ++k) dx[idx + k] = x[i][k] - x0[i][k];
        } else {
            for (int k = 0; k < 3; ++k) dx[idx + k] = x[i][k] - x0[i][k];
            const Quat q0 = q4(x0[i] + 3), q = q4(x[i] + 3);
            const Quat rel = qmul(qinv(q0), q);
            const double sgn = rel.w < 0.0 ? -2.0 : 2.0;
            dx[idx + 3] = sgn * rel.x, dx[idx + 4] = sgn * rel.y, dx[idx + 5] = sgn * rel.z;
        }
    }
    for (int i = 0; i < n; ++i) {
        double s = r[i];
        for (int k = 0; k < n; ++k) s += J[i * n + k] * dx[k];
        residual[i] = s;
    }
    if (jacobians)
        for (int b = 0; b < n_blocks; ++b) {
            double* Jb = jacobians[b];
            if (!Jb) continue;
            const int size = block_size[b], idx = block_idx[b], local = size == 7 ? 6 : size;
            for (int i = 0; i < n; ++i)
                for (int c = 0; c < size; ++c) Jb[i * size + c] = c < local ? J[i * n + idx + c] : 0.0;
        }
    return FVGS_OK;
}

// --------------------------------------------------------------------------
// Visual-inertial normal equations
// --------------------------------------------------------------------------
}  // extern "C"

namespace {

// The linearised factors of the two-state problem as one system over the 30
// local dimensions [pose_i 6 | speedbias_i 9 | pose_j 6 | speedbias_j 9]:
// A = sum J^T J, b = sum J^T r; the cost 0.5 sum |r|^2.
int vi_system(fvgs_preint* P, const double* JtJ_imu, const double* Jtr_imu, double eps, const double* prior_J,
              const double* prior_r, const double* prior_x0, const double* pose_i, const double* sb_i,
              const double* pose_j, const double* sb_j, double A[900], double b[30], double* cost) {
    const int N = 30;
    for (int i = 0; i < N * N; ++i) A[i] = 0.0;
    for (int i = 0; i < N; ++i) b[i] = 0.0;
    double c = 0.0;
    // rows of one factor: residual r (m) and its Jacobian over the 30 dims
    auto add = [&](const double* r, const double* J, int m) {
        for (int a = 0; a < N; ++a) {
            double s = 0.0;
            for (int k = 0; k < m; ++k) s += J[k * N + a] * r[k];
            b[a] += s;
            for (int d = a; d < N; ++d) {
                double t = 0.0;
                for (int k = 0; k < m; ++k) t += J[k * N + a] * J[k * N + d];
                A[a * N + d] += t;
                if (d != a) A[d * N + a] += t;
            }
        }
        for (int k = 0; k < m; ++k) c += r[k] * r[k];
    };
    // RGB-D pseudo factor on pose_j
    {
        double rs[6], Js[36];
        const int st = fvgs_pseudo_factor(JtJ_imu, Jtr_imu, eps, rs, Js);
        if (st != FVGS_OK) return st;
        std::vector<double> J(6 * N, 0.0);
        for (int k = 0; k < 6; ++k)
            for (int d = 0; d < 6; ++d) J[k * N + 15 + d] = Js[k * 6 + d];
        add(rs, J.data(), 6);
    }
    // IMU factor between i and j
    {
        double r[15], Jpi[105], Jsi[135], Jpj[105], Jsj[135];
        const int st = fvgs_imu_factor(P, pose_i, sb_i, pose_j, sb_j, r, Jpi, Jsi, Jpj, Jsj);
        if (st != FVGS_OK) return st;
        std::vector<double> J(15 * N, 0.0);
        for (int k = 0; k < 15; ++k) {
            for (int d = 0; d < 6; ++d) {
                J[k * N + d] = Jpi[k * 7 + d];
                J[k * N + 15 + d] = Jpj[k * 7 + d];
            }
            for (int d = 0; d < 9; ++d) {
                J[k * N + 6 + d] = Jsi[k * 9 + d];
                J[k * N + 21 + d] = Jsj[k * 9 + d];
            }
        }
        add(r, J.data(), 15);
    }
    // marginalization prior on state i
    if (prior_J) {
        const int bs[2] = {7, 9}, bi[2] = {0, 6};
        const double* x[2] = {pose_i, sb_i};
        const double* x0[2] = {prior_x0, prior_x0 + 7};
        double r[15], Jp[105], Js[135];
        double* jac[2] = {Jp, Js};
        const int st = fvgs_marginal_prior_evaluate(prior_J, prior_r, 15, 2, bs, bi, x, x0, r, jac);
        if (st != FVGS_OK) return st;
        std::vector<double> J(15 * N, 0.0);
        for (int k = 0; k < 15; ++k) {
            for (int d = 0; d < 6; ++d) J[k * N + d] = Jp[k * 7 + d];
            for (int d = 0; d < 9; ++d) J[k * N + 6 + d] = Js[k * 9 + d];
        }
        add(r, J.data(), 15);
    }
    if (cost) *cost = 0.5 * c;
    return FVGS_OK;
}

// x = -A^-1 b for symmetric A (n x n): Cholesky, or the eigen-thresholded
// pseudo-inverse (eigenvalues above 1e-12 of the largest) if A is not
// positive definite.
void solve_spd(const double* A, const double* b, int n, double* x) {
    std::vector<double> L((size_t)n * n, 0.0);
    bool pd = true;
    for (int j = 0; j < n && pd; ++j) {
        double s = A[j * n + j];
        for (int k = 0; k < j; ++k) s -= L[j * n + k] * L[j * n + k];
        if (!(s > 0.0)) {
            pd = false;
            break;
        }
        const double ljj = std::sqrt(s);
        L[j * n + j] = ljj;
        for (int i = j + 1; i < n; ++i) {
            double t = A[i * n + j];
            for (int k = 0; k < j; ++k) t -= L[i * n + k] * L[j * n + k];
            L[i * n + j] = t / ljj;
        }
    }
    if (pd) {
        std::vector<double> y(n);
        for (int i = 0; i < n; ++i) {
            double s = b[i];
            for (int k = 0; k < i; ++k) s -= L[i * n + k] * y[k];
            y[i] = s / L[i * n + i];
        }
        for (int i = n - 1; i >= 0; --i) {
            double s = y[i];
            for (int k = i + 1; k < n; ++k) s -= L[k * n + i] * x[k];
            x[i] = s / L[i * n + i];
        }
        for (int i = 0; i < n; ++i) x[i] = -x[i];
        return;
    }
    std::vector<double> w(n), V((size_t)n * n);
    sym_eig(A, n, w.data(), V.data());
    const double wmax = w[n - 1];
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    for (int k = 0; k < n; ++k) {
        if (!(w[k] > 1e-12 * wmax)) continue;
        double proj = 0.0;
        for (int i = 0; i < n; ++i) proj += V[i * n + k] * b[i];
        for (int i = 0; i < n; ++i) x[i] -= V[i * n + k] * proj / w[k];
    }
}

// PoseLocalParameterization::Plus: p + dp, (q (x) [dtheta / 2, 1]) normalised.
void pose_plus(double* pose, const double* d) {
    for (int k = 0; k < 3; ++k) pose[k] += d[k];
    const Quat q = q4(pose + 3);
    const Quat dq = {0.5 * d[3], 0.5 * d[4], 0.5 * d[5], 1.0};
    const Quat n = qnormalized(qmul(q, dq));
    pose[3] = n.x, pose[4] = n.y, pose[5] = n.z, pose[6] = n.w;
}

}  // namespace

extern "C" {

int fvgs_vi_step(fvgs_preint* P, const double JtJ_imu[36], const double Jtr_imu[6], double eps,
                 const double* prior_J, const double* prior_r, const double* prior_x0, double pose_i[7],
                 double speedbias_i[9], double pose_j[7], double speedbias_j[9], double* cost, double delta[30]) {
    if (!P || !JtJ_imu || !Jtr_imu || !pose_i || !speedbias_i || !pose_j || !speedbias_j) return FVGS_E_INVALID;
    if (prior_J && (!prior_r || !prior_x0)) return FVGS_E_INVALID;
    double A[900], b[30];
    const int st = vi_system(P, JtJ_imu, Jtr_imu, eps, prior_J, prior_r, prior_x0, pose_i, speedbias_i, pose_j,
                             speedbias_j, A, b, cost);
    if (st != FVGS_OK) return st;
    double d[30] = {};
    if (prior_J) {
        solve_spd(A, b, 30, d);
    } else {
        // state i fixed: the 15-dim system of state j
        double Aj[225], bj[15], dj[15];
        for (int r = 0; r < 15; ++r) {
            bj[r] = b[15 + r];
            for (int c = 0; c < 15; ++c) Aj[r * 15 + c] = A[(15 + r) * 30 + 15 + c];
        }
        solve_spd(Aj, bj, 15, dj);
        for (int k = 0; k < 15; ++k) d[15 + k] = dj[k];
    }
    for (int k = 0; k < 30; ++k)
        if (!std::isfinite(d[k])) return FVGS_E_STATE;
    if (prior_J) {
        pose_plus(pose_i, d);
        for (int k = 0; k < 9; ++k) speedbias_i[k] += d[6 + k];
    }
    pose_plus(pose_j, d + 15);
    for (int k = 0; k < 9; ++k) speedbias_j[k] += d[21 + k];
    if (delta) std::memcpy(delta, d, sizeof(d));
    return FVGS_OK;
}

int fvgs_vi_marginalize(fvgs_preint* P, const double JtJ_imu[36], const double Jtr_imu[6], double eps,
                        const double* prior_J, const double* prior_r, const double* prior_x0,
                        const double pose_i[7], const double speedbias_i[9], const double pose_j[7],
                        const double speedbias_j[9], double new_J[225], double new_r[15], double new_x0[16]) {
    if (!P || !JtJ_imu || !Jtr_imu || !pose_i || !speedbias_i || !pose_j || !speedbias_j || !new_J || !new_r ||
        !new_x0)
        return FVGS_E_INVALID;
    if (prior_J && (!prior_r || !prior_x0)) return FVGS_E_INVALID;
    double A[900], b[30];
    const int st = vi_system(P, JtJ_imu, Jtr_imu, eps, prior_J, prior_r, prior_x0, pose_i, speedbias_i, pose_j,
                             speedbias_j, A, b, nullptr);
    if (st != FVGS_OK) return st;
    const int ms = fvgs_marginalize(A, b, 15, 15, 1e-8, new_J, new_r);
    if (ms != FVGS_OK) return ms;
    std::memcpy(new_x0, pose_j, 7 * sizeof(double));
    std::memcpy(new_x0 + 7, speedbias_j, 9 * sizeof(double));
    return FVGS_OK;
}

}  // extern "C"
