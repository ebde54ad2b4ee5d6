// track.cu -- fused tracking kernel (forward blend + RGB-D pose Jacobian +
// per-tile J^T J / J^T r reduction), the frame reduction, and the on-device
// Gauss-Newton pose update, for sm_103a.
//
// Reference: getRgbdPoseJacobians (src/GSCudaKernels.cu:922-1392), the host
// reduction and sign convention of GSSlam::computeRgbdPoseJacobians
// (src/GSSlam.cu:2205-2226), the eigen-regularised pseudo factor of
// RgbdPoseCostFunction::Evaluate (src/RgbdPoseCost.cu:57-106) and the pose
// update PoseLocalParameterization::Plus (src/PoseLocalParameterization.cpp:22-44).
//
// Per-pixel semantics are the reference's (each pixel scans its tile list,
// thresholds 0.99 / 1/255 / 1e-4 / 0.5 / 1e-3, the pass-1-only v<=0 skip, the
// reference Jacobian's second pass over the first n_contrib entries; the
// analytic Jacobian accumulates its terms in the forward pass, with the final
// colour factored out -- track_tile.cuh).  The arithmetic is reorganised for
// the GPU without changing the mathematics:
//  * every per-Gaussian colour term is rank one (Jt_cam = jt_dl (x) alpha*dC),
//    so J_pose * JtJ_cam * J_pose^T becomes one 21-FMA update with
//    u = (jt_dl, d * (ray x jt_dl)) instead of the reference's 3x3 and 6x3
//    products; with jt_dl = g / d that is u = (g / d, ray x g), so the
//    per-pixel depth enters through one reciprocal;
//  * per-Gaussian factors of u (the mean's ray, -f * ray) are computed once
//    per staged batch; the per-pixel depth takes the compensated evaluation
//    only where its two-FMA value may have cancelled; reciprocals are the
//    one-ulp rcp.approx;
//  * terms are accumulated in the camera frame (translation rows without R)
//    and rotated once per frame, in FP64, by diag(R, I);
//  * the 27 per-thread sums are reduced by a 31-shuffle butterfly
//    reduce-scatter, then across the 8 warps in a fixed order, and written
//    once per tile (no atomics: results are run-to-run deterministic).
#include <cooperative_groups.h>

#include "track_tile.cuh"

namespace cg = cooperative_groups;

namespace fvgs {


// The per-frame kernel: one CTA per tile of one session.
template <int TW, int TH, bool RENDER_ONLY, bool REF_LAYOUT = false, int MIN_CTAS = 4, bool TMA = false,
          int BATCH = kBatch, bool ANALYTIC = false, bool COMP = false>
__global__ void __launch_bounds__(TW * TH, MIN_CTAS) track_tile_kernel(TrackArgs a, const __grid_constant__ RecMaps maps) {
    pdl_begin();
    extern __shared__ __align__(128) unsigned char s_dyn[];
    if (TMA) {
        if (threadIdx.x == 0) tma_bar_init(&body_tma_stage<TW, TH, BATCH, ANALYTIC>(s_dyn).bar);
        __syncthreads();
    }
    track_tile_body<TW, TH, RENDER_ONLY, REF_LAYOUT, TMA, BATCH, ANALYTIC, COMP>(a, maps, blockIdx.x, s_dyn);
}

// Cholesky of a symmetric 6x6 (lower factor in L); false if not positive
// definite.  Fully unrolled so everything stays in registers.
__device__ __forceinline__ bool chol6(const double A[6][6], double L[6][6]) {
#pragma unroll
    for (int j = 0; j < 6; ++j) {
        double s = A[j][j];
#pragma unroll
        for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
        if (!(s > 0.0)) return false;
        const double ljj = sqrt(s);
        L[j][j] = ljj;
#pragma unroll
        for (int i = j + 1; i < 6; ++i) {
            double t = A[i][j];
#pragma unroll
            for (int k = 0; k < j; ++k) t -= L[i][k] * L[j][k];
            L[i][j] = t / ljj;
        }
#pragma unroll
        for (int i = 0; i < j; ++i) L[i][j] = 0.0;
    }
    return true;
}

// delta = -sum_{lambda_i > eps} (u_i . g / lambda_i) u_i for symmetric H:
// the Gauss-Newton step of the pseudo residual / Jacobian pair that
// RgbdPoseCostFunction::Evaluate builds from the eigen-decomposition of JtJ
// (src/RgbdPoseCost.cu:57-78).  When H - eps*I is positive definite every
// eigenvalue is kept and the step is exactly -H^-1 g (Cholesky); otherwise a
// cyclic Jacobi eigen-decomposition drops the small eigenvalues.
__device__ __noinline__ void pseudo_step(const double H[6][6], const double g[6], double eps, double delta[6]) {
    double L[6][6];
    double He[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) He[i][j] = H[i][j] - (i == j ? eps : 0.0);
    if (chol6(He, L) && chol6(H, L)) {
        double y[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) {
            double s = g[i];
#pragma unroll
            for (int k = 0; k < i; ++k) s -= L[i][k] * y[k];
            y[i] = s / L[i][i];
        }
#pragma unroll
        for (int i = 5; i >= 0; --i) {
            double s = y[i];
#pragma unroll
            for (int k = i + 1; k < 6; ++k) s -= L[k][i] * delta[k];
            delta[i] = s / L[i][i];
        }
#pragma unroll
        for (int i = 0; i < 6; ++i) delta[i] = -delta[i];
        return;
    }
    double A[6][6], V[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) {
            A[i][j] = H[i][j];
            V[i][j] = (i == j) ? 1.0 : 0.0;
        }
    for (int sweep = 0; sweep < 30; ++sweep) {
        double off = 0.0, tot = 0.0;
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
            for (int j = 0; j < 6; ++j) {
                tot += A[i][j] * A[i][j];
                if (i != j) off += A[i][j] * A[i][j];
            }
        if (off <= 1e-30 * tot) break;
#pragma unroll
        for (int p = 0; p < 5; ++p)
#pragma unroll
            for (int q = p + 1; q < 6; ++q) {
                const double apq = A[p][q];
                if (apq != 0.0) {
                    const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                    const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                    const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const double akp = A[k][p], akq = A[k][q];
                        A[k][p] = cs * akp - sn * akq;
                        A[k][q] = sn * akp + cs * akq;
                    }
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const double apk = A[p][k], aqk = A[q][k];
                        A[p][k] = cs * apk - sn * aqk;
                        A[q][k] = sn * apk + cs * aqk;
                    }
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const double vkp = V[k][p], vkq = V[k][q];
                        V[k][p] = cs * vkp - sn * vkq;
                        V[k][q] = sn * vkp + cs * vkq;
                    }
                }
            }
    }
#pragma unroll
    for (int k = 0; k < 6; ++k) delta[k] = 0.0;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const double lam = A[i][i];
        if (lam > eps) {
            double ug = 0.0;
#pragma unroll
            for (int k = 0; k < 6; ++k) ug += V[k][i] * g[k];
#pragma unroll
            for (int k = 0; k < 6; ++k) delta[k] -= (ug / lam) * V[k][i];
        }
    }
}

__device__ __forceinline__ double shfl_d(double v, int src) { return __shfl_sync(kFullMask, v, src); }

// 1/x for finite positive x: the PTX rcp.approx.ftz.f64 estimate refined by
// two Newton steps r += r (1 - x r), each doubling the correct bits, to within
// an ulp or two of the correctly rounded reciprocal.  FP64 division is a long
// dependent sequence on this part, and the factorisation and pose step below
// are latency chains.
__device__ __forceinline__ double rcp_newton(double x) {
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    r = fma(r, fma(-x, r, 1.0), r);
    return fma(r, fma(-x, r, 1.0), r);
}

// Lower-triangle lane map: lane l < 21 holds entry (i, j), i >= j,
// l = i (i + 1) / 2 + j.
__device__ __forceinline__ int tri_index(int i, int j) { return i * (i + 1) / 2 + j; }

// Warp-parallel LDL^T factorisation of a symmetric 6x6 held as one
// lower-triangle entry per lane (lanes >= 21 idle), without square roots: on
// return lane tri_index(i, j) holds L[i][j] (i > j, unit diagonal implied) or
// D[i] (i == j).  Returns false (uniformly) when a pivot is not positive, i.e.
// the matrix is not positive definite.  Lane k < 6 also ends with 1 / D[k]
// in inv_d.
__device__ __forceinline__ bool warp_ldl6(double& m, int li, int lj, double& inv_d) {
    const int lane = threadIdx.x & 31;
    const bool act = lane < 21;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const double dk = shfl_d(m, tri_index(k, k));
        if (!(dk > 0.0 && dk <= 1e300)) return false;
        const double inv = rcp_newton(dk);
        if (lane == k) inv_d = inv;
        // entries still holding L(i, k) D(k) for i > k
        const double lik = shfl_d(m, (act && li > k) ? tri_index(li, k) : 0);
        const double ljk = shfl_d(m, (act && lj > k) ? tri_index(lj, k) : 0);
        if (act && lj > k) m = fma(-lik * inv, ljk, m);
        if (act && lj == k && li > k) m *= inv;
    }
    return true;
}

// Frame reduction + (optionally) the Gauss-Newton pose update, one cluster of
// kRedCtas CTAs: warp k of the cluster sums tiles k, k + 8 kRedCtas, ... with
// lane l < 27 holding column l (Kahan-compensated FP32, fixed order), the
// CTA combines its warps in FP64, and CTA 0 gathers the CTAs' sums over
// distributed shared memory in rank order (deterministic).  The total is
// rotated to the world frame by diag(R, I) and written as out[42] = JtJ[36]
// symmetric, Jtr[6] negated (src/GSSlam.cu:2205-2226); then the pseudo-factor
// step of RgbdPoseCostFunction (src/RgbdPoseCost.cu:57-78) and
// PoseLocalParameterization::Plus on the device pose.
//
// FP64 is issued slowly on this part, so the 6x6 work is spread over lanes:
// warp 0 factors H - eps*I (all eigenvalues > eps exactly when it is positive
// definite, and then the eigen-regularised step equals -H^-1 g), warp 1 factors
// H and solves; only a failed test falls back to a one-thread Jacobi
// eigen-decomposition that drops the small eigenvalues.
constexpr int kRedCtas = 8;
constexpr int kRedUnroll = 28;

// Column col of list tile t's partial sum from its `split` partial rows, in
// the order of a whole 16 x 16 CTA's sum (cta_partial_sum): 2 rows = the
// upper and lower 16 x 8 halves; 4 rows = the 8 x 8 quarters in row-major
// order, ((q00 + q10) + (q01 + q11)).
__device__ __forceinline__ float tile_partial_sum(const float* __restrict__ tile_out, int t, int split, int col) {
    const float* r = tile_out + (size_t)t * split * FVGS_POSEDATA_FLOATS + col;
    if (split == 2) return __fadd_rn(r[0], r[FVGS_POSEDATA_FLOATS]);
    if (split == 4)
        return __fadd_rn(__fadd_rn(r[0], r[FVGS_POSEDATA_FLOATS]),
                         __fadd_rn(r[2 * FVGS_POSEDATA_FLOATS], r[3 * FVGS_POSEDATA_FLOATS]));
    return r[0];
}

template <bool DO_GN>
__device__ __forceinline__ void track_reduce_body(const float* __restrict__ tile_out, int num_tiles, int split,
                                                  DevPose* pose, double* out, double eig_eps, double* step_out) {
    __shared__ double s_w[8][32];
    __shared__ double s_part[32];
    __shared__ double s_tot[27];
    __shared__ double s_R[9];
    __shared__ int s_pd;
    cg::cluster_group cluster = cg::this_cluster();
    const unsigned rank = cluster.block_rank();
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    const int col = lane < FVGS_POSEDATA_FLOATS ? lane : 0;
    const int stride = kRedCtas * 8;
    // the pose the step is applied to, loaded now so its latency overlaps the sums
    float pq[4] = {0.f, 0.f, 0.f, 0.f};
    double pqd[4] = {0.0, 0.0, 0.0, 0.0}, ptd[3] = {0.0, 0.0, 0.0};
    if (DO_GN && rank == 0 && w == 1) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            pq[k] = pose->q[k];
            pqd[k] = pose->qd[k];
        }
#pragma unroll
        for (int k = 0; k < 3; ++k) ptd[k] = pose->td[k];
    }
    // every load of a round is issued before the (ordered) compensated adds
    float sum = 0.f, comp = 0.f;
    for (int t0 = (int)rank * 8 + w; t0 < num_tiles; t0 += kRedUnroll * stride) {
        float x[kRedUnroll];
#pragma unroll
        for (int u = 0; u < kRedUnroll; ++u) {
            const int t = t0 + u * stride;
            x[u] = t < num_tiles ? tile_partial_sum(tile_out, t, split, col) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < kRedUnroll; ++u) {
            if (t0 + u * stride < num_tiles) {
                const float y = __fsub_rn(x[u], comp);
                const float s = __fadd_rn(sum, y);
                comp = __fsub_rn(__fsub_rn(s, sum), y);
                sum = s;
            }
        }
    }
    s_w[w][lane] = lane < FVGS_POSEDATA_FLOATS ? (double)sum - (double)comp : 0.0;
    __syncthreads();
    if (w == 0) {
        double c = 0.0;
#pragma unroll
        for (int ww = 0; ww < 8; ++ww) c += s_w[ww][lane];
        s_part[lane] = c;
    }
    cluster.sync();  // every CTA's column sums are visible cluster-wide
    if (rank == 0 && w == 0 && lane < FVGS_POSEDATA_FLOATS) {
        double c = 0.0;
#pragma unroll
        for (int r = 0; r < kRedCtas; ++r) c += cluster.map_shared_rank(s_part, r)[lane];
        s_tot[lane] = c;
    }
    cluster.sync();  // CTA 0 has read the remote sums; the others may leave
    if (rank != 0) return;
    if (w >= 2) return;
    // ---- CTA 0, warps 0 and 1 only; named barrier 1 over 64 threads ----
    // lane l < 21 holds lower-triangle entry (li, lj) of a symmetric 6x6
    int li = 0, lj = 0;
    if (lane < 21) {
        while (tri_index(li + 1, 0) <= lane) ++li;
        lj = lane - tri_index(li, 0);
    }
    auto Ac = [&](int a, int b) {
        const int hi = a > b ? a : b, lo = a > b ? b : a;
        // upper-triangle row-major index of (lo, hi) among the 21 JtJ sums
        return s_tot[6 + lo * 6 - lo * (lo - 1) / 2 + (hi - lo)];
    };
    if (!DO_GN) {
        // world-frame JtJ = D A D^T and Jtr = -(D b), D = diag(R, I)
        if (w == 1 && lane < 9) {
            const double qx = pose->q[0], qy = pose->q[1], qz = pose->q[2], qw = pose->q[3];
            const int i = lane / 3, j = lane % 3;
            const double q[3] = {qx, qy, qz};
            double r;
            if (i == j) {
                const double a = q[(i + 1) % 3], b2 = q[(i + 2) % 3];
                r = 1.0 - 2.0 * (a * a + b2 * b2);
            } else {
                // off-diagonal: 2 (q_i q_j -/+ w q_k), sign + when (i, j) is (1,0), (2,1), (0,2)
                const int k = 3 - i - j;
                const bool plus = (i == (j + 1) % 3);
                r = 2.0 * (q[i] * q[j] + (plus ? qw * q[k] : -qw * q[k]));
            }
            s_R[lane] = r;
        }
        asm volatile("bar.sync 1, 64;" ::: "memory");
        if (w != 0) return;
        if (lane < 21) {
            double m;
            if (li < 3) {  // then lj < 3
                double s = 0.0;
#pragma unroll
                for (int a2 = 0; a2 < 3; ++a2)
#pragma unroll
                    for (int b2 = 0; b2 < 3; ++b2) s = fma(s_R[li * 3 + a2] * Ac(a2, b2), s_R[lj * 3 + b2], s);
                m = s;
            } else if (lj < 3) {
                double s = 0.0;
#pragma unroll
                for (int b2 = 0; b2 < 3; ++b2) s = fma(Ac(li, b2), s_R[lj * 3 + b2], s);
                m = s;
            } else {
                m = Ac(li, lj);
            }
            out[li * 6 + lj] = m;
            out[lj * 6 + li] = m;
        } else if (lane < 27) {
            const int i = lane - 21;
            out[36 + i] = i < 3 ? -(s_R[i * 3] * s_tot[0] + s_R[i * 3 + 1] * s_tot[1] + s_R[i * 3 + 2] * s_tot[2])
                                : -s_tot[i];
        }
        return;
    }
    // Gauss-Newton step.  With H = D A D^T and g = -(D b) the step
    // -H^-1 g equals D x for A x = b, and H, A share their eigenvalues, so the
    // camera-frame system is factored and only the step is rotated.
    double m = lane < 21 ? Ac(li, lj) : 0.0;
    if (w == 0) {
        if (lane < 21 && li == lj) m -= eig_eps;
        double inv_d;
        const bool pd = warp_ldl6(m, li, lj, inv_d);
        if (lane == 0) s_pd = pd ? 1 : 0;
        asm volatile("bar.sync 1, 64;" ::: "memory");
        return;
    }
    // warp 1
    double inv_d = 0.0;
    const bool pdh = warp_ldl6(m, li, lj, inv_d);
    asm volatile("bar.sync 1, 64;" ::: "memory");
    double xv = lane < 6 ? s_tot[lane] : 0.0;  // lane k < 6 ends with x[k]
    if (s_pd && pdh) {
        // L y = b (unit lower)
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double yk = shfl_d(xv, k);
            const double lik = shfl_d(m, (lane < 6 && lane > k) ? tri_index(lane, k) : 0);
            if (lane < 6 && lane > k) xv = fma(-lik, yk, xv);
        }
        // D z = y
        if (lane < 6) xv *= inv_d;
        // L^T x = z (unit upper)
#pragma unroll
        for (int k = 5; k >= 0; --k) {
            const double xk = shfl_d(xv, k);
            const double lki = shfl_d(m, (lane < k) ? tri_index(k, lane) : 0);
            if (lane < k) xv = fma(-lki, xk, xv);
        }
    } else {
        // rare: some eigenvalue <= eps -- exact eigen-decomposition on one lane
        double dl[6] = {0, 0, 0, 0, 0, 0};
        if (lane == 0) {
            double A[6][6], g[6];
            for (int i = 0; i < 6; ++i) {
                for (int j = 0; j < 6; ++j) A[i][j] = Ac(i, j);
                g[i] = -s_tot[i];
            }
            pseudo_step(A, g, eig_eps, dl);
        }
#pragma unroll
        for (int k = 0; k < 6; ++k) {
            const double d = shfl_d(dl[k], 0);
            if (lane == k) xv = d;
        }
    }
    double x[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) x[k] = shfl_d(xv, k);
    if (lane != 0) return;
    // delta = (R x_t, x_r), R of the pose the Jacobians were taken at
    const double qx = pq[0], qy = pq[1], qz = pq[2], qw = pq[3];
    const double R[3][3] = {
        {1.0 - 2.0 * (qy * qy + qz * qz), 2.0 * (qx * qy - qw * qz), 2.0 * (qx * qz + qw * qy)},
        {2.0 * (qx * qy + qw * qz), 1.0 - 2.0 * (qx * qx + qz * qz), 2.0 * (qy * qz - qw * qx)},
        {2.0 * (qx * qz - qw * qy), 2.0 * (qy * qz + qw * qx), 1.0 - 2.0 * (qx * qx + qy * qy)}};
    double delta[6];
#pragma unroll
    for (int i = 0; i < 3; ++i) delta[i] = R[i][0] * x[0] + R[i][1] * x[1] + R[i][2] * x[2];
#pragma unroll
    for (int i = 3; i < 6; ++i) delta[i] = x[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        ptd[k] += delta[k];
        pose->td[k] = ptd[k];
    }
    const double ax = pqd[0], ay = pqd[1], az = pqd[2], aw = pqd[3];
    const double bx = 0.5 * delta[3], by = 0.5 * delta[4], bz = 0.5 * delta[5];
    double nx = aw * bx + ax + (ay * bz - az * by);
    double ny = aw * by + ay + (az * bx - ax * bz);
    double nz = aw * bz + az + (ax * by - ay * bx);
    double nw = aw - (ax * bx + ay * by + az * bz);
    // 1 / |n| by the FP32 estimate and two Newton steps r *= (3 - n2 r^2) / 2
    // (about 2^-22, 2^-44, then rounding): the quaternion is within O(|delta|^2)
    // of unit length, and FP64 square root and division are long chains here
    const double n2 = nx * nx + ny * ny + nz * nz + nw * nw;
    double inn = (double)rsqrtf((float)n2);
    inn = inn * fma(-0.5 * n2, inn * inn, 1.5);
    inn = inn * fma(-0.5 * n2, inn * inn, 1.5);
    nx *= inn;
    ny *= inn;
    nz *= inn;
    nw *= inn;
    pose->qd[0] = nx;
    pose->qd[1] = ny;
    pose->qd[2] = nz;
    pose->qd[3] = nw;
#pragma unroll
    for (int k = 0; k < 3; ++k) pose->t[k] = (float)ptd[k];
    pose->q[0] = (float)nx;
    pose->q[1] = (float)ny;
    pose->q[2] = (float)nz;
    pose->q[3] = (float)nw;
    if (step_out)
#pragma unroll
        for (int k = 0; k < 6; ++k) step_out[k] = delta[k];
}

template <bool DO_GN>
__global__ void __cluster_dims__(kRedCtas, 1, 1) __launch_bounds__(256)
    track_reduce_kernel(const float* __restrict__ tile_out, int num_tiles, int split, DevPose* pose, double* out,
                        double eig_eps, double* step_out) {
    pdl_begin();
    track_reduce_body<DO_GN>(tile_out, num_tiles, split, pose, out, eig_eps, step_out);
}

// The frame reduction and Gauss-Newton step of many sessions in one launch:
// cluster k (CTAs kRedCtas k .. kRedCtas k + kRedCtas - 1) takes jobs[k].
__global__ void __cluster_dims__(kRedCtas, 1, 1) __launch_bounds__(256)
    track_reduce_batch_kernel(const ReduceJob* __restrict__ jobs) {
    pdl_begin();
    const ReduceJob& j = jobs[blockIdx.x / kRedCtas];
    track_reduce_body<true>(j.tile_out, j.num_tiles, j.split > 1 ? j.split : 1, j.pose, j.out, j.eig_eps, j.step_out);
}

namespace {

using TrackKernel = void (*)(TrackArgs, RecMaps);

struct KernelPick {
    TrackKernel fn = nullptr;
    int threads = 0;
    size_t smem = 0;
};

template <int TW, int TH, bool RENDER_ONLY, bool REF_LAYOUT, int MIN_CTAS, bool TMA, int BATCH, bool ANALYTIC,
          bool COMP = false>
KernelPick pick() {
    return {track_tile_kernel<TW, TH, RENDER_ONLY, REF_LAYOUT, MIN_CTAS, TMA, BATCH, ANALYTIC, COMP>, TW * TH,
            body_smem_bytes<TW, TH, BATCH, ANALYTIC, TMA>()};
}

// Tiles of 8 x 8 and 32 x 8: the staging batch is the only launch choice;
// MIN_CTAS gives the register budget of the 16 x 16 kernels' variant 1 for
// the analytic Jacobian (80 per thread) and of variant 0 otherwise (64).
template <int TW, int TH, bool ANALYTIC>
KernelPick pick_shape(int variant) {
    constexpr int M = (ANALYTIC ? 768 : 1024) / (TW * TH);
    const int batch = track_variant_batch(variant);
    if (batch == 128) return pick<TW, TH, false, false, M, false, 128, ANALYTIC>();
    if (batch == 512) return pick<TW, TH, false, false, M, false, 512, ANALYTIC>();
    return pick<TW, TH, false, false, M, false, 256, ANALYTIC>();
}

// The kernel of a tracking launch: tile shape, Jacobian mode and launch
// variant (the autotuner's choice; the arithmetic and its order are the same
// in all variants of a shape).
KernelPick pick_track(const TrackArgs& a, bool have_maps) {
    const bool analytic = !(a.quirks & FVGS_Q_POSE_JAC_APPROX);
    const int tw = a.tile_w ? a.tile_w : kTW, th = a.tile_h ? a.tile_h : kTH;
    if (a.compensated && (!analytic || tw != kTW || th != kTH)) return {};
    const int split = a.split > 1 ? a.split : 1;
    if (split > 1 && (a.compensated || a.render_only || tw != kTW || th != kTH)) return {};
    if (a.render_only) {
        if (tw != kTW || th != kTH) return {};
        return pick<16, 16, true, false, 4, false, kBatch, false>();
    }
    if (tw == 8 && th == 8) return analytic ? pick_shape<8, 8, true>(a.variant) : pick_shape<8, 8, false>(a.variant);
    if (tw == 32 && th == 8)
        return analytic ? pick_shape<32, 8, true>(a.variant) : pick_shape<32, 8, false>(a.variant);
    if (tw != kTW || th != kTH) return {};
    if (analytic && a.compensated) return pick<16, 16, false, false, 3, false, 256, true, true>();
    // 16 x 16 lists over 2 or 4 CTAs (the split matches the variant)
    if (split != track_variant_split(a.variant)) return {};
    if (a.variant == 5)
        return analytic ? pick<16, 8, false, false, 6, false, 128, true>()
                        : pick<16, 8, false, false, 8, false, 128, false>();
    if (a.variant == 6)
        return analytic ? pick<8, 8, false, false, 12, false, 128, true>()
                        : pick<8, 8, false, false, 16, false, 128, false>();
    if (analytic) {
        // analytic Jacobian: plain staging (no TMA variant), one CTA per SM
        // fewer than the reference Jacobian's variants (its fused pass holds
        // the colour-Jacobian sums: 80 registers at three CTAs, 128 at two)
        if (a.variant == 1) return pick<16, 16, false, false, 2, false, 256, true>();
        if (a.variant == 7) return pick<16, 16, false, false, 2, false, 128, true>();
        if (a.variant == 3) return pick<16, 16, false, false, 3, false, 128, true>();
        if (a.variant == 4) return pick<16, 16, false, false, 3, false, 512, true>();
        return pick<16, 16, false, false, 3, false, 256, true>();
    }
    if (a.variant == 1) return pick<16, 16, false, false, 3, false, 256, false>();
    if (a.variant == 7) return pick<16, 16, false, false, 2, false, 256, false>();
    if (a.variant == 3) return pick<16, 16, false, false, 4, false, 128, false>();
    if (a.variant == 4) return pick<16, 16, false, false, 4, false, 512, false>();
    if (a.variant == 2 && have_maps) return pick<16, 16, false, false, 4, true, 256, false>();
    return pick<16, 16, false, false, 4, false, 256, false>();
}

}  // namespace

cudaError_t track_configure_device() {
    // every instantiation pick_track can return
    for (int render = 0; render < 2; ++render)
        for (int q = 0; q < 2; ++q)
            for (int shape = 0; shape < 3; ++shape)
                for (int v = 0; v < 2 * kTrackVariants; ++v) {
                    TrackArgs a{};
                    a.compensated = v >= kTrackVariants && !render && !q && shape == 0;
                    a.render_only = render;
                    a.quirks = q ? FVGS_Q_POSE_JAC_APPROX : 0u;
                    a.tile_w = shape == 0 ? 16 : (shape == 1 ? 8 : 32);
                    a.tile_h = shape == 0 ? 16 : 8;
                    a.variant = v % kTrackVariants;
                    if (shape == 0 && !a.compensated && !render) a.split = track_variant_split(a.variant);
                    const KernelPick k = pick_track(a, true);
                    if (!k.fn) continue;
                    const cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(k.fn),
                                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                               (int)k.smem);
                    if (e != cudaSuccess) return e;
                }
    const cudaError_t e = cudaFuncSetAttribute(reinterpret_cast<const void*>(track_tile_kernel<16, 16, false, true>),
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)body_smem_bytes<16, 16, kBatch, false, false>());
    if (e != cudaSuccess) return e;
    return track_batch_configure_device();
}

cudaError_t launch_track(const TrackArgs& a, const RecMaps* maps, cudaStream_t s) {
    const int T = a.ntx * a.nty * (a.split > 1 ? a.split : 1);
    if (T <= 0) return cudaSuccess;
    if (!a.render_only && !(a.quirks & FVGS_Q_POSE_JAC_APPROX) && (!a.geo0 || !a.geo1)) return cudaErrorInvalidValue;
    if (a.variant == 2 && !a.render_only && (a.quirks & FVGS_Q_POSE_JAC_APPROX) &&
        (a.tile_w == 0 || a.tile_w == kTW) && (a.tile_h == 0 || a.tile_h == kTH) && (!maps || !a.st_flags))
        return cudaErrorInvalidValue;
    const KernelPick k = pick_track(a, maps != nullptr);
    if (!k.fn) return cudaErrorInvalidValue;
    RecMaps m{};
    if (maps) m = *maps;
    return launch_chained(k.fn, dim3(T), dim3(k.threads), k.smem, s, a, m);
}

cudaError_t launch_track_ref_layout(const TrackArgs& a, cudaStream_t s) {
    const int T = a.ntx * a.nty;
    if (T <= 0) return cudaSuccess;
    return launch_chained(track_tile_kernel<16, 16, false, true>, dim3(T), dim3(kPix),
                          body_smem_bytes<16, 16, kBatch, false, false>(), s, a, RecMaps{});
}

cudaError_t launch_track_reduce(const float* tile_out, int num_tiles, int split, DevPose* pose, double* out,
                                cudaStream_t s) {
    return launch_chained(track_reduce_kernel<false>, dim3(kRedCtas), dim3(256), 0, s, tile_out, num_tiles,
                          split > 1 ? split : 1, pose, out, 0.0, static_cast<double*>(nullptr));
}

cudaError_t launch_track_reduce_batch(const ReduceJob* jobs, int n_jobs, cudaStream_t s) {
    if (n_jobs <= 0) return cudaSuccess;
    return launch_chained(track_reduce_batch_kernel, dim3(kRedCtas * n_jobs), dim3(256), 0, s, jobs);
}

cudaError_t launch_track_reduce_gn(const float* tile_out, int num_tiles, int split, DevPose* pose, double* out,
                                   double eig_eps, double* step_out, cudaStream_t s) {
    return launch_chained(track_reduce_kernel<true>, dim3(kRedCtas), dim3(256), 0, s, tile_out, num_tiles,
                          split > 1 ? split : 1, pose, out, eig_eps, step_out);
}

}  // namespace fvgs

