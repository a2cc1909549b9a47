// sm_icp.h - arithmetic of one symmetric point-to-plane ICP step and of rigid-pose
// handling, shared by the CUDA kernels and the CPU oracle.
//
// Follows icp.cpp:39-121 (symmetric_rigid_matching / minimizePointToPlaneMetric) and
// util.cpp:209-232 (transformPointCloud). Precision design: the 21 + 6 entries of the
// normal equations and the centroid sums are accumulated in FP32 with Kahan compensation;
// only the 6x6 solve and the pose composition run in FP64. Both sides use the same
// summation layout, so the GPU and the oracle produce bit-identical poses: kIcpSlots
// strided partial sums (slot = source index mod kIcpSlots, ascending within a slot), merged
// by fixed binary trees - within each group of 32 slots (offsets 16..1), over the
// kIcpThreads / 32 groups of a block (offsets 8..1), then over the kIcpBlocks blocks
// (offsets 2..1; a candidate's blocks form one thread-block cluster).
#pragma once

#include "sm_linalg.h"
#include "sm_math.h"

namespace smi {

constexpr int kIcpThreads = 512;                       // ICP reduction CTA size
constexpr int kIcpBlocks  = 4;                         // CTAs per candidate and reduction
constexpr int kIcpSlots   = kIcpThreads * kIcpBlocks;  // strided partial sums

// Kahan-compensated FP32 accumulator; value() = s - c.
struct KahanF {
    float s, c;
    SM_HD void init() {
        s = 0.0f;
        c = 0.0f;
    }
    SM_HD void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c             = (t - s) - y;
        s             = t;
    }
    // merge another partial: its sum, then its negated compensation, as two more terms
    SM_HD void merge(const KahanF &o) {
        add(o.s);
        add(-o.c);
    }
    SM_HD float value() const { return s - c; }
};

// A rigid pose as a row-major 3x4 [R | t] in float.
struct Pose34 {
    float m[12];
};

SM_HD void pose_identity(Pose34 &p) {
    for (int i = 0; i < 12; i++)
        p.m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

// x' = R x + t with Eigen's 3-term order r0*x + (r1*y + r2*z), then + t.
SM_HD void pose_apply(const Pose34 &T, float x, float y, float z, float &ox, float &oy,
                      float &oz) {
    ox = (T.m[0] * x + (T.m[1] * y + T.m[2] * z)) + T.m[3];
    oy = (T.m[4] * x + (T.m[5] * y + T.m[6] * z)) + T.m[7];
    oz = (T.m[8] * x + (T.m[9] * y + T.m[10] * z)) + T.m[11];
}
SM_HD void pose_rotate(const Pose34 &T, float x, float y, float z, float &ox, float &oy,
                       float &oz) {
    ox = T.m[0] * x + (T.m[1] * y + T.m[2] * z);
    oy = T.m[4] * x + (T.m[5] * y + T.m[6] * z);
    oz = T.m[8] * x + (T.m[9] * y + T.m[10] * z);
}

// out = a * b, evaluated in FP64 and rounded to float.
SM_HD Pose34 pose_mul(const Pose34 &a, const Pose34 &b) {
    Pose34 o;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 4; j++) {
            double s = (j == 3) ? (double)a.m[i * 4 + 3] : 0.0;
            for (int k = 0; k < 3; k++)
                s += (double)a.m[i * 4 + k] * (double)b.m[k * 4 + j];
            o.m[i * 4 + j] = (float)s;
        }
    }
    return o;
}

// Number of accumulated quantities of one ICP step.
constexpr int kNumMoments = 6;  // sum of source and target points (centroids)
constexpr int kNumSystem  = 27; // 21 upper-triangular A entries + 6 entries of b

// Terms of one correspondence (icp.cpp:56-65): with p, q centred source / target points
// and n = n_p + n_q, x = [(p+q) x n ; n], b_i = (p-q).n; contributes x x^T to A and b_i x
// to b. All in float, as the reference computes them.
SM_HD void system_terms(float px, float py, float pz, float qx, float qy, float qz, float nx,
                        float ny, float nz, float out[kNumSystem]) {
    const float sx = px + qx, sy = py + qy, sz = pz + qz;
    float       x[6];
    x[0]           = sy * nz - sz * ny;
    x[1]           = sz * nx - sx * nz;
    x[2]           = sx * ny - sy * nx;
    x[3]           = nx;
    x[4]           = ny;
    x[5]           = nz;
    const float bi = (px - qx) * nx + ((py - qy) * ny + (pz - qz) * nz);
    int         k  = 0;
    for (int i = 0; i < 6; i++)
        for (int j = i; j < 6; j++)
            out[k++] = x[i] * x[j];
    for (int i = 0; i < 6; i++)
        out[21 + i] = bi * x[i];
}

// Solve A u = -b (FP64 Cholesky, pseudo-inverse fallback) and compose the pose
// (icp.cpp:68-86): theta = atan(|a~|) with sin/cos taken exactly as |a~|/sqrt(1+|a~|^2) and
// 1/sqrt(1+|a~|^2), R_i = I + sin W + (1-cos) W^2, R = R_i^2,
// t = R_i^2 (-Pmean) + R_i (cos * t~) + Qmean.
SM_HD void system_matrix(const float sys[kNumSystem], double A[6][6], double r[6]) {
    int k = 0;
    SML_UNROLL
    for (int i = 0; i < 6; i++)
        SML_UNROLL
        for (int j = i; j < 6; j++) {
            A[i][j] = (double)sys[k];
            A[j][i] = A[i][j];
            k++;
        }
    SML_UNROLL
    for (int i = 0; i < 6; i++)
        r[i] = -(double)sys[21 + i];
}

// The step's pose from the solution u = (rotation vector a~, translation) of the system.
SM_HD Pose34 step_pose(const double u[6], const float Pm[3], const float Qm[3]);

SM_HD Pose34 solve_step(const float sys[kNumSystem], const float Pm[3], const float Qm[3]) {
    double A[6][6], r[6], u[6];
    system_matrix(sys, A, r);
    if (!sml::cholesky6(A, r, u)) {
        double A2[6][6], r2[6]; // rank-deficient: pseudo-inverse on its own copy
        system_matrix(sys, A2, r2);
        sml::pinv6(A2, r2, u);
    }
    return step_pose(u, Pm, Qm);
}

#if defined(__CUDACC__)
// solve_step by one warp (every lane calls it and gets the pose): the Cholesky factorisation
// runs one row per lane (sml::cholesky6_warp); identical results.
__device__ __forceinline__ Pose34 solve_step_warp(const float sys[kNumSystem], const float Pm[3],
                                                  const float Qm[3]) {
    double A[6][6], r[6], u[6];
    system_matrix(sys, A, r);
    if (!sml::cholesky6_warp(A, r, u)) {
        double A2[6][6], r2[6];
        system_matrix(sys, A2, r2);
        sml::pinv6(A2, r2, u);
    }
    return step_pose(u, Pm, Qm);
}
#endif

SM_HD Pose34 step_pose(const double u[6], const float Pm[3], const float Qm[3]) {
    const double an = sml::dsqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
    const double h  = sml::dsqrt(1.0 + an * an);
    const double cs = 1.0 / h, sn = an * cs;
    double       a[3] = {0.0, 0.0, 0.0};
    if (an > 0.0) {
        const double ia = 1.0 / an;
        a[0]            = u[0] * ia;
        a[1]            = u[1] * ia;
        a[2]            = u[2] * ia;
    }
    // W = [a]x and W^2 = a a^T - (a.a) I; R_i = I + sin(t) W + (1 - cos(t)) W^2 with
    // sin(t) = sn, cos(t) = cs, and R = R_i^2 = I + sin(2t) W + (1 - cos(2t)) W^2 with
    // sin(2t) = 2 sn cs, 1 - cos(2t) = 2 sn^2 (the same rotation, by the double angle)
    const double W[3][3] = {{0.0, -a[2], a[1]}, {a[2], 0.0, -a[0]}, {-a[1], a[0], 0.0}};
    const double aa      = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
    const double s1 = sn, c1 = 1.0 - cs, s2 = 2.0 * sn * cs, c2 = 2.0 * sn * sn;
    double       Ri[3][3], R[3][3];
    SML_UNROLL
    for (int i = 0; i < 3; i++)
        SML_UNROLL
        for (int j = 0; j < 3; j++) {
            const double w2 = a[i] * a[j] - (i == j ? aa : 0.0);
            const double id = i == j ? 1.0 : 0.0;
            Ri[i][j]        = id + s1 * W[i][j] + c1 * w2;
            R[i][j]         = id + s2 * W[i][j] + c2 * w2;
        }
    const double tt[3] = {cs * u[3], cs * u[4], cs * u[5]};
    Pose34       o;
    SML_UNROLL
    for (int i = 0; i < 3; i++) {
        double t = 0.0;
        SML_UNROLL
        for (int m = 0; m < 3; m++)
            t += R[i][m] * (-(double)Pm[m]) + Ri[i][m] * tt[m];
        t += (double)Qm[i];
        SML_UNROLL
        for (int j = 0; j < 3; j++)
            o.m[i * 4 + j] = (float)R[i][j];
        o.m[i * 4 + 3] = (float)t;
    }
    return o;
}

// Pose record of one voting candidate: T (3x4), quaternion (w,x,y,z), rotation angle,
// votes -- 18 floats, the layout of the pose list.
constexpr int kPoseFloats = 18;

// Pose::updatePose (type.cpp:53-59): quaternion and rotation angle of T's rotation.
SM_HD void pose_record(const float T[12], float votes, float out[kPoseFloats]) {
    double R[9], q[4];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            R[i * 3 + j] = (double)T[i * 4 + j];
    sml::mat_to_quat(R, q);
    for (int i = 0; i < 12; i++)
        out[i] = T[i];
    for (int i = 0; i < 4; i++)
        out[12 + i] = (float)q[i];
    out[16] = sml::quat_angle(q);
    out[17] = votes;
}

// Candidate pose of ppf.cpp:393-405: T = RT_s^-1 * Rx(alpha) * RT_m, with the rigid
// inverse [R^T | -R^T t], cos/sin of the float angle from the shared float functions and
// the products in FP64.
SM_HD void candidate_pose(const smm::RT &rs, const smm::RT &rm, float alpha, float votes,
                          float out[kPoseFloats]) {
    const double ca = (double)smm::cosf_(alpha), sa = (double)smm::sinf_(alpha);
    double       XM[3][4];
    for (int j = 0; j < 4; j++) {
        const double r0 = j < 3 ? (double)rm.r[j] : (double)rm.t[0];
        const double r1 = j < 3 ? (double)rm.r[3 + j] : (double)rm.t[1];
        const double r2 = j < 3 ? (double)rm.r[6 + j] : (double)rm.t[2];
        XM[0][j]        = r0;
        XM[1][j]        = ca * r1 - sa * r2;
        XM[2][j]        = sa * r1 + ca * r2;
    }
    float T[12];
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 4; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++)
                s += (double)rs.r[k * 3 + i] * XM[k][j];
            if (j == 3)
                for (int k = 0; k < 3; k++)
                    s -= (double)rs.r[k * 3 + i] * (double)rs.t[k];
            T[i * 4 + j] = (float)s;
        }
    }
    pose_record(T, votes, out);
}

} // namespace smi
