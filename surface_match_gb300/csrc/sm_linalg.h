// sm_linalg.h - small fixed-size FP64 linear algebra of the matching path (normal
// eigensolve, quaternion averaging, ICP 6x6 solve, pose conversions), shared by the CUDA
// kernels and the CPU oracle. Only +, -, *, / and sqrt are used, so with FMA contraction
// off (nvcc --fmad=false, gcc -ffp-contract=off) the results are bit-identical on both.
//
// The reference uses Eigen for these steps (util.cpp:262-267 SelfAdjointEigenSolver::
// computeDirect, util.cpp:563-576 EigenSolver<Matrix4f>, icp.cpp:68 JacobiSVD, type.cpp:
// 53-59 matrix->AngleAxis/Quaternion); Eigen is not vendored with the reference, so these
// are written from the textbook methods named at each function and agree with the
// reference to rounding, not bit-for-bit.
#pragma once

#include "sm_math.h"

#if defined(__CUDACC__)
#define SML_HD __host__ __device__ __forceinline__
#else
#define SML_HD inline
#endif
// Full unrolling of fixed-size loops on the device, so small matrices stay in registers
// (the operations and their order are unchanged).
#if defined(__CUDA_ARCH__)
#define SML_UNROLL _Pragma("unroll")
#else
#define SML_UNROLL
#endif

namespace sml {

SML_HD double dsqrt(double a) {
#if defined(__CUDA_ARCH__)
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}
SML_HD double dabs(double a) { return a < 0.0 ? -a : a; }

// Cyclic Jacobi eigen-decomposition of a symmetric N x N matrix (Golub & Van Loan,
// "Matrix Computations", 8.5): each rotation zeroes a_pq and, by symmetry, updates only the
// diagonal pair and the off-diagonal entries of rows p and q. Sweeps stop once the
// off-diagonal mass falls below 1e-24 of the matrix's (relative size 1e-12, far below the
// float precision of every result taken from it). A is destroyed (its upper triangle holds
// the state); d[i] are the eigenvalues, column i of V the matching unit eigenvector. Fixed
// sweep order, so the result is reproducible.
template <int N> SML_HD void jacobi_eig(double A[N][N], double V[N][N], double d[N]) {
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            V[i][j] = (i == j) ? 1.0 : 0.0;
    double scale = 0.0;
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            scale += A[i][j] * A[i][j];
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0;
        for (int p = 0; p < N - 1; p++)
            for (int q = p + 1; q < N; q++)
                off += A[p][q] * A[p][q];
        if (!(off > scale * 1e-24))
            break;
        for (int p = 0; p < N - 1; p++) {
            for (int q = p + 1; q < N; q++) {
                const double apq = A[p][q];
                if (apq == 0.0)
                    continue;
                // t = sgn(theta) / (|theta| + sqrt(theta^2 + 1)) with theta = dq / (2 apq),
                // multiplied through by 2 |apq| (one division fewer)
                const double dq = A[q][q] - A[p][p];
                const double t2 = 2.0 * apq;
                double       t  = t2 / (dabs(dq) + dsqrt(dq * dq + t2 * t2));
                if (dq < 0.0)
                    t = -t;
                const double c = 1.0 / dsqrt(t * t + 1.0);
                const double s = t * c;
                A[p][p]        = A[p][p] - t * apq;
                A[q][q]        = A[q][q] + t * apq;
                A[p][q]        = 0.0;
                for (int r = 0; r < N; r++) {
                    if (r == p || r == q)
                        continue;
                    // a_rp, a_rq in the upper triangle
                    double &arp = r < p ? A[r][p] : A[p][r];
                    double &arq = r < q ? A[r][q] : A[q][r];
                    const double g = arp, h = arq;
                    arp            = c * g - s * h;
                    arq            = s * g + c * h;
                }
                for (int k = 0; k < N; k++) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p]          = c * vkp - s * vkq;
                    V[k][q]          = s * vkp + c * vkq;
                }
            }
        }
    }
    for (int i = 0; i < N; i++)
        d[i] = A[i][i];
}

// Normal of a 3x3 covariance: the unit eigenvector of its smallest eigenvalue, in closed
// form (the reference solves this 3x3 problem directly too, util.cpp:262-267
// SelfAdjointEigenSolver::computeDirect). The smallest root of the characteristic cubic
// p(l) = l^3 - c2 l^2 + c1 l - c0 is found by Newton's method from a Gershgorin lower bound:
// p is negative, increasing and concave left of its smallest root, so the iterates rise
// monotonically to it; iteration stops when they no longer increase. An FP32 pass of the
// same iteration supplies a start just below the root, so that few FP64 steps remain. The eigenvector is the
// longest cross product of two rows of A - l I. Where the smallest eigenvalue is repeated
// (rows of A - l I parallel or zero) a unit vector orthogonal to the longest row is taken,
// and e_x for A = qI. FP64 throughout, basic operations only, so GPU and CPU agree bit for bit.
SML_HD void normal_from_cov(const double C[6] /*xx xy xz yy yz zz*/, float out[3]) {
    const double a00 = C[0], a01 = C[1], a02 = C[2], a11 = C[3], a12 = C[4], a22 = C[5];
    const double c2 = a00 + a11 + a22;
    const double c1 = (a00 * a11 - a01 * a01) + (a00 * a22 - a02 * a02) + (a11 * a22 - a12 * a12);
    const double c0 = a00 * (a11 * a22 - a12 * a12) - a01 * (a01 * a22 - a12 * a02) +
                      a02 * (a01 * a12 - a11 * a02);
    // Gershgorin lower bound of the spectrum (and not above 0: covariances are PSD)
    double l = a00 - (dabs(a01) + dabs(a02));
    const double g1 = a11 - (dabs(a01) + dabs(a12)), g2 = a22 - (dabs(a02) + dabs(a12));
    l = g1 < l ? g1 : l;
    l = g2 < l ? g2 : l;
    l = l < 0.0 ? l : 0.0;
    {
        // the same iteration in FP32 first (a fraction of the FP64 cost); its root, moved
        // down by 1e-4 of the trace (far above the FP32 error), starts the FP64 iterations
        // when p is still negative there, i.e. when it lies below the root
        const float f2 = (float)c2, f1 = (float)c1, f0 = (float)c0;
        float       lf = (float)l;
        for (int it = 0; it < 100; it++) {
            const float pv = ((lf - f2) * lf + f1) * lf - f0;
            const float dv = (3.0f * lf - 2.0f * f2) * lf + f1;
            if (!(dv > 0.0f) || !(pv < 0.0f))
                break;
            const float nl = lf - pv / dv;
            if (!(nl > lf))
                break;
            lf = nl;
        }
        const double l1 = (double)lf - 1e-4 * (c2 > 0.0 ? c2 : 0.0);
        if (l1 > l && ((l1 - c2) * l1 + c1) * l1 - c0 < 0.0)
            l = l1;
    }
    for (int it = 0; it < 100; it++) {
        const double pv = ((l - c2) * l + c1) * l - c0;
        const double dv = (3.0 * l - 2.0 * c2) * l + c1;
        if (!(dv > 0.0) || !(pv < 0.0))
            break;
        const double nl = l - pv / dv;
        if (!(nl > l))
            break;
        l = nl;
    }
    // rows of M = A - l I and their cross products
    const double r0[3] = {a00 - l, a01, a02}, r1[3] = {a01, a11 - l, a12}, r2[3] = {a02, a12, a22 - l};
    const double x01[3] = {r0[1] * r1[2] - r0[2] * r1[1], r0[2] * r1[0] - r0[0] * r1[2],
                           r0[0] * r1[1] - r0[1] * r1[0]};
    const double x02[3] = {r0[1] * r2[2] - r0[2] * r2[1], r0[2] * r2[0] - r0[0] * r2[2],
                           r0[0] * r2[1] - r0[1] * r2[0]};
    const double x12[3] = {r1[1] * r2[2] - r1[2] * r2[1], r1[2] * r2[0] - r1[0] * r2[2],
                           r1[0] * r2[1] - r1[1] * r2[0]};
    const double n01 = x01[0] * x01[0] + x01[1] * x01[1] + x01[2] * x01[2];
    const double n02 = x02[0] * x02[0] + x02[1] * x02[1] + x02[2] * x02[2];
    const double n12 = x12[0] * x12[0] + x12[1] * x12[1] + x12[2] * x12[2];
    const double m0  = r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2];
    const double m1  = r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2];
    const double m2  = r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2];
    const double mmax = m0 > m1 ? (m0 > m2 ? m0 : m2) : (m1 > m2 ? m1 : m2);
    double v[3], nv;
    if (n01 >= n02 && n01 >= n12) {
        v[0] = x01[0], v[1] = x01[1], v[2] = x01[2], nv = n01;
    } else if (n02 >= n12) {
        v[0] = x02[0], v[1] = x02[1], v[2] = x02[2], nv = n02;
    } else {
        v[0] = x12[0], v[1] = x12[1], v[2] = x12[2], nv = n12;
    }
    if (!(nv > mmax * mmax * 1e-20)) {
        // repeated smallest eigenvalue: any unit vector orthogonal to the longest row
        const double *r = m0 >= m1 && m0 >= m2 ? r0 : (m1 >= m2 ? r1 : r2);
        if (!(mmax > 0.0)) {
            out[0] = 1.0f;
            out[1] = 0.0f;
            out[2] = 0.0f;
            return;
        }
        // cross with the axis least aligned with r
        const double ax = dabs(r[0]), ay = dabs(r[1]), az = dabs(r[2]);
        if (ax <= ay && ax <= az) { // r x e_x
            v[0] = 0.0, v[1] = r[2], v[2] = -r[1];
        } else if (ay <= az) { // r x e_y
            v[0] = -r[2], v[1] = 0.0, v[2] = r[0];
        } else { // r x e_z
            v[0] = r[1], v[1] = -r[0], v[2] = 0.0;
        }
        nv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    }
    const double inv = 1.0 / dsqrt(nv);
    out[0]           = (float)(v[0] * inv);
    out[1]           = (float)(v[1] * inv);
    out[2]           = (float)(v[2] * inv);
}

SML_HD double det3(double a, double b, double c, double d, double e, double f, double g, double h,
                   double i) {
    return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

// Determinant of B without row r and column c (both in 0..3).
SML_HD double minor4(const double B[4][4], int r, int c) {
    int rr[3], cc[3], nr = 0, nc = 0;
    for (int k = 0; k < 4; k++) {
        if (k != r)
            rr[nr++] = k;
        if (k != c)
            cc[nc++] = k;
    }
    return det3(B[rr[0]][cc[0]], B[rr[0]][cc[1]], B[rr[0]][cc[2]], B[rr[1]][cc[0]],
                B[rr[1]][cc[1]], B[rr[1]][cc[2]], B[rr[2]][cc[0]], B[rr[2]][cc[1]],
                B[rr[2]][cc[2]]);
}

// Average of M unit quaternions from the upper triangle S of sum q q^T: the unit
// eigenvector of the largest eigenvalue of A = S / M (Markley, Cheng, Crassidis & Oshman,
// "Averaging Quaternions", 2007; the reference takes it from EigenSolver<Matrix4f>,
// util.cpp:563-576), in closed form. The largest root of the characteristic quartic
// p(l) = det(l I - A) = l^4 - c3 l^3 + c2 l^2 - c1 l + c0 is found by Newton's method from
// a Gershgorin upper bound: right of its largest root p is positive, increasing and convex,
// so the iterates fall monotonically to it; iteration stops when they no longer decrease.
// For a simple root, adj(A - l I) is a multiple of v v^T: its column with the largest
// diagonal entry is the eigenvector. Where that entry vanishes against the matrix scale
// (a repeated largest eigenvalue) the cyclic Jacobi decomposition decides. The sign is
// fixed by w >= 0 (q and -q are the same rotation). FP64, basic operations only, so GPU
// and CPU agree bit for bit.
SML_HD void quat_average_from_sum(const double S[10] /*upper triangle of sum q q^T*/, int M,
                                  double q[4]) {
    double A[4][4];
    int    k = 0;
    for (int i = 0; i < 4; i++)
        for (int j = i; j < 4; j++) {
            A[i][j] = S[k] / (double)M;
            A[j][i] = A[i][j];
            k++;
        }
    const double c3 = ((A[0][0] + A[1][1]) + A[2][2]) + A[3][3];
    double       c2 = 0.0, c1 = 0.0;
    for (int i = 0; i < 3; i++)
        for (int j = i + 1; j < 4; j++)
            c2 += A[i][i] * A[j][j] - A[i][j] * A[i][j];
    for (int i = 0; i < 4; i++)
        c1 += minor4(A, i, i);
    const double c0 = (A[0][0] * minor4(A, 0, 0) - A[0][1] * minor4(A, 0, 1)) +
                      (A[0][2] * minor4(A, 0, 2) - A[0][3] * minor4(A, 0, 3));
    double l = 0.0;
    for (int i = 0; i < 4; i++) {
        double r = A[i][i];
        for (int j = 0; j < 4; j++)
            if (j != i)
                r += dabs(A[i][j]);
        l = (i == 0 || r > l) ? r : l;
    }
    for (int it = 0; it < 100; it++) {
        const double pv = (((l - c3) * l + c2) * l - c1) * l + c0;
        const double dv = ((4.0 * l - 3.0 * c3) * l + 2.0 * c2) * l - c1;
        if (!(dv > 0.0) || !(pv > 0.0))
            break;
        const double nl = l - pv / dv;
        if (!(nl < l))
            break;
        l = nl;
    }
    double B[4][4];
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            B[i][j] = i == j ? A[i][j] - l : A[i][j];
    int    jc = 0;
    double dj = 0.0;
    for (int j = 0; j < 4; j++) {
        const double d = dabs(minor4(B, j, j));
        if (j == 0 || d > dj) {
            dj = d;
            jc = j;
        }
    }
    double v[4], n = 0.0;
    if (c3 > 0.0 && dj > 1e-9 * (c3 * c3 * c3)) {
        for (int i = 0; i < 4; i++) {
            const double m = minor4(B, i, jc);
            v[i]           = ((i + jc) & 1) ? -m : m;
            n += v[i] * v[i];
        }
    } else {
        double V[4][4], d[4];
        jacobi_eig<4>(A, V, d);
        int best = 0;
        for (int i = 1; i < 4; i++)
            if (d[i] > d[best])
                best = i;
        for (int i = 0; i < 4; i++) {
            v[i] = V[i][best];
            n += v[i] * v[i];
        }
    }
    if (!(n > 0.0)) {
        q[0] = 1.0;
        q[1] = q[2] = q[3] = 0.0;
        return;
    }
    const double inv = (v[0] < 0.0 ? -1.0 : 1.0) / dsqrt(n);
    for (int i = 0; i < 4; i++)
        q[i] = v[i] * inv;
}

// Unit quaternion (w,x,y,z) -> row-major rotation matrix.
SML_HD void quat_to_mat(const double q[4], double R[9]) {
    const double w = q[0], x = q[1], y = q[2], z = q[3];
    const double tx = 2.0 * x, ty = 2.0 * y, tz = 2.0 * z;
    const double twx = tx * w, twy = ty * w, twz = tz * w;
    const double txx = tx * x, txy = ty * x, txz = tz * x;
    const double tyy = ty * y, tyz = tz * y, tzz = tz * z;
    R[0]             = 1.0 - (tyy + tzz);
    R[1]             = txy - twz;
    R[2]             = txz + twy;
    R[3]             = txy + twz;
    R[4]             = 1.0 - (txx + tzz);
    R[5]             = tyz - twx;
    R[6]             = txz - twy;
    R[7]             = tyz + twx;
    R[8]             = 1.0 - (txx + tyy);
}

// Rotation matrix -> unit quaternion (w,x,y,z), Shepperd's method (largest-pivot branch).
SML_HD void mat_to_quat(const double R[9], double q[4]) {
    const double tr = R[0] + R[4] + R[8];
    if (tr > 0.0) {
        double t = dsqrt(tr + 1.0);
        q[0]     = 0.5 * t;
        t        = 0.5 / t;
        q[1]     = (R[7] - R[5]) * t;
        q[2]     = (R[2] - R[6]) * t;
        q[3]     = (R[3] - R[1]) * t;
    } else {
        int i = 0;
        if (R[4] > R[0])
            i = 1;
        if (R[8] > R[i * 4])
            i = 2;
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        double    t = dsqrt(R[i * 4] - R[j * 4] - R[k * 4] + 1.0);
        double    v[3];
        v[i] = 0.5 * t;
        t    = 0.5 / t;
        q[0] = (R[k * 3 + j] - R[j * 3 + k]) * t;
        v[j] = (R[j * 3 + i] + R[i * 3 + j]) * t;
        v[k] = (R[k * 3 + i] + R[i * 3 + k]) * t;
        q[1] = v[0];
        q[2] = v[1];
        q[3] = v[2];
    }
}

// Rotation angle in [0, pi] of a unit quaternion: 2 atan2(|v|, |w|) (AngleAxis from
// quaternion), evaluated with the shared float atan2.
SML_HD float quat_angle(const double q[4]) {
    const double n = dsqrt(q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    if (n == 0.0)
        return 0.0f;
    return 2.0f * smm::atan2f_((float)n, (float)dabs(q[0]));
}

// Solve the symmetric 6x6 system A u = r by Cholesky (A = L L^T). Returns false when a
// pivot is not positive relative to the matrix scale; the caller then uses the
// eigen-decomposition pseudo-inverse below.
SML_HD bool cholesky6(const double A[6][6], const double r[6], double u[6]) {
    double L[6][6], inv[6]; // inv[j] = 1 / L[j][j]: one division per pivot
    double dmax = 0.0;
    SML_UNROLL
    for (int i = 0; i < 6; i++)
        dmax = A[i][i] > dmax ? A[i][i] : dmax;
    if (!(dmax > 0.0))
        return false;
    SML_UNROLL
    for (int j = 0; j < 6; j++) {
        double s = A[j][j];
        SML_UNROLL
        for (int k = 0; k < j; k++)
            s -= L[j][k] * L[j][k];
        if (!(s > dmax * 1e-13))
            return false;
        const double ljj = dsqrt(s);
        L[j][j]          = ljj;
        inv[j]           = 1.0 / ljj;
        SML_UNROLL
        for (int i = j + 1; i < 6; i++) {
            double t = A[i][j];
            SML_UNROLL
            for (int k = 0; k < j; k++)
                t -= L[i][k] * L[j][k];
            L[i][j] = t * inv[j];
        }
    }
    double y[6];
    SML_UNROLL
    for (int i = 0; i < 6; i++) {
        double t = r[i];
        SML_UNROLL
        for (int k = 0; k < i; k++)
            t -= L[i][k] * y[k];
        y[i] = t * inv[i];
    }
    SML_UNROLL
    for (int i = 5; i >= 0; i--) {
        double t = y[i];
        SML_UNROLL
        for (int k = 5; k > i; k--) // descending k: the order of the warp version's column sweep
            t -= L[k][i] * u[k];
        u[i] = t * inv[i];
    }
    return true;
}

#if defined(__CUDACC__)
// cholesky6 by one warp, one row per lane (lanes 0-5; every lane calls it): per column the
// pivot's square root, then all rows' updates and divisions at once; the triangular solves
// column by column. Each element sees the same operations in the same order as cholesky6,
// so the results are identical; every lane gets u. Returns false where cholesky6 does.
__device__ __forceinline__ bool cholesky6_warp(const double A[6][6], const double r[6], double u[6]) {
    const int lane = threadIdx.x & 31;
    const int row  = lane < 6 ? lane : 5;
    double    Lr[6]; // row `row` of L
    double    inv  = 0.0; // 1 / L[row][row]
    double    dmax = 0.0;
    SML_UNROLL
    for (int i = 0; i < 6; i++)
        dmax = A[i][i] > dmax ? A[i][i] : dmax;
    if (!(dmax > 0.0))
        return false;
    SML_UNROLL
    for (int j = 0; j < 6; j++) {
        // the pivot row j: s = A[j][j] - sum_k L[j][k]^2 (lane j), broadcast
        double s = A[j][j];
        SML_UNROLL
        for (int k = 0; k < j; k++) {
            const double ljk = __shfl_sync(0xffffffffu, Lr[k], j);
            s -= ljk * ljk;
        }
        if (!(s > dmax * 1e-13))
            return false;
        const double ljj  = dsqrt(s);
        const double invj = 1.0 / ljj;
        if (row == j)
            inv = invj;
        // rows i > j: t = A[i][j] - sum_k L[i][k] L[j][k], L[i][j] = t * (1 / L[j][j])
        double t = A[row][j];
        SML_UNROLL
        for (int k = 0; k < j; k++)
            t -= Lr[k] * __shfl_sync(0xffffffffu, Lr[k], j);
        Lr[j] = row == j ? ljj : (row > j ? t * invj : 0.0);
    }
    // forward: y_i = (r_i - sum_{k<i} L[i][k] y_k) * (1 / L[i][i]), column by column
    double ti = r[row], y[6];
    SML_UNROLL
    for (int k = 0; k < 6; k++) {
        const double yk = __shfl_sync(0xffffffffu, ti * inv, k);
        y[k]            = yk;
        if (row > k)
            ti -= Lr[k] * yk;
    }
    // back: u_i = (y_i - sum_{k>i, descending} L[k][i] u_k) * (1 / L[i][i]); L[k][i] is row k's
    double tb = y[row];
    SML_UNROLL
    for (int k = 5; k >= 0; k--) {
        const double uk  = __shfl_sync(0xffffffffu, tb * inv, k);
        u[k]             = uk;
        double lki = 0.0; // L[k][row] held by lane k
        SML_UNROLL
        for (int i = 0; i < 6; i++) {
            const double v = __shfl_sync(0xffffffffu, Lr[i], k);
            if (i == row)
                lki = v;
        }
        if (row < k)
            tb -= lki * uk;
    }
    return true;
}
#endif

// Least-squares / minimum-norm solve of a symmetric PSD 6x6 system through its
// eigen-decomposition, discarding eigenvalues below 1e-6 of the largest (rank-deficient
// cases the reference handles with JacobiSVD, icp.cpp:68).
SML_HD void pinv6(const double Ain[6][6], const double r[6], double u[6]) {
    double A[6][6], V[6][6], d[6];
    for (int i = 0; i < 6; i++)
        for (int j = 0; j < 6; j++)
            A[i][j] = Ain[i][j];
    jacobi_eig<6>(A, V, d);
    double dmax = 0.0;
    for (int i = 0; i < 6; i++)
        dmax = dabs(d[i]) > dmax ? dabs(d[i]) : dmax;
    for (int i = 0; i < 6; i++)
        u[i] = 0.0;
    for (int k = 0; k < 6; k++) {
        if (!(dabs(d[k]) > dmax * 1e-6))
            continue;
        double c = 0.0;
        for (int i = 0; i < 6; i++)
            c += V[i][k] * r[i];
        c /= d[k];
        for (int i = 0; i < 6; i++)
            u[i] += c * V[i][k];
    }
}

} // namespace sml
