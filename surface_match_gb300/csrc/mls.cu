// mls.cu - moving-least-squares normals and surface projection of listed points
// (estimateNormalMLS, util.cpp:336-457, declared in privateUtil.h:13).
//
// For each listed point p, over its neighbours closer than the radius (strict <, the k-d
// tree's radius search, util.cpp:357-362; points with fewer than 3 are left unchanged):
//   1. PCA plane: centroid c, covariance, n = eigenvector of the smallest eigenvalue
//      (util.cpp:368-381); the normal output takes n here already, as the reference writes
//      it before its later exits.
//   2. The query projected on the plane, m = p - (n.(p - c)) n, and a tangent frame:
//      v = a unit vector orthogonal to n (Eigen's unitOrthogonal), u = n x v
//      (util.cpp:385-390).
//   3. A weighted least-squares fit of the heights f = (q - m).n over the tangent
//      coordinates by the polynomial of total degree `order` with monomials u^a v^b in the
//      order a = 0..order, b = 0..order-a; weights exp(-|q - m|^2 / r^2)
//      (util.cpp:392-436). Order <= 1 with fewer neighbours than coefficients stops at 1.
//   4. The point moves to the fit's value at the origin, m + c0 n, and the normal is
//      n - c_u u - c_v v, normalised (c_u, c_v: the coefficients of u and v, indices
//      order+1 and 1), then oriented toward the viewpoint (or +z) with the invert rule of
//      the normal estimator (util.cpp:439-455).
//
// Deterministic two-phase form: neighbourhoods always read the positions at the start of
// the call, and results go to separate outputs (the reference projects points in place
// while other threads read them as neighbours). Where the weighted system is not positive
// definite (Eigen's LLT then reports a numerical issue and its solve returns an unspecified
// vector) the point keeps the PCA normal, as for a non-finite solution.
//
// One warp per listed point over a hashed grid of cell just above the radius, so the 3x3x3
// block holds every neighbour. Sums are FP32 Kahan per lane, merged in FP64; the fit runs
// in coordinates scaled by 1/r (the same polynomial, better conditioned); the small
// systems are solved in FP64.
#include <cmath>

#include "sm_device.cuh"
#include "sm_icp.h"
#include "sm_linalg.h"
#include "sm_stages.h"

namespace sm {
namespace {

constexpr int kMlsWarps    = 8;
constexpr int kMlsMaxCoeff = (kMlsMaxOrder + 1) * (kMlsMaxOrder + 2) / 2;          // 15
constexpr int kMlsMaxEnt   = kMlsMaxCoeff * (kMlsMaxCoeff + 1) / 2 + kMlsMaxCoeff; // 135
constexpr int kMlsPerLane  = (kMlsMaxEnt + 31) / 32;                               // 5

struct MlsArgs {
    smd::HGridView g; // the finite points; cell side >= 1.02 radius
    const float4  *pos;
    const int     *ids;
    int            m;
    float          r, r2;
    int            order, nc;
    int            invert, hasVp;
    float          vx, vy, vz;
    float         *outXyz, *outNrm; // n x 3, pre-filled with the inputs
};

__device__ __forceinline__ bool finite3f(float x, float y, float z) {
    return isfinite(x) && isfinite(y) && isfinite(z);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Exponents (a, b) of monomial k, in the order a = 0..order, b = 0..order-a.
__device__ __forceinline__ void monomial(int k, int order, int &a, int &b) {
    a = 0;
    while (k > order - a) {
        k -= order - a + 1;
        a++;
    }
    b = k;
}

// Entry e of the fit's sums: the upper triangle of the Gram matrix row by row (k <= l),
// then the right-hand side. Returns the exponents of u and v in the entry's term and whether
// it carries the height.
__device__ __forceinline__ void entry_terms(int e, int nc, int order, int &A, int &B, bool &rhs) {
    const int ng = nc * (nc + 1) / 2;
    int       k = 0, l = 0;
    if (e < ng) {
        rhs = false;
        while (e >= nc - k) {
            e -= nc - k;
            k++;
        }
        l = k + e;
    } else {
        rhs = true;
        k   = e - ng;
    }
    int ak, bk, al = 0, bl = 0;
    monomial(k, order, ak, bk);
    if (!rhs)
        monomial(l, order, al, bl);
    A = ak + al;
    B = bk + bl;
}

__device__ __forceinline__ float powi(float x, int e) {
    float r = 1.0f;
    for (int i = 0; i < e; i++)
        r *= x;
    return r;
}

// In-place Cholesky solve of the SPD system G c = b (n <= kMlsMaxCoeff, G row-major full);
// false when a pivot is not positive or the solution is not finite.
__device__ bool cholesky_solve(double *G, double *b, int n) {
    for (int j = 0; j < n; j++) {
        double d = G[j * n + j];
        for (int k = 0; k < j; k++)
            d -= G[j * n + k] * G[j * n + k];
        if (!(d > 0.0))
            return false;
        const double s = sqrt(d);
        G[j * n + j]   = s;
        for (int i = j + 1; i < n; i++) {
            double v = G[i * n + j];
            for (int k = 0; k < j; k++)
                v -= G[i * n + k] * G[j * n + k];
            G[i * n + j] = v / s;
        }
    }
    for (int i = 0; i < n; i++) { // L y = b
        double v = b[i];
        for (int k = 0; k < i; k++)
            v -= G[i * n + k] * b[k];
        b[i] = v / G[i * n + i];
    }
    for (int i = n - 1; i >= 0; i--) { // L^T c = y
        double v = b[i];
        for (int k = i + 1; k < n; k++)
            v -= G[k * n + i] * b[k];
        b[i] = v / G[i * n + i];
        if (!isfinite(b[i]))
            return false;
    }
    return true;
}

__global__ void __launch_bounds__(kMlsWarps * 32) k_mls(MlsArgs a) {
    __shared__ double sSys[kMlsWarps][kMlsMaxCoeff * kMlsMaxCoeff + kMlsMaxCoeff];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int t    = blockIdx.x * kMlsWarps + wid;
    if (t >= a.m)
        return; // warp-uniform
    const int    id = a.ids[t];
    const float4 q  = a.pos[id];
    if (!finite3f(q.x, q.y, q.z))
        return; // a search from a non-finite point finds nothing
    int c[3];
    smd::grid_cc(a.g, q.x, q.y, q.z, c);
    const float r2 = a.r2;

    // 1. count and centroid (offsets from q)
    smi::KahanF s0[3];
    int         cnt = 0;
    for (int d = 0; d < 3; d++)
        s0[d].init();
    smd::warp_block27(a.g, q.x, q.y, q.z, c, r2, [&](const float4 &p, bool valid) {
        if (valid && smm::dist2(q.x, q.y, q.z, p.x, p.y, p.z) < r2) {
            cnt++;
            s0[0].add(p.x - q.x);
            s0[1].add(p.y - q.y);
            s0[2].add(p.z - q.z);
        }
        return false;
    });
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (cnt < 3)
        return;
    const double inv = 1.0 / (double)cnt;
    const float  cx = (float)((double)q.x + warp_sum((double)s0[0].value()) * inv);
    const float  cy = (float)((double)q.y + warp_sum((double)s0[1].value()) * inv);
    const float  cz = (float)((double)q.z + warp_sum((double)s0[2].value()) * inv);

    // covariance about the centroid
    smi::KahanF s1[6];
    for (int e = 0; e < 6; e++)
        s1[e].init();
    smd::warp_block27(a.g, q.x, q.y, q.z, c, r2, [&](const float4 &p, bool valid) {
        if (valid && smm::dist2(q.x, q.y, q.z, p.x, p.y, p.z) < r2) {
            const float dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
            s1[0].add(dx * dx);
            s1[1].add(dx * dy);
            s1[2].add(dx * dz);
            s1[3].add(dy * dy);
            s1[4].add(dy * dz);
            s1[5].add(dz * dz);
        }
        return false;
    });
    double C[6];
    for (int e = 0; e < 6; e++)
        C[e] = warp_sum((double)s1[e].value());
    float n[3];
    sml::normal_from_cov(C, n);
    float *outN = a.outNrm + 3 * (size_t)id;
    float *outP = a.outXyz + 3 * (size_t)id;
    if (lane == 0) {
        outN[0] = n[0];
        outN[1] = n[1];
        outN[2] = n[2];
    }

    // 2. projection on the plane and the tangent frame
    const float dist = n[0] * (q.x - cx) + n[1] * (q.y - cy) + n[2] * (q.z - cz);
    const float mx = q.x - dist * n[0], my = q.y - dist * n[1], mz = q.z - dist * n[2];
    float       v[3];
    if (!(fabsf(n[0]) <= fabsf(n[2]) * 1e-5f) || !(fabsf(n[1]) <= fabsf(n[2]) * 1e-5f)) {
        const float h = smm::fdiv(1.0f, smm::fsqrt(n[0] * n[0] + n[1] * n[1]));
        v[0]          = -n[1] * h;
        v[1]          = n[0] * h;
        v[2]          = 0.0f;
    } else {
        const float h = smm::fdiv(1.0f, smm::fsqrt(n[1] * n[1] + n[2] * n[2]));
        v[0]          = 0.0f;
        v[1]          = -n[2] * h;
        v[2]          = n[1] * h;
    }
    const float u[3] = {n[1] * v[2] - n[2] * v[1], n[2] * v[0] - n[0] * v[2],
                        n[0] * v[1] - n[1] * v[0]};
    const int   nc   = a.nc;
    if (a.order <= 1 && nc > cnt)
        return;

    // 3. the fit's sums; lane L owns entries L, L + 32, ... and adds every neighbour's term
    const int ne = nc * (nc + 1) / 2 + nc;
    int       eA[kMlsPerLane], eB[kMlsPerLane];
    bool      eR[kMlsPerLane];
    smi::KahanF acc[kMlsPerLane];
#pragma unroll
    for (int k = 0; k < kMlsPerLane; k++) {
        acc[k].init();
        eA[k] = eB[k] = 0;
        eR[k]         = false;
        const int e   = lane + 32 * k;
        if (e < ne)
            entry_terms(e, nc, a.order, eA[k], eB[k], eR[k]);
    }
    const float invR = smm::fdiv(1.0f, a.r);
    smd::warp_block27(a.g, q.x, q.y, q.z, c, r2, [&](const float4 &p, bool valid) {
        float w = 0.0f, uc = 0.0f, vc = 0.0f, fc = 0.0f;
        if (valid && smm::dist2(q.x, q.y, q.z, p.x, p.y, p.z) < r2) {
            const float dx = p.x - mx, dy = p.y - my, dz = p.z - mz;
            w  = expf(-smm::fdiv(dx * dx + dy * dy + dz * dz, r2));
            uc = (dx * u[0] + dy * u[1] + dz * u[2]) * invR;
            vc = (dx * v[0] + dy * v[1] + dz * v[2]) * invR;
            fc = (dx * n[0] + dy * n[1] + dz * n[2]) * invR;
        }
        unsigned live = __ballot_sync(0xffffffffu, w > 0.0f);
        while (live) {
            const int   j  = __ffs(live) - 1;
            live &= live - 1;
            const float wj = __shfl_sync(0xffffffffu, w, j);
            const float uj = __shfl_sync(0xffffffffu, uc, j);
            const float vj = __shfl_sync(0xffffffffu, vc, j);
            const float fj = __shfl_sync(0xffffffffu, fc, j);
#pragma unroll
            for (int k = 0; k < kMlsPerLane; k++)
                if (lane + 32 * k < ne) {
                    const float term = wj * powi(uj, eA[k]) * powi(vj, eB[k]);
                    acc[k].add(eR[k] ? term * fj : term);
                }
        }
        return false;
    });
    double *S = sSys[wid]; // G (nc x nc, full), then b
#pragma unroll
    for (int k = 0; k < kMlsPerLane; k++) {
        int e = lane + 32 * k;
        if (e < ne) {
            const double val = (double)acc[k].value();
            if (eR[k]) {
                S[nc * nc + (e - nc * (nc + 1) / 2)] = val;
            } else {
                int row = 0;
                while (e >= nc - row) {
                    e -= nc - row;
                    row++;
                }
                const int col      = row + e;
                S[row * nc + col] = val;
                S[col * nc + row] = val;
            }
        }
    }
    __syncwarp();
    if (lane == 0) {
        double *G = S, *b = S + nc * nc;
        if (cholesky_solve(G, b, nc)) {
            // 4. coefficients back to unscaled coordinates: c0 scales by r, the linear
            // terms are slopes and do not change
            const float c0 = (float)(b[0] * (double)a.r);
            const float cv = (float)b[1], cu = (float)b[a.order + 1];
            const float px = mx + c0 * n[0], py = my + c0 * n[1], pz = mz + c0 * n[2];
            float       nx = n[0] - cu * u[0] - cv * v[0], ny = n[1] - cu * u[1] - cv * v[1],
                  nz = n[2] - cu * u[2] - cv * v[2];
            const float nn = nx * nx + ny * ny + nz * nz;
            if (nn > 0.0f) {
                const float s = smm::fsqrt(nn);
                nx            = smm::fdiv(nx, s);
                ny            = smm::fdiv(ny, s);
                nz            = smm::fdiv(nz, s);
            }
            const float d = a.hasVp ? nx * (a.vx - px) + ny * (a.vy - py) + nz * (a.vz - pz) : nz;
            if (a.invert ? d > 0.0f : d < 0.0f) {
                nx = -nx;
                ny = -ny;
                nz = -nz;
            }
            outP[0] = px;
            outP[1] = py;
            outP[2] = pz;
            outN[0] = nx;
            outN[1] = ny;
            outN[2] = nz;
        }
    }
}

__global__ void k_fill_nan(float *x, long long n) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n)
        x[i] = __int_as_float(0x7fc00000);
}

} // namespace

void estimate_normals_mls(Ctx &c, const float4 *pos, const int *valid, int nvalid, const Box &box,
                          const int *ids, int m, float radius, int order, bool invert,
                          const float *vp, float *outXyz, float *outNrm) {
    const float r  = std::fabs(radius);
    const float r2 = radius * radius;
    if (m <= 0 || nvalid <= 0 || !(r2 > 0.0f))
        return; // no point has a neighbour within a zero radius
    HGrid G;
    build_hgrid(c, pos, valid, nvalid, box, r * 1.02f, G, "mls.g");
    MlsArgs a;
    a.g      = G.view();
    a.pos    = pos;
    a.ids    = ids;
    a.m      = m;
    a.r      = r;
    a.r2     = r2;
    a.order  = order;
    a.nc     = (order + 1) * (order + 2) / 2;
    a.invert = invert ? 1 : 0;
    a.hasVp  = vp && std::isfinite(vp[0]) && std::isfinite(vp[1]) && std::isfinite(vp[2]);
    a.vx     = a.hasVp ? vp[0] : 0.f;
    a.vy     = a.hasVp ? vp[1] : 0.f;
    a.vz     = a.hasVp ? vp[2] : 0.f;
    a.outXyz = outXyz;
    a.outNrm = outNrm;
    k_mls<<<nblocks(m, kMlsWarps), kMlsWarps * 32, 0, c.stream>>>(a);
    SM_LAUNCH_CHECK();
}

void fill_nan(Ctx &c, float *x, long long n) {
    if (n <= 0)
        return;
    k_fill_nan<<<nblocks(n, 256), 256, 0, c.stream>>>(x, n);
    SM_LAUNCH_CHECK();
}

} // namespace sm
