// sm_math.h - IEEE-float arithmetic of the point-pair-feature hot path, shared by the CUDA
// kernels and the CPU oracle so that quantised keys, alpha angles and vote bins are
// bit-identical on both sides by construction.
//
// Build rules that make this header deterministic:
//   * device: nvcc --fmad=false (no FMA contraction), IEEE division and square root
//     (__fdiv_rn / __fsqrt_rn are called explicitly below);
//   * host:   -ffp-contract=off -fno-fast-math (aarch64 gcc contracts by default).
//
// The reference computes these quantities with xsimd (SIMD lanes) and glibc libm (scalar
// tails), neither of which is vendored with the reference; their exact polynomials are not
// available, so the transcendental functions here are written from the Cephes Math Library
// (S. L. Moshier, atanf.c / asinf.c / sinf.c): argument reduction followed by its published
// minimax polynomials. They are accurate to a few float ulp (checked against libm in the
// tests); agreement with the reference binary is therefore pinned only up to that accuracy,
// while agreement between the GPU and the oracle is exact.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SM_HD __host__ __device__ __forceinline__
#else
#define SM_HD inline
#include <cmath>
#endif

namespace smm {

// float constants as the reference spells them: M_PI rounded to float, and
// ppf.cpp:24 `const float M_2PI = 2 * M_PI`.
constexpr float kPiF   = 3.14159265358979323846f;
constexpr float k2PiF  = (float)(2.0 * 3.14159265358979323846);
constexpr float kPio2F = 1.57079632679489661923f;
constexpr float kPio4F = 0.785398163397448309616f;
constexpr double kPiD  = 3.14159265358979323846;

SM_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

SM_HD float fsqrt(float a) {
#if defined(__CUDA_ARCH__)
    return __fsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}

SM_HD float fabs_(float a) {
#if defined(__CUDA_ARCH__)
    return fabsf(a);
#else
    return std::fabs(a);
#endif
}

SM_HD float ffloor(float a) {
#if defined(__CUDA_ARCH__)
    return floorf(a);
#else
    return std::floor(a);
#endif
}

SM_HD float fceil(float a) {
#if defined(__CUDA_ARCH__)
    return ceilf(a);
#else
    return std::ceil(a);
#endif
}

SM_HD float fcopysign(float a, float s) {
#if defined(__CUDA_ARCH__)
    return copysignf(a, s);
#else
    return std::copysign(a, s);
#endif
}

SM_HD bool fisnan(float a) { return a != a; }

// ---------------------------------------------------------------------------------------
// Cephes-method transcendental functions (float).
// ---------------------------------------------------------------------------------------

// atan(x): reduction to |x| <= tan(pi/8) via the identities atan(x) = pi/2 - atan(1/x)
// and atan(x) = pi/4 + atan((x-1)/(x+1)), then a degree-9 odd minimax polynomial.
SM_HD float atanf_(float xx) {
    float x = fabs_(xx);
    float y;
    if (x > 2.414213562373095f) {
        y = kPio2F;
        x = -fdiv(1.0f, x);
    } else if (x > 0.4142135623730950f) {
        y = kPio4F;
        x = fdiv(x - 1.0f, x + 1.0f);
    } else {
        y = 0.0f;
    }
    const float z = x * x;
    const float p = ((8.05374449538e-2f * z - 1.38776856032e-1f) * z + 1.99777106478e-1f) * z -
                    3.33329491539e-1f;
    y = y + (p * z * x + x);
    return xx < 0.0f ? -y : y;
}

// atan2(y, x) with the C99 conventions for signed zeros: atan2(+-0, x<0 or -0) = +-pi,
// atan2(+-0, x>0 or +0) = +-0, atan2(y!=0, +-0) = +-pi/2. NaN in, NaN out.
SM_HD float atan2f_(float y, float x) {
    if (fisnan(x) || fisnan(y))
        return x + y;
    if (y == 0.0f) {
        const bool xneg = (x < 0.0f) || (x == 0.0f && fcopysign(1.0f, x) < 0.0f);
        return xneg ? fcopysign(kPiF, y) : y;
    }
    if (x == 0.0f)
        return fcopysign(kPio2F, y);
    float a = atanf_(fdiv(y, x));
    if (x < 0.0f)
        a = (y > 0.0f) ? a + kPiF : a - kPiF;
    return a;
}

// asin(x) on |x| <= 1: for |x| > 1/2 use asin(x) = pi/2 - 2 asin(sqrt((1-x)/2)).
SM_HD float asinf_(float xx) {
    float a = fabs_(xx);
    if (a > 1.0f)
        return fdiv(0.0f, 0.0f);
    if (a < 1.0e-4f)
        return xx;
    float x, z;
    bool  big = false;
    if (a > 0.5f) {
        z   = 0.5f * (1.0f - a);
        x   = fsqrt(z);
        big = true;
    } else {
        x = a;
        z = x * x;
    }
    const float p = (((4.2163199048e-2f * z + 2.4181311049e-2f) * z + 4.5470025998e-2f) * z +
                     7.4953002686e-2f) * z + 1.6666752422e-1f;
    z = p * z * x + x;
    if (big) {
        z = z + z;
        z = kPio2F - z;
    }
    return xx < 0.0f ? -z : z;
}

SM_HD float acosf_(float x) {
    if (x < -1.0f || x > 1.0f)
        return fdiv(0.0f, 0.0f);
    if (x < -0.5f)
        return kPiF - 2.0f * asinf_(fsqrt(0.5f * (1.0f + x)));
    if (x > 0.5f)
        return 2.0f * asinf_(fsqrt(0.5f * (1.0f - x)));
    return kPio2F - asinf_(x);
}

// sin / cos: octant reduction with a three-part (Cody-Waite) pi/4, then the degree-7 sine
// or degree-8 cosine polynomial on |x| <= pi/4. Arguments here are angles in [-2pi, 2pi].
constexpr float kFopiF = 1.27323954473516f; // 4/pi
constexpr float kDp1F  = 0.78515625f;
constexpr float kDp2F  = 2.4187564849853515625e-4f;
constexpr float kDp3F  = 3.77489497744594108e-8f;

SM_HD float poly_sin_(float x, float z) {
    return ((-1.9515295891e-4f * z + 8.3321608736e-3f) * z - 1.6666654611e-1f) * z * x + x;
}
SM_HD float poly_cos_(float z) {
    return ((2.443315711809948e-5f * z - 1.388731625493765e-3f) * z + 4.166664568298827e-2f) *
               z * z -
           0.5f * z + 1.0f;
}

SM_HD float sinf_(float xx) {
    float x    = fabs_(xx);
    bool  neg  = xx < 0.0f;
    int   j    = (int)(kFopiF * x);
    float y    = (float)j;
    if (j & 1) {
        j += 1;
        y += 1.0f;
    }
    j &= 7;
    if (j > 3) {
        neg = !neg;
        j -= 4;
    }
    x             = ((x - y * kDp1F) - y * kDp2F) - y * kDp3F;
    const float z = x * x;
    const float r = (j == 1 || j == 2) ? poly_cos_(z) : poly_sin_(x, z);
    return neg ? -r : r;
}

SM_HD float cosf_(float xx) {
    float x   = fabs_(xx);
    bool  neg = false;
    int   j   = (int)(kFopiF * x);
    float y   = (float)j;
    if (j & 1) {
        j += 1;
        y += 1.0f;
    }
    j &= 7;
    if (j > 3) {
        neg = !neg;
        j -= 4;
    }
    if (j > 1)
        neg = !neg;
    x             = ((x - y * kDp1F) - y * kDp2F) - y * kDp3F;
    const float z = x * x;
    const float r = (j == 1 || j == 2) ? poly_sin_(x, z) : poly_cos_(z);
    return neg ? -r : r;
}

// ---------------------------------------------------------------------------------------
// MurmurHash3_x86_32 (Austin Appleby, public domain) of the four quantised feature words,
// key length 16 bytes, seed 42 (util.cpp:643-695 scalar, util.cpp:732-777 SIMD).
// ---------------------------------------------------------------------------------------
SM_HD uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

SM_HD uint32_t murmur_mix_(uint32_t h, uint32_t k) {
    k *= 0xcc9e2d51u;
    k = rotl32(k, 15);
    k *= 0x1b873593u;
    h ^= k;
    return rotl32(h, 13) * 5u + 0xe6546b64u;
}

SM_HD uint32_t murmur4(uint32_t w0, uint32_t w1, uint32_t w2, uint32_t w3) {
    uint32_t h = 42u;
    h          = murmur_mix_(h, w0);
    h          = murmur_mix_(h, w1);
    h          = murmur_mix_(h, w2);
    h          = murmur_mix_(h, w3);
    h ^= 16u;
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

} // namespace smm
#include <algorithm>
#include <vector>
namespace smm {
// (host) Largest number of entries one reference point has in a bucket (refs[b0..b1)): a hit on
// the bucket adds at most this many votes to any accumulator cell, so the sum over a
// keypoint's hits bounds its largest cell (it picks the accumulator's counter width).
inline uint32_t bucket_max_ref_multiplicity(const uint32_t *refs, uint32_t b0, uint32_t b1) {
    std::vector<uint32_t> t(refs + b0, refs + b1);
    std::sort(t.begin(), t.end());
    uint32_t best = t.empty() ? 0u : 1u, run = 1;
    for (size_t i = 1; i < t.size(); i++) {
        run  = t[i] == t[i - 1] ? run + 1 : 1;
        best = run > best ? run : best;
    }
    return best;
}

// splitmix64 finaliser (S. Vigna): fingerprint mixing of accumulator cells.
SM_HD uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// float -> uint32 conversion of a non-negative quantised value. NaN (only reachable for a
// zero-length pair, which two distinct sampled points never form) maps to 0x80000000, the
// x86 "integer indefinite" value, on both host and device.
SM_HD uint32_t f2u_(float v) { return fisnan(v) ? 0x80000000u : (uint32_t)v; }
SM_HD uint32_t f2i_(float v) { return fisnan(v) ? 0x80000000u : (uint32_t)(int)v; }

// ---------------------------------------------------------------------------------------
// Point-pair feature. The reference evaluates the pairs of one reference point in 8-wide
// AVX blocks (util.cpp:779-820) and the last (rows mod 8) pairs with scalar Eigen code
// (util.cpp:712-730, 822-824). The two paths differ in rounding (ceil vs. truncation of the
// quantised words, and the summation order of the 3-vector reductions), so the row's
// position selects the rule: `block` = the row lies in a full 8-lane block.
// ---------------------------------------------------------------------------------------
constexpr int kLanes = 8; // xsimd batch<float> width under -mavx (CMakeLists.txt:44)

// angle between a and b as atan2(|a x b|, a.b); block: (x+y)+z sums, tail: Eigen x+(y+z).
SM_HD float angle_block_(float ax, float ay, float az, float bx, float by, float bz) {
    const float i = ay * bz - az * by;
    const float j = az * bx - ax * bz;
    const float k = ax * by - ay * bx;
    const float c = fsqrt((i * i + j * j) + k * k);
    const float d = (ax * bx + ay * by) + az * bz;
    return atan2f_(c, d);
}
SM_HD float angle_tail_(float ax, float ay, float az, float bx, float by, float bz) {
    const float i = ay * bz - az * by;
    const float j = az * bx - ax * bz;
    const float k = ax * by - ay * bx;
    const float c = fsqrt(i * i + (j * j + k * k));
    const float d = ax * bx + (ay * by + az * bz);
    return atan2f_(c, d);
}

// Quantised, hashed PPF key of pair (p1,n1) -> (p2,n2).
SM_HD uint32_t ppf_key(bool block, float p1x, float p1y, float p1z, float n1x, float n1y,
                       float n1z, float p2x, float p2y, float p2z, float n2x, float n2y,
                       float n2z, float angleStep, float distStep) {
    const float dx = p2x - p1x;
    const float dy = p2y - p1y;
    const float dz = p2z - p1z;
    if (block) {
        const float dn = fsqrt((dx * dx + dy * dy) + dz * dz);
        const float ux = fdiv(dx, dn), uy = fdiv(dy, dn), uz = fdiv(dz, dn);
        const float f1 = angle_block_(ux, uy, uz, n1x, n1y, n1z);
        const float f2 = angle_block_(ux, uy, uz, n2x, n2y, n2z);
        const float f3 = angle_block_(n1x, n1y, n1z, n2x, n2y, n2z);
        return murmur4(f2u_(fceil(fdiv(f1, angleStep))), f2u_(fceil(fdiv(f2, angleStep))),
                       f2u_(fceil(fdiv(f3, angleStep))), f2u_(fceil(fdiv(dn, distStep))));
    }
    const float dn = fsqrt(dx * dx + (dy * dy + dz * dz));
    float       f1 = 0.0f, f2 = 0.0f, f3 = 0.0f;
    if (dn > 0.0f) {
        const float ux = fdiv(dx, dn), uy = fdiv(dy, dn), uz = fdiv(dz, dn);
        f1 = angle_tail_(ux, uy, uz, n1x, n1y, n1z);
        f2 = angle_tail_(ux, uy, uz, n2x, n2y, n2z);
        f3 = angle_tail_(n1x, n1y, n1z, n2x, n2y, n2z);
    }
    return murmur4(f2i_(fdiv(f1, angleStep)), f2i_(fdiv(f2, angleStep)),
                   f2i_(fdiv(f3, angleStep)), f2i_(fdiv(dn, distStep)));
}

// transformRT (util.cpp:459-475): rotation taking n onto +x about the axis (0, n_z, -n_y),
// angle acos(n_x), as the Rodrigues matrix c*I + s*[a]x + (1-c)*a*a^T, and t = -R p.
struct RT {
    float r[9]; // row-major
    float t[3];
};

SM_HD RT transform_rt(float px, float py, float pz, float nx, float ny, float nz) {
    const float angle = acosf_(nx);
    float       ax = 0.0f, ay = nz, az = -ny;
    if (ny == 0.0f && nz == 0.0f) {
        ax = 0.0f;
        ay = 1.0f;
        az = 0.0f;
    }
    const float sq = ax * ax + (ay * ay + az * az);
    if (sq > 0.0f) {
        const float s = fsqrt(sq);
        ax            = fdiv(ax, s);
        ay            = fdiv(ay, s);
        az            = fdiv(az, s);
    }
    const float s = sinf_(angle), c = cosf_(angle);
    const float sx = s * ax, sy = s * ay, sz = s * az;
    const float omc = 1.0f - c;
    const float cx = omc * ax, cy = omc * ay, cz = omc * az;
    RT          o;
    float       m;
    m      = cx * ay;
    o.r[1] = m - sz;
    o.r[3] = m + sz;
    m      = cx * az;
    o.r[2] = m + sy;
    o.r[6] = m - sy;
    m      = cy * az;
    o.r[5] = m - sx;
    o.r[7] = m + sx;
    o.r[0] = cx * ax + c;
    o.r[4] = cy * ay + c;
    o.r[8] = cz * az + c;
    o.t[0] = -(o.r[0] * px + (o.r[1] * py + o.r[2] * pz));
    o.t[1] = -(o.r[3] * px + (o.r[4] * py + o.r[5] * pz));
    o.t[2] = -(o.r[6] * px + (o.r[7] * py + o.r[8] * pz));
    return o;
}

// computeAlpha: angle of RT*p2 about the x axis (util.cpp:829-872 block, 477-484 tail).
SM_HD float alpha_of(bool block, const RT &rt, float x, float y, float z) {
    float my, mz;
    if (block) {
        my = ((rt.r[3] * x + rt.r[4] * y) + rt.r[5] * z) + rt.t[1];
        mz = ((rt.r[6] * x + rt.r[7] * y) + rt.r[8] * z) + rt.t[2];
    } else {
        my = (rt.r[3] * x + (rt.r[4] * y + rt.r[5] * z)) + rt.t[1];
        mz = (rt.r[6] * x + (rt.r[7] * y + rt.r[8] * z)) + rt.t[2];
    }
    const float a = atan2f_(mz * -1.0f, my);
    if (sinf_(a) * mz > 0.0f)
        return a * -1.0f;
    return a;
}

// Angle-bin of one bucket entry (ppf.cpp:316-340). `block` = the entry lies in a full
// 8-lane block of its bucket. `as` is the scene alpha; `asTail` = float(as - (double)pi),
// precomputed once per pair for the scalar tail. smax = float(A-1) / M_2PI.
SM_HD uint32_t vote_bin(bool block, float am, float as, float asTail, float smax) {
    float v;
    if (block) {
        const float vs = as - kPiF;
        v              = am - vs;
        if (v > k2PiF)
            v = v - k2PiF;
        if (v < 0.0f)
            v = v + k2PiF;
    } else {
        v = am - asTail;
        if (v < 0.0f)
            v = v + k2PiF;
        if (v > k2PiF)
            v = v - k2PiF;
    }
    return (uint32_t)ffloor(smax * v);
}

SM_HD float alpha_tail_shift(float as) { return (float)((double)as - kPiD); }

// Pose rotation angle for candidate bin j (ppf.cpp:402): float(M_2PI*j/(A-1)) - (double)pi.
SM_HD float candidate_angle(int j, int maxAngleIndex) {
    return (float)((double)fdiv(k2PiF * (float)j, (float)maxAngleIndex) - kPiD);
}

// nanoflann L2 metric for DIM = 3 (nanoflann.hpp:545-579): ((d0^2 + d1^2) + d2^2), d = q - p.
SM_HD float dist2(float qx, float qy, float qz, float px, float py, float pz) {
    const float d0 = qx - px, d1 = qy - py, d2 = qz - pz;
    return (d0 * d0 + d1 * d1) + d2 * d2;
}

} // namespace smm
