/*
 * util.h - the reference's public point-cloud helpers (util.h:8-21), header-only over
 * ppf::PointCloud: sampleMesh (area-weighted surface samples of a triangle mesh,
 * util.cpp:20-84), removeNan (util.cpp:86-105), extraIndices (util.cpp:141-161),
 * normalizeNormal (util.cpp:163-176), computeBoundingBox (util.cpp:178-207) and
 * transformPointCloud (util.cpp:209-232), with the same signatures and results.
 * sampleMesh draws from a generator seeded by std::random_device, as the reference does;
 * the overload with a seed makes a draw repeatable.
 */
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <random>
#include <vector>

#include "ppf.h"

namespace ppf {
namespace util_detail {

inline Vec3f v3(float x, float y, float z) { return Vec3f(x, y, z); }
inline Vec3f sub(const Vec3f &a, const Vec3f &b) { return v3(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline Vec3f cross(const Vec3f &a, const Vec3f &b) {
    return v3(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline float norm(const Vec3f &a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }
// a / |a|, and a itself when |a| = 0 (Eigen's normalized())
inline Vec3f normalized(const Vec3f &a) {
    const float n = norm(a);
    return n > 0.0f ? v3(a[0] / n, a[1] / n, a[2] / n) : a;
}
inline bool finite(const Vec3f &a) {
    return std::isfinite(a[0]) && std::isfinite(a[1]) && std::isfinite(a[2]);
}

} // namespace util_detail

// Points spread over the triangles in proportion to their areas, about one per radius^2 of
// surface: triangle i takes the points up to round(cumulative area share x count), each at
// uniform barycentric coordinates (a, b, c) = (1 - sqrt r1, sqrt r1 (1 - r2), sqrt r1 r2),
// with the triangle's unit normal. An empty mesh gives an empty cloud.
inline PointCloud sampleMesh(const PointCloud &pc, float radius, uint32_t seed) {
    using namespace util_detail;
    if (pc.face.empty())
        return {};
    const std::size_t  nt = pc.face.size();
    std::vector<float> cdf(nt);
    std::vector<Vec3f> nrm(nt);
    float              area = 0.0f;
    for (std::size_t i = 0; i < nt; i++) {
        const Vec3f &p0 = pc.point[pc.face[i][0]], &p1 = pc.point[pc.face[i][1]],
                    &p2 = pc.point[pc.face[i][2]];
        const Vec3f  k  = cross(sub(p1, p0), sub(p2, p0));
        cdf[i]          = norm(k) / 2.0f;
        nrm[i]          = normalized(k);
        area += cdf[i];
    }
    cdf[0] = cdf[0] / area;
    for (std::size_t i = 1; i < nt; i++)
        cdf[i] = cdf[i] / area + cdf[i - 1];
    cdf[nt - 1]        = 1.0f;
    const int     npts = (int)(area / (radius * radius));
    std::mt19937  mt(seed);
    std::uniform_real_distribution<float> u(0.0f, 1.0f);
    PointCloud    out;
    out.point.resize(npts > 0 ? npts : 0);
    out.normal.resize(out.point.size());
    std::size_t k = 0;
    for (std::size_t i = 0; i < nt; i++) {
        const std::size_t end = (std::size_t)std::round(cdf[i] * npts);
        const Vec3f &p0 = pc.point[pc.face[i][0]], &p1 = pc.point[pc.face[i][1]],
                    &p2 = pc.point[pc.face[i][2]];
        while (k < end && k < out.point.size()) {
            const float  r1 = u(mt), r2 = u(mt);
            const double s  = std::sqrt((double)r1);
            const double a = 1.0 - s, b = s * (1.0 - r2), c = s * r2;
            out.point[k]   = v3((float)(a * p0[0] + b * p1[0] + c * p2[0]),
                                (float)(a * p0[1] + b * p1[1] + c * p2[1]),
                                (float)(a * p0[2] + b * p1[2] + c * p2[2]));
            out.normal[k]  = nrm[i];
            k++;
        }
    }
    out.box = pc.box;
    return out;
}

inline PointCloud sampleMesh(const PointCloud &pc, float radius) {
    std::random_device rd;
    return sampleMesh(pc, radius, (uint32_t)rd());
}

// Indices of the points with finite coordinates (and finite normals when checkNormal and
// the cloud has normals), ascending.
inline std::vector<int> removeNan(const PointCloud &pc, bool checkNormal = false) {
    const bool       cn = checkNormal && pc.hasNormal();
    std::vector<int> keep;
    keep.reserve(pc.size());
    for (std::size_t i = 0; i < pc.size(); i++)
        if (util_detail::finite(pc.point[i]) && (!cn || util_detail::finite(pc.normal[i])))
            keep.push_back((int)i);
    return keep;
}

// The bounding box of all points, or of the points validIndices names.
inline BoundingBox computeBoundingBox(const PointCloud &pc, const std::vector<int> &validIndices = {}) {
    Vec3f mn = validIndices.empty() ? pc.point[0] : pc.point[validIndices[0]];
    Vec3f mx = mn;
    auto  fold = [&](const Vec3f &p) {
        for (int d = 0; d < 3; d++) {
            if (p[d] > mx[d])
                mx[d] = p[d];
            else if (p[d] < mn[d])
                mn[d] = p[d];
        }
    };
    if (validIndices.empty())
        for (const Vec3f &p : pc.point)
            fold(p);
    else
        for (int i : validIndices)
            fold(pc.point[i]);
    return BoundingBox(mn, mx);
}

// The points `indices` names (unit normals when the cloud has normals), keeping the box
// unless it is empty.
inline PointCloud extraIndices(const PointCloud &pc, const std::vector<std::size_t> &indices) {
    PointCloud out;
    const bool hasN = pc.hasNormal();
    out.point.resize(indices.size());
    if (hasN)
        out.normal.resize(indices.size());
    for (std::size_t i = 0; i < indices.size(); i++) {
        out.point[i] = pc.point[indices[i]];
        if (hasN)
            out.normal[i] = util_detail::normalized(pc.normal[indices[i]]);
    }
    out.box = pc.box;
    if (out.box.diameter() == 0 && !out.point.empty())
        out.box = computeBoundingBox(out);
    return out;
}

// Unit normals, reversed when invert.
inline void normalizeNormal(PointCloud &pc, bool invert = false) {
    for (Vec3f &n : pc.normal) {
        const Vec3f u = util_detail::normalized(n);
        n             = invert ? util_detail::v3(-u[0], -u[1], -u[2]) : u;
    }
}

// R p + t for every point (R n for the normals when useNormal and present), the triangles
// kept, the box recomputed.
inline PointCloud transformPointCloud(const PointCloud &pc, const Mat4f &pose, bool useNormal = true) {
    PointCloud out;
    const bool doN = pc.hasNormal() && useNormal;
    out.point.resize(pc.size());
    if (doN)
        out.normal.resize(pc.size());
    auto rot = [&](const Vec3f &v, bool translate) {
        float r[3];
        for (int i = 0; i < 3; i++)
            r[i] = pose(i, 0) * v[0] + pose(i, 1) * v[1] + pose(i, 2) * v[2] +
                   (translate ? pose(i, 3) : 0.0f);
        return util_detail::v3(r[0], r[1], r[2]);
    };
    for (std::size_t i = 0; i < pc.size(); i++) {
        out.point[i] = rot(pc.point[i], true);
        if (doN)
            out.normal[i] = rot(pc.normal[i], false);
    }
    out.face = pc.face;
    if (!out.point.empty())
        out.box = computeBoundingBox(out);
    return out;
}

} // namespace ppf
