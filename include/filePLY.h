/*
 * filePLY.h - PLY point-cloud / mesh files for ppf::PointCloud (the reference's filePLY.h:6-9:
 * readPLY, writePLY), header-only, written from the PLY format description (Turk, "The PLY
 * Polygon File Format"): ASCII and binary (either byte order) files, any scalar property
 * type, list properties. readPLY takes the vertex element's x, y, z (and nx, ny, nz when all
 * three are present) and the face element's vertex_indices / vertex_index lists; polygons
 * with more than three corners are cut into triangles by ear clipping (a corner is an ear
 * when it is convex about the polygon's normal and no other corner lies in its triangle,
 * seen along z), as the reference does (filePLY.cpp:44-98). Every other element and
 * property is skipped. Like the reference, failures print a message and return false.
 * writePLY writes float x, y, z (+ nx, ny, nz) and uchar/uint triangle lists, binary
 * little-endian unless write_ascii.
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "ppf.h"

namespace ppf {
namespace ply_detail {

enum class Fmt { Ascii, LittleEndian, BigEndian };

struct Property {
    std::string name;
    std::string type;      // scalar type (the list's item type for lists)
    std::string countType; // list count type, empty for scalars
};

struct Element {
    std::string           name;
    long long             count = 0;
    std::vector<Property> props;
};

inline int type_size(const std::string &t) {
    if (t == "char" || t == "uchar" || t == "int8" || t == "uint8")
        return 1;
    if (t == "short" || t == "ushort" || t == "int16" || t == "uint16")
        return 2;
    if (t == "int" || t == "uint" || t == "int32" || t == "uint32" || t == "float" ||
        t == "float32")
        return 4;
    if (t == "double" || t == "float64")
        return 8;
    return 0;
}

inline bool host_little_endian() {
    const uint16_t one = 1;
    unsigned char  b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// One binary scalar of type t from `in` as a double (byte order swapped when needed).
inline bool read_binary(std::istream &in, const std::string &t, bool swap, double &out) {
    const int     n = type_size(t);
    unsigned char b[8];
    if (n == 0 || !in.read(reinterpret_cast<char *>(b), n))
        return false;
    if (swap)
        for (int i = 0; i < n / 2; i++) {
            const unsigned char x = b[i];
            b[i]                  = b[n - 1 - i];
            b[n - 1 - i]          = x;
        }
    if (t == "char" || t == "int8") {
        int8_t v;
        std::memcpy(&v, b, 1);
        out = v;
    } else if (t == "uchar" || t == "uint8") {
        out = b[0];
    } else if (t == "short" || t == "int16") {
        int16_t v;
        std::memcpy(&v, b, 2);
        out = v;
    } else if (t == "ushort" || t == "uint16") {
        uint16_t v;
        std::memcpy(&v, b, 2);
        out = v;
    } else if (t == "int" || t == "int32") {
        int32_t v;
        std::memcpy(&v, b, 4);
        out = v;
    } else if (t == "uint" || t == "uint32") {
        uint32_t v;
        std::memcpy(&v, b, 4);
        out = v;
    } else if (t == "float" || t == "float32") {
        float v;
        std::memcpy(&v, b, 4);
        out = v;
    } else {
        double v;
        std::memcpy(&v, b, 8);
        out = v;
    }
    return true;
}

// Even-odd crossing test of (x, y) against the triangle a, b, c seen along z.
inline bool inside_xy(const Vec3f &a, const Vec3f &b, const Vec3f &c, double x, double y) {
    const Vec3f *v[3] = {&a, &b, &c};
    bool         in   = false;
    for (int i = 0; i < 3; i++) {
        const Vec3f &p = *v[i], &q = *v[(i + 1) % 3];
        const double py = p[1], qy = q[1];
        if ((py <= y && qy > y) || (qy <= y && py > y)) {
            const double cx = (double)(q[0] - p[0]) * (y - py) / (qy - py) + p[0];
            if (cx < x)
                in = !in;
        }
    }
    return in;
}

inline Vec3f sub3(const Vec3f &a, const Vec3f &b) { return Vec3f(a[0] - b[0], a[1] - b[1], a[2] - b[2]); }
inline Vec3f cross3(const Vec3f &a, const Vec3f &b) {
    return Vec3f(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]);
}
inline float dot3(const Vec3f &a, const Vec3f &b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Triangles of polygon `idx` (corners in order) appended to `faces`; false when no ear is
// left before three corners remain.
inline bool triangulate(const std::vector<Vec3f> &pts, std::vector<int> idx,
                        std::vector<Vec3i> &faces) {
    for (int i : idx)
        if (i < 0 || (size_t)i >= pts.size())
            return false;
    int   n = (int)idx.size();
    Vec3f nrm(0, 0, 0);
    if (n > 3) {
        for (int i = 0; i < n; i++) {
            const Vec3f c = cross3(sub3(pts[idx[(i + 1) % n]], pts[idx[i]]),
                                   sub3(pts[idx[(i + 2) % n]], pts[idx[(i + 1) % n]]));
            nrm           = Vec3f(nrm[0] + c[0], nrm[1] + c[1], nrm[2] + c[2]);
        }
        const float l = std::sqrt(dot3(nrm, nrm));
        nrm           = Vec3f(nrm[0] / l, nrm[1] / l, nrm[2] / l);
    }
    while (n > 3) {
        bool cut = false;
        for (int i = 1; i < n - 1 && !cut; i++) {
            const Vec3f &a = pts[idx[i - 1]], &b = pts[idx[i]], &c = pts[idx[i + 1]];
            if (!(dot3(nrm, cross3(sub3(b, a), sub3(c, b))) > 0.0f))
                continue;
            bool ear = true;
            for (int j = 0; j < n && ear; j++) {
                if (j >= i - 1 && j <= i + 1)
                    continue;
                ear = !inside_xy(a, b, c, pts[idx[j]][0], pts[idx[j]][1]);
            }
            if (ear) {
                faces.push_back(Vec3i(idx[i - 1], idx[i], idx[i + 1]));
                idx.erase(idx.begin() + i);
                n--;
                cut = true;
            }
        }
        if (!cut)
            return false;
    }
    if (n == 3)
        faces.push_back(Vec3i(idx[0], idx[1], idx[2]));
    return true;
}

inline bool fail(const std::string &msg) {
    std::cout << "Read PLY failed: " << msg << std::endl;
    return false;
}

} // namespace ply_detail

inline bool readPLY(const std::string &filename, PointCloud &mesh) {
    using namespace ply_detail;
    std::ifstream in(filename, std::ios::binary);
    if (!in)
        return fail("unable to open file: " + filename);
    std::string line;
    if (!std::getline(in, line) || line.compare(0, 3, "ply") != 0)
        return fail("unable to parse header.");
    Fmt                  fmt = Fmt::Ascii;
    std::vector<Element> elems;
    bool                 ended = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        std::istringstream ls(line);
        std::string        kw;
        ls >> kw;
        if (kw == "format") {
            std::string f;
            ls >> f;
            if (f == "ascii")
                fmt = Fmt::Ascii;
            else if (f == "binary_little_endian")
                fmt = Fmt::LittleEndian;
            else if (f == "binary_big_endian")
                fmt = Fmt::BigEndian;
            else
                return fail("unable to parse header.");
        } else if (kw == "element") {
            Element e;
            ls >> e.name >> e.count;
            if (!ls || e.count < 0)
                return fail("unable to parse header.");
            elems.push_back(e);
        } else if (kw == "property") {
            if (elems.empty())
                return fail("unable to parse header.");
            Property    p;
            std::string t;
            ls >> t;
            if (t == "list")
                ls >> p.countType >> p.type >> p.name;
            else {
                p.type = t;
                ls >> p.name;
            }
            if (!ls || type_size(p.type) == 0 ||
                (!p.countType.empty() && type_size(p.countType) == 0))
                return fail("unable to parse header.");
            elems.back().props.push_back(p);
        } else if (kw == "end_header") {
            ended = true;
            break;
        }
    }
    if (!ended)
        return fail("unable to parse header.");
    const bool swap = fmt != Fmt::Ascii && ((fmt == Fmt::LittleEndian) != host_little_endian());
    long long  nv   = 0;
    for (const Element &e : elems)
        if (e.name == "vertex")
            nv = e.count;
    if (nv <= 0)
        return fail("number of vertex <= 0.");
    mesh.point.assign((size_t)nv, Vec3f(0, 0, 0));
    mesh.normal.clear();
    mesh.face.clear();
    auto read_value = [&](const std::string &t, double &v) {
        if (fmt == Fmt::Ascii)
            return (bool)(in >> v);
        return read_binary(in, t, swap, v);
    };
    for (const Element &e : elems) {
        int ix[6] = {-1, -1, -1, -1, -1, -1}, face = -1;
        for (int k = 0; k < (int)e.props.size(); k++) {
            const Property &p     = e.props[k];
            const char     *nm[6] = {"x", "y", "z", "nx", "ny", "nz"};
            if (e.name == "vertex" && p.countType.empty())
                for (int a = 0; a < 6; a++)
                    if (p.name == nm[a])
                        ix[a] = k;
            if (e.name == "face" && !p.countType.empty() &&
                (p.name == "vertex_indices" || p.name == "vertex_index") && face < 0)
                face = k;
        }
        const bool hasN = e.name == "vertex" && ix[3] >= 0 && ix[4] >= 0 && ix[5] >= 0;
        if (hasN)
            mesh.normal.assign((size_t)nv, Vec3f(0, 0, 0));
        std::vector<double> vals(e.props.size());
        std::vector<int>    poly;
        for (long long r = 0; r < e.count; r++) {
            for (int k = 0; k < (int)e.props.size(); k++) {
                const Property &p = e.props[k];
                if (p.countType.empty()) {
                    if (!read_value(p.type, vals[k]))
                        return fail("unable to read file: " + filename);
                    continue;
                }
                double cnt;
                if (!read_value(p.countType, cnt) || cnt < 0)
                    return fail("unable to read file: " + filename);
                if (k == face)
                    poly.assign((size_t)cnt, 0);
                for (long long j = 0; j < (long long)cnt; j++) {
                    double v;
                    if (!read_value(p.type, v))
                        return fail("unable to read file: " + filename);
                    if (k == face)
                        poly[(size_t)j] = (int)v;
                }
            }
            if (e.name == "vertex") {
                for (int a = 0; a < 3; a++)
                    mesh.point[(size_t)r][a] = ix[a] >= 0 ? (float)vals[ix[a]] : 0.0f;
                if (hasN)
                    for (int a = 0; a < 3; a++)
                        mesh.normal[(size_t)r][a] = (float)vals[ix[3 + a]];
            } else if (face >= 0 && !triangulate(mesh.point, poly, mesh.face)) {
                return fail("A polygon in the mesh could not be decomposed into triangles.");
            }
        }
    }
    return true;
}

inline bool writePLY(const std::string &filename, const PointCloud &mesh,
                     bool write_ascii = false) {
    if (mesh.empty()) {
        std::cout << "Write PLY failed: mesh has 0 vertices." << std::endl;
        return false;
    }
    std::ofstream out(filename, std::ios::binary);
    if (!out) {
        std::cout << "Write PLY failed: unable to open file: " << filename << std::endl;
        return false;
    }
    const bool normals = mesh.hasNormal();
    out << "ply\nformat " << (write_ascii ? "ascii" : "binary_little_endian") << " 1.0\n"
        << "element vertex " << mesh.point.size() << "\n"
        << "property float x\nproperty float y\nproperty float z\n";
    if (normals)
        out << "property float nx\nproperty float ny\nproperty float nz\n";
    out << "element face " << mesh.face.size() << "\n"
        << "property list uchar uint vertex_indices\nend_header\n";
    const bool swap = !ply_detail::host_little_endian();
    auto put = [&](const void *p, int n) {
        unsigned char b[4];
        std::memcpy(b, p, n);
        if (swap)
            for (int i = 0; i < n / 2; i++) {
                const unsigned char x = b[i];
                b[i]                  = b[n - 1 - i];
                b[n - 1 - i]          = x;
            }
        out.write(reinterpret_cast<const char *>(b), n);
    };
    for (size_t i = 0; i < mesh.point.size(); i++) {
        float v[6] = {mesh.point[i][0], mesh.point[i][1], mesh.point[i][2], 0, 0, 0};
        if (normals)
            for (int a = 0; a < 3; a++)
                v[3 + a] = mesh.normal[i][a];
        const int nv = normals ? 6 : 3;
        if (write_ascii) {
            for (int a = 0; a < nv; a++) {
                char buf[32];
                std::snprintf(buf, sizeof buf, "%.9g", v[a]);
                out << buf << (a + 1 < nv ? " " : "\n");
            }
        } else {
            for (int a = 0; a < nv; a++)
                put(&v[a], 4);
        }
    }
    for (size_t i = 0; i < mesh.face.size(); i++) {
        const uint32_t f[3] = {(uint32_t)mesh.face[i][0], (uint32_t)mesh.face[i][1],
                               (uint32_t)mesh.face[i][2]};
        if (write_ascii) {
            out << "3 " << f[0] << " " << f[1] << " " << f[2] << "\n";
        } else {
            const unsigned char three = 3;
            put(&three, 1);
            for (int a = 0; a < 3; a++)
                put(&f[a], 4);
        }
    }
    return (bool)out;
}

} // namespace ppf
