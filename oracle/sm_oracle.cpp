// oracle/sm_oracle.cpp - TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's ppf::Detector::trainModel / matchScene hot path
// (ppf.cpp:36-147, 149-510; util.cpp; icp.cpp). It is the checker for the GPU library and
// the timed CPU baseline; the product never links, loads or calls it.
//
// Two search-order modes share one pipeline:
//   ORC_MODE_REF  - the reference's orders: k-d tree (oracle/kdtree.h, a restatement of
//                   the vendored nanoflann) for greedy sampling order, radius-search
//                   neighbour order (decides the SIMD/tail lane rule of every pair) and
//                   nearest-neighbour tie-breaking.
//   ORC_MODE_GRID - the GPU's orders: 8-phase grid greedy sampling (sm_grid.h), neighbour
//                   lists by ascending point index, exact (distance, index) tie-breaking.
// Everything else is the same code in both modes. The float arithmetic of keys, alpha
// angles, vote bins, normals, clustering and ICP comes from the headers the kernels use
// (sm_math.h, sm_linalg.h, sm_icp.h, sm_grid.h), so GRID mode is bit-identical to the GPU.
//
// Deterministic resolutions of the reference's order-dependent or racy parts (the
// reference is run single-threaded for parity; these choices are shared with the GPU):
//   H3 normals: two-phase estimation (all neighbourhoods from the positions at the start
//      of the call, then smoothing with raw normals), instead of in-place updates whose
//      result depends on visiting order (util.cpp:269, 292-306).
//   H4 sorts: stable sorts (votes desc, then list order) where the reference uses
//      std::sort (util.cpp:487, ppf.cpp:498); pose list in keypoint order (the reference
//      appends under omp critical, ppf.cpp:407).
//   Accumulations: centroid/covariance in FP32 Kahan per point; ICP sums in FP32 Kahan over
//      smi::kIcpSlots strided partials merged by a fixed tree (the GPU's layout, sm_icp.h).
//      ORC_PREC_FP64 runs the same pipeline with FP64 accumulation (the precision reference).
#include "../surface_match_gb300/csrc/sm_grid.h"
#include "../surface_match_gb300/csrc/sm_icp.h"
#include "../surface_match_gb300/csrc/sm_linalg.h"
#include "../surface_match_gb300/csrc/sm_math.h"
#include "kdtree.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using orc::V3;

namespace {

enum { ORC_MODE_REF = 0, ORC_MODE_GRID = 1 };

thread_local std::string g_err;

bool finite3(const V3 &v) { return std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z); }

// Eigen 3-vector norm order: x*x + (y*y + z*z).
float norm3(float x, float y, float z) { return smm::fsqrt(x * x + (y * y + z * z)); }

V3 normalized(const V3 &n) {
    float sq = n.x * n.x + (n.y * n.y + n.z * n.z);
    if (sq > 0.0f) {
        float s = smm::fsqrt(sq);
        return {n.x / s, n.y / s, n.z / s};
    }
    return n;
}

struct Box {
    V3 mn{0, 0, 0}, mx{0, 0, 0};
    float diameter() const { return norm3(mx.x - mn.x, mx.y - mn.y, mx.z - mn.z); }
    V3    center() const { return {(mn.x + mx.x) / 2.f, (mn.y + mx.y) / 2.f, (mn.z + mx.z) / 2.f}; }
};

// computeBoundingBox (util.cpp:178-207) over the valid points.
Box bbox_of(const std::vector<V3> &p, const std::vector<int> &valid) {
    Box b;
    if (valid.empty())
        return b;
    b.mn = b.mx = p[valid[0]];
    for (int idx : valid) {
        const V3 &q = p[idx];
        if (q.x > b.mx.x) b.mx.x = q.x; else if (q.x < b.mn.x) b.mn.x = q.x;
        if (q.y > b.mx.y) b.mx.y = q.y; else if (q.y < b.mn.y) b.mn.y = q.y;
        if (q.z > b.mx.z) b.mx.z = q.z; else if (q.z < b.mn.z) b.mn.z = q.z;
    }
    return b;
}

// ---------------------------------------------------------------------------------------
// Exact grid searches (GRID mode): results are the (squared distance, index)-smallest
// points, so they do not depend on the order in which cells are visited.
// ---------------------------------------------------------------------------------------
struct Grid {
    float              org[3], g;
    int                dim[3];
    std::vector<int>   start; // per cell, CSR into ids
    std::vector<int>   ids;   // point ids, cell-major, ascending inside a cell
    const std::vector<V3> *pts = nullptr;

    void build(const std::vector<V3> &P, const std::vector<int> &sub, const Box &box, float cell) {
        pts    = &P;
        org[0] = box.mn.x;
        org[1] = box.mn.y;
        org[2] = box.mn.z;
        float ext[3] = {box.mx.x - box.mn.x, box.mx.y - box.mn.y, box.mx.z - box.mn.z};
        g            = cell;
        for (int a = 0; a < 3; a++)
            dim[a] = smg::dim_of(ext[a], g);
        long long nc = (long long)dim[0] * dim[1] * dim[2];
        start.assign(nc + 1, 0);
        std::vector<int> cellOf(sub.size());
        for (size_t i = 0; i < sub.size(); i++) {
            cellOf[i] = cell_index(P[sub[i]]);
            start[cellOf[i] + 1]++;
        }
        for (long long c = 0; c < nc; c++)
            start[c + 1] += start[c];
        ids.resize(sub.size());
        std::vector<int> fill(start.begin(), start.end() - 1);
        std::vector<int> order(sub.size());
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return sub[a] < sub[b]; });
        for (int o : order)
            ids[fill[cellOf[o]]++] = sub[o];
    }
    void cc(const V3 &p, int c[3]) const {
        c[0] = smg::coord(p.x, org[0], g, dim[0]);
        c[1] = smg::coord(p.y, org[1], g, dim[1]);
        c[2] = smg::coord(p.z, org[2], g, dim[2]);
    }
    int cell_index(const V3 &p) const {
        int c[3];
        cc(p, c);
        return (c[2] * dim[1] + c[1]) * dim[0] + c[0];
    }
    // visit all cells at Chebyshev distance exactly s from c (clipped to the grid)
    template <class F> void shell(const int c[3], int s, F &&f) const {
        for (int z = c[2] - s; z <= c[2] + s; z++) {
            if (z < 0 || z >= dim[2]) continue;
            for (int y = c[1] - s; y <= c[1] + s; y++) {
                if (y < 0 || y >= dim[1]) continue;
                bool edgeYZ = (z == c[2] - s || z == c[2] + s || y == c[1] - s || y == c[1] + s);
                for (int x = c[0] - s; x <= c[0] + s; x++) {
                    if (x < 0 || x >= dim[0]) continue;
                    if (!edgeYZ && x != c[0] - s && x != c[0] + s) continue;
                    int cell = (z * dim[1] + y) * dim[0] + x;
                    for (int k = start[cell]; k < start[cell + 1]; k++)
                        f(ids[k]);
                }
            }
        }
    }
    int max_shell(const int c[3]) const {
        int m = 0;
        for (int a = 0; a < 3; a++)
            m = std::max(m, std::max(c[a], dim[a] - 1 - c[a]));
        return m;
    }
    // k nearest by (d2, id); returns count (<= k)
    int knn(const V3 &q, int k, int *oi, float *od) const {
        int c[3];
        cc(q, c);
        int   n = 0;
        int   ms = max_shell(c);
        for (int s = 0; s <= ms; s++) {
            shell(c, s, [&](int id) {
                const V3 &p = (*pts)[id];
                float     d = smm::dist2(q.x, q.y, q.z, p.x, p.y, p.z);
                if (n == k && !(d < od[k - 1] || (d == od[k - 1] && id < oi[k - 1])))
                    return;
                int i = (n < k) ? n++ : k - 1;
                while (i > 0 && (od[i - 1] > d || (od[i - 1] == d && oi[i - 1] > id))) {
                    od[i] = od[i - 1];
                    oi[i] = oi[i - 1];
                    i--;
                }
                od[i] = d;
                oi[i] = id;
            });
            float b = smg::ring_bound(s, g);
            if (n == k && od[k - 1] < b * b)
                break;
        }
        return n;
    }
    // nearest within squared radius limit (limit = +inf for unbounded); -1 if none
    int nn(const V3 &q, float limit2, float &outd) const {
        int c[3];
        cc(q, c);
        int   best = -1;
        float bd   = FLT_MAX;
        int   ms   = max_shell(c);
        for (int s = 0; s <= ms; s++) {
            shell(c, s, [&](int id) {
                const V3 &p = (*pts)[id];
                float     d = smm::dist2(q.x, q.y, q.z, p.x, p.y, p.z);
                if (d < bd || (d == bd && id < best)) {
                    bd   = d;
                    best = id;
                }
            });
            float b = smg::ring_bound(s, g);
            if (best >= 0 && bd < b * b)
                break;
            if (b * b > limit2)
                break;
        }
        outd = bd;
        return best;
    }
    bool any_within(const V3 &q, float r2) const {
        int c[3];
        cc(q, c);
        int  ms = max_shell(c);
        bool hit = false;
        for (int s = 0; s <= ms && !hit; s++) {
            shell(c, s, [&](int id) {
                if (hit) return;
                const V3 &p = (*pts)[id];
                if (smm::dist2(q.x, q.y, q.z, p.x, p.y, p.z) < r2) hit = true;
            });
            float b = smg::ring_bound(s, g);
            if (b * b >= r2)
                break;
        }
        return hit;
    }
};

// 8-phase grid greedy thinning over `sub` (any order); returns kept ids ascending. Cells of
// side smg::thin_cell are held sparse (only occupied cells), as the GPU's hashed grid: a
// point is kept unless a kept point of its 3x3x3 cell block lies within the step, visiting
// phase by phase, cell by cell (cells of one phase do not interact) and by ascending index.
std::vector<int> grid_sample(const std::vector<V3> &P, const std::vector<int> &sub,
                             const Box &box, float step) {
    if (!(step > 0.0f)) { // nothing lies at a squared distance below zero: all kept
        std::vector<int> out(sub);
        std::sort(out.begin(), out.end());
        return out;
    }
    float       ext[3] = {box.mx.x - box.mn.x, box.mx.y - box.mn.y, box.mx.z - box.mn.z};
    const float g      = smg::thin_cell(step, ext);
    int         dim[3];
    for (int a = 0; a < 3; a++)
        dim[a] = smg::dim_of(ext[a], g);
    auto key_of = [&](int x, int y, int z) {
        return ((uint64_t)z * (uint64_t)dim[1] + (uint64_t)y) * (uint64_t)dim[0] + (uint64_t)x;
    };
    // points by (cell key, id)
    std::vector<std::pair<uint64_t, int>> pk(sub.size());
    for (size_t i = 0; i < sub.size(); i++) {
        const V3 &p = P[sub[i]];
        pk[i]       = {key_of(smg::coord(p.x, box.mn.x, g, dim[0]), smg::coord(p.y, box.mn.y, g, dim[1]),
                        smg::coord(p.z, box.mn.z, g, dim[2])),
                 sub[i]};
    }
    std::sort(pk.begin(), pk.end());
    std::vector<uint64_t>            cellKey;
    std::vector<std::pair<int, int>> range;
    std::unordered_map<uint64_t, int> cellOf;
    for (size_t i = 0; i < pk.size();) {
        size_t j = i;
        while (j < pk.size() && pk[j].first == pk[i].first)
            j++;
        cellOf[pk[i].first] = (int)range.size();
        range.push_back({(int)i, (int)j});
        cellKey.push_back(pk[i].first);
        i = j;
    }
    const float                   r2 = step * step;
    std::vector<char>             kept(P.size(), 0);
    std::vector<std::vector<int>> keptIn(range.size());
    const uint64_t                xy = (uint64_t)dim[0] * (uint64_t)dim[1];
    for (int phase = 0; phase < 8; phase++) {
        for (size_t ci = 0; ci < range.size(); ci++) {
            const uint64_t key = cellKey[ci];
            const int      x = (int)(key % (uint64_t)dim[0]), y = (int)((key / (uint64_t)dim[0]) % (uint64_t)dim[1]);
            const int      z = (int)(key / xy);
            if (smg::phase_of(x, y, z) != phase) continue;
            for (int k = range[ci].first; k < range[ci].second; k++) {
                const int id = pk[k].second;
                const V3 &q  = P[id];
                bool      ok = true;
                for (int dz = -1; dz <= 1 && ok; dz++)
                    for (int dy = -1; dy <= 1 && ok; dy++)
                        for (int dx = -1; dx <= 1 && ok; dx++) {
                            const int xx = x + dx, yy = y + dy, zz = z + dz;
                            if (xx < 0 || yy < 0 || zz < 0 || xx >= dim[0] || yy >= dim[1] ||
                                zz >= dim[2])
                                continue;
                            const auto it = cellOf.find(key_of(xx, yy, zz));
                            if (it == cellOf.end()) continue;
                            for (int o : keptIn[it->second]) {
                                const V3 &p = P[o];
                                if (smm::dist2(p.x, p.y, p.z, q.x, q.y, q.z) < r2) {
                                    ok = false;
                                    break;
                                }
                            }
                        }
                if (ok) {
                    kept[id] = 1;
                    keptIn[ci].push_back(id);
                }
            }
        }
    }
    std::vector<int> out;
    for (int id : sub)
        if (kept[id]) out.push_back(id);
    std::sort(out.begin(), out.end());
    return out;
}

// samplePointCloud (util.cpp:107-139), single-threaded: greedy in tree leaf order.
std::vector<int> kd_sample(const orc::KdTree &tree, float step, std::vector<int> *ioi) {
    size_t            size = tree.vAcc.size();
    std::vector<char> keep(tree.data->size(), 1);
    float             r2 = step * step;
    std::vector<int>  result;
    if (ioi) ioi->assign(size, -1);
    std::vector<std::pair<int, float>> found;
    for (size_t i = 0; i < size; i++) {
        int index = tree.vAcc[i];
        if (index == -1 || !keep[index]) continue;
        result.push_back(index);
        if (ioi) (*ioi)[i] = index;
        const V3 &p    = (*tree.data)[index];
        float     q[3] = {p.x, p.y, p.z};
        tree.radiusSearch(q, r2, found);
        for (auto &f : found) keep[f.first] = 0;
    }
    return result;
}

// ---------------------------------------------------------------------------------------
// Model / scene state
// ---------------------------------------------------------------------------------------
struct TrainParam {
    float featDistanceStepRel        = 0.04f;
    int   featAngleResolution        = 30;
    float poseRefRelSamplingDistance = 0.01f;
    int   knnNormal                  = 10;
    int   smoothNormal               = 1;
};

struct MatchParam {
    int   numMatches              = 1;
    int   knnNormal               = 10;
    int   smoothNormal            = 1;
    int   invertNormal            = 0;
    float maxOverlapDistRel       = 0.5f;
    float maxOverlapDistAbs       = 0.0f;
    int   sparsePoseRefinement    = 1;
    int   densePoseRefinement     = 1;
    int   poseRefNumSteps         = 5;
    float poseRefDistThresholdRel = 0.1f;
    float poseRefDistThresholdAbs = 0.0f;
    float poseRefScoringDistRel   = 0.01f;
    float poseRefScoringDistAbs   = 0.0f;
};

struct Model {
    float                 samplingDistanceRel = 0.04f;
    TrainParam            tp;
    std::vector<V3>       sp, sn, rp, rn; // sampled / resampled points and normals
    Box                   box;
    std::vector<uint32_t> keys;          // ascending
    std::vector<uint32_t> offs;          // keys.size() + 1
    std::vector<uint32_t> refs;          // entries, per bucket in insertion order
    std::vector<float>    alphas;
    std::unordered_map<uint32_t, uint32_t> slot; // key -> bucket
    std::vector<uint32_t> maxMult; // per bucket: most entries of one reference point
};

// Per-bucket multiplicities of the finished table (the GPU keeps them in its table slots).
void finish_table(Model &m) {
    m.maxMult.resize(m.keys.size());
    for (size_t b = 0; b < m.keys.size(); b++)
        m.maxMult[b] = smm::bucket_max_ref_multiplicity(m.refs.data(), m.offs[b], m.offs[b + 1]);
}

// Normal estimation (estimateNormal / computeNormal, util.cpp:234-334) in the two-phase
// form. `knn(q, k, idx, d2)` returns the k nearest points of q in the full cloud, sorted.
template <class KNN>
void estimate_normals(std::vector<V3> &P, std::vector<V3> &N, const std::vector<int> &ids, int k,
                      bool smooth, bool invert, const V3 &vp, bool fp64, int nthreads, KNN &&knn) {
    if (k < 3) k = 3;
    std::vector<int> need;
    std::vector<char> mark(P.size(), 0);
    std::vector<std::vector<int>> nb(P.size());
    // neighbourhoods of the requested points (positions at the start of the call)
    std::vector<int> todo;
    for (int id : ids)
        if (!finite3(N[id])) { todo.push_back(id); mark[id] = 1; }
    std::vector<std::vector<int>> nbTodo(todo.size());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (long t = 0; t < (long)todo.size(); t++) {
        std::vector<int>   oi(k);
        std::vector<float> od(k);
        int                n = knn(P[todo[t]], k, oi.data(), od.data());
        nbTodo[t].assign(oi.begin(), oi.begin() + n);
    }
    for (size_t t = 0; t < todo.size(); t++) nb[todo[t]] = nbTodo[t];
    need = todo;
    if (smooth) {
        for (int id : todo)
            for (int j : nb[id])
                if (!mark[j] && !finite3(N[j])) { mark[j] = 2; need.push_back(j); }
        std::vector<int> extra(need.begin() + todo.size(), need.end());
        std::vector<std::vector<int>> nbExtra(extra.size());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
        for (long t = 0; t < (long)extra.size(); t++) {
            std::vector<int>   oi(k);
            std::vector<float> od(k);
            int                n = knn(P[extra[t]], k, oi.data(), od.data());
            nbExtra[t].assign(oi.begin(), oi.begin() + n);
        }
        for (size_t t = 0; t < extra.size(); t++) nb[extra[t]] = nbExtra[t];
    }
    // phase A: centroid + covariance (FP32 Kahan, or FP64) and PCA normal
    std::vector<V3> cen(need.size()), nrm(need.size());
    std::vector<char> ok(need.size(), 0);
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
    for (long t = 0; t < (long)need.size(); t++) {
        const std::vector<int> &L = nb[need[t]];
        int m = (int)L.size();
        if (m < 3) continue;
        double C[6];
        V3     c;
        if (!fp64) {
            smi::KahanF sx, sy, sz;
            sx.init(); sy.init(); sz.init();
            for (int j : L) { sx.add(P[j].x); sy.add(P[j].y); sz.add(P[j].z); }
            c = {sx.value() / (float)m, sy.value() / (float)m, sz.value() / (float)m};
            smi::KahanF a[6];
            for (auto &e : a) e.init();
            for (int j : L) {
                float dx = P[j].x - c.x, dy = P[j].y - c.y, dz = P[j].z - c.z;
                a[0].add(dx * dx); a[1].add(dx * dy); a[2].add(dx * dz);
                a[3].add(dy * dy); a[4].add(dy * dz); a[5].add(dz * dz);
            }
            for (int e = 0; e < 6; e++) C[e] = (double)a[e].value();
        } else {
            double sx = 0, sy = 0, sz = 0;
            for (int j : L) { sx += P[j].x; sy += P[j].y; sz += P[j].z; }
            double cx = sx / m, cy = sy / m, cz = sz / m;
            for (double &e : C) e = 0;
            for (int j : L) {
                double dx = P[j].x - cx, dy = P[j].y - cy, dz = P[j].z - cz;
                C[0] += dx * dx; C[1] += dx * dy; C[2] += dx * dz;
                C[3] += dy * dy; C[4] += dy * dz; C[5] += dz * dz;
            }
            c = {(float)cx, (float)cy, (float)cz};
        }
        float n3[3];
        sml::normal_from_cov(C, n3);
        cen[t] = c;
        nrm[t] = {n3[0], n3[1], n3[2]};
        ok[t]  = 1;
    }
    for (size_t t = 0; t < need.size(); t++)
        if (ok[t]) { N[need[t]] = nrm[t]; P[need[t]] = cen[t]; }
    // phase B: smoothing with the raw normals of the neighbourhood
    if (smooth) {
        std::vector<V3> sm(todo.size());
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 256)
        for (long t = 0; t < (long)todo.size(); t++) {
            int       id = todo[t];
            const V3 &n0 = N[id];
            float sx = 0, sy = 0, sz = 0;
            for (int j : nb[id]) {
                const V3 &n = N[j];
                float d = n.x * n0.x + (n.y * n0.y + n.z * n0.z);
                if (d > 0) { sx += n.x; sy += n.y; sz += n.z; }
                else { sx -= n.x; sy -= n.y; sz -= n.z; }
            }
            sm[t] = normalized({sx, sy, sz});
        }
        for (size_t t = 0; t < todo.size(); t++)
            if (nb[todo[t]].size() >= 3) N[todo[t]] = sm[t];
    }
    // phase C: orientation of the requested points toward the viewpoint (or +z)
    bool hasVp = finite3(vp);
    for (int id : ids) {
        V3   &n = N[id];
        float d;
        if (hasVp) {
            const V3 &p = P[id];
            float vx = vp.x - p.x, vy = vp.y - p.y, vz = vp.z - p.z;
            d = n.x * vx + (n.y * vy + n.z * vz);
        } else
            d = n.x * 0.0f + (n.y * 0.0f + n.z * 1.0f);
        bool flip = invert ? (d > 0.f) : (d < 0.f);
        if (flip) n = {-n.x, -n.y, -n.z};
    }
}

// Hash-table build of trainModel (ppf.cpp:105-143), single-threaded insertion order.
void build_table(Model &m) {
    const auto &P = m.sp;
    const auto &N = m.sn;
    const size_t Nm = P.size();
    float diam      = m.box.diameter();
    float angleStep = smm::k2PiF / (float)m.tp.featAngleResolution;
    float distStep  = diam * m.tp.featDistanceStepRel;
    size_t vec      = Nm - Nm % smm::kLanes;
    std::unordered_map<uint32_t, std::pair<std::vector<uint32_t>, std::vector<float>>> table;
    std::vector<uint32_t> order;
    for (size_t i = 0; i < Nm; i++) {
        const V3 &p1 = P[i], &n1 = N[i];
        if (!finite3(n1)) continue;
        smm::RT rt = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
        for (size_t j = 0; j < Nm; j++) {
            bool  block = j < vec;
            float a     = smm::alpha_of(block, rt, P[j].x, P[j].y, P[j].z);
            if (i == j || std::isnan(a)) continue;
            uint32_t key = smm::ppf_key(block, p1.x, p1.y, p1.z, n1.x, n1.y, n1.z, P[j].x, P[j].y,
                                        P[j].z, N[j].x, N[j].y, N[j].z, angleStep, distStep);
            auto it = table.find(key);
            if (it == table.end()) {
                order.push_back(key);
                it = table.emplace(key, std::make_pair(std::vector<uint32_t>(), std::vector<float>())).first;
            }
            it->second.first.push_back((uint32_t)i);
            it->second.second.push_back(a);
        }
    }
    std::sort(order.begin(), order.end());
    m.keys = order;
    m.offs.assign(1, 0);
    m.refs.clear();
    m.alphas.clear();
    m.slot.clear();
    for (size_t b = 0; b < order.size(); b++) {
        auto &e = table[order[b]];
        m.refs.insert(m.refs.end(), e.first.begin(), e.first.end());
        m.alphas.insert(m.alphas.end(), e.second.begin(), e.second.end());
        m.offs.push_back((uint32_t)m.refs.size());
        m.slot[order[b]] = (uint32_t)b;
    }
    finish_table(m);
}

Model *train(const float *xyz, const float *nrm, int64_t n, float sdRel, const TrainParam &tp,
             int mode, int nthreads) {
    if (sdRel > 1 || sdRel < 0) { g_err = "Invalid Input: samplingDistanceRel range mismatch in trainModel"; return nullptr; }
    if (n <= 0) { g_err = "Invalid Input: empty model in trainModel"; return nullptr; }
    std::vector<V3> P(n), N;
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    bool hasN = nrm != nullptr;
    if (hasN) {
        N.resize(n);
        for (int64_t i = 0; i < n; i++) N[i] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
    }
    std::vector<int> valid;
    for (int64_t i = 0; i < n; i++)
        if (finite3(P[i]) && (!hasN || finite3(N[i]))) valid.push_back((int)i);
    if (valid.empty()) { g_err = "Invalid Input: empty model in trainModel"; return nullptr; }
    Box   box  = bbox_of(P, valid);
    float diam = box.diameter();
    float sampleStep   = diam * sdRel;
    float reSampleStep = diam * tp.poseRefRelSamplingDistance;
    Model *m = new Model();
    m->samplingDistanceRel = sdRel;
    m->tp = tp;
    m->box = box;
    std::vector<int> idx1, idx2;
    if (!hasN) N.assign(n, V3{NAN, NAN, NAN});
    if (mode == ORC_MODE_REF) {
        orc::KdTree tree(P, valid, box.mn, box.mx);
        idx1 = kd_sample(tree, sampleStep, nullptr);
        idx2 = kd_sample(tree, reSampleStep, nullptr);
        auto knn = [&](const V3 &q, int k, int *oi, float *od) {
            orc::KnnSet<64> rs(k);
            float qq[3] = {q.x, q.y, q.z};
            tree.findNeighbors(rs, qq);
            for (int i = 0; i < k; i++) { oi[i] = rs.idx[i]; od[i] = rs.dist[i]; }
            return rs.count;
        };
        if (!hasN) {
            estimate_normals(P, N, idx1, tp.knnNormal, tp.smoothNormal, false, V3{NAN, NAN, NAN}, false, nthreads, knn);
            estimate_normals(P, N, idx2, tp.knnNormal, tp.smoothNormal, false, V3{NAN, NAN, NAN}, false, nthreads, knn);
        }
    } else {
        idx1 = grid_sample(P, valid, box, sampleStep);
        idx2 = grid_sample(P, valid, box, reSampleStep);
        if (!hasN) {
            float ext[3] = {box.mx.x - box.mn.x, box.mx.y - box.mn.y, box.mx.z - box.mn.z};
            Grid G;
            G.build(P, valid, box, smg::query_cell(sampleStep * 0.25f, ext));
            auto knn = [&](const V3 &q, int k, int *oi, float *od) { return G.knn(q, k, oi, od); };
            estimate_normals(P, N, idx1, tp.knnNormal, tp.smoothNormal, false, V3{NAN, NAN, NAN}, false, nthreads, knn);
            G.build(P, valid, box, smg::query_cell(sampleStep * 0.25f, ext));
            estimate_normals(P, N, idx2, tp.knnNormal, tp.smoothNormal, false, V3{NAN, NAN, NAN}, false, nthreads, knn);
        }
    }
    if (hasN)
        for (auto &v : N) v = normalized(v);
    // extraIndices (util.cpp:141-161): copy and normalise the normals once more
    for (int id : idx1) { m->sp.push_back(P[id]); m->sn.push_back(normalized(N[id])); }
    for (int id : idx2) { m->rp.push_back(P[id]); m->rn.push_back(normalized(N[id])); }
    build_table(*m);
    return m;
}

// ---------------------------------------------------------------------------------------
// Matching
// ---------------------------------------------------------------------------------------
struct PoseRec {
    smi::Pose34 T;
    float       q[4];  // w x y z
    float       angle; // rotation angle in [0, pi]
    float       votes;
};

void pose_update(PoseRec &p) { // Pose::updatePose (type.cpp:53-59)
    float rec[smi::kPoseFloats];
    smi::pose_record(p.T.m, p.votes, rec);
    memcpy(p.q, rec + 12, 16);
    p.angle = rec[16];
}

struct KpOut {
    int      searched = 0, skipped = 1; // skipped: 1 = NaN normal, 2 = below vote threshold
    int64_t  hits = 0, votes = 0, bound = 0; // bound: sum of the hits' bucket multiplicities
    uint64_t accHash = 0;
    int      nc = 0;
    float    cv[3];
    int      cr[3], ca[3];
    int      npose = 0;
    PoseRec  poses[3];
};

// Order-independent accumulator fingerprint: sum over cells of splitmix64(index, count).
uint64_t acc_hash(const std::vector<int> &acc) {
    uint64_t h = 0;
    for (size_t i = 0; i < acc.size(); i++)
        if (acc[i]) h += smm::mix64(((uint64_t)i << 32) | (uint32_t)acc[i]);
    return h;
}

// The per-keypoint body of the voting loop (ppf.cpp:263-409) for neighbour list `nbrs`
// (point ids in search order, self included).
void vote_keypoint(const Model &m, const std::vector<V3> &P, const std::vector<V3> &N, int pid,
                   const std::vector<int> &nbrs, float voteThreshold, std::vector<int> &acc,
                   KpOut &o, std::vector<int> *accOut) {
    const V3 &p1 = P[pid], &n1 = N[pid];
    o.searched = (int)nbrs.size();
    if (!finite3(n1)) { o.skipped = 1; return; }
    if ((float)o.searched < voteThreshold) { o.skipped = 2; return; }
    o.skipped = 0;
    const int   A         = m.tp.featAngleResolution;
    const float diam      = m.box.diameter();
    const float angleStep = smm::k2PiF / (float)A;
    const float distStep  = diam * m.tp.featDistanceStepRel;
    const float smax      = (float)(A - 1) / smm::k2PiF;
    const size_t refNum   = m.sp.size();
    acc.assign(refNum * A, 0);
    std::vector<int> rows;
    rows.reserve(nbrs.size());
    for (int id : nbrs)
        if (id != pid) rows.push_back(id);
    size_t  R   = rows.size();
    size_t  vec = R - R % smm::kLanes;
    smm::RT rt  = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
    for (size_t r = 0; r < R; r++) {
        bool      block = r < vec;
        const V3 &p2 = P[rows[r]], &n2 = N[rows[r]];
        uint32_t  key = smm::ppf_key(block, p1.x, p1.y, p1.z, n1.x, n1.y, n1.z, p2.x, p2.y, p2.z,
                                     n2.x, n2.y, n2.z, angleStep, distStep);
        float as = smm::alpha_of(block, rt, p2.x, p2.y, p2.z);
        auto  it = m.slot.find(key);
        if (it == m.slot.end() || std::isnan(as)) continue;
        uint32_t b0 = m.offs[it->second], b1 = m.offs[it->second + 1];
        uint32_t B = b1 - b0, bvec = B - B % smm::kLanes;
        float asT = smm::alpha_tail_shift(as);
        o.hits++;
        o.votes += B;
        o.bound += m.maxMult[it->second];
        for (uint32_t e = 0; e < B; e++) {
            uint32_t bin = smm::vote_bin(e < bvec, m.alphas[b0 + e], as, asT, smax);
            if (bin > (uint32_t)(A - 1)) bin = A - 1; // unreachable; keeps the index in range
            acc[(size_t)m.refs[b0 + e] * A + bin]++;
        }
    }
    o.accHash = acc_hash(acc);
    if (accOut) *accOut = acc;
    // peaks (ppf.cpp:363-391): top 3 by (vote desc, ref asc)
    const float thre = voteThreshold / 2.0f;
    o.nc = 0;
    for (size_t i = 0; i < refNum; i++) {
        const int *b = &acc[i * A];
        int total = 0;
        for (int j = 0; j < A; j++) total += b[j];
        if ((float)total < thre) continue;
        int j = 0;
        for (int t = 1; t < A; t++) if (b[t] > b[j]) j = t;
        int vote = b[j];
        if ((float)vote < thre) continue;
        vote += (j == 0) ? b[A - 1] : b[j - 1];
        vote += (j == A - 1) ? b[0] : b[j + 1];
        float fv = (float)vote;
        int   pos = o.nc;
        while (pos > 0 && o.cv[pos - 1] < fv) pos--;
        if (pos >= 3) continue;
        int last = std::min(o.nc, 2);
        for (int t = last; t > pos; t--) { o.cv[t] = o.cv[t - 1]; o.cr[t] = o.cr[t - 1]; o.ca[t] = o.ca[t - 1]; }
        o.cv[pos] = fv; o.cr[pos] = (int)i; o.ca[pos] = j;
        if (o.nc < 3) o.nc++;
    }
    if (o.nc == 0) return;
    // poses (ppf.cpp:393-409): T = RT_s^-1 * Rx(alpha) * RT_m
    const float thr2 = (float)((double)o.cv[0] * 0.95);
    for (int c = 0; c < o.nc; c++) {
        if (o.cv[c] < thr2) continue;
        const V3 &pm = m.sp[o.cr[c]], &nm = m.sn[o.cr[c]];
        smm::RT rm = smm::transform_rt(pm.x, pm.y, pm.z, nm.x, nm.y, nm.z);
        float   al = smm::candidate_angle(o.ca[c], A - 1);
        float   rec[smi::kPoseFloats];
        smi::candidate_pose(rt, rm, al, o.cv[c], rec);
        PoseRec pr;
        memcpy(pr.T.m, rec, 48);
        memcpy(pr.q, rec + 12, 16);
        pr.angle = rec[16];
        pr.votes = rec[17];
        o.poses[o.npose++] = pr;
    }
}

// Greedy first-fit leader clustering: an item joins the first earlier leader it is
// compatible with, else becomes a leader. Shared by clusterPose (util.cpp:499-520) and
// clusterPose2 (util.cpp:522-551). Returns leader index per item (itself for leaders).
template <class Compat> std::vector<int> leaders(int n, Compat &&compat) {
    std::vector<int> lead(n, -1), heads;
    for (int i = 0; i < n; i++) {
        for (int h : heads)
            if (compat(i, h)) { lead[i] = h; break; }
        if (lead[i] < 0) { lead[i] = i; heads.push_back(i); }
    }
    return lead;
}

std::vector<PoseRec> cluster_poses(const std::vector<PoseRec> &poseList, float distThr,
                                   float angThr, const V3 &center, float maxOverlap,
                                   std::vector<int> *clusterSizes) {
    // sortPoses (stable) + clusterPose
    std::vector<int> ord(poseList.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return poseList[a].votes > poseList[b].votes; });
    std::vector<PoseRec> sorted;
    for (int i : ord) sorted.push_back(poseList[i]);
    auto lead = leaders((int)sorted.size(), [&](int i, int h) {
        const PoseRec &a = sorted[i], &b = sorted[h];
        float d   = norm3(a.T.m[3] - b.T.m[3], a.T.m[7] - b.T.m[7], a.T.m[11] - b.T.m[11]);
        float phi = std::fabs(a.angle - b.angle);
        return d < distThr && phi < angThr;
    });
    // avgClusters (util.cpp:579-601), clusters in creation order
    std::vector<int> heads;
    std::vector<std::vector<int>> members;
    std::vector<int> slotOf(sorted.size(), -1);
    for (size_t i = 0; i < sorted.size(); i++) {
        if (lead[i] == (int)i) { slotOf[i] = (int)heads.size(); heads.push_back((int)i); members.emplace_back(); }
        members[slotOf[lead[i]]].push_back((int)i);
    }
    std::vector<PoseRec> avg;
    for (auto &mem : members) {
        float px = 0, py = 0, pz = 0, votes = 0;
        double S[10] = {0};
        for (int i : mem) {
            const PoseRec &p = sorted[i];
            px += p.T.m[3]; py += p.T.m[7]; pz += p.T.m[11];
            votes += p.votes;
            double v[4] = {p.q[0], p.q[1], p.q[2], p.q[3]};
            int k = 0;
            for (int a = 0; a < 4; a++) for (int b = a; b < 4; b++) S[k++] += v[a] * v[b];
        }
        float  cnt = (float)mem.size();
        double q[4], R[9];
        sml::quat_average_from_sum(S, (int)mem.size(), q);
        sml::quat_to_mat(q, R);
        PoseRec o;
        for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) o.T.m[i * 4 + j] = (float)R[i * 3 + j];
        o.T.m[3] = px / cnt; o.T.m[7] = py / cnt; o.T.m[11] = pz / cnt;
        for (int i = 0; i < 4; i++) o.q[i] = (float)q[i];
        o.angle = sml::quat_angle(q);
        o.votes = votes;
        avg.push_back(o);
        if (clusterSizes) clusterSizes->push_back((int)mem.size());
    }
    // sortPoses (stable) + clusterPose2
    std::vector<int> ord2(avg.size());
    std::iota(ord2.begin(), ord2.end(), 0);
    std::stable_sort(ord2.begin(), ord2.end(), [&](int a, int b) { return avg[a].votes > avg[b].votes; });
    std::vector<PoseRec> s2;
    for (int i : ord2) s2.push_back(avg[i]);
    std::vector<V3> tr(s2.size());
    for (size_t i = 0; i < s2.size(); i++) {
        smi::pose_apply(s2[i].T, center.x, center.y, center.z, tr[i].x, tr[i].y, tr[i].z);
    }
    float thr2 = maxOverlap * maxOverlap;
    auto  lead2 = leaders((int)s2.size(), [&](int i, int h) {
        float dx = tr[h].x - tr[i].x, dy = tr[h].y - tr[i].y, dz = tr[h].z - tr[i].z;
        return dx * dx + (dy * dy + dz * dz) < thr2;
    });
    std::vector<PoseRec> out;
    std::vector<int>     outSlot(s2.size(), -1);
    for (size_t i = 0; i < s2.size(); i++) {
        if (lead2[i] == (int)i) { outSlot[i] = (int)out.size(); out.push_back(s2[i]); }
        else out[outSlot[lead2[i]]].votes += s2[i].votes;
    }
    return out;
}

// ICP (icp.cpp:123-278) on correspondences from `nn(point, limit2, d2) -> id`.
struct IcpResult {
    smi::Pose34 pose;
    bool        converged = false;
    int         type = 0, iterations = 0;
    float       mse = FLT_MAX;
};

struct IcpCrit {
    int   iterations;
    float rejectDist, mseMin, mseMax, tolerance;
};

// FP32 Kahan partials over kIcpSlots strided slots, merged by the GPU's fixed trees (32
// slots of a warp, the warps of a block, then the blocks; sm_icp.h).
struct StridedSum {
    int         width;
    bool        fp64;
    std::vector<smi::KahanF> part;
    std::vector<double>      dpart;
    explicit StridedSum(int w, bool f64) : width(w), fp64(f64), part(smi::kIcpSlots * w), dpart(w, 0.0) {
        for (auto &k : part) k.init();
    }
    void add(int i, const float *v) {
        int t = i % smi::kIcpSlots;
        for (int c = 0; c < width; c++) {
            part[t * width + c].add(v[c]);
            dpart[c] += (double)v[c];
        }
    }
    void add_d(int i, const double *v) { // FP64 mode terms
        (void)i;
        for (int c = 0; c < width; c++) dpart[c] += v[c];
    }
    float result(int c) const {
        if (fp64) return (float)dpart[c];
        const int   NW = smi::kIcpThreads / 32, NB = smi::kIcpBlocks;
        smi::KahanF bs[NB];
        for (int b = 0; b < NB; b++) {
            smi::KahanF ws[NW];
            for (int w = 0; w < NW; w++) {
                smi::KahanF a[32];
                for (int l = 0; l < 32; l++) a[l] = part[(b * smi::kIcpThreads + w * 32 + l) * width + c];
                for (int off = 16; off >= 1; off /= 2)
                    for (int l = 0; l < off; l++) a[l].merge(a[l + off]);
                ws[w] = a[0];
            }
            for (int off = NW / 2; off >= 1; off /= 2)
                for (int l = 0; l < off; l++) ws[l].merge(ws[l + off]);
            bs[b] = ws[0];
        }
        for (int off = NB / 2; off >= 1; off /= 2)
            for (int l = 0; l < off; l++) bs[l].merge(bs[l + off]);
        return bs[0].value();
    }
};

template <class NN>
IcpResult icp_regist(const std::vector<V3> &sp, const std::vector<V3> &sn,
                     const std::vector<V3> &P, const std::vector<V3> &N, size_t dstSize,
                     const smi::Pose34 &init, const IcpCrit &cr, bool fp64, int nthreads, NN &&nn,
                     float *trace = nullptr) {
    IcpResult res;
    res.pose = init;
    const size_t ns = sp.size();
    std::vector<int>   nnId(ns);
    std::vector<float> nnD(ns);
    std::vector<V3>    x(ns), xn(ns);
    std::unordered_map<int, int> winner;
    winner.reserve(ns * 2);
    (void)dstSize;
    const float rej2 = cr.rejectDist * cr.rejectDist;
    while (res.iterations < cr.iterations) {
        // correspondences
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (long i = 0; i < (long)ns; i++) {
            smi::pose_apply(res.pose, sp[i].x, sp[i].y, sp[i].z, x[i].x, x[i].y, x[i].z);
            smi::pose_rotate(res.pose, sn[i].x, sn[i].y, sn[i].z, xn[i].x, xn[i].y, xn[i].z);
            float d;
            int   j = nn(x[i], rej2, d);
            nnId[i] = (j >= 0 && d <= rej2) ? j : -1;
            nnD[i]  = d;
        }
        winner.clear();
        for (size_t i = 0; i < ns; i++) {
            int j = nnId[i];
            if (j < 0) continue;
            auto it = winner.find(j);
            if (it == winner.end()) winner[j] = (int)i;
            else if (nnD[i] < nnD[it->second]) it->second = (int)i;
        }
        std::vector<int> pairs;
        for (size_t i = 0; i < ns; i++)
            if (nnId[i] >= 0 && winner[nnId[i]] == (int)i) pairs.push_back((int)i);
        size_t cnt = pairs.size();
        smi::Pose34 step;
        float       mse = FLT_MAX;
        if (cnt >= 6) {
            StridedSum mom(6, fp64);
            for (int i : pairs) {
                const V3 &q = P[nnId[i]];
                float v[6] = {x[i].x, x[i].y, x[i].z, q.x, q.y, q.z};
                mom.add(i, v);
            }
            float Pm[3], Qm[3];
            for (int c = 0; c < 3; c++) {
                Pm[c] = mom.result(c) / (float)cnt;
                Qm[c] = mom.result(3 + c) / (float)cnt;
            }
            StridedSum sys(smi::kNumSystem, fp64);
            for (int i : pairs) {
                const V3 &q = P[nnId[i]], &qn = N[nnId[i]];
                float t[smi::kNumSystem];
                if (!fp64) {
                    smi::system_terms(x[i].x - Pm[0], x[i].y - Pm[1], x[i].z - Pm[2], q.x - Qm[0],
                                      q.y - Qm[1], q.z - Qm[2], xn[i].x + qn.x, xn[i].y + qn.y,
                                      xn[i].z + qn.z, t);
                    sys.add(i, t);
                } else {
                    double p3[3] = {x[i].x - (double)Pm[0], x[i].y - (double)Pm[1], x[i].z - (double)Pm[2]};
                    double q3[3] = {q.x - (double)Qm[0], q.y - (double)Qm[1], q.z - (double)Qm[2]};
                    double n3[3] = {(double)xn[i].x + qn.x, (double)xn[i].y + qn.y, (double)xn[i].z + qn.z};
                    double s3[3] = {p3[0] + q3[0], p3[1] + q3[1], p3[2] + q3[2]};
                    double xv[6] = {s3[1] * n3[2] - s3[2] * n3[1], s3[2] * n3[0] - s3[0] * n3[2],
                                    s3[0] * n3[1] - s3[1] * n3[0], n3[0], n3[1], n3[2]};
                    double bi = (p3[0] - q3[0]) * n3[0] + (p3[1] - q3[1]) * n3[1] + (p3[2] - q3[2]) * n3[2];
                    double td[smi::kNumSystem];
                    int k = 0;
                    for (int a = 0; a < 6; a++) for (int b = a; b < 6; b++) td[k++] = xv[a] * xv[b];
                    for (int a = 0; a < 6; a++) td[21 + a] = bi * xv[a];
                    sys.add_d(i, td);
                }
            }
            float S[smi::kNumSystem];
            for (int c = 0; c < smi::kNumSystem; c++) S[c] = sys.result(c);
            step = smi::solve_step(S, Pm, Qm);
            // mean residual distance after the step
            std::vector<float> dist(cnt);
#pragma omp parallel for num_threads(nthreads) schedule(static)
            for (long k = 0; k < (long)cnt; k++) {
                int i = pairs[k];
                V3  y;
                smi::pose_apply(step, x[i].x, x[i].y, x[i].z, y.x, y.y, y.z);
                float d;
                nn(y, FLT_MAX, d);
                dist[k] = smm::fsqrt(d);
            }
            StridedSum ms(1, fp64);
            for (size_t k = 0; k < cnt; k++) ms.add(pairs[k], &dist[k]);
            mse = ms.result(0) / (float)cnt;
            if (trace && res.iterations < 32) {
                trace[res.iterations * 4 + 2] = Pm[0];
                trace[res.iterations * 4 + 3] = step.m[3];
            }
        }
        if (trace && res.iterations < 32) {
            trace[res.iterations * 4]     = (float)cnt;
            trace[res.iterations * 4 + 1] = mse;
            if (cnt < 6) trace[res.iterations * 4 + 3] = 0.0f;
        }
        // regist loop logic (icp.cpp:233-272)
        bool conv = (cnt > 6) && (mse < cr.mseMax);
        if (conv) res.converged = true;
        bool stop = false;
        if (cnt < 6) {
            res.type = 3;
            stop     = true;
        } else {
            if (mse < cr.mseMin) { res.type = 1; stop = true; }
            float rate = (res.mse - mse) / res.mse;
            if (rate < cr.tolerance) { res.type = 2; stop = true; }
            if (res.iterations++ >= cr.iterations) { res.type = 0; stop = true; }
            if (rate > 0) {
                res.mse  = mse;
                res.pose = smi::pose_mul(step, res.pose);
            }
        }
        if (stop) break;
    }
    return res;
}

struct MatchOut {
    std::vector<int>     sampled, keypoints, resampled;
    std::vector<V3>      P, N; // final positions / normals of the scene
    std::vector<int>     nbrOff, nbrIds; // per keypoint neighbour lists (search order)
    std::vector<KpOut>   kp;
    std::vector<PoseRec> poseList, clustered;
    std::vector<int>     clusterSizes;
    std::vector<float>   candScore;   // per clustered candidate: final score or -1
    std::vector<int>     candStatus;  // 0 ok, 1 votes, 2 sparse nc, 3 sparse score, 4 dense nc, 5 dense score
    std::vector<PoseRec> candPose;
    std::vector<float>   candTrace;   // 258 floats per candidate (layout of the GPU trace)
    std::vector<PoseRec> results;     // [score in votes field]
    std::vector<std::vector<int>> accDump; // full accumulators of the first dumpK keypoints
    double               tStage[8] = {0};
};

MatchOut *match(const Model &m, const float *xyz, const float *nrm, int64_t n, const float *vp3,
                float sdRel, float kpFrac, float minScore, const MatchParam &mp, int mode,
                int nthreads, int fp64, int dumpK) {
    if (sdRel > 1 || sdRel < 0) { g_err = "Invalid Input: samplingDistanceRel range mismatch in matchScene"; return nullptr; }
    if (kpFrac > 1 || kpFrac < 0) { g_err = "Invalid Input: keyPointFraction range mismatch in matchScene"; return nullptr; }
    if (minScore > 1 || minScore < 0) { g_err = "Invalid Input: minScore range mismatch in matchScene"; return nullptr; }
    if (n <= 0) { g_err = "Invalid Input: empty scene in matchScene"; return nullptr; }
    MatchOut *o = new MatchOut();
    auto &P = o->P;
    auto &N = o->N;
    P.resize(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    bool hasN = nrm != nullptr;
    if (hasN) { N.resize(n); for (int64_t i = 0; i < n; i++) N[i] = {nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]}; }
    else N.assign(n, V3{NAN, NAN, NAN});
    V3 vp = vp3 ? V3{vp3[0], vp3[1], vp3[2]} : V3{NAN, NAN, NAN};
    std::vector<int> valid;
    for (int64_t i = 0; i < n; i++)
        if (finite3(P[i]) && (!hasN || finite3(N[i]))) valid.push_back((int)i);
    Box box = bbox_of(P, valid);
    float ext[3] = {box.mx.x - box.mn.x, box.mx.y - box.mn.y, box.mx.z - box.mn.z};

    const float  diam        = m.box.diameter();
    const size_t refNum      = m.sp.size();
    const float  sqDiam      = diam * diam;
    const float  reSampleStep = diam * m.tp.poseRefRelSamplingDistance;
    const float  sampleStep  = diam * sdRel;
    const float  angleStep   = smm::k2PiF / (float)m.tp.featAngleResolution;

    std::unique_ptr<orc::KdTree> tree;
    std::vector<int> ioi, ioi2;
    Grid gq; // full-cloud query grid (GRID mode)
    auto grid_knn = [&](const V3 &q, int k, int *oi, float *od) { return gq.knn(q, k, oi, od); };
    auto kd_knn = [&](const V3 &q, int k, int *oi, float *od) {
        orc::KnnSet<64> rs(k);
        float qq[3] = {q.x, q.y, q.z};
        tree->findNeighbors(rs, qq);
        for (int i = 0; i < k; i++) { oi[i] = rs.idx[i]; od[i] = rs.dist[i]; }
        return rs.count;
    };
    if (mode == ORC_MODE_REF) {
        tree.reset(new orc::KdTree(P, valid, box.mn, box.mx));
        o->sampled = kd_sample(*tree, sampleStep, &ioi);
    } else {
        o->sampled = grid_sample(P, valid, box, sampleStep);
        gq.build(P, valid, box, smg::query_cell(sampleStep * 0.25f, ext));
    }
    if (!hasN) {
        if (mode == ORC_MODE_REF)
            estimate_normals(P, N, o->sampled, mp.knnNormal, mp.smoothNormal, mp.invertNormal, vp, fp64, nthreads, kd_knn);
        else
            estimate_normals(P, N, o->sampled, mp.knnNormal, mp.smoothNormal, mp.invertNormal, vp, fp64, nthreads, grid_knn);
    } else {
        for (auto &v : N) v = normalized(v);
    }
    const float keyStep = smm::fsqrt(1.f / kpFrac) * sampleStep;
    if (mode == ORC_MODE_REF) {
        tree->reduce(ioi);
        o->keypoints = kd_sample(*tree, keyStep, nullptr);
    } else {
        o->keypoints = grid_sample(P, o->sampled, box, keyStep);
    }
    const float voteThreshold = (float)refNum * minScore;
    float maxOverlapDist = 0;
    if (mp.maxOverlapDistRel > 0) maxOverlapDist = diam * mp.maxOverlapDistRel;
    if (mp.maxOverlapDistAbs > 0) maxOverlapDist = mp.maxOverlapDistAbs;
    float refDist = 0;
    if (mp.poseRefDistThresholdRel > 0) refDist = diam * mp.poseRefDistThresholdRel;
    if (mp.poseRefDistThresholdAbs > 0) refDist = mp.poseRefDistThresholdAbs;
    float scoreDist = 0;
    if (mp.poseRefScoringDistRel > 0) scoreDist = diam * mp.poseRefScoringDistRel;
    if (mp.poseRefScoringDistAbs > 0) scoreDist = mp.poseRefScoringDistAbs;

    // neighbour lists
    const size_t K = o->keypoints.size();
    std::vector<std::vector<int>> nb(K);
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4)
    for (long c = 0; c < (long)K; c++) {
        const V3 &p = P[o->keypoints[c]];
        if (mode == ORC_MODE_REF) {
            std::vector<std::pair<int, float>> f;
            float q[3] = {p.x, p.y, p.z};
            tree->radiusSearch(q, sqDiam, f);
            for (auto &e : f) nb[c].push_back(e.first);
        } else {
            for (int id : o->sampled) {
                const V3 &s = P[id];
                if (smm::dist2(p.x, p.y, p.z, s.x, s.y, s.z) < sqDiam) nb[c].push_back(id);
            }
        }
    }
    o->nbrOff.assign(1, 0);
    for (size_t c = 0; c < K; c++) {
        o->nbrIds.insert(o->nbrIds.end(), nb[c].begin(), nb[c].end());
        o->nbrOff.push_back((int)o->nbrIds.size());
    }
    // voting
    o->kp.resize(K);
    if (dumpK > 0) o->accDump.resize(std::min<size_t>(dumpK, K));
#pragma omp parallel num_threads(nthreads)
    {
        std::vector<int> acc;
#pragma omp for schedule(dynamic, 1)
        for (long c = 0; c < (long)K; c++)
            vote_keypoint(m, P, N, o->keypoints[c], nb[c], voteThreshold, acc, o->kp[c],
                          c < (long)o->accDump.size() ? &o->accDump[c] : nullptr);
    }
    for (size_t c = 0; c < K; c++)
        for (int t = 0; t < o->kp[c].npose; t++) o->poseList.push_back(o->kp[c].poses[t]);
    // clustering
    o->clustered = cluster_poses(o->poseList, 0.1f * diam, angleStep, m.box.center(), maxOverlapDist, &o->clusterSizes);

    // ICP
    IcpCrit sparse{5, refDist, sampleStep * 0.5f, sampleStep, 0.05f};
    IcpCrit dense{mp.poseRefNumSteps, refDist, reSampleStep * 0.5f, sampleStep, 0.05f};
    if (mp.densePoseRefinement) {
        if (mode == ORC_MODE_REF) {
            tree->restore();
            o->resampled = kd_sample(*tree, reSampleStep, &ioi2);
            if (!hasN) estimate_normals(P, N, o->resampled, mp.knnNormal, false, mp.invertNormal, vp, fp64, nthreads, kd_knn);
        } else {
            o->resampled = grid_sample(P, valid, box, reSampleStep);
            if (!hasN) {
                gq.build(P, valid, box, smg::query_cell(sampleStep * 0.25f, ext));
                estimate_normals(P, N, o->resampled, mp.knnNormal, false, mp.invertNormal, vp, fp64, nthreads, grid_knn);
            }
        }
    }
    Grid gS, gR, gF;
    if (mode == ORC_MODE_GRID) {
        gS.build(P, o->sampled, box, smg::query_cell(sampleStep, ext));
        if (mp.densePoseRefinement) gR.build(P, o->resampled, box, smg::query_cell(reSampleStep * 2.0f, ext));
        gF.build(P, valid, box, smg::query_cell(scoreDist > 0 ? scoreDist : sampleStep, ext));
    }
    auto nn_in = [&](Grid &g, const std::vector<int> *reduceIoi) {
        return [&, reduceIoi](const V3 &q, float lim2, float &d) -> int {
            if (mode == ORC_MODE_GRID) return g.nn(q, lim2, d);
            orc::KnnSet<1> rs(1);
            float qq[3] = {q.x, q.y, q.z};
            tree->findNeighbors(rs, qq);
            d = rs.dist[0];
            return rs.count ? rs.idx[0] : -1;
        };
    };
    const float score2 = scoreDist * scoreDist;
    auto inliers = [&](const std::vector<V3> &src, const smi::Pose34 &T) {
        long cnt = 0;
#pragma omp parallel for num_threads(nthreads) reduction(+ : cnt)
        for (long i = 0; i < (long)src.size(); i++) {
            V3 y;
            smi::pose_apply(T, src[i].x, src[i].y, src[i].z, y.x, y.y, y.z);
            if (mode == ORC_MODE_GRID) {
                if (gF.any_within(y, score2)) cnt++;
            } else {
                orc::KnnSet<1> rs(1);
                float qq[3] = {y.x, y.y, y.z};
                tree->findNeighbors(rs, qq);
                if (rs.count && rs.dist[0] < score2) cnt++;
            }
        }
        return (int)cnt;
    };
    for (auto &c : o->clustered) {
        smi::Pose34 pose = c.T;
        float       score = c.votes;
        int         status = 0;
        std::vector<float> tr(258, -1.0f);
        if (score < voteThreshold) status = 1;
        if (!status && mp.sparsePoseRefinement) {
            if (mode == ORC_MODE_REF) { tree->restore(); tree->reduce(ioi); }
            auto r = icp_regist(m.sp, m.sn, P, N, o->sampled.size(), pose, sparse, fp64, nthreads, nn_in(gS, &ioi), tr.data());
            if (!r.converged) status = 2;
            else {
                pose = r.pose;
                if (mode == ORC_MODE_REF) tree->restore();
                int in = inliers(m.sp, pose);
                tr[256] = (float)in;
                score = std::min(1.f, in / float(refNum));
                if (score < minScore) status = 3;
            }
        }
        if (!status && mp.sparsePoseRefinement && mp.densePoseRefinement) {
            if (mode == ORC_MODE_REF) { tree->restore(); tree->reduce(ioi2); }
            auto r = icp_regist(m.rp, m.rn, P, N, o->resampled.size(), pose, dense, fp64, nthreads, nn_in(gR, &ioi2), tr.data() + 128);
            if (!r.converged) status = 4;
            else {
                pose = r.pose;
                if (mode == ORC_MODE_REF) tree->restore();
                int in = inliers(m.rp, pose);
                tr[257] = (float)in;
                score = std::min(1.f, in / float(m.rp.size()));
                if (score < minScore) status = 5;
            }
        }
        if (!status && (mp.sparsePoseRefinement || mp.densePoseRefinement) && score < minScore) status = 5;
        PoseRec pr;
        pr.T = pose;
        pr.votes = score;
        o->candStatus.push_back(status);
        o->candScore.push_back(status ? -1.f : score);
        o->candPose.push_back(pr);
        o->candTrace.insert(o->candTrace.end(), tr.begin(), tr.end());
        if (!status) {
            o->results.push_back(pr);
            if ((int)o->results.size() >= mp.numMatches) break;
        }
    }
    std::stable_sort(o->results.begin(), o->results.end(), [](const PoseRec &a, const PoseRec &b) { return a.votes > b.votes; });
    return o;
}

} // namespace

// ---------------------------------------------------------------------------------------
// C ABI for the test harness (ctypes)
// ---------------------------------------------------------------------------------------
extern "C" {

struct orc_train_param {
    float featDistanceStepRel;
    int   featAngleResolution;
    float poseRefRelSamplingDistance;
    int   knnNormal;
    int   smoothNormal;
};

struct orc_match_param {
    int   numMatches, knnNormal, smoothNormal, invertNormal;
    float maxOverlapDistRel, maxOverlapDistAbs;
    int   sparsePoseRefinement, densePoseRefinement, poseRefNumSteps;
    float poseRefDistThresholdRel, poseRefDistThresholdAbs, poseRefScoringDistRel, poseRefScoringDistAbs;
};

const char *orc_last_error() { return g_err.c_str(); }

void *orc_train(const float *xyz, const float *nrm, int64_t n, float sdRel, const orc_train_param *p,
                int mode, int nthreads) {
    TrainParam tp;
    tp.featDistanceStepRel        = p->featDistanceStepRel;
    tp.featAngleResolution        = p->featAngleResolution;
    tp.poseRefRelSamplingDistance = p->poseRefRelSamplingDistance;
    tp.knnNormal                  = p->knnNormal;
    tp.smoothNormal               = p->smoothNormal;
    return train(xyz, nrm, n, sdRel, tp, mode, nthreads);
}

void orc_model_free(void *m) { delete (Model *)m; }

// sizes: [n_sampled, n_resampled, n_keys, n_entries]
void orc_model_sizes(void *mp, int64_t *out) {
    Model *m = (Model *)mp;
    out[0] = (int64_t)m->sp.size();
    out[1] = (int64_t)m->rp.size();
    out[2] = (int64_t)m->keys.size();
    out[3] = (int64_t)m->refs.size();
}

// box[6] = min xyz, max xyz; diam
void orc_model_export(void *mp, float *sp, float *sn, float *rp, float *rn, float *box,
                      uint32_t *keys, uint32_t *offs, uint32_t *refs, float *alphas) {
    Model *m = (Model *)mp;
    for (size_t i = 0; i < m->sp.size(); i++) {
        memcpy(sp + 3 * i, &m->sp[i], 12);
        memcpy(sn + 3 * i, &m->sn[i], 12);
    }
    for (size_t i = 0; i < m->rp.size(); i++) {
        memcpy(rp + 3 * i, &m->rp[i], 12);
        memcpy(rn + 3 * i, &m->rn[i], 12);
    }
    box[0] = m->box.mn.x; box[1] = m->box.mn.y; box[2] = m->box.mn.z;
    box[3] = m->box.mx.x; box[4] = m->box.mx.y; box[5] = m->box.mx.z;
    memcpy(keys, m->keys.data(), m->keys.size() * 4);
    memcpy(offs, m->offs.data(), m->offs.size() * 4);
    memcpy(refs, m->refs.data(), m->refs.size() * 4);
    memcpy(alphas, m->alphas.data(), m->alphas.size() * 4);
}

// Build a model from arrays (a table produced elsewhere, e.g. by the GPU trainer).
void *orc_model_import(int64_t ns, const float *sp, const float *sn, int64_t nr, const float *rp,
                       const float *rn, const float *box, int64_t nk, const uint32_t *keys,
                       const uint32_t *offs, const uint32_t *refs, const float *alphas,
                       const orc_train_param *p, float sdRel) {
    Model *m = new Model();
    m->samplingDistanceRel        = sdRel;
    m->tp.featDistanceStepRel        = p->featDistanceStepRel;
    m->tp.featAngleResolution        = p->featAngleResolution;
    m->tp.poseRefRelSamplingDistance = p->poseRefRelSamplingDistance;
    m->tp.knnNormal                  = p->knnNormal;
    m->tp.smoothNormal               = p->smoothNormal;
    for (int64_t i = 0; i < ns; i++) { m->sp.push_back({sp[3 * i], sp[3 * i + 1], sp[3 * i + 2]}); m->sn.push_back({sn[3 * i], sn[3 * i + 1], sn[3 * i + 2]}); }
    for (int64_t i = 0; i < nr; i++) { m->rp.push_back({rp[3 * i], rp[3 * i + 1], rp[3 * i + 2]}); m->rn.push_back({rn[3 * i], rn[3 * i + 1], rn[3 * i + 2]}); }
    m->box.mn = {box[0], box[1], box[2]};
    m->box.mx = {box[3], box[4], box[5]};
    m->keys.assign(keys, keys + nk);
    m->offs.assign(offs, offs + nk + 1);
    m->refs.assign(refs, refs + offs[nk]);
    m->alphas.assign(alphas, alphas + offs[nk]);
    for (int64_t b = 0; b < nk; b++) m->slot[keys[b]] = (uint32_t)b;
    finish_table(*m);
    return m;
}

void *orc_match(void *model, const float *xyz, const float *nrm, int64_t n, const float *vp,
                float sdRel, float kpFrac, float minScore, const orc_match_param *p, int mode,
                int nthreads, int fp64, int dumpK) {
    MatchParam mp;
    mp.numMatches = p->numMatches; mp.knnNormal = p->knnNormal; mp.smoothNormal = p->smoothNormal;
    mp.invertNormal = p->invertNormal; mp.maxOverlapDistRel = p->maxOverlapDistRel;
    mp.maxOverlapDistAbs = p->maxOverlapDistAbs; mp.sparsePoseRefinement = p->sparsePoseRefinement;
    mp.densePoseRefinement = p->densePoseRefinement; mp.poseRefNumSteps = p->poseRefNumSteps;
    mp.poseRefDistThresholdRel = p->poseRefDistThresholdRel; mp.poseRefDistThresholdAbs = p->poseRefDistThresholdAbs;
    mp.poseRefScoringDistRel = p->poseRefScoringDistRel; mp.poseRefScoringDistAbs = p->poseRefScoringDistAbs;
    return match(*(Model *)model, xyz, nrm, n, vp, sdRel, kpFrac, minScore, mp, mode, nthreads, fp64, dumpK);
}

void orc_match_free(void *r) { delete (MatchOut *)r; }

// Field sizes / copies of a match result. Field ids:
//  0 sampled ids (int32)     1 keypoint ids (int32)     2 resampled ids (int32)
//  3 positions (f32 x3)      4 normals (f32 x3)         5 nbr offsets (int32, K+1)
//  6 nbr ids (int32)         7 per-keypoint stats (int64 x8: searched, skipped, hits,
//    votes, accHash, ncand, npose, counter bound)                   8 candidates (f32 x9: v0 r0 a0 ..)
//  9 pose list (f32 x18: 12 pose, 4 q, angle, votes)   10 clustered (f32 x18)
// 11 cluster sizes (int32)  12 candidate status (int32) 13 candidate score (f32)
// 14 candidate pose (f32 x12)  15 results (f32 x13: 12 pose + score)
// 16 accumulator dump (int32, dumpK x refNum x A)
int64_t orc_res_size(void *rp, int field) {
    MatchOut *r = (MatchOut *)rp;
    switch (field) {
        case 0: return r->sampled.size();
        case 1: return r->keypoints.size();
        case 2: return r->resampled.size();
        case 3: case 4: return r->P.size() * 3;
        case 5: return r->nbrOff.size();
        case 6: return r->nbrIds.size();
        case 7: return r->kp.size() * 8;
        case 8: return r->kp.size() * 9;
        case 9: return r->poseList.size() * 18;
        case 10: return r->clustered.size() * 18;
        case 11: return r->clusterSizes.size();
        case 12: return r->candStatus.size();
        case 13: return r->candScore.size();
        case 14: return r->candPose.size() * 12;
        case 15: return r->results.size() * 13;
        case 16: { int64_t s = 0; for (auto &a : r->accDump) s += a.size(); return s; }
        case 17: return r->candTrace.size();
    }
    return -1;
}

static void put_pose(float *d, const PoseRec &p) {
    memcpy(d, p.T.m, 48);
    memcpy(d + 12, p.q, 16);
    d[16] = p.angle;
    d[17] = p.votes;
}

void orc_res_get(void *rp, int field, void *dst) {
    MatchOut *r = (MatchOut *)rp;
    switch (field) {
        case 0: memcpy(dst, r->sampled.data(), r->sampled.size() * 4); break;
        case 1: memcpy(dst, r->keypoints.data(), r->keypoints.size() * 4); break;
        case 2: memcpy(dst, r->resampled.data(), r->resampled.size() * 4); break;
        case 3: memcpy(dst, r->P.data(), r->P.size() * 12); break;
        case 4: memcpy(dst, r->N.data(), r->N.size() * 12); break;
        case 5: memcpy(dst, r->nbrOff.data(), r->nbrOff.size() * 4); break;
        case 6: memcpy(dst, r->nbrIds.data(), r->nbrIds.size() * 4); break;
        case 7: {
            int64_t *d = (int64_t *)dst;
            for (size_t c = 0; c < r->kp.size(); c++) {
                auto &k = r->kp[c];
                int64_t v[8] = {k.searched, k.skipped, k.hits, k.votes, (int64_t)k.accHash, k.nc, k.npose, k.bound};
                memcpy(d + 8 * c, v, 64);
            }
            break;
        }
        case 8: {
            float *d = (float *)dst;
            for (size_t c = 0; c < r->kp.size(); c++) {
                auto &k = r->kp[c];
                for (int t = 0; t < 3; t++) {
                    d[9 * c + 3 * t]     = t < k.nc ? k.cv[t] : -1.f;
                    d[9 * c + 3 * t + 1] = t < k.nc ? (float)k.cr[t] : -1.f;
                    d[9 * c + 3 * t + 2] = t < k.nc ? (float)k.ca[t] : -1.f;
                }
            }
            break;
        }
        case 9: for (size_t i = 0; i < r->poseList.size(); i++) put_pose((float *)dst + 18 * i, r->poseList[i]); break;
        case 10: for (size_t i = 0; i < r->clustered.size(); i++) put_pose((float *)dst + 18 * i, r->clustered[i]); break;
        case 11: memcpy(dst, r->clusterSizes.data(), r->clusterSizes.size() * 4); break;
        case 12: memcpy(dst, r->candStatus.data(), r->candStatus.size() * 4); break;
        case 13: memcpy(dst, r->candScore.data(), r->candScore.size() * 4); break;
        case 14: for (size_t i = 0; i < r->candPose.size(); i++) memcpy((float *)dst + 12 * i, r->candPose[i].T.m, 48); break;
        case 15:
            for (size_t i = 0; i < r->results.size(); i++) {
                memcpy((float *)dst + 13 * i, r->results[i].T.m, 48);
                ((float *)dst)[13 * i + 12] = r->results[i].votes;
            }
            break;
        case 17: memcpy(dst, r->candTrace.data(), r->candTrace.size() * 4); break;
        case 16: {
            int *d = (int *)dst;
            for (auto &a : r->accDump) { memcpy(d, a.data(), a.size() * 4); d += a.size(); }
            break;
        }
    }
}

// Standalone voting stage on caller-supplied scene state (stage parity): positions and
// normals of the scene, keypoint ids, and per-keypoint neighbour lists in search order.
// stats/cands as fields 7 / 8; acc (optional) receives dumpK full accumulators.
void orc_vote_stage(void *model, const float *pts, const float *nrms, int64_t n, const int *kp,
                    int64_t K, const int *nbrOff, const int *nbrIds, float minScore, int nthreads,
                    int64_t *stats, float *cands, float *poses18, int dumpK, int *acc) {
    Model &m = *(Model *)model;
    std::vector<V3> P(n), N(n);
    for (int64_t i = 0; i < n; i++) {
        P[i] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
        N[i] = {nrms[3 * i], nrms[3 * i + 1], nrms[3 * i + 2]};
    }
    const float voteThreshold = (float)m.sp.size() * minScore;
    std::vector<KpOut> out(K);
    std::vector<std::vector<int>> dump(std::min<int64_t>(dumpK, K));
#pragma omp parallel num_threads(nthreads)
    {
        std::vector<int> a;
#pragma omp for schedule(dynamic, 1)
        for (long c = 0; c < (long)K; c++) {
            std::vector<int> nb(nbrIds + nbrOff[c], nbrIds + nbrOff[c + 1]);
            vote_keypoint(m, P, N, kp[c], nb, voteThreshold, a, out[c], c < (long)dump.size() ? &dump[c] : nullptr);
        }
    }
    for (int64_t c = 0; c < K; c++) {
        auto &k = out[c];
        int64_t v[8] = {k.searched, k.skipped, k.hits, k.votes, (int64_t)k.accHash, k.nc, k.npose, k.bound};
        memcpy(stats + 8 * c, v, 64);
        for (int t = 0; t < 3; t++) {
            cands[9 * c + 3 * t]     = t < k.nc ? k.cv[t] : -1.f;
            cands[9 * c + 3 * t + 1] = t < k.nc ? (float)k.cr[t] : -1.f;
            cands[9 * c + 3 * t + 2] = t < k.nc ? (float)k.ca[t] : -1.f;
            if (poses18) {
                if (t < k.npose) put_pose(poses18 + 54 * c + 18 * t, k.poses[t]);
                else for (int e = 0; e < 18; e++) poses18[54 * c + 18 * t + e] = 0.f;
            }
        }
    }
    if (acc)
        for (auto &d : dump) { memcpy(acc, d.data(), d.size() * 4); acc += d.size(); }
}

// Shared-math probes for the unit tests.
float orc_atan2f(float y, float x) { return smm::atan2f_(y, x); }
float orc_acosf(float x) { return smm::acosf_(x); }
float orc_sinf(float x) { return smm::sinf_(x); }
float orc_cosf(float x) { return smm::cosf_(x); }
uint32_t orc_murmur4(const uint32_t *w) { return smm::murmur4(w[0], w[1], w[2], w[3]); }

// k-d tree probes (compared against the vendored nanoflann where the reference is
// present): vAcc order after the build, and a radius search.
int64_t orc_kd_probe(const float *xyz, int64_t n, const float *box, const float *q, float r2,
                     int *vacc, int *found, int64_t maxFound) {
    std::vector<V3> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    std::vector<int> valid(n);
    std::iota(valid.begin(), valid.end(), 0);
    orc::KdTree t(P, valid, V3{box[0], box[1], box[2]}, V3{box[3], box[4], box[5]});
    memcpy(vacc, t.vAcc.data(), n * 4);
    std::vector<std::pair<int, float>> f;
    t.radiusSearch(q, r2, f);
    for (int64_t i = 0; i < (int64_t)f.size() && i < maxFound; i++) found[i] = f[i].first;
    return (int64_t)f.size();
}

// samplePointCloud (util.cpp:107-139) on the full tree of all n points: kept ids in tree
// order into out (capacity n); returns their count.
int64_t orc_kd_sample(const float *xyz, int64_t n, const float *box, float step, int *out) {
    std::vector<V3> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    std::vector<int> valid(n);
    std::iota(valid.begin(), valid.end(), 0);
    orc::KdTree t(P, valid, V3{box[0], box[1], box[2]}, V3{box[3], box[4], box[5]});
    std::vector<int> r = kd_sample(t, step, nullptr);
    memcpy(out, r.data(), r.size() * 4);
    return (int64_t)r.size();
}

} // extern "C"

extern "C" void orc_kd_knn(const float *xyz, int64_t n, const float *box, const float *qs,
                           int64_t nq, int k, int *idx, float *dist) {
    std::vector<V3> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    std::vector<int> valid(n);
    std::iota(valid.begin(), valid.end(), 0);
    orc::KdTree t(P, valid, V3{box[0], box[1], box[2]}, V3{box[3], box[4], box[5]});
    for (int64_t j = 0; j < nq; j++) {
        orc::KnnSet<64> rs(k);
        t.findNeighbors(rs, qs + 3 * j);
        for (int i = 0; i < k; i++) {
            idx[(int64_t)k * j + i]  = rs.idx[i];
            dist[(int64_t)k * j + i] = rs.dist[i];
        }
    }
}

// Grid-search probe for the exactness tests: k nearest, nearest within a limit and
// any-within-radius of each query over all points, on a grid of cell side `cell`.
extern "C" void orc_grid_probe(const float *xyz, int64_t n, const float *qs, int64_t nq,
                               float cell, int k, float limit2, float r2, int *knnIdx,
                               float *knnDist, int *nnIdx, float *nnDist, int *within) {
    std::vector<V3> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    std::vector<int> all(n);
    std::iota(all.begin(), all.end(), 0);
    Box b = bbox_of(P, all);
    Grid G;
    G.build(P, all, b, cell);
    for (int64_t j = 0; j < nq; j++) {
        V3 q{qs[3 * j], qs[3 * j + 1], qs[3 * j + 2]};
        std::vector<int>   oi(k, -1);
        std::vector<float> od(k, -1.f);
        G.knn(q, k, oi.data(), od.data());
        for (int i = 0; i < k; i++) { knnIdx[j * k + i] = oi[i]; knnDist[j * k + i] = od[i]; }
        float d;
        nnIdx[j]  = G.nn(q, limit2, d);
        nnDist[j] = d;
        within[j] = G.any_within(q, r2) ? 1 : 0;
    }
}

// estimateNormalMLS (util.cpp:336-457) restated in FP64 and unscaled coordinates, the
// reference's steps in its order: neighbours closer than the radius (the k-d tree's float
// metric, nanoflann.hpp:545-579, over the finite points, found here by a scan in index
// order); fewer than 3 leave the point unchanged (util.cpp:363-364); PCA normal of the
// neighbourhood (util.cpp:368-381); the query projected on its plane and the frame
// v = unitOrthogonal(n), u = n x v (util.cpp:383-390); order <= 1 with fewer neighbours
// than coefficients stops there (util.cpp:393-394); the weighted polynomial fit solved by
// Cholesky (util.cpp:395-436); the point and normal from the fit and the orientation
// (util.cpp:439-455). Neighbourhoods read the input positions (two-phase, like the GPU).
// status[i] of listed point i: 0 unchanged, 1 PCA normal only, 2 moved onto the fit.
namespace {

// Eigen's unitOrthogonal for 3-vectors: (-y, x, 0) normalised unless x and y are both
// much smaller than z (|.| <= 1e-5 |z|, the float dummy precision), else (0, -z, y)
// normalised.
void unit_orthogonal(const double n[3], double v[3]) {
    const double eps = 1e-5;
    if (!(std::fabs(n[0]) <= std::fabs(n[2]) * eps) || !(std::fabs(n[1]) <= std::fabs(n[2]) * eps)) {
        const double h = 1.0 / std::sqrt(n[0] * n[0] + n[1] * n[1]);
        v[0] = -n[1] * h, v[1] = n[0] * h, v[2] = 0.0;
    } else {
        const double h = 1.0 / std::sqrt(n[1] * n[1] + n[2] * n[2]);
        v[0] = 0.0, v[1] = -n[2] * h, v[2] = n[1] * h;
    }
}

// G c = b for symmetric positive definite G (row-major n x n), by the LLT factorisation;
// false when a pivot is not positive or the solution is not finite.
bool llt_solve(std::vector<double> G, std::vector<double> &b, int n) {
    for (int j = 0; j < n; j++) {
        double d = G[j * n + j];
        for (int k = 0; k < j; k++) d -= G[j * n + k] * G[j * n + k];
        if (!(d > 0.0)) return false;
        G[j * n + j] = std::sqrt(d);
        for (int i = j + 1; i < n; i++) {
            double v = G[i * n + j];
            for (int k = 0; k < j; k++) v -= G[i * n + k] * G[j * n + k];
            G[i * n + j] = v / G[j * n + j];
        }
    }
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < i; k++) b[i] -= G[i * n + k] * b[k];
        b[i] /= G[i * n + i];
    }
    for (int i = n - 1; i >= 0; i--) {
        for (int k = i + 1; k < n; k++) b[i] -= G[k * n + i] * b[k];
        b[i] /= G[i * n + i];
        if (!std::isfinite(b[i])) return false;
    }
    return true;
}

} // namespace

extern "C" void orc_mls(const float *xyz, int64_t n, const int64_t *idx, int64_t m, float radius,
                        int order, int invert, const float *vp, float *outXyz, float *outNrm,
                        int *status) {
    const float r2 = radius * radius;
    const int   nc = (order + 1) * (order + 2) / 2;
    const bool  hasVp = vp && std::isfinite(vp[0]) && std::isfinite(vp[1]) && std::isfinite(vp[2]);
    std::vector<int> fin;
    for (int64_t j = 0; j < n; j++)
        if (std::isfinite(xyz[3 * j]) && std::isfinite(xyz[3 * j + 1]) && std::isfinite(xyz[3 * j + 2]))
            fin.push_back((int)j);
    for (int64_t t = 0; t < m; t++) {
        const int64_t id = idx[t];
        status[t]        = 0;
        const float  qx = xyz[3 * id], qy = xyz[3 * id + 1], qz = xyz[3 * id + 2];
        std::vector<int> nb;
        if (std::isfinite(qx) && std::isfinite(qy) && std::isfinite(qz))
            for (int j : fin)
                if (smm::dist2(qx, qy, qz, xyz[3 * j], xyz[3 * j + 1], xyz[3 * j + 2]) < r2)
                    nb.push_back(j);
        if (nb.size() < 3) continue;
        // PCA
        double c[3] = {0, 0, 0};
        for (int j : nb)
            for (int a = 0; a < 3; a++) c[a] += xyz[3 * j + a];
        for (int a = 0; a < 3; a++) c[a] /= (double)nb.size();
        double C[6] = {0, 0, 0, 0, 0, 0};
        for (int j : nb) {
            const double d[3] = {xyz[3 * j] - c[0], xyz[3 * j + 1] - c[1], xyz[3 * j + 2] - c[2]};
            C[0] += d[0] * d[0], C[1] += d[0] * d[1], C[2] += d[0] * d[2];
            C[3] += d[1] * d[1], C[4] += d[1] * d[2], C[5] += d[2] * d[2];
        }
        float nf[3];
        sml::normal_from_cov(C, nf);
        const double nv[3] = {nf[0], nf[1], nf[2]};
        for (int a = 0; a < 3; a++) outNrm[3 * id + a] = nf[a];
        status[t] = 1;
        // plane projection and frame
        const double dpl  = -(nv[0] * c[0] + nv[1] * c[1] + nv[2] * c[2]);
        const double dist = qx * nv[0] + qy * nv[1] + qz * nv[2] + dpl;
        const double mean[3] = {qx - dist * nv[0], qy - dist * nv[1], qz - dist * nv[2]};
        double       v[3], u[3];
        unit_orthogonal(nv, v);
        u[0] = nv[1] * v[2] - nv[2] * v[1];
        u[1] = nv[2] * v[0] - nv[0] * v[2];
        u[2] = nv[0] * v[1] - nv[1] * v[0];
        if (order <= 1 && nc > (int)nb.size()) continue;
        // weighted polynomial fit of the heights
        std::vector<double> G((size_t)nc * nc, 0.0), b(nc, 0.0), P(nc);
        for (int j : nb) {
            const double d[3] = {xyz[3 * j] - mean[0], xyz[3 * j + 1] - mean[1], xyz[3 * j + 2] - mean[2]};
            const double w  = std::exp(-(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) / (double)r2);
            const double uc = d[0] * u[0] + d[1] * u[1] + d[2] * u[2];
            const double vc = d[0] * v[0] + d[1] * v[1] + d[2] * v[2];
            const double f  = d[0] * nv[0] + d[1] * nv[1] + d[2] * nv[2];
            int    k    = 0;
            double uPow = 1;
            for (int ui = 0; ui <= order; ui++) {
                double vPow = 1;
                for (int vi = 0; vi <= order - ui; vi++) {
                    P[k++] = uPow * vPow;
                    vPow *= vc;
                }
                uPow *= uc;
            }
            for (int a = 0; a < nc; a++) {
                b[a] += w * P[a] * f;
                for (int e = 0; e < nc; e++) G[(size_t)a * nc + e] += w * P[a] * P[e];
            }
        }
        if (!llt_solve(G, b, nc)) continue;
        const double p[3] = {mean[0] + b[0] * nv[0], mean[1] + b[0] * nv[1], mean[2] + b[0] * nv[2]};
        double       nn[3];
        for (int a = 0; a < 3; a++) nn[a] = nv[a] - b[order + 1] * u[a] - b[1] * v[a];
        const double len = std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        if (len > 0)
            for (int a = 0; a < 3; a++) nn[a] /= len;
        const double o = hasVp ? nn[0] * (vp[0] - p[0]) + nn[1] * (vp[1] - p[1]) + nn[2] * (vp[2] - p[2])
                               : nn[2];
        const bool flip = invert ? o > 0.0 : o < 0.0;
        for (int a = 0; a < 3; a++) {
            outXyz[3 * id + a] = (float)p[a];
            outNrm[3 * id + a] = (float)(flip ? -nn[a] : nn[a]);
        }
        status[t] = 2;
    }
}
