// oracle/kdtree.h - TEST INFRASTRUCTURE ONLY (the oracle's k-d tree; never linked into the
// product library).
//
// Restatement of the k-d tree the reference builds through its vendored, locally modified
// nanoflann (kdtree/kdtree.h:52-161, kdtree/nanoflann.hpp v0x155), kept to the points that
// decide sampling order, neighbour order and tie-breaking:
//   * build: root box = the user box (kdtree.h:135-144); middle split on the widest box
//     side among sides within (1-1e-5) of the widest, cut at the box middle clamped to the
//     points' range (nanoflann.hpp:1290-1339); two-pass in-place partition on < and <=
//     the cut value with unsigned indices (nanoflann.hpp:1352-1393); leaves of at most
//     10 points; node bounds tightened bottom-up (nanoflann.hpp:1120-1176). The root box
//     is replaced by the tight box of all points after the build, as nanoflann passes
//     root_bbox_ by reference into divideTree.
//   * search: depth first, nearer child first by (val-divlow)+(val-divhigh) < 0, far child
//     visited when mindist <= worst distance (nanoflann.hpp:1846-1930); leaf entries equal
//     to INVALID_INDEX (-1) are skipped (the local modification used by reduce(), kdtree.h
//     :146-157); squared distance ((d0^2+d1^2)+d2^2) with d = query - point.
//   * radius result set: keeps dist < r^2, unsorted, in visiting order (nanoflann.hpp:
//     374-420). kNN result set: insertion sort with strict '>' so the first-found point
//     wins ties (nanoflann.hpp:180-233).
// The tree keeps a pointer to the live position array: normal estimation moves points to
// their neighbourhood centroid (util.cpp:269) after the build, and searches then evaluate
// distances on the moved positions against the build-time node bounds, as the reference
// does through KDTreeVectorOfVectorsAdaptor::m_data.
// Deviation (documented): vAcc is initialised with the valid indices themselves; the
// vendored nanoflann uses 0..count-1 (nanoflann.hpp:1798-1804), which is identical for
// clouds without NaN points and wrong for clouds with them.
#pragma once

#include <algorithm>
#include <cfloat>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace orc {

struct V3 {
    float x, y, z;
    float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

struct KdNode {
    int   child1 = -1, child2 = -1; // -1 = leaf
    int   left = 0, right = 0;       // leaf range in vAcc
    int   divfeat = 0;
    float divlow = 0, divhigh = 0;
};

struct Interval {
    float low, high;
};

struct RadiusSet {
    float                          radius;
    std::vector<std::pair<int, float>> *out;
    float worst() const { return radius; }
    bool  add(float d, int idx) {
        if (d < radius)
            out->emplace_back(idx, d);
        return true;
    }
};

template <int K> struct KnnSet {
    int   idx[K];
    float dist[K];
    int   cap, count = 0;
    explicit KnnSet(int c) : cap(c) {
        for (int i = 0; i < K; i++) {
            idx[i]  = -1;
            dist[i] = FLT_MAX;
        }
    }
    float worst() const { return dist[cap - 1]; }
    bool  add(float d, int index) {
        int i;
        for (i = count; i > 0; --i) {
            if (dist[i - 1] > d) {
                if (i < cap) {
                    dist[i] = dist[i - 1];
                    idx[i]  = idx[i - 1];
                }
            } else
                break;
        }
        if (i < cap) {
            dist[i] = d;
            idx[i]  = index;
        }
        if (count < cap)
            count++;
        return true;
    }
};

class KdTree {
public:
    const std::vector<V3> *data = nullptr;
    std::vector<int>       vAcc, vAccTmp;
    std::vector<KdNode>    nodes;
    int                    root = -1;
    Interval               rootBox[3];
    size_t                 leafMax = 10;

    KdTree(const std::vector<V3> &pts, const std::vector<int> &valid, const V3 &bmin,
           const V3 &bmax, size_t leafMaxSize = 10)
        : data(&pts), leafMax(leafMaxSize) {
        vAcc = valid;
        if (vAcc.empty())
            return;
        rootBox[0] = {bmin.x, bmax.x};
        rootBox[1] = {bmin.y, bmax.y};
        rootBox[2] = {bmin.z, bmax.z};
        nodes.reserve(2 * (vAcc.size() / 5 + 1));
        root = divide(0, vAcc.size(), rootBox);
    }

    float pt(int idx, int dim) const { return (*data)[idx][dim]; }

    // reduce()/restore() of kdtree.h:146-157.
    void reduce(const std::vector<int> &indices) {
        vAccTmp = std::move(vAcc);
        vAcc    = indices;
    }
    void restore() {
        if (vAccTmp.empty())
            return;
        vAcc = std::move(vAccTmp);
        vAccTmp.clear();
    }

    template <class RS> void findNeighbors(RS &rs, const float *q) const {
        if (root < 0)
            return;
        float dists[3] = {0, 0, 0};
        float dist     = 0;
        for (int i = 0; i < 3; i++) {
            if (q[i] < rootBox[i].low) {
                dists[i] = (q[i] - rootBox[i].low) * (q[i] - rootBox[i].low);
                dist += dists[i];
            }
            if (q[i] > rootBox[i].high) {
                dists[i] = (q[i] - rootBox[i].high) * (q[i] - rootBox[i].high);
                dist += dists[i];
            }
        }
        searchLevel(rs, q, root, dist, dists);
    }

    void radiusSearch(const float *q, float r2, std::vector<std::pair<int, float>> &out) const {
        out.clear();
        RadiusSet rs{r2, &out};
        findNeighbors(rs, q);
    }

private:
    void computeMinMax(size_t ind, size_t count, int dim, float &mn, float &mx) const {
        mn = pt(vAcc[ind], dim);
        mx = mn;
        for (size_t i = 1; i < count; ++i) {
            float v = pt(vAcc[ind + i], dim);
            if (v < mn)
                mn = v;
            if (v > mx)
                mx = v;
        }
    }

    void planeSplit(size_t ind, size_t count, int cutfeat, float cutval, size_t &lim1,
                    size_t &lim2) {
        size_t left = 0, right = count - 1;
        for (;;) {
            while (left <= right && pt(vAcc[ind + left], cutfeat) < cutval)
                ++left;
            while (right && left <= right && pt(vAcc[ind + right], cutfeat) >= cutval)
                --right;
            if (left > right || !right)
                break;
            std::swap(vAcc[ind + left], vAcc[ind + right]);
            ++left;
            --right;
        }
        lim1  = left;
        right = count - 1;
        for (;;) {
            while (left <= right && pt(vAcc[ind + left], cutfeat) <= cutval)
                ++left;
            while (right && left <= right && pt(vAcc[ind + right], cutfeat) > cutval)
                --right;
            if (left > right || !right)
                break;
            std::swap(vAcc[ind + left], vAcc[ind + right]);
            ++left;
            --right;
        }
        lim2 = left;
    }

    void middleSplit(size_t ind, size_t count, size_t &index, int &cutfeat, float &cutval,
                     const Interval *bbox) {
        const float EPS      = 0.00001f;
        float       maxSpan  = bbox[0].high - bbox[0].low;
        for (int i = 1; i < 3; ++i) {
            float span = bbox[i].high - bbox[i].low;
            if (span > maxSpan)
                maxSpan = span;
        }
        float maxSpread = -1;
        cutfeat         = 0;
        float minElem = 0, maxElem = 0;
        for (int i = 0; i < 3; ++i) {
            float span = bbox[i].high - bbox[i].low;
            if (span > (1 - EPS) * maxSpan) {
                float mn, mx;
                computeMinMax(ind, count, i, mn, mx);
                float spread = mx - mn;
                if (spread > maxSpread) {
                    cutfeat   = i;
                    maxSpread = spread;
                    minElem   = mn;
                    maxElem   = mx;
                }
            }
        }
        float splitVal = (bbox[cutfeat].low + bbox[cutfeat].high) / 2;
        if (splitVal < minElem)
            cutval = minElem;
        else if (splitVal > maxElem)
            cutval = maxElem;
        else
            cutval = splitVal;
        size_t lim1, lim2;
        planeSplit(ind, count, cutfeat, cutval, lim1, lim2);
        if (lim1 > count / 2)
            index = lim1;
        else if (lim2 < count / 2)
            index = lim2;
        else
            index = count / 2;
    }

    int divide(size_t left, size_t right, Interval *bbox) {
        int id = (int)nodes.size();
        nodes.emplace_back();
        if ((right - left) <= leafMax) {
            nodes[id].left  = (int)left;
            nodes[id].right = (int)right;
            for (int i = 0; i < 3; ++i) {
                bbox[i].low  = pt(vAcc[left], i);
                bbox[i].high = pt(vAcc[left], i);
            }
            for (size_t k = left + 1; k < right; ++k) {
                for (int i = 0; i < 3; ++i) {
                    float v = pt(vAcc[k], i);
                    if (bbox[i].low > v)
                        bbox[i].low = v;
                    if (bbox[i].high < v)
                        bbox[i].high = v;
                }
            }
        } else {
            size_t idx;
            int    cutfeat;
            float  cutval;
            middleSplit(left, right - left, idx, cutfeat, cutval, bbox);
            nodes[id].divfeat = cutfeat;
            Interval lb[3] = {bbox[0], bbox[1], bbox[2]};
            lb[cutfeat].high = cutval;
            int c1           = divide(left, left + idx, lb);
            Interval rb[3] = {bbox[0], bbox[1], bbox[2]};
            rb[cutfeat].low = cutval;
            int c2          = divide(left + idx, right, rb);
            nodes[id].child1  = c1;
            nodes[id].child2  = c2;
            nodes[id].divlow  = lb[cutfeat].high;
            nodes[id].divhigh = rb[cutfeat].low;
            for (int i = 0; i < 3; ++i) {
                bbox[i].low  = std::min(lb[i].low, rb[i].low);
                bbox[i].high = std::max(lb[i].high, rb[i].high);
            }
        }
        return id;
    }

    template <class RS>
    bool searchLevel(RS &rs, const float *q, int nodeId, float mindist, float *dists) const {
        const KdNode &node = nodes[nodeId];
        if (node.child1 < 0) {
            float worst = rs.worst();
            for (int i = node.left; i < node.right; ++i) {
                int acc = vAcc[i];
                if (acc == -1)
                    continue;
                const V3 &p  = (*data)[acc];
                float     d0 = q[0] - p.x, d1 = q[1] - p.y, d2 = q[2] - p.z;
                float     d  = 0;
                d += d0 * d0;
                d += d1 * d1;
                d += d2 * d2;
                if (d < worst) {
                    if (!rs.add(d, acc))
                        return false;
                }
            }
            return true;
        }
        int   idx   = node.divfeat;
        float val   = q[idx];
        float diff1 = val - node.divlow;
        float diff2 = val - node.divhigh;
        int   best, other;
        float cutDist;
        if ((diff1 + diff2) < 0) {
            best    = node.child1;
            other   = node.child2;
            cutDist = (val - node.divhigh) * (val - node.divhigh);
        } else {
            best    = node.child2;
            other   = node.child1;
            cutDist = (val - node.divlow) * (val - node.divlow);
        }
        if (!searchLevel(rs, q, best, mindist, dists))
            return false;
        float dst  = dists[idx];
        mindist    = mindist + cutDist - dst;
        dists[idx] = cutDist;
        if (mindist * 1.0f <= rs.worst()) {
            if (!searchLevel(rs, q, other, mindist, dists))
                return false;
        }
        dists[idx] = dst;
        return true;
    }
};

} // namespace orc
