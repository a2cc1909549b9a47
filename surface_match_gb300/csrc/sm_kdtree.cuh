// sm_kdtree.cuh - device view of the reference-order k-d tree and its searches.
//
// The reference searches its scene through a locally modified nanoflann k-d tree
// (kdtree/kdtree.h:52-161, kdtree/nanoflann.hpp v0x155): middle-split nodes, leaves of at
// most 10 points, depth-first search that visits the nearer child first and the farther
// one only while the accumulated lower bound `mindist` stays within the result set's worst
// distance (nanoflann.hpp:1846-1930), leaf entries equal to INVALID_INDEX skipped (the
// reduce() of kdtree.h:146-157). Every result of the reference that depends on search
// order or pruning - which points a radius search finds after points have moved, which of
// equally distant points a k-nearest search keeps, the order of a radius search's results
// - follows from that procedure. The functions here are that procedure, one query per
// thread, on a tree built on the GPU with the reference's split rules (kdtree.cu).
//
// Node layout (one int4 per node, so a search step is one load):
//   internal: {divlow bits, divhigh bits, child1 | divfeat << 30, split}; child2 = child1+1,
//             child1 holds the tree positions [node left, split); child1 < 2^30, so the
//             word is never -1 (it is negative for divfeat 2)
//   leaf:     {left, right, -1, 0}: tree positions [left, right) of vacc
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sm_math.h"

namespace smk {

constexpr int kLeafMax  = 10; // leaf_max_size (kdtree.h:67, ppf.cpp:197)
constexpr int kMaxDepth = 64; // deepest supported tree (the build fails loudly beyond)

struct KdView {
    const int4   *nd;   // nodes (root = 0)
    const float  *box;  // root's tight box: lo xyz, hi xyz (nanoflann's root_bbox_)
    const int    *vacc; // per tree position: point id, or -1 where reduce() excluded it
    const float4 *pos;  // live point positions by id (normal estimation moves points)
    // per node: nonzero when its subtree holds a point of vacc (nullptr: all do). A search
    // that skips a subtree without points finds and changes nothing the reference's would
    // not: entering it adds no point and its bounds are restored on the way out.
    const int    *nonEmpty = nullptr;
    // tree-ordered live positions, w = point id bits (-1: excluded); when set, a leaf scan
    // reads one record per entry instead of vacc and then pos
    const float4 *tpos = nullptr;
};

__device__ __forceinline__ bool is_leaf(const int4 &n) { return n.z == -1; }
__device__ __forceinline__ int  child1_of(const int4 &n) { return n.z & 0x3FFFFFFF; }
__device__ __forceinline__ int  divfeat_of(const int4 &n) { return (n.z >> 30) & 3; }

// computeInitialDistances (nanoflann.hpp:1950-1970): per-axis squared distance of the query
// to the root box and their sum, accumulated in axis order.
__device__ __forceinline__ float init_dists(const KdView &t, const float q[3], float d[3]) {
    float s = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        d[a]           = 0.0f;
        const float lo = t.box[a], hi = t.box[3 + a];
        if (q[a] < lo) {
            d[a] = (q[a] - lo) * (q[a] - lo);
            s += d[a];
        }
        if (q[a] > hi) {
            d[a] = (q[a] - hi) * (q[a] - hi);
            s += d[a];
        }
    }
    return s;
}

// L2_Adaptor::evalMetric for 3 components: ((0 + d0^2) + d1^2) + d2^2 with d = q - p.
__device__ __forceinline__ float eval_metric(const float q[3], const float4 &p) {
    const float d0 = q[0] - p.x, d1 = q[1] - p.y, d2 = q[2] - p.z;
    float       d  = 0.0f;
    d += d0 * d0;
    d += d1 * d1;
    d += d2 * d2;
    return d;
}

// KNNResultSet (nanoflann.hpp:180-233) for k <= K: insertion by strict '>', so of equally
// distant points the first one found stays first; worst = the k-th distance (max float
// until k points are held).
template <int K> struct KnnSet {
    int   idx[K];
    float dist[K];
    int   cap, count;
    __device__ void init(int k) {
        cap   = k;
        count = 0;
#pragma unroll
        for (int i = 0; i < K; i++) {
            idx[i]  = -1;
            dist[i] = 3.402823466e38f;
        }
    }
    __device__ __forceinline__ float worst() const { return dist[cap - 1]; }
    __device__ __forceinline__ void add(float d, int id, int /*pos*/) {
        int i;
        for (i = count; i > 0; --i) {
            if (dist[i - 1] > d) {
                if (i < cap) {
                    dist[i] = dist[i - 1];
                    idx[i]  = idx[i - 1];
                }
            } else {
                break;
            }
        }
        if (i < cap) {
            dist[i] = d;
            idx[i]  = id;
        }
        if (count < cap)
            count++;
    }
};

// The one-nearest result set (KNNResultSet with capacity 1).
struct NnSet {
    int   idx;
    float dist;
    int   count;
    __device__ void init() {
        idx   = -1;
        dist  = 3.402823466e38f;
        count = 0;
    }
    __device__ __forceinline__ float worst() const { return dist; }
    __device__ __forceinline__ void add(float d, int id, int) {
        if (!(dist > d) && count > 0)
            return;
        dist  = d;
        idx   = id;
        count = 1;
    }
};

// findNeighbors + searchLevel (nanoflann.hpp:1846-1930) iteratively: a frame per pending
// far child keeps the node's entry state, so the far child is entered exactly when and
// with the bound the recursion would use. Returns false when the tree is deeper than the
// frame stack (the build rejects such trees, so this does not happen).
template <class RS> __device__ bool kd_search(const KdView &t, const float q[3], RS &rs) {
    struct Frame {
        int   other, idx;
        float cut, mind, d[3];
    };
    Frame st[kMaxDepth];
    int   sp = 0;
    float dists[3];
    float mindist = init_dists(t, q, dists);
    int   v       = 0;
    for (;;) {
        const int4 n = t.nd[v];
        if (is_leaf(n)) {
            const float worst = rs.worst();
            for (int i = n.x; i < n.y; i++) {
                float4 p;
                int    id;
                if (t.tpos) {
                    p  = t.tpos[i];
                    id = __float_as_int(p.w);
                    if (id < 0)
                        continue;
                } else {
                    id = t.vacc[i];
                    if (id < 0)
                        continue;
                    p = t.pos[id];
                }
                const float d = eval_metric(q, p);
                if (d < worst)
                    rs.add(d, id, i);
            }
            // resume the deepest pending far child that passes its bound
            v = -1;
            while (sp > 0) {
                const Frame &f   = st[--sp];
                const float  dst = f.d[f.idx];
                const float  md  = f.mind + f.cut - dst;
                if (md * 1.0f <= rs.worst()) {
                    dists[0]      = f.d[0];
                    dists[1]      = f.d[1];
                    dists[2]      = f.d[2];
                    dists[f.idx]  = f.cut;
                    mindist       = md;
                    v             = f.other;
                    break;
                }
            }
            if (v < 0)
                return true;
            continue;
        }
        const int   idx   = divfeat_of(n);
        const float val   = q[idx];
        const float dlow  = __int_as_float(n.x), dhigh = __int_as_float(n.y);
        const float diff1 = val - dlow, diff2 = val - dhigh;
        const int   c1    = child1_of(n);
        int         best, other;
        float       cut;
        if ((diff1 + diff2) < 0.0f) {
            best  = c1;
            other = c1 + 1;
            cut   = (val - dhigh) * (val - dhigh);
        } else {
            best  = c1 + 1;
            other = c1;
            cut   = (val - dlow) * (val - dlow);
        }
        const bool bestIn  = !t.nonEmpty || t.nonEmpty[best];
        const bool otherIn = !t.nonEmpty || t.nonEmpty[other];
        if (bestIn) {
            if (otherIn) {
                if (sp >= kMaxDepth)
                    return false;
                Frame &f = st[sp++];
                f.other  = other;
                f.idx    = idx;
                f.cut    = cut;
                f.mind   = mindist;
                f.d[0]   = dists[0];
                f.d[1]   = dists[1];
                f.d[2]   = dists[2];
            }
            v = best;
            continue;
        }
        // the near child holds no point: its search would return at once, so the far child
        // is checked now with the bound the search computes after it
        if (otherIn) {
            const float dst = dists[idx];
            const float md  = mindist + cut - dst;
            if (md * 1.0f <= rs.worst()) {
                dists[idx] = cut;
                mindist    = md;
                v          = other;
                continue;
            }
        }
        // neither child is entered: resume the deepest pending far child
        v = -1;
        while (sp > 0) {
            const Frame &f   = st[--sp];
            const float  dst = f.d[f.idx];
            const float  md  = f.mind + f.cut - dst;
            if (md * 1.0f <= rs.worst()) {
                dists[0]     = f.d[0];
                dists[1]     = f.d[1];
                dists[2]     = f.d[2];
                dists[f.idx] = f.cut;
                mindist      = md;
                v            = f.other;
                break;
            }
        }
        if (v < 0)
            return true;
    }
}

// Whether a radius search of radius^2 `worst` from q reaches tree position `ip` without
// being pruned above it (the leaf's own `dist < worst` test is the caller's), and the
// position's depth-first rank key for that query: bit (63 - depth) set where the path takes
// the far child, so that larger keys are visited later. The walk follows the search's
// steps along the root-to-leaf path of `ip`: the bound changes only where the path enters
// a far child.
__device__ __forceinline__ bool kd_reaches(const KdView &t, const float q[3], int ip, float worst,
                                           uint64_t *key) {
    float    dists[3];
    float    mindist = init_dists(t, q, dists);
    uint64_t k       = 0;
    int      depth   = 0;
    int      v       = 0;
    for (;;) {
        const int4 n = t.nd[v];
        if (is_leaf(n))
            break;
        const int   idx    = divfeat_of(n);
        const float val    = q[idx];
        const float dlow   = __int_as_float(n.x), dhigh = __int_as_float(n.y);
        const bool  best1  = ((val - dlow) + (val - dhigh)) < 0.0f;
        const bool  in1    = ip < n.w;
        if (in1 != best1) {
            const float cut = best1 ? (val - dhigh) * (val - dhigh) : (val - dlow) * (val - dlow);
            const float dst = dists[idx];
            mindist         = mindist + cut - dst;
            dists[idx]      = cut;
            if (!(mindist * 1.0f <= worst))
                return false;
            if (depth < 64)
                k |= 1ull << (63 - depth);
        }
        v = child1_of(n) + (in1 ? 0 : 1);
        depth++;
    }
    *key = k;
    return true;
}

} // namespace smk
