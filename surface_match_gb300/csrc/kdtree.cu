// kdtree.cu - the reference-order k-d tree on the GPU: build, searches, and the greedy
// sampler in tree order.
//
// Reference counterparts: KDTreeVectorOfVectorsAdaptor (kdtree/kdtree.h:52-161) over the
// vendored nanoflann (kdtree/nanoflann.hpp: divideTree 1120-1176, middleSplit_ 1290-1339,
// planeSplit 1352-1393, searchLevel 1846-1930) and samplePointCloud (util.cpp:107-139).
//
// Build. nanoflann splits a node's index range [left, right) recursively: the cut axis is
// the one of largest point spread among the axes whose box side is within (1 - 1e-5) of
// the widest, the cut value the box middle clamped to the points' range, and the range is
// reordered by two in-place Hoare passes (values < cut to the front, then values <= cut).
// Each pass has a closed form: with T the number of elements that go to the front, the
// j-th element of the front part that does not belong there is swapped with the j-th
// element from the back of the rear part that does - so a pass is a prefix sum and a
// batch of disjoint swaps. The GPU builds all nodes of one depth at once (segments of the
// position array, one kernel per step, prefix sums over the whole array) until every open
// range holds at most kSmall points; those finish in one CTA each, in shared memory, with
// the same steps. Node bounds are then tightened bottom-up (divlow/divhigh are the
// children's tight bounds, the root box becomes the tight box of all points, as nanoflann
// does through its by-reference bbox).
//
// Greedy sampling in tree order. The reference keeps a point unless an already kept point's
// radius search found it, visiting points in tree position order (util.cpp:107-139). Each
// point's fate depends only on the earlier points within the step: it is dropped once a
// kept one reaches it, and kept once all of them are decided and none of the kept ones
// reaches it. The GPU counts those earlier points per point (neighbourhoods from grid cells
// of side >= step, each cell's points in tree order), then decides points as their counts
// run out, through a device queue: every point is handled exactly once, and decisions
// travel along the dependency chains of the greedy order. "Reaches" is the reference's
// radius search membership: squared distance below step^2 and not pruned by the search
// above the point's leaf - decided by walking the point's root-to-leaf path
// (smk::kd_reaches) unless the distance bound proves the pruning cannot happen (points
// moved by normal estimation can leave their leaf's box).
#include <climits>
#include <cmath>

#include "sm_kdtree.cuh"
#include "sm_stages.h"

namespace sm {
using namespace smd;
using smk::KdView;

namespace {

struct GridParamsK {
    float org[3], g;
    int   dim[3];
};

constexpr int kSmall    = 1024; // ranges of at most this many points finish in one CTA
constexpr int kSmallSeg = 96;   // open sub-ranges per level inside that CTA (> 10 points each: <= 93)

// An open range of the build (one future node) and its split.
struct Seg {
    int   left, right, node, cutfeat;
    float lo[3], hi[3]; // the box nanoflann passes down (parent box cut at the split)
    int   mn[3], mx[3]; // ordered-int min / max of the points (computeMinMax)
    float cutval;
    int   index;    // split offset from left
    int   child[2]; // next-level segment of each child (-1: leaf or small range)
    int   depth;    // depth of the node (root 0)
};

// Lanes add their point's ordered coordinates to the bounds of their range (s < 0: none);
// a warp whose lanes share one range reduces first and adds once.
template <class S>
__device__ __forceinline__ void add_bounds(S *seg, int s, const float4 &p) {
    const int  o[3] = {f2ord(p.x), f2ord(p.y), f2ord(p.z)};
    const int  s0   = __shfl_sync(0xffffffffu, s, 0);
    const bool same = __all_sync(0xffffffffu, s == s0);
    if (same) {
        if (s0 < 0)
            return;
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = __reduce_min_sync(0xffffffffu, o[a]);
            hi[a] = __reduce_max_sync(0xffffffffu, o[a]);
        }
        if ((threadIdx.x & 31) == 0)
            for (int a = 0; a < 3; a++) {
                atomicMin(&seg[s0].mn[a], lo[a]);
                atomicMax(&seg[s0].mx[a], hi[a]);
            }
        return;
    }
    if (s >= 0)
        for (int a = 0; a < 3; a++) {
            atomicMin(&seg[s].mn[a], o[a]);
            atomicMax(&seg[s].mx[a], o[a]);
        }
}

__device__ __forceinline__ float coord_of(const float4 &p, int a) {
    return a == 0 ? p.x : (a == 1 ? p.y : p.z);
}

// middleSplit_'s choice of axis and cut value (nanoflann.hpp:1290-1329).
__device__ void choose_cut(const float lo[3], const float hi[3], const int mn[3], const int mx[3],
                           int &cutfeat, float &cutval) {
    const float EPS     = 0.00001f;
    float       maxSpan = hi[0] - lo[0];
    for (int i = 1; i < 3; ++i) {
        const float span = hi[i] - lo[i];
        if (span > maxSpan)
            maxSpan = span;
    }
    float maxSpread = -1.0f, minElem = 0.0f, maxElem = 0.0f;
    cutfeat = 0;
    for (int i = 0; i < 3; ++i) {
        const float span = hi[i] - lo[i];
        if (span > (1.0f - EPS) * maxSpan) {
            const float a = ord2f(mn[i]), b = ord2f(mx[i]);
            const float spread = b - a;
            if (spread > maxSpread) {
                cutfeat   = i;
                maxSpread = spread;
                minElem   = a;
                maxElem   = b;
            }
        }
    }
    const float splitVal = (lo[cutfeat] + hi[cutfeat]) / 2.0f;
    if (splitVal < minElem)
        cutval = minElem;
    else if (splitVal > maxElem)
        cutval = maxElem;
    else
        cutval = splitVal;
}

// middleSplit_'s split offset from the two partition limits (nanoflann.hpp:1333-1338).
__device__ __forceinline__ int split_index(int count, int lim1, int lim2) {
    if (lim1 > count / 2)
        return lim1;
    if (lim2 < count / 2)
        return lim2;
    return count / 2;
}

__device__ __forceinline__ int4 leaf_node(int l, int r) { return make_int4(l, r, -1, 0); }

// ---- top levels: one kernel per step over the whole position array -------------------
__global__ void k_kd_root(Seg *seg, Seg *small, int m, Box box, int4 *nd, int *parent, int *cnt) {
    Seg s{};
    s.left  = 0;
    s.right = m;
    s.node  = 0;
    s.depth = 0;
    for (int a = 0; a < 3; a++) {
        s.lo[a] = box.mn[a];
        s.hi[a] = box.mx[a];
        s.mn[a] = INT_MAX;
        s.mx[a] = INT_MIN;
    }
    s.child[0] = s.child[1] = -1;
    seg[0]     = s;
    parent[0]  = -1;
    cnt[0]     = 1;                    // nodes
    cnt[4]     = m > kSmall ? 1 : 0;  // open ranges of the first level
    if (m <= smk::kLeafMax) {
        nd[0] = leaf_node(0, m);
    } else if (m <= kSmall) {
        small[0] = s;                  // the whole cloud is one small range
        cnt[2]   = 1;
    }
}

__global__ void k_kd_init(const float4 *__restrict__ pos, const int *__restrict__ ids, int m,
                          float4 *__restrict__ rec, int *__restrict__ segOf, Seg *__restrict__ seg) {
    const int i  = blockIdx.x * blockDim.x + threadIdx.x;
    float4    p  = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < m) {
        const int id = ids[i];
        p            = pos[id];
        rec[i]       = make_float4(p.x, p.y, p.z, __int_as_float(id));
        segOf[i]     = 0;
    }
    add_bounds(seg, i < m ? 0 : -1, p);
}

__global__ void k_kd_cut(Seg *__restrict__ seg, const int *__restrict__ nseg) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *nseg)
        return;
    Seg &S = seg[s];
    choose_cut(S.lo, S.hi, S.mn, S.mx, S.cutfeat, S.cutval);
}

// pass 1: value < cut over [left, right); pass 2: value <= cut over [left + lim1, right)
__device__ __forceinline__ int pass_start(const Seg &S, int pass, const int *g1) {
    return pass == 1 ? S.left : S.left + (g1[S.right] - g1[S.left]);
}

__global__ void k_kd_flags(const float4 *__restrict__ rec, const int *__restrict__ segOf, int m,
                           const Seg *__restrict__ seg, int pass, const int *__restrict__ g1,
                           int *__restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > m)
        return;
    int f = 0;
    if (i < m) {
        const int s = segOf[i];
        if (s >= 0) {
            const Seg &S = seg[s];
            if (i >= pass_start(S, pass, g1)) {
                const float x = coord_of(rec[i], S.cutfeat);
                f             = pass == 1 ? (x < S.cutval) : (x <= S.cutval);
            }
        }
    }
    flag[i] = f;
}

// The back part's misplaced elements record their positions by rank from the back.
__global__ void k_kd_rank(const int *__restrict__ segOf, int m, const Seg *__restrict__ seg,
                          int pass, const int *__restrict__ g1, const int *__restrict__ flag,
                          const int *__restrict__ g, int *__restrict__ badR) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || !flag[i])
        return;
    const int s = segOf[i];
    if (s < 0)
        return;
    const Seg &S = seg[s];
    const int  a = pass_start(S, pass, g1);
    if (i < a)
        return;
    const int T = g[S.right] - g[a], lt = g[i] - g[a];
    if (i - a >= T)
        badR[a + (T - lt - 1)] = i;
}

// The front part's misplaced elements swap with their partners (disjoint pairs).
__global__ void k_kd_swap(float4 *__restrict__ rec, const int *__restrict__ segOf, int m,
                          const Seg *__restrict__ seg, int pass, const int *__restrict__ g1,
                          const int *__restrict__ flag, const int *__restrict__ g,
                          const int *__restrict__ badR) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || flag[i])
        return;
    const int s = segOf[i];
    if (s < 0)
        return;
    const Seg &S = seg[s];
    const int  a = pass_start(S, pass, g1);
    if (i < a)
        return;
    const int T = g[S.right] - g[a], lt = g[i] - g[a];
    if (i - a < T) {
        const int    p = badR[a + (i - a - lt)];
        const float4 x = rec[i];
        rec[i]         = rec[p];
        rec[p]         = x;
    }
}

// Children of every open range: nodes, leaves, small ranges and next-level ranges.
__global__ void k_kd_children(Seg *__restrict__ seg, const int *__restrict__ nseg,
                              const int *__restrict__ g1, const int *__restrict__ g2,
                              int4 *__restrict__ nd, int *__restrict__ parent,
                              int *__restrict__ nodeCount, Seg *__restrict__ next,
                              int *__restrict__ nnext, Seg *__restrict__ small,
                              int *__restrict__ nsmall, int *__restrict__ depthErr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= *nseg)
        return;
    Seg      &S     = seg[s];
    const int count = S.right - S.left;
    const int lim1  = g1[S.right] - g1[S.left];
    const int lim2  = lim1 + (g2[S.right] - g2[S.left + lim1]);
    const int index = split_index(count, lim1, lim2);
    S.index         = index;
    const int c1    = atomicAdd(nodeCount, 2);
    nd[S.node]      = make_int4(0, 0, c1 | (S.cutfeat << 30), S.left + index);
    if (S.depth + 1 >= smk::kMaxDepth)
        atomicExch(depthErr, 1);
    for (int k = 0; k < 2; k++) {
        const int l = k == 0 ? S.left : S.left + index;
        const int r = k == 0 ? S.left + index : S.right;
        Seg       C{};
        C.left  = l;
        C.right = r;
        C.node  = c1 + k;
        for (int a = 0; a < 3; a++) {
            C.lo[a] = S.lo[a];
            C.hi[a] = S.hi[a];
            C.mn[a] = INT_MAX;
            C.mx[a] = INT_MIN;
        }
        if (k == 0)
            C.hi[S.cutfeat] = S.cutval;
        else
            C.lo[S.cutfeat] = S.cutval;
        C.child[0] = C.child[1] = -1;
        C.depth    = S.depth + 1;
        parent[c1 + k]          = S.node;
        S.child[k]              = -1;
        if (r - l <= smk::kLeafMax) {
            nd[c1 + k] = leaf_node(l, r);
        } else if (r - l <= kSmall) {
            small[atomicAdd(nsmall, 1)] = C;
        } else {
            const int id = atomicAdd(nnext, 1);
            next[id]     = C;
            S.child[k]   = id;
        }
    }
}

// Next-level segment of every position, and the next level's point bounds.
__global__ void k_kd_advance(const float4 *__restrict__ rec, int *__restrict__ segOf, int m,
                             const Seg *__restrict__ seg, Seg *__restrict__ next) {
    const int i  = blockIdx.x * blockDim.x + threadIdx.x;
    int       ns = -1;
    float4    p  = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < m) {
        const int s = segOf[i];
        if (s >= 0) {
            const Seg &S = seg[s];
            ns           = S.child[i < S.left + S.index ? 0 : 1];
            segOf[i]     = ns;
            p            = rec[i];
        }
    }
    add_bounds(next, ns, p);
}

// ---- small ranges: one CTA of 1024 threads, one position per thread -------------------
struct SubSeg {
    int   left, right, node, cutfeat;
    float lo[3], hi[3];
    int   mn[3], mx[3];
    float cutval;
    int   index, child[2], depth;
};

__global__ void __launch_bounds__(kSmall)
    k_kd_small(const Seg *__restrict__ small, float4 *__restrict__ rec, int4 *__restrict__ nd,
               int *__restrict__ parent, int *__restrict__ nodeCount, int *__restrict__ err) {
    __shared__ float4 r[kSmall];
    __shared__ short  sid[kSmall];
    __shared__ int    sc1[kSmall + 1], sc2[kSmall + 1], bad[kSmall];
    __shared__ SubSeg ss[2][kSmallSeg];
    __shared__ int    nsub[2];
    __shared__ int    wsum[33];
    const Seg S0  = small[blockIdx.x];
    const int n   = S0.right - S0.left;
    const int t   = threadIdx.x;
    if (t < n)
        r[t] = rec[S0.left + t];
    sid[t] = (short)(t < n ? 0 : -1);
    if (t == 0) {
        SubSeg z{};
        z.left  = 0;
        z.right = n;
        z.node  = S0.node;
        z.depth = S0.depth;
        for (int a = 0; a < 3; a++) {
            z.lo[a] = S0.lo[a];
            z.hi[a] = S0.hi[a];
            z.mn[a] = INT_MAX;
            z.mx[a] = INT_MIN;
        }
        ss[0][0] = z;
        nsub[0]  = 1;
        nsub[1]  = 0;
    }
    __syncthreads();
    int cur = 0;
    while (nsub[cur] > 0) {
        SubSeg *L = ss[cur];
        SubSeg *N = ss[cur ^ 1];
        // point bounds per open range
        add_bounds(L, sid[t], r[t]);
        __syncthreads();
        if (t < nsub[cur])
            choose_cut(L[t].lo, L[t].hi, L[t].mn, L[t].mx, L[t].cutfeat, L[t].cutval);
        __syncthreads();
        for (int pass = 1; pass <= 2; pass++) {
            int *sc = pass == 1 ? sc1 : sc2;
            int  f  = 0;
            int  a  = 0;
            if (sid[t] >= 0) {
                const SubSeg &Q = L[sid[t]];
                a = pass == 1 ? Q.left : Q.left + (sc1[Q.right] - sc1[Q.left]);
                if (t >= a) {
                    const float x = coord_of(r[t], Q.cutfeat);
                    f             = pass == 1 ? (x < Q.cutval) : (x <= Q.cutval);
                }
            }
            int tot;
            const int ex = block_excl_scan(f, wsum, &tot);
            sc[t]        = ex;
            if (t == 0)
                sc[kSmall] = tot;
            __syncthreads();
            int T = 0, lt = 0;
            if (sid[t] >= 0 && t >= a) {
                const SubSeg &Q = L[sid[t]];
                T               = sc[Q.right] - sc[a];
                lt              = sc[t] - sc[a];
                if (f && t - a >= T)
                    bad[a + (T - lt - 1)] = t;
            }
            __syncthreads();
            float4 mine = r[t], other = mine;
            int    p    = -1;
            if (sid[t] >= 0 && t >= a && !f && t - a < T) {
                p     = bad[a + (t - a - lt)];
                other = r[p];
            }
            __syncthreads();
            if (p >= 0) {
                r[t] = other;
                r[p] = mine;
            }
            __syncthreads();
        }
        if (t == 0)
            nsub[cur ^ 1] = 0;
        __syncthreads();
        if (t < nsub[cur]) {
            SubSeg   &Q     = L[t];
            const int count = Q.right - Q.left;
            const int lim1  = sc1[Q.right] - sc1[Q.left];
            const int lim2  = lim1 + (sc2[Q.right] - sc2[Q.left + lim1]);
            const int index = split_index(count, lim1, lim2);
            Q.index         = index;
            const int c1    = atomicAdd(nodeCount, 2);
            nd[Q.node]      = make_int4(0, 0, c1 | (Q.cutfeat << 30), S0.left + Q.left + index);
            if (Q.depth + 1 >= smk::kMaxDepth)
                atomicExch(err, 1);
            for (int k = 0; k < 2; k++) {
                const int l = k == 0 ? Q.left : Q.left + index;
                const int rr = k == 0 ? Q.left + index : Q.right;
                parent[c1 + k] = Q.node;
                Q.child[k]     = -1;
                if (rr - l <= smk::kLeafMax) {
                    nd[c1 + k] = leaf_node(S0.left + l, S0.left + rr);
                } else {
                    const int id = atomicAdd(&nsub[cur ^ 1], 1);
                    if (id >= kSmallSeg) {
                        atomicExch(err, 2);
                        continue;
                    }
                    SubSeg C{};
                    C.left  = l;
                    C.right = rr;
                    C.node  = c1 + k;
                    C.depth = Q.depth + 1;
                    for (int a = 0; a < 3; a++) {
                        C.lo[a] = Q.lo[a];
                        C.hi[a] = Q.hi[a];
                        C.mn[a] = INT_MAX;
                        C.mx[a] = INT_MIN;
                    }
                    if (k == 0)
                        C.hi[Q.cutfeat] = Q.cutval;
                    else
                        C.lo[Q.cutfeat] = Q.cutval;
                    N[id]      = C;
                    Q.child[k] = id;
                }
            }
        }
        __syncthreads();
        if (t == 0 && nsub[cur ^ 1] > kSmallSeg)
            nsub[cur ^ 1] = 0; // overflow reported through err; stop
        if (sid[t] >= 0) {
            const SubSeg &Q = L[sid[t]];
            sid[t]          = (short)Q.child[t < Q.left + Q.index ? 0 : 1];
        }
        __syncthreads();
        cur ^= 1;
    }
    if (t < n)
        rec[S0.left + t] = r[t];
}

// ---- finish: tight boxes bottom-up, split bounds, per-position indexes ----------------
__global__ void k_kd_finish(int4 *__restrict__ nd, const int *__restrict__ parent,
                            const int *__restrict__ nodeCount, const float4 *__restrict__ rec,
                            float *__restrict__ box, int *__restrict__ arrive,
                            int *__restrict__ vacc, int *__restrict__ leafOf,
                            int *__restrict__ treePos) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= *nodeCount)
        return;
    const int4 n = nd[v];
    if (!smk::is_leaf(n))
        return;
    float lo[3], hi[3];
    {
        const float4 p = rec[n.x];
        lo[0] = hi[0] = p.x;
        lo[1] = hi[1] = p.y;
        lo[2] = hi[2] = p.z;
    }
    for (int i = n.x; i < n.y; i++) {
        const float4 p  = rec[i];
        const float  c3[3] = {p.x, p.y, p.z};
        for (int a = 0; a < 3; a++) {
            if (lo[a] > c3[a])
                lo[a] = c3[a];
            if (hi[a] < c3[a])
                hi[a] = c3[a];
        }
        const int id = __float_as_int(p.w);
        vacc[i]      = id;
        leafOf[i]    = v;
        treePos[id]  = i;
    }
    for (int a = 0; a < 3; a++) {
        box[6 * v + a]     = lo[a];
        box[6 * v + 3 + a] = hi[a];
    }
    // the second child to finish tightens the parent
    int u = v;
    for (;;) {
        const int p = parent[u];
        if (p < 0)
            return;
        __threadfence();
        if (atomicAdd(&arrive[p], 1) == 0)
            return;
        __threadfence();
        const int4 pn = nd[p];
        const int  c1 = smk::child1_of(pn), cf = smk::divfeat_of(pn);
        const volatile float *b1 = box + 6 * c1;
        const volatile float *b2 = box + 6 * (c1 + 1);
        for (int a = 0; a < 3; a++) {
            box[6 * p + a]     = fminf(b1[a], b2[a]);
            box[6 * p + 3 + a] = fmaxf(b1[3 + a], b2[3 + a]);
        }
        nd[p].x = __float_as_int(b1[3 + cf]); // divlow: child1's upper bound on the cut axis
        nd[p].y = __float_as_int(b2[cf]);     // divhigh: child2's lower bound
        u       = p;
    }
}

// ---- greedy sampling in tree order ---------------------------------------------------
constexpr uint32_t  kNoCell   = 1u << 23; // sort key of positions reduce() excluded
constexpr int       kSpBs     = 256;
constexpr long long kSpIdle   = 1ll << 22; // polls of an unwritten queue slot before giving up
constexpr int       kSpUnroll = 4;         // neighbourhood entries in flight per lane

struct SampleArgs {
    KdView          t;
    float           org[3], g;
    int             dim[3];
    const float4   *ent;      // cell runs: {x, y, z, tree position bits}, tree order in a run
    const float    *ex;       // the entries' excursions from their leaves' build-time boxes
    const int      *cellOf;   // per entry: its cell's occupied rank (-1 past the active ones)
    const int      *cellRank; // dense cell -> occupied rank (-1: empty)
    const int      *cellList; // occupied rank -> dense cell
    const int      *cellBeg;  // occupied rank -> its run [beg, end) of the entries
    const int      *cellEnd;
    int            *open;     // occupied rank -> its points not yet decided
    int            *cnt;      // per entry: earlier points within the step not yet decided
    int            *dec;      // per entry: 0 open, 1 kept, 2 dropped
    int            *queue;    // entries in the order they were decided (-1: not written)
    int            *head, *tail;
    const int      *nact;     // number of entries of active points (device)
    int             m;
    float           r2;
    double          safe2;
    int            *keptFlag; // per tree position
    int            *err;      // a bounded wait expired
};

__device__ __forceinline__ int ld_vol(const int *p) { return *(const volatile int *)p; }

// Distance of a (moved) point from its leaf's build-time box.
__device__ __forceinline__ double excursion(const float *box, const float4 &p) {
    const float c[3] = {p.x, p.y, p.z};
    double      s    = 0.0;
    for (int a = 0; a < 3; a++) {
        const double lo = box[a], hi = box[3 + a], x = c[a];
        const double o  = x < lo ? lo - x : (x > hi ? x - hi : 0.0);
        s += o * o;
    }
    return sqrt(s);
}

// Whether the radius search from kept point q reaches the point p at tree position ip
// (radiusSearch membership, nanoflann.hpp:1736-1749): distance first; the search's
// lower bound at any node above p's leaf is at most (|q - p| + excursion)^2, so the path
// walk is needed only near the radius or for points that left their leaf's box. The
// margin covers the float rounding of the search's running bound.
__device__ __forceinline__ bool reaches(const SampleArgs &a, const float4 &q, const float4 &p,
                                        int ip, double e) {
    const float qq[3] = {q.x, q.y, q.z};
    const float d     = smk::eval_metric(qq, p);
    if (!(d < a.r2))
        return false;
    const double b = sqrt((double)d) + e;
    if (b * b < a.safe2)
        return true;
    uint64_t key;
    return smk::kd_reaches(a.t, qq, ip, a.r2, &key);
}

__global__ void k_sp_keys(const int *__restrict__ vaccA, const float4 *__restrict__ pos, int m,
                          GridParamsK gp, uint32_t *__restrict__ key, uint32_t *__restrict__ val) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const int id = vaccA[i];
    uint32_t  k  = kNoCell;
    if (id >= 0) {
        const float4 p  = pos[id];
        const int    cx = smg::coord(p.x, gp.org[0], gp.g, gp.dim[0]);
        const int    cy = smg::coord(p.y, gp.org[1], gp.g, gp.dim[1]);
        const int    cz = smg::coord(p.z, gp.org[2], gp.g, gp.dim[2]);
        k               = (uint32_t)((cz * gp.dim[1] + cy) * gp.dim[0] + cx);
    }
    key[i] = k;
    val[i] = (uint32_t)i;
}

__global__ void k_sp_heads(const uint32_t *__restrict__ key, int m, int *__restrict__ head) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k > m)
        return;
    head[k] = (k < m && key[k] != kNoCell && (k == 0 || key[k - 1] != key[k])) ? 1 : 0;
}

__global__ void k_sp_cells(const uint32_t *__restrict__ key, int m, const int *__restrict__ head,
                           const int *__restrict__ rank, int *__restrict__ cellRank,
                           int *__restrict__ cellList, int *__restrict__ cellBeg,
                           int *__restrict__ cellEnd, int *__restrict__ cellOf,
                           int *__restrict__ open, int *__restrict__ nact) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m)
        return;
    if (key[k] == kNoCell) {
        cellOf[k] = -1;
        return;
    }
    const int r = rank[k] + head[k] - 1; // the run's occupied rank
    cellOf[k]   = r;
    atomicAdd(&open[r], 1);
    if (head[k]) {
        cellRank[key[k]] = r;
        cellList[r]      = (int)key[k];
        cellBeg[r]       = k;
    }
    if (k == m - 1 || key[k + 1] != key[k])
        cellEnd[r] = k + 1;
    if (k == m - 1 || key[k + 1] == kNoCell)
        *nact = k + 1; // the active entries sort first
}

// The cell runs' points in run order: {x, y, z, tree position bits} and the point's
// excursion from its leaf's build-time box.
__global__ void k_sp_entries(const uint32_t *__restrict__ sortPos, int m, KdView t,
                             const float *__restrict__ nodeBox, const int *__restrict__ leafOf,
                             float4 *__restrict__ ent, float *__restrict__ ex) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m)
        return;
    const int ip = (int)sortPos[k];
    const int id = t.vacc[ip];
    if (id < 0)
        return;
    const float4 p = t.pos[id];
    ent[k]         = make_float4(p.x, p.y, p.z, __int_as_float(ip));
    ex[k]          = (float)excursion(nodeBox + 6 * (size_t)leafOf[ip], p);
}

// The 27 cells around a cell: lane l < 27 gets the first entry of neighbour l's run; returns
// the lane's exclusive prefix of the runs' lengths and writes their total to tot.
// With onlyOpen, cells whose points are all decided count as empty: a decided point needs
// nothing from its neighbours any more.
__device__ __forceinline__ int nb_runs(const SampleArgs &a, int cid, int &nb, int &tot,
                                       bool onlyOpen) {
    const int lane = threadIdx.x & 31;
    const int cx = cid % a.dim[0], cy = (cid / a.dim[0]) % a.dim[1], cz = cid / (a.dim[0] * a.dim[1]);
    nb      = 0;
    int len = 0;
    if (lane < 27) {
        const int x = cx + lane % 3 - 1, y = cy + (lane / 3) % 3 - 1, z = cz + lane / 9 - 1;
        if (x >= 0 && y >= 0 && z >= 0 && x < a.dim[0] && y < a.dim[1] && z < a.dim[2]) {
            const int nr = a.cellRank[(z * a.dim[1] + y) * a.dim[0] + x];
            if (nr >= 0 && !(onlyOpen && ld_vol(&a.open[nr]) == 0)) {
                nb  = a.cellBeg[nr];
                len = a.cellEnd[nr] - nb;
            }
        }
    }
    const int incl = warp_incl_scan(len);
    tot            = __shfl_sync(0xffffffffu, incl, 31);
    return incl - len;
}

// Entry of flattened neighbourhood index t: binary search over the lanes' prefixes.
__device__ __forceinline__ int nb_entry(int t, int excl, int nb) {
    int lo = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1) {
        const int mid = lo + step;
        const int ev  = __shfl_sync(0xffffffffu, excl, mid & 31);
        if (mid < 27 && ev <= t)
            lo = mid;
    }
    return __shfl_sync(0xffffffffu, nb, lo) + (t - __shfl_sync(0xffffffffu, excl, lo));
}

// Step 1, a warp per point p: the earlier points (lower tree position) within the step of
// p - squared distance from that point to p below step^2, the first test of its radius
// search. p's decision waits for theirs. Points without any are kept at once and queued.
__global__ void __launch_bounds__(kSpBs) k_sp_count(SampleArgs a) {
    const int lane = threadIdx.x & 31;
    const int nw   = (int)(((long long)gridDim.x * blockDim.x) >> 5);
    for (int k = (int)((blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5); k < a.m; k += nw) {
        if (a.cellOf[k] < 0)
            break; // past the active entries
        const float4 p  = a.ent[k];
        const int    ip = __float_as_int(p.w);
        int          nb, tot;
        const int    excl = nb_runs(a, a.cellList[a.cellOf[k]], nb, tot, false);
        int          cnt  = 0;
        for (int base = 0; base < tot; base += 32 * kSpUnroll) {
            int    kb[kSpUnroll];
            float4 b[kSpUnroll];
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                kb[u] = nb_entry(min(base + u * 32 + lane, tot - 1), excl, nb);
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                b[u] = a.ent[max(kb[u], 0)];
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                if (base + u * 32 + lane < tot && __float_as_int(b[u].w) < ip) {
                    const float bq[3] = {b[u].x, b[u].y, b[u].z};
                    cnt += smk::eval_metric(bq, p) < a.r2 ? 1 : 0;
                }
        }
        cnt = __reduce_add_sync(0xffffffffu, cnt);
        if (lane == 0) {
            a.cnt[k] = cnt;
            if (cnt == 0) {
                a.dec[k]                      = 1;
                a.queue[atomicAdd(a.tail, 1)] = k;
                atomicSub(&a.open[a.cellOf[k]], 1);
            }
        }
    }
}

// Decide entry p (open -> fate) and queue it, unless it is decided already.
__device__ __forceinline__ void sp_push(const SampleArgs &a, int p, int fate) {
    if (atomicCAS(&a.dec[p], 0, fate) == 0) {
        atomicSub(&a.open[a.cellOf[p]], 1);
        const int slot = atomicAdd(a.tail, 1);
        __threadfence();
        atomicExch(&a.queue[slot], p);
    }
}

// Step 2, a warp per queued point b, in queue order (every active point is queued exactly
// once). A kept b drops every later point its search reaches (and queues it); every other
// later point within the step that is still open counts b as decided, and the last of its
// earlier points to be decided queues it as kept. Dropping happens before counting, so a
// point that a kept point reaches never runs out of count. Each queued point waits only on
// points queued before it, so the warps that took the earliest slots always progress.
__global__ void __launch_bounds__(kSpBs) k_sp_run(SampleArgs a) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int slot = 0;
        if (lane == 0)
            slot = atomicAdd(a.head, 1);
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot >= *a.nact)
            return;
        int b = -1;
        if (lane == 0) {
            for (long long it = 0;; it++) {
                b = ld_vol(&a.queue[slot]);
                if (b >= 0)
                    break;
                if (ld_vol(a.err) || it > kSpIdle) {
                    atomicExch(a.err, 1);
                    break;
                }
                __nanosleep(32);
            }
        }
        b = __shfl_sync(0xffffffffu, b, 0);
        if (b < 0)
            return;
        __threadfence();
        const int    fate = ld_vol(&a.dec[b]);
        const float4 q    = a.ent[b];
        const int    iq   = __float_as_int(q.w);
        if (fate == 1 && lane == 0)
            a.keptFlag[iq] = 1;
        int         nb, tot;
        // only neighbour cells that still hold an undecided point: after a kept point's
        // wave of drops most cells around a dropped point are settled
        const int   excl  = nb_runs(a, a.cellList[a.cellOf[b]], nb, tot, true);
        const float qq[3] = {q.x, q.y, q.z};
        for (int base = 0; base < tot; base += 32 * kSpUnroll) {
            int    kp[kSpUnroll];
            float4 p[kSpUnroll];
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                kp[u] = nb_entry(min(base + u * 32 + lane, tot - 1), excl, nb);
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                p[u] = a.ent[max(kp[u], 0)];
            // the later points within the step that are still open
            bool live[kSpUnroll];
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                live[u] = base + u * 32 + lane < tot && __float_as_int(p[u].w) > iq &&
                          smk::eval_metric(qq, p[u]) < a.r2;
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                live[u] = live[u] && ld_vol(&a.dec[kp[u]]) == 0;
            bool count[kSpUnroll];
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++) {
                count[u] = false;
                if (!live[u])
                    continue;
                if (fate == 1 && reaches(a, q, p[u], __float_as_int(p[u].w), (double)a.ex[kp[u]])) {
                    sp_push(a, kp[u], 2);
                    continue;
                }
                count[u] = true;
            }
            __threadfence();
            int old[kSpUnroll];
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                old[u] = count[u] ? atomicSub(&a.cnt[kp[u]], 1) : 0;
#pragma unroll
            for (int u = 0; u < kSpUnroll; u++)
                if (old[u] == 1) {
                    __threadfence();
                    sp_push(a, kp[u], 1);
                }
        }
    }
}

__global__ void k_sp_out(const int *__restrict__ flag, const int *__restrict__ pre, int m,
                         const int *__restrict__ vaccA, int *__restrict__ outIds,
                         int *__restrict__ ioi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const bool kept = flag[i] != 0;
    if (kept)
        outIds[pre[i]] = vaccA[i];
    if (ioi)
        ioi[i] = kept ? vaccA[i] : -1;
}

// ---- k-nearest searches on the tree (one query per thread) -----------------------------
// Query t: position qpos[t], or pos[list[t]] when qpos is null; t < *nq (device count).
// Writes its k nearest ids in the reference's order (distance, then first found) and
// their squared distances; cnt[t] = how many were found.
__global__ void k_kd_knn(KdView t, const float4 *__restrict__ qpos, const int *__restrict__ list,
                         const int *__restrict__ nq, int k, int *__restrict__ nbr,
                         float *__restrict__ dist, int *__restrict__ cnt, int *__restrict__ err,
                         const float4 *__restrict__ nrm, int *__restrict__ need) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= *nq)
        return;
    const float4 p    = qpos ? qpos[i] : t.pos[list[i]];
    const float  q[3] = {p.x, p.y, p.z};
    smk::KnnSet<kMaxKnn> rs;
    rs.init(k);
    if (!smk::kd_search(t, q, rs))
        atomicExch(err, 1);
    for (int j = 0; j < k; j++) {
        const int id           = j < rs.count ? rs.idx[j] : -1;
        nbr[(size_t)i * k + j] = id;
        if (dist)
            dist[(size_t)i * k + j] = rs.dist[j];
        // with smoothing, neighbours that still need a normal are marked for estimation
        if (need && id >= 0 && need[id] == 0) {
            const float4 n = nrm[id];
            if (!(isfinite(n.x) && isfinite(n.y) && isfinite(n.z)))
                need[id] = 1;
        }
    }
    if (cnt)
        cnt[i] = rs.count;
}

// ---- the voting stage's radius searches (ppf.cpp:273-276) -------------------------------
constexpr int kRlBs  = 256;
constexpr int kTailN = 7; // rows % 8 < 8

struct TailKey {
    uint64_t key;
    int                pos, cand; // tree position, candidate index
};
__device__ __forceinline__ bool tail_after(const TailKey &a, const TailKey &b) {
    return a.key > b.key || (a.key == b.key && a.pos > b.pos);
}

// One CTA per keypoint over the candidates (the sampled points): membership of the radius
// search of radius^2 r2 in the reduced tree (distance and the search's pruning), as a
// bitmask over the candidate list; the member count; and the candidates of the last
// (rows mod 8) rows other than the keypoint itself in the search's depth-first order -
// the rows the reference evaluates one by one after its 8-lane blocks.
__global__ void __launch_bounds__(kRlBs)
    k_kd_radius(KdView t, const int *__restrict__ treePos, const int *__restrict__ kp, int K,
                const int *__restrict__ cand, int ncand, float r2, uint32_t *__restrict__ mask,
                int words, int *__restrict__ count, int *__restrict__ tail) {
    __shared__ TailKey sk[kRlBs];
    __shared__ int     sh[33];
    const int c = blockIdx.x;
    if (c >= K)
        return;
    const int    pid  = kp[c];
    const float4 p    = t.pos[pid];
    const float  q[3] = {p.x, p.y, p.z};
    TailKey      top[kTailN];
    for (int k = 0; k < kTailN; k++)
        top[k] = TailKey{0ull, -1, -1};
    int       nTop = 0, S = 0;
    bool      self = false;
    uint32_t *mrow = mask + (size_t)c * words;
    for (int j0 = 0; j0 < ncand; j0 += kRlBs) {
        const int j   = j0 + threadIdx.x;
        bool      mem = false;
        if (j < ncand) {
            const int id = cand[j];
            const float d = smk::eval_metric(q, t.pos[id]);
            if (d < r2) {
                const int ip = treePos[id];
                uint64_t  key;
                mem = smk::kd_reaches(t, q, ip, r2, &key);
                self = self || (mem && id == pid);
                if (mem && id != pid) {
                    TailKey e{key, ip, j};
                    // keep the kTailN latest in search order, sorted latest first
                    int at = nTop < kTailN ? nTop : kTailN;
                    while (at > 0 && tail_after(e, top[at - 1]))
                        at--;
                    if (at < kTailN) {
                        for (int k = (nTop < kTailN ? nTop : kTailN - 1); k > at; k--)
                            top[k] = top[k - 1];
                        top[at] = e;
                        if (nTop < kTailN)
                            nTop++;
                    }
                }
            }
        }
        const uint32_t b = __ballot_sync(0xffffffffu, mem);
        if ((threadIdx.x & 31) == 0 && ((j0 + threadIdx.x) >> 5) < words)
            mrow[(j0 + threadIdx.x) >> 5] = b;
        S += mem ? 1 : 0;
    }
    int tot;
    block_excl_scan(S, sh, &tot);
    // rows = the members other than the keypoint (which its own search finds)
    const int rows = tot - (__syncthreads_or(self ? 1 : 0) ? 1 : 0);
    const int need = rows % 8;
    // the `need` latest rows: rounds of a block-wide maximum over the threads' lists
    int head = 0;
    for (int r = 0; r < need; r++) {
        sk[threadIdx.x] = head < nTop ? top[head] : TailKey{0ull, -1, -1};
        __syncthreads();
        for (int o = kRlBs / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o && tail_after(sk[threadIdx.x + o], sk[threadIdx.x]))
                sk[threadIdx.x] = sk[threadIdx.x + o];
            __syncthreads();
        }
        const TailKey w = sk[0];
        if (head < nTop && top[head].pos == w.pos && top[head].cand == w.cand)
            head++;
        if (threadIdx.x == 0)
            tail[(size_t)c * kTailN + r] = w.cand;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        count[c] = tot;
        for (int r = need; r < kTailN; r++)
            tail[(size_t)c * kTailN + r] = -1;
    }
}

// The CSR list of keypoint blockIdx.x: its members in candidate order except the tail
// rows, then the tail rows (the voting stage marks the last rows % 8 rows of a list as the
// reference's one-by-one rows).
__global__ void __launch_bounds__(kRlBs)
    k_kd_fill(const uint32_t *__restrict__ mask, int words, const int *__restrict__ cand,
              int ncand, const int *__restrict__ off, const int *__restrict__ tail,
              int *__restrict__ ids) {
    __shared__ int sh[33];
    __shared__ int sT[kTailN];
    const int c = blockIdx.x;
    if (threadIdx.x < kTailN)
        sT[threadIdx.x] = tail[(size_t)c * kTailN + threadIdx.x];
    __syncthreads();
    int nt = 0;
    for (int k = 0; k < kTailN; k++)
        nt += sT[k] >= 0 ? 1 : 0;
    const uint32_t *mrow = mask + (size_t)c * words;
    int            *out  = ids + off[c];
    const int       len  = off[c + 1] - off[c];
    int             base = 0;
    for (int j0 = 0; j0 < ncand; j0 += kRlBs) {
        const int j  = j0 + threadIdx.x;
        bool      in = j < ncand && ((mrow[j >> 5] >> (j & 31)) & 1u);
        if (in)
            for (int k = 0; k < kTailN; k++)
                if (sT[k] == j)
                    in = false;
        int       tot;
        const int ex = block_excl_scan(in ? 1 : 0, sh, &tot);
        if (in)
            out[base + ex] = cand[j];
        base += tot;
    }
    // the tail rows last, in search order (earliest first)
    if (threadIdx.x == 0)
        for (int k = nt - 1, o = len - nt; k >= 0; k--, o++)
            out[o] = cand[sT[k]];
}

// Leaves holding an active position flag themselves and their ancestors (a walk stops at
// an ancestor another walk has flagged).
__global__ void k_kd_nonempty(const int4 *__restrict__ nd, const int *__restrict__ parent,
                              int nnodes, const int *__restrict__ vacc, int *__restrict__ flags) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nnodes)
        return;
    const int4 n = nd[v];
    if (!smk::is_leaf(n))
        return;
    bool any = false;
    for (int i = n.x; i < n.y && !any; i++)
        any = vacc[i] >= 0;
    for (int u = v; any && u >= 0; u = parent[u])
        if (atomicExch(&flags[u], 1) == 1)
            break;
}

__global__ void k_kd_tpos(const int *__restrict__ vacc, int m, const float4 *__restrict__ pos,
                          float4 *__restrict__ tpos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const int id = vacc[i];
    if (id < 0) {
        tpos[i] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        return;
    }
    const float4 p = pos[id];
    tpos[i]        = make_float4(p.x, p.y, p.z, __int_as_float(id));
}

} // namespace

// =======================================================================================
void build_kdtree(Ctx &c, const float4 *pos, int npoints, const int *ids, int m, const Box &box,
                  KdTree &T, const std::string &tag) {
    if (m >= (1 << 28))
        throw Error(SM_ERR_CAPACITY, "k-d tree over more than 2^28 points is not supported");
    T.m       = m;
    T.npoints = npoints;
    const int cap = std::max(2 * m, 1);
    T.nd      = c.arena.get<int4>(tag + ".nd", cap);
    T.box     = c.arena.get<float>(tag + ".box", (size_t)6 * cap);
    T.vacc    = c.arena.get<int>(tag + ".vacc", std::max(m, 1));
    T.leafOf  = c.arena.get<int>(tag + ".leaf", std::max(m, 1));
    T.treePos = c.arena.get<int>(tag + ".tpos", std::max(npoints, 1));
    T.rec     = c.arena.get<float4>(tag + ".rec", std::max(m, 1));
    int *parent  = c.arena.get<int>(tag + ".par", cap);
    T.parent     = parent;
    int *arrive  = c.arena.get<int>(tag + ".arr", cap);
    int *cnt     = c.arena.get<int>(tag + ".cnt", 8); // nodes, nnext, nsmall, err
    int *segOf   = c.arena.get<int>(tag + ".segof", std::max(m, 1));
    int *flag    = c.arena.get<int>(tag + ".flag", (size_t)m + 1);
    int *g1      = c.arena.get<int>(tag + ".g1", (size_t)m + 1);
    int *g2      = c.arena.get<int>(tag + ".g2", (size_t)m + 1);
    int *badR    = c.arena.get<int>(tag + ".badr", std::max(m, 1));
    const int maxSeg = std::max(m / (smk::kLeafMax + 1) + 2, 2);
    Seg *segA  = c.arena.get<Seg>(tag + ".segA", maxSeg);
    Seg *segB  = c.arena.get<Seg>(tag + ".segB", maxSeg);
    Seg *small = c.arena.get<Seg>(tag + ".small", maxSeg);
    SM_CUDA(cudaMemsetAsync(cnt, 0, 8 * sizeof(int), c.stream));
    SM_CUDA(cudaMemsetAsync(T.treePos, 0xff, (size_t)std::max(npoints, 1) * 4, c.stream));
    if (m == 0)
        return;
    int *nseg = cnt + 4; // open ranges of the current level (device)
    k_kd_root<<<1, 1, 0, c.stream>>>(segA, small, m, box, T.nd, parent, cnt);
    SM_LAUNCH_CHECK();
    k_kd_init<<<nblocks(m, 256), 256, 0, c.stream>>>(pos, ids, m, T.rec, segOf, segA);
    SM_LAUNCH_CHECK();
    int hostSeg = m > kSmall ? 1 : 0;
    Seg *cur = segA, *nxt = segB;
    const int gm = nblocks((long long)m + 1, 256);
    while (hostSeg > 0) {
        k_kd_cut<<<nblocks(hostSeg, 128), 128, 0, c.stream>>>(cur, nseg);
        SM_LAUNCH_CHECK();
        for (int pass = 1; pass <= 2; pass++) {
            int *g = pass == 1 ? g1 : g2;
            k_kd_flags<<<gm, 256, 0, c.stream>>>(T.rec, segOf, m, cur, pass, g1, flag);
            SM_LAUNCH_CHECK();
            scan_excl(c, flag, g, (long long)m + 1, tag + ".scan", false);
            k_kd_rank<<<gm, 256, 0, c.stream>>>(segOf, m, cur, pass, g1, flag, g, badR);
            SM_LAUNCH_CHECK();
            k_kd_swap<<<gm, 256, 0, c.stream>>>(T.rec, segOf, m, cur, pass, g1, flag, g, badR);
            SM_LAUNCH_CHECK();
        }
        SM_CUDA(cudaMemsetAsync(cnt + 1, 0, sizeof(int), c.stream));
        k_kd_children<<<nblocks(hostSeg, 128), 128, 0, c.stream>>>(
            cur, nseg, g1, g2, T.nd, parent, cnt, nxt, cnt + 1, small, cnt + 2, cnt + 3);
        SM_LAUNCH_CHECK();
        k_kd_advance<<<nblocks(m, 256), 256, 0, c.stream>>>(T.rec, segOf, m, cur, nxt);
        SM_LAUNCH_CHECK();
        SM_CUDA(cudaMemcpyAsync(nseg, cnt + 1, sizeof(int), cudaMemcpyDeviceToDevice, c.stream));
        SM_CUDA(cudaMemcpyAsync(c.hostCounts, cnt, 4 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        c.sync_checked();
        hostSeg = c.hostCounts[1];
        std::swap(cur, nxt);
        if (c.hostCounts[3])
            throw Error(SM_ERR_CAPACITY, "k-d tree deeper than " + std::to_string(smk::kMaxDepth));
    }
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, cnt, 4 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync_checked();
    const int nsmall = c.hostCounts[2];
    if (nsmall > 0) {
        k_kd_small<<<nsmall, kSmall, 0, c.stream>>>(small, T.rec, T.nd, parent, cnt, cnt + 3);
        SM_LAUNCH_CHECK();
    }
    SM_CUDA(cudaMemsetAsync(arrive, 0, (size_t)cap * 4, c.stream));
    k_kd_finish<<<nblocks(cap, 256), 256, 0, c.stream>>>(T.nd, parent, cnt, T.rec, T.box, arrive,
                                                         T.vacc, T.leafOf, T.treePos);
    SM_LAUNCH_CHECK();
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, cnt, 4 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync_checked();
    T.nnodes = c.hostCounts[0];
    if (c.hostCounts[3] == 1)
        throw Error(SM_ERR_CAPACITY, "k-d tree deeper than " + std::to_string(smk::kMaxDepth));
    if (c.hostCounts[3] == 2)
        throw Error(SM_ERR_CAPACITY, "k-d tree build: too many open ranges in a small range");
}

int kd_sample(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos, float step,
              const Box &box, int *outIds, int *ioi, const std::string &tag) {
    const int m = T.m;
    if (m <= 0)
        return 0;
    const int *vaccA = vaccActive ? vaccActive : T.vacc;
    float      ext[3] = {box.ext(0), box.ext(1), box.ext(2)};
    GridParamsK gp;
    gp.g = smg::sample_cell(step, ext);
    for (int a = 0; a < 3; a++) {
        gp.org[a] = box.mn[a];
        gp.dim[a] = smg::dim_of(ext[a], gp.g);
    }
    const long long nc = (long long)gp.dim[0] * gp.dim[1] * gp.dim[2];
    uint32_t *key   = c.arena.get<uint32_t>(tag + ".key", m);
    uint32_t *val   = c.arena.get<uint32_t>(tag + ".val", m);
    int      *head  = c.arena.get<int>(tag + ".head", (size_t)m + 1);
    int      *rank  = c.arena.get<int>(tag + ".rank", (size_t)m + 1);
    int      *cRank = c.arena.get<int>(tag + ".crank", nc);
    k_sp_keys<<<nblocks(m, 256), 256, 0, c.stream>>>(vaccA, pos, m, gp, key, val);
    SM_LAUNCH_CHECK();
    radix_sort_pairs(c, key, val, m, 24, tag);
    k_sp_heads<<<nblocks((long long)m + 1, 256), 256, 0, c.stream>>>(key, m, head);
    SM_LAUNCH_CHECK();
    const int ncells = scan_excl(c, head, rank, (long long)m + 1, tag + ".hs", true);
    int    *cellList = c.arena.get<int>(tag + ".clist", std::max(ncells, 1));
    int    *cellBeg  = c.arena.get<int>(tag + ".cbeg", std::max(ncells, 1));
    int    *cellEnd  = c.arena.get<int>(tag + ".cend", std::max(ncells, 1));
    int    *cellOf   = c.arena.get<int>(tag + ".cof", m);
    float4 *ent      = c.arena.get<float4>(tag + ".ent", m);
    float  *ex       = c.arena.get<float>(tag + ".ex", m);
    int    *cnt      = c.arena.get<int>(tag + ".cnt", m);
    int    *open     = c.arena.get<int>(tag + ".open", std::max(ncells, 1));
    int    *dec      = c.arena.get<int>(tag + ".dec", m);
    int    *queue    = c.arena.get<int>(tag + ".q", m);
    int    *flag     = c.arena.get<int>(tag + ".flag", (size_t)m + 1);
    int    *ctl      = c.arena.get<int>(tag + ".ctl", 4); // head, tail, active entries, error
    SM_CUDA(cudaMemsetAsync(cRank, 0xff, (size_t)nc * 4, c.stream));
    SM_CUDA(cudaMemsetAsync(flag, 0, ((size_t)m + 1) * 4, c.stream));
    SM_CUDA(cudaMemsetAsync(ctl, 0, 4 * sizeof(int), c.stream));
    SM_CUDA(cudaMemsetAsync(dec, 0, (size_t)m * 4, c.stream));
    SM_CUDA(cudaMemsetAsync(open, 0, (size_t)std::max(ncells, 1) * 4, c.stream));
    SM_CUDA(cudaMemsetAsync(queue, 0xff, (size_t)m * 4, c.stream));
    k_sp_cells<<<nblocks(m, 256), 256, 0, c.stream>>>(key, m, head, rank, cRank, cellList, cellBeg,
                                                     cellEnd, cellOf, open, ctl + 2);
    SM_LAUNCH_CHECK();
    k_sp_entries<<<nblocks(m, 256), 256, 0, c.stream>>>(val, m, T.view(vaccA, pos), T.box,
                                                        T.leafOf, ent, ex);
    SM_LAUNCH_CHECK();
    SampleArgs a{};
    a.t = T.view(vaccA, pos);
    for (int d = 0; d < 3; d++) {
        a.org[d] = gp.org[d];
        a.dim[d] = gp.dim[d];
    }
    a.g        = gp.g;
    a.ent      = ent;
    a.ex       = ex;
    a.cellOf   = cellOf;
    a.cellRank = cRank;
    a.cellList = cellList;
    a.cellBeg  = cellBeg;
    a.cellEnd  = cellEnd;
    a.cnt      = cnt;
    a.open     = open;
    a.dec      = dec;
    a.queue    = queue;
    a.head     = ctl;
    a.tail     = ctl + 1;
    a.nact     = ctl + 2;
    a.m        = m;
    a.r2       = step * step;
    a.safe2    = (double)a.r2 * (1.0 - 1e-4);
    a.keptFlag = flag;
    a.err      = ctl + 3;
    if (ncells > 0) {
        int nsm = 0;
        SM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
        const int wpb = kSpBs / 32;
        k_sp_count<<<std::min(nblocks(m, wpb), nsm * 16), kSpBs, 0, c.stream>>>(a);
        SM_LAUNCH_CHECK();
        // the queue's consumers: each queued point is taken by one warp, in queue order
        k_sp_run<<<std::min(nblocks(m, wpb), nsm * 4), kSpBs, 0, c.stream>>>(a);
        SM_LAUNCH_CHECK();
    }
    int *pre = c.arena.get<int>(tag + ".pre", (size_t)m + 1);
    scan_excl(c, flag, pre, (long long)m + 1, tag + ".os", false);
    k_sp_out<<<nblocks(m, 256), 256, 0, c.stream>>>(flag, pre, m, vaccA, outIds, ioi);
    SM_LAUNCH_CHECK();
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, pre + m, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SM_CUDA(cudaMemcpyAsync(c.hostCounts + 1, ctl + 3, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync_checked();
    if (c.hostCounts[1])
        throw Error(SM_ERR_RUNTIME, "tree-order sampler: a bounded wait expired");
    return c.hostCounts[0];
}

void kd_knn(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos,
            const float4 *qpos, const int *list, const int *nq, int nqMax, int k, int *nbr,
            float *dist, int *cnt, const float4 *nrm, int *need) {
    if (nqMax <= 0 || T.m <= 0)
        return;
    if (k < 1 || k > kMaxKnn)
        throw Error(SM_ERR_RANGE, "knnNormal larger than " + std::to_string(kMaxKnn) + " is not supported");
    int    *err  = c.arena.get<int>("kd.knn.err", 1);
    float4 *tpos = c.arena.get<float4>("kd.knn.tpos", T.m);
    SM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
    kd_tree_positions(c, T, vaccActive, pos, tpos);
    k_kd_knn<<<nblocks(nqMax, 128), 128, 0, c.stream>>>(T.view(vaccActive, pos, nullptr, tpos), qpos,
                                                        list, nq, k, nbr, dist, cnt, err, nrm, need);
    SM_LAUNCH_CHECK();
}

int kd_vote_lists(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos,
                  const int *kp, int K, const int *cand, int ncand, float r2, int **offOut,
                  int **idsOut, const std::string &tag) {
    int *off = c.arena.get<int>(tag + ".off", (size_t)K + 1);
    *offOut  = off;
    if (K <= 0) {
        *idsOut = c.arena.get<int>(tag + ".ids", 1);
        return 0;
    }
    const int words = std::max((ncand + 31) / 32, 1);
    uint32_t *mask  = c.arena.get<uint32_t>(tag + ".mask", (size_t)K * words);
    int      *cnt   = c.arena.get<int>(tag + ".cnt", (size_t)K + 1);
    int      *tail  = c.arena.get<int>(tag + ".tail", (size_t)K * kTailN);
    SM_CUDA(cudaMemsetAsync(mask, 0, (size_t)K * words * 4, c.stream));
    SM_CUDA(cudaMemsetAsync(cnt + K, 0, sizeof(int), c.stream));
    k_kd_radius<<<K, kRlBs, 0, c.stream>>>(T.view(vaccActive, pos), T.treePos, kp, K, cand, ncand,
                                            r2, mask, words, cnt, tail);
    SM_LAUNCH_CHECK();
    const int total = scan_excl(c, cnt, off, (long long)K + 1, tag + ".scan", true);
    int      *ids   = c.arena.get<int>(tag + ".ids", std::max(total, 1));
    *idsOut         = ids;
    k_kd_fill<<<K, kRlBs, 0, c.stream>>>(mask, words, cand, ncand, off, tail, ids);
    SM_LAUNCH_CHECK();
    return total;
}

void kd_mark_nonempty(Ctx &c, const KdTree &T, const int *vaccActive, int *flags) {
    if (T.nnodes <= 0)
        return;
    SM_CUDA(cudaMemsetAsync(flags, 0, (size_t)T.nnodes * 4, c.stream));
    k_kd_nonempty<<<nblocks(T.nnodes, 256), 256, 0, c.stream>>>(T.nd, T.parent, T.nnodes,
                                                                vaccActive ? vaccActive : T.vacc,
                                                                flags);
    SM_LAUNCH_CHECK();
}

void kd_tree_positions(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos,
                       float4 *tpos) {
    if (T.m <= 0)
        return;
    k_kd_tpos<<<nblocks(T.m, 256), 256, 0, c.stream>>>(vaccActive ? vaccActive : T.vacc, T.m, pos,
                                                        tpos);
    SM_LAUNCH_CHECK();
}

} // namespace sm
