// icp.cu - pose refinement and scoring of matchScene (ppf.cpp:422-495): ICP::regist
// (icp.cpp:214-278) with findCorresponds (icp.cpp:123-167), the symmetric point-to-plane
// step (icp.cpp:39-121) and inliner (util.cpp:628-641).
//
// All candidates are refined at once; the searches spread each candidate's source points
// over many CTAs, so the whole GPU works even for a handful of candidates. One ICP iteration
// is four launches: correspondences (one warp per source point on the grid cell walker; per
// scene point the closest source point wins a 64-bit atomicMin of (distance bits, source
// index), which is the reference's "first minimum in model order" without its O(n*m)
// grouping scan); pair selection, pair count, centroids, normal-equation terms and the FP64
// solve in one thread-block cluster per candidate; residual distances; and their reduction +
// the convergence logic in one cluster per candidate. Every reduction has the same fixed
// layout: kIcpSlots slots (slot = source index mod kIcpSlots, a thread each), each a Kahan sum
// over its source points in ascending order, merged by a fixed tree (warp, the CTA's warps,
// then the cluster's CTAs through distributed shared memory) - the layout the CPU oracle
// emulates, so poses are bit-identical. The selection walk over the candidates
// (numMatches) runs on the host afterwards and only reads the per-candidate results.
#include <cfloat>

#include <cooperative_groups.h>

#include "sm_icp.h"
#include "sm_stages.h"

namespace sm {
using namespace smd;
namespace cg = cooperative_groups;

namespace {

constexpr int kT  = 256;              // search CTAs: a warp (or a thread) per point
constexpr int kW  = kT / 32;
constexpr int kR  = smi::kIcpThreads; // reduction CTAs: a slot per thread
constexpr int kRW = kR / 32;
constexpr int kRC = smi::kIcpBlocks;  // reduction CTAs per candidate: one thread-block cluster
constexpr int kFitU = 4;              // pairs whose loads a reduction thread has in flight
constexpr int kTraceIters  = 32;
constexpr int kTraceFloats = 2 * kTraceIters * 4 + 2;

// Per-candidate state, resident in global memory across the launches of one refinement.
struct Cand {
    smi::Pose34 M, keep, step;
    float       Pm[3], Qm[3];
    float       resMse, mse, score;
    int         cnt, iterations, converged, stop, status, active, inl, pad;
};

struct Stage {
    const float4 *src, *srcN; // model points / normals
    int           n, nb;      // points, CTAs per candidate
    HGridView     G;          // scene subset grid (pts.w = subset rank)
    const float4 *dPos, *dNrm; // the subset's positions / normals by rank
    int           nDst;
    int           iters;
    float         mseMin, mseMax, rej2;
    int           traceOff; // 0 sparse, 1 dense
    // reference search order: nearest points from the k-d tree reduced to the stage's
    // subset (rankOf maps a point id to its subset rank); tree.nd == nullptr: the grid G
    smk::KdView   tree;
    const int    *rankOf;
};

struct Work {
    Cand               *cand;
    const float4       *pos, *nrm;
    int                *nnId;   // ncand x maxSrc: subset rank of the pair's scene point (-1 none)
    int                *nnR;    // ncand x maxSrc: the same, kept through pair selection
    int                *nnPrev; // ncand x maxSrc: nearest subset point of the last iteration
    float4             *x4;     // ncand x maxSrc: moved source point, w = squared distance
    float4             *n4;     // ncand x maxSrc: rotated source normal
    float              *resid;  // ncand x maxSrc: residual distance of each pair
    unsigned long long *win;    // ncand x maxDst
    int                 maxSrc, maxDst;
    float              *trace;  // ncand x kTraceFloats (nullable)
    unsigned long long *live;   // (candidate, source point) searches of K1 (nullable: not counted)
};

__device__ __forceinline__ unsigned long long win_key(float d, int i) {
    return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)i;
}

__device__ __forceinline__ bool cand_live(const Cand &c, const Stage &s) {
    return c.active && !c.stop && c.iterations < s.iters;
}

// K1: correspondences, one warp per source point (warp-cooperative grid search)
__global__ void __launch_bounds__(kT, 4) k_corr(Work w, Stage s, int usePrev) {
    chain_enter(); // launched chained
    const int ci   = blockIdx.y;
    const int lane = threadIdx.x & 31;
    int       i    = blockIdx.x * kW + (threadIdx.x >> 5);
    // the first source point is read together with the candidate's state
    float4 sp = i < s.n ? s.src[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 sn = i < s.n ? s.srcN[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const Cand &C = w.cand[ci];
    if (!cand_live(C, s))
        return; // (a candidate that is not live has no nearest points of this stage)
    if (w.live && blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(w.live, (unsigned long long)s.n);
    for (; i < s.n; i += gridDim.x * kW) {
        const size_t o = (size_t)ci * w.maxSrc + i;
        float4       x, y;
        if (i != blockIdx.x * kW + (threadIdx.x >> 5)) {
            sp = s.src[i];
            sn = s.srcN[i];
        }
        // written by this candidate's previous iteration of this stage (usePrev: not the
        // first iteration), a rank of this stage's subset or -1
        const int jp = usePrev ? w.nnPrev[o] : -1;
        float4    qp = make_float4(0.f, 0.f, 0.f, 0.f);
        if (jp >= 0 && jp < s.nDst)
            qp = s.dPos[jp];
        smi::pose_apply(C.M, sp.x, sp.y, sp.z, x.x, x.y, x.z);
        smi::pose_rotate(C.M, sn.x, sn.y, sn.z, y.x, y.y, y.z);
        // the last iteration's nearest point of this stage bounds the search exactly
        float lim = s.rej2;
        if (jp >= 0 && jp < s.nDst)
            lim = fminf(lim, smm::dist2(x.x, x.y, x.z, qp.x, qp.y, qp.z));
        float      d;
        const int  j  = warp_nn_walk(s.G, x.x, x.y, x.z, lim, d); // subset rank
        const bool ok = j >= 0 && d <= s.rej2;
        if (lane == 0) {
            w.nnPrev[o] = j;
            x.w         = d;
            y.w         = 0.0f;
            w.x4[o]     = x;
            w.n4[o]     = y;
            w.nnId[o]   = ok ? j : -1;
            w.nnR[o]    = ok ? j : -1;
            if (ok)
                atomicMin(&w.win[(size_t)ci * w.maxDst + j], win_key(d, i));
        }
    }
}

// K1 with the reference's search: one thread per source point, the nearest point of the
// reduced k-d tree (findClosestPoint, util.cpp:603-626: a 1-nearest search from the root,
// with the tree's pruning) - the same pair rules as k_corr.
__global__ void __launch_bounds__(kT) k_corr_tree(Work w, Stage s) {
    chain_enter(); // launched chained
    const int   ci = blockIdx.y;
    const Cand &C  = w.cand[ci];
    if (!cand_live(C, s))
        return;
    if (w.live && blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(w.live, (unsigned long long)s.n);
    for (int i = blockIdx.x * kT + threadIdx.x; i < s.n; i += gridDim.x * kT) {
        const size_t o  = (size_t)ci * w.maxSrc + i;
        const float4 sp = s.src[i], sn = s.srcN[i];
        float4       x, y;
        smi::pose_apply(C.M, sp.x, sp.y, sp.z, x.x, x.y, x.z);
        smi::pose_rotate(C.M, sn.x, sn.y, sn.z, y.x, y.y, y.z);
        const float q[3] = {x.x, x.y, x.z};
        smk::NnSet  rs;
        rs.init();
        smk::kd_search(s.tree, q, rs);
        const int   j  = rs.count ? s.rankOf[rs.idx] : -1;
        const float d  = rs.dist;
        const bool  ok = j >= 0 && d <= s.rej2;
        w.nnPrev[o] = j;
        x.w         = d;
        y.w         = 0.0f;
        w.x4[o]     = x;
        w.n4[o]     = y;
        w.nnId[o]   = ok ? j : -1;
        w.nnR[o]    = ok ? j : -1;
        if (ok)
            atomicMin(&w.win[(size_t)ci * w.maxDst + j], win_key(d, i));
    }
}

// K4 with the reference's search: residual of each pair, one thread per pair.
__global__ void __launch_bounds__(kT) k_resid_tree(Work w, Stage s) {
    chain_enter(); // launched chained
    const int   ci = blockIdx.y;
    const Cand &C  = w.cand[ci];
    if (!cand_live(C, s) || C.cnt < 6)
        return;
    for (int i = blockIdx.x * kT + threadIdx.x; i < s.n; i += gridDim.x * kT) {
        const size_t o = (size_t)ci * w.maxSrc + i;
        if (w.nnId[o] < 0)
            continue;
        const float4 x = w.x4[o];
        float        y[3];
        smi::pose_apply(C.step, x.x, x.y, x.z, y[0], y[1], y[2]);
        smk::NnSet rs;
        rs.init();
        smk::kd_search(s.tree, y, rs);
        w.resid[o] = smm::fsqrt(rs.dist);
    }
}

// The reductions of one refinement iteration run in one thread-block cluster of kRC CTAs
// (kR threads each) per candidate, with the fixed layout of sm_icp.h: slot t (CTA t / kR,
// thread t % kR) sums, with Kahan, the terms of the pairs i = t, t + kIcpSlots, ... in
// ascending order; each CTA merges its slots by the tree (warp shfl_down offsets 16..1, then
// warp 0 over the warp partials, offsets kRW/2..1) and publishes its totals in its shared
// memory; rank 0 reads the kRC partials through distributed shared memory and merges them
// by the block tree (offsets kRC/2..1). No global fence or counter between CTAs, and the
// centroids, the normal equations and the solve share one launch.
template <int W> __device__ void block_tree(smi::KahanF (&v)[W], float (*red)[W][2]) {
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1)
        for (int k = 0; k < W; k++) {
            smi::KahanF o;
            o.s = __shfl_down_sync(0xffffffffu, v[k].s, off);
            o.c = __shfl_down_sync(0xffffffffu, v[k].c, off);
            v[k].merge(o);
        }
    if (lane == 0)
        for (int k = 0; k < W; k++) {
            red[wp][k][0] = v[k].s;
            red[wp][k][1] = v[k].c;
        }
    __syncthreads();
    if (wp == 0) {
        for (int k = 0; k < W; k++) {
            v[k].s = lane < kRW ? red[lane][k][0] : 0.f;
            v[k].c = lane < kRW ? red[lane][k][1] : 0.f;
        }
#pragma unroll
        for (int off = kRW / 2; off >= 1; off >>= 1)
            for (int k = 0; k < W; k++) {
                smi::KahanF o;
                o.s = __shfl_down_sync(0xffffffffu, v[k].s, off);
                o.c = __shfl_down_sync(0xffffffffu, v[k].c, off);
                v[k].merge(o);
            }
    }
    __syncthreads(); // red may be reused
}

__device__ __forceinline__ int block_sum_int(int x, int *red) {
    x = __reduce_add_sync(0xffffffffu, x);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = x;
    __syncthreads();
    int t = 0;
    for (int k = 0; k < kRW; k++)
        t += red[k];
    __syncthreads();
    return t;
}

// Rank 0's warp 0: the cluster's kRC published partials (lane r < kRC reads CTA r's through
// distributed shared memory), merged by the block tree; lane 0 ends with the totals.
template <int W>
__device__ void cluster_merge(cg::cluster_group &cl, float (*part)[2], smi::KahanF (&v)[W]) {
    const int lane = threadIdx.x & 31;
    for (int k = 0; k < W; k++) {
        float ps = 0.f, pc = 0.f;
        if (lane < kRC) {
            const float *rp = cl.map_shared_rank(&part[k][0], (unsigned)lane);
            ps              = rp[0];
            pc              = rp[1];
        }
        v[k].s = ps;
        v[k].c = pc;
    }
#pragma unroll
    for (int off = kRC / 2; off >= 1; off >>= 1)
        for (int k = 0; k < W; k++) {
            smi::KahanF o;
            o.s = __shfl_down_sync(0xffffffffu, v[k].s, off);
            o.c = __shfl_down_sync(0xffffffffu, v[k].c, off);
            v[k].merge(o);
        }
}

// K2: pair selection (the closest source point per scene point: the atomicMin winner), pair
// count and centroids, then the normal-equation terms of the pairs and the FP64 solve.
__global__ void __cluster_dims__(kRC, 1, 1) __launch_bounds__(kR) k_fit(Work w, Stage s) {
    chain_enter(); // launched chained
    __shared__ float red[kRW][smi::kNumSystem][2];
    __shared__ float part[smi::kNumSystem][2]; // this CTA's totals, read by rank 0
    __shared__ int   ired[kRW];
    __shared__ int   pcnt;
    __shared__ float sPQ[6]; // rank 0: the centroids, read by every CTA
    __shared__ int   sTotal;
    cg::cluster_group cl = cg::this_cluster();
    const int         rk = (int)cl.block_rank();
    const int         ci = blockIdx.x / kRC;
    Cand             &C  = w.cand[ci];
    if (!cand_live(C, s))
        return; // (the whole cluster: one candidate)
    int          *nnId = w.nnId + (size_t)ci * w.maxSrc;
    const int    *nnR  = w.nnR + (size_t)ci * w.maxSrc;
    const float4 *x4   = w.x4 + (size_t)ci * w.maxSrc;
    const float4 *n4   = w.n4 + (size_t)ci * w.maxSrc;
    const int     slot = rk * kR + threadIdx.x;
    smi::KahanF   m[6];
    for (int k = 0; k < 6; k++)
        m[k].init();
    // a thread's pairs i = slot, slot + kIcpSlots, ... in ascending order, kFitU of them
    // loaded at once (their loads are independent; the sums still take them in order)
    int cnt = 0;
    for (int base = slot; base < s.n; base += kFitU * smi::kIcpSlots) {
        int                r[kFitU];
        float4             x[kFitU], q[kFitU];
        unsigned long long wk[kFitU];
#pragma unroll
        for (int u = 0; u < kFitU; u++) {
            const int i = base + u * smi::kIcpSlots;
            r[u]        = i < s.n ? nnR[i] : -1;
        }
#pragma unroll
        for (int u = 0; u < kFitU; u++) {
            wk[u] = 0ull;
            if (r[u] >= 0) {
                x[u]  = x4[base + u * smi::kIcpSlots];
                wk[u] = w.win[(size_t)ci * w.maxDst + r[u]];
                q[u]  = s.dPos[r[u]];
            }
        }
#pragma unroll
        for (int u = 0; u < kFitU; u++) {
            const int i = base + u * smi::kIcpSlots;
            if (r[u] < 0)
                continue;
            if (wk[u] != win_key(x[u].w, i)) {
                nnId[i] = -1; // this thread reads it again below
                continue;
            }
            cnt++;
            m[0].add(x[u].x);
            m[1].add(x[u].y);
            m[2].add(x[u].z);
            m[3].add(q[u].x);
            m[4].add(q[u].y);
            m[5].add(q[u].z);
        }
    }
    const int cntB = block_sum_int(cnt, ired);
    block_tree<6>(m, reinterpret_cast<float (*)[6][2]>(&red[0][0][0]));
    if (threadIdx.x == 0) {
        for (int k = 0; k < 6; k++) {
            part[k][0] = m[k].s;
            part[k][1] = m[k].c;
        }
        pcnt = cntB;
    }
    cl.sync(); // the partials are published
    if (rk == 0 && threadIdx.x < 32) {
        smi::KahanF mm[6];
        cluster_merge<6>(cl, part, mm);
        if (threadIdx.x == 0) {
            int total = 0;
            for (int r = 0; r < kRC; r++)
                total += *cl.map_shared_rank(&pcnt, (unsigned)r);
            const float fc = (float)total;
            for (int k = 0; k < 3; k++) {
                C.Pm[k]    = smm::fdiv(mm[k].value(), fc);
                C.Qm[k]    = smm::fdiv(mm[3 + k].value(), fc);
                sPQ[k]     = C.Pm[k];
                sPQ[3 + k] = C.Qm[k];
            }
            C.cnt  = total;
            sTotal = total;
        }
    }
    cl.sync(); // rank 0 has read the partials and published the centroids
    const float *pq    = cl.map_shared_rank(sPQ, 0u);
    const float  Pm0   = pq[0], Pm1 = pq[1], Pm2 = pq[2];
    const float  Qm0   = pq[3], Qm1 = pq[4], Qm2 = pq[5];
    const int    total = *cl.map_shared_rank(&sTotal, 0u);
    cl.sync(); // every CTA has read rank 0's centroids (rank 0 may leave after this)
    if (total < 6)
        return;
    smi::KahanF v[smi::kNumSystem];
    for (int k = 0; k < smi::kNumSystem; k++)
        v[k].init();
    for (int base = slot; base < s.n; base += 2 * smi::kIcpSlots) {
        int    id[2];
        float4 x[2], xn[2], q[2], qn[2];
#pragma unroll
        for (int u = 0; u < 2; u++) {
            const int i = base + u * smi::kIcpSlots;
            id[u]       = i < s.n ? nnId[i] : -1;
        }
#pragma unroll
        for (int u = 0; u < 2; u++)
            if (id[u] >= 0) {
                const int i = base + u * smi::kIcpSlots;
                x[u]        = x4[i];
                xn[u]       = n4[i];
                q[u]        = s.dPos[id[u]];
                qn[u]       = s.dNrm[id[u]];
            }
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (id[u] < 0)
                continue;
            float t[smi::kNumSystem];
            smi::system_terms(x[u].x - Pm0, x[u].y - Pm1, x[u].z - Pm2, q[u].x - Qm0,
                              q[u].y - Qm1, q[u].z - Qm2, xn[u].x + qn[u].x, xn[u].y + qn[u].y,
                              xn[u].z + qn[u].z, t);
            for (int k = 0; k < smi::kNumSystem; k++)
                v[k].add(t[k]);
        }
    }
    block_tree<smi::kNumSystem>(v, red);
    if (threadIdx.x == 0)
        for (int k = 0; k < smi::kNumSystem; k++) {
            part[k][0] = v[k].s;
            part[k][1] = v[k].c;
        }
    cl.sync(); // the partials are published
    if (rk == 0 && threadIdx.x < 32) {
        cluster_merge<smi::kNumSystem>(cl, part, v);
        cl.sync(); // (rank 0 has read every partial: the others may leave)
        // the totals are on lane 0; warp 0 solves with one row of the system per lane
        float sys[smi::kNumSystem];
        for (int k = 0; k < smi::kNumSystem; k++)
            sys[k] = __shfl_sync(0xffffffffu, v[k].value(), 0);
        const float       pm[3] = {Pm0, Pm1, Pm2}, qm[3] = {Qm0, Qm1, Qm2};
        const smi::Pose34 st    = smi::solve_step_warp(sys, pm, qm);
        if (threadIdx.x == 0)
            C.step = st;
    } else {
        cl.sync();
    }
}

// K4: residual distance of each pair after the step, one warp per pair
__global__ void __launch_bounds__(kT, 5) k_resid(Work w, Stage s) {
    chain_enter(); // launched chained
    const int   ci = blockIdx.y;
    const Cand &C  = w.cand[ci];
    if (!cand_live(C, s) || C.cnt < 6)
        return;
    for (int i = blockIdx.x * kW + (threadIdx.x >> 5); i < s.n; i += gridDim.x * kW) {
        const size_t o = (size_t)ci * w.maxSrc + i;
        if (w.nnId[o] < 0)
            continue;
        const float4 x = w.x4[o];
        const float4 q = s.dPos[w.nnId[o]];
        float        y0, y1, y2, d;
        smi::pose_apply(C.step, x.x, x.y, x.z, y0, y1, y2);
        // the pair's scene point bounds the search exactly
        warp_nn_walk(s.G, y0, y1, y2, smm::dist2(y0, y1, y2, q.x, q.y, q.z), d);
        if ((threadIdx.x & 31) == 0)
            w.resid[(size_t)ci * w.maxSrc + i] = smm::fsqrt(d);
    }
}

// K5: mean residual, the regist loop logic (icp.cpp:233-272), winner reset; one cluster per
// candidate (the same layout as K2), rank 0's thread 0 runs the logic
__global__ void __cluster_dims__(kRC, 1, 1) __launch_bounds__(kR) k_update(Work w, Stage s) {
    chain_enter(); // launched chained
    __shared__ float red[kRW][1][2];
    __shared__ float part[1][2];
    cg::cluster_group cl = cg::this_cluster();
    const int         rk = (int)cl.block_rank();
    const int         ci = blockIdx.x / kRC;
    Cand             &C  = w.cand[ci];
    if (!cand_live(C, s))
        return;
    const int  slot = rk * kR + threadIdx.x;
    const int *nnR  = w.nnR + (size_t)ci * w.maxSrc;
    for (int i = slot; i < s.n; i += smi::kIcpSlots)
        if (nnR[i] >= 0)
            w.win[(size_t)ci * w.maxDst + nnR[i]] = ~0ull;
    const int cnt = C.cnt;
    float     mse = FLT_MAX;
    if (cnt >= 6) {
        const float *D    = w.resid + (size_t)ci * w.maxSrc;
        const int   *nnId = w.nnId + (size_t)ci * w.maxSrc;
        smi::KahanF  v[1];
        v[0].init();
        for (int base = slot; base < s.n; base += kFitU * smi::kIcpSlots) {
            int   id[kFitU];
            float d[kFitU];
#pragma unroll
            for (int u = 0; u < kFitU; u++) {
                const int i = base + u * smi::kIcpSlots;
                id[u]       = i < s.n ? nnId[i] : -1;
                d[u]        = i < s.n ? D[i] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < kFitU; u++)
                if (id[u] >= 0)
                    v[0].add(d[u]);
        }
        block_tree<1>(v, red);
        if (threadIdx.x == 0) {
            part[0][0] = v[0].s;
            part[0][1] = v[0].c;
        }
        cl.sync(); // the partials are published
        if (rk == 0 && threadIdx.x < 32) {
            cluster_merge<1>(cl, part, v);
            if (threadIdx.x == 0)
                mse = smm::fdiv(v[0].value(), (float)cnt);
        }
        cl.sync(); // rank 0 has read every partial: the others may leave
    }
    if (rk != 0 || threadIdx.x != 0)
        return;
    if (w.trace && C.iterations < kTraceIters) {
        float *t = w.trace + (size_t)ci * kTraceFloats + (s.traceOff * kTraceIters + C.iterations) * 4;
        t[0]     = (float)cnt;
        t[1]     = mse;
        t[2]     = cnt >= 6 ? C.Pm[0] : -1.0f;
        t[3]     = cnt >= 6 ? C.step.m[3] : 0.0f;
    }
    if (cnt > 6 && mse < s.mseMax)
        C.converged = 1;
    int stop = 0;
    if (cnt < 6) {
        stop = 1;
    } else {
        if (mse < s.mseMin)
            stop = 1;
        const float rate = smm::fdiv(C.resMse - mse, C.resMse);
        if (rate < 0.05f)
            stop = 1;
        if (C.iterations++ >= s.iters)
            stop = 1;
        if (rate > 0.0f) {
            C.resMse = mse;
            C.M      = smi::pose_mul(C.step, C.M);
        }
    }
    C.stop = stop;
}

__global__ void k_init(Work w, const float *__restrict__ cands, int ncand, float voteThreshold,
                       int sparse) {
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= ncand)
        return;
    Cand        &C = w.cand[ci];
    const float *P = cands + (size_t)ci * smi::kPoseFloats;
    for (int e = 0; e < 12; e++)
        C.M.m[e] = P[e];
    C.keep   = C.M;
    C.score  = P[17];
    C.status = P[17] < voteThreshold ? 1 : 0;
    C.active = (C.status == 0 && sparse) ? 1 : 0;
    if (w.trace)
        for (int e = 0; e < kTraceFloats; e++)
            w.trace[(size_t)ci * kTraceFloats + e] = -1.0f;
}

__global__ void k_stage_begin(Work w, int ncand) {
    chain_enter(); // launched chained
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= ncand)
        return;
    Cand &C      = w.cand[ci];
    C.resMse     = FLT_MAX;
    C.iterations = 0;
    C.converged  = 0;
    C.stop       = 0;
    C.inl        = 0;
}

// After a refinement: failed candidates get their status; converged ones keep the pose.
__global__ void k_stage_end(Work w, int ncand, int failStatus) {
    chain_enter(); // launched chained
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= ncand)
        return;
    Cand &C = w.cand[ci];
    if (!C.active)
        return;
    if (!C.converged) {
        C.status = failStatus;
        C.active = 0;
    } else {
        C.keep = C.M;
    }
}

// Inliers of each candidate: source points with a scene point closer than the scoring
// distance, one warp per point (warp_any_within).
__global__ void __launch_bounds__(kT, 6) k_inliers(Work w, const float4 *__restrict__ src, int n,
                                                HGridView F, float r2) {
    chain_enter(); // launched chained
    __shared__ int sc[kW];
    const int      ci = blockIdx.y;
    const Cand    &C  = w.cand[ci];
    if (!C.active)
        return;
    const int lane = threadIdx.x & 31;
    int       c    = 0;
    for (int i = blockIdx.x * kW + (threadIdx.x >> 5); i < n; i += gridDim.x * kW) {
        float x, y, z;
        smi::pose_apply(C.M, src[i].x, src[i].y, src[i].z, x, y, z);
        c += warp_any_within(F, x, y, z, r2) ? 1 : 0;
    }
    if (lane == 0)
        sc[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < kW; k++)
            t += sc[k];
        if (t)
            atomicAdd(&w.cand[ci].inl, t);
    }
}

// Inliers with the reference's search: the nearest point of the full tree closer than the
// scoring distance (inliner, util.cpp:628-641), one thread per source point.
__global__ void __launch_bounds__(kT) k_inliers_tree(Work w, const float4 *__restrict__ src, int n,
                                                     smk::KdView F, float r2) {
    chain_enter(); // launched chained
    __shared__ int sc[kW];
    const int      ci = blockIdx.y;
    const Cand    &C  = w.cand[ci];
    if (!C.active)
        return;
    int c = 0;
    for (int i = blockIdx.x * kT + threadIdx.x; i < n; i += gridDim.x * kT) {
        float q[3];
        smi::pose_apply(C.M, src[i].x, src[i].y, src[i].z, q[0], q[1], q[2]);
        smk::NnSet rs;
        rs.init();
        smk::kd_search(F, q, rs);
        c += (rs.count && rs.dist < r2) ? 1 : 0;
    }
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0)
        sc[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < kW; k++)
            t += sc[k];
        if (t)
            atomicAdd(&w.cand[ci].inl, t);
    }
}

__global__ void k_score(Work w, int ncand, int n, float minScore, int failStatus, int slot) {
    chain_enter(); // launched chained
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= ncand)
        return;
    Cand &C = w.cand[ci];
    if (!C.active)
        return;
    if (w.trace)
        w.trace[(size_t)ci * kTraceFloats + 2 * kTraceIters * 4 + slot] = (float)C.inl;
    C.score = fminf(1.0f, smm::fdiv((float)C.inl, (float)n));
    if (C.score < minScore) {
        C.status = failStatus;
        C.active = 0;
    }
}

__global__ void k_finish(Work w, int ncand, int refine, float minScore, int *status, float *score,
                         float *pose) {
    chain_enter(); // launched chained
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci >= ncand)
        return;
    Cand &C = w.cand[ci];
    if (!C.status && refine && C.score < minScore)
        C.status = 5;
    status[ci] = C.status;
    score[ci]  = C.status ? -1.0f : C.score;
    for (int e = 0; e < 12; e++)
        pose[(size_t)ci * 12 + e] = C.keep.m[e];
}


void run_stage(Ctx &c, Work &w, const Stage &s, int ncand) {
    const dim3 gc(ncand * kRC);                               // reductions: a cluster per candidate
    const dim3 gw(std::max(1, nblocks(s.n, kW)), ncand); // warp kernels: a warp per point
    const dim3 gt(std::max(1, nblocks(s.n, kT)), ncand); // tree searches: a thread per point
    const bool tree = s.tree.nd != nullptr;
    launch_chained(c, k_stage_begin, nblocks(ncand, 128), 128, 0, w, ncand);
    for (int it = 0; it < s.iters; it++) {
        cudaEvent_t t0 = c.clock.begin(c.stream);
        if (tree)
            launch_chained(c, k_corr_tree, gt, kT, 0, w, s);
        else
            launch_chained(c, k_corr, gw, kT, 0, w, s, it > 0 ? 1 : 0);
        c.clock.end(c.stream, t0, KernelClock::kCorr, 0.0); // bytes from the live count
        t0 = c.clock.begin(c.stream);
        launch_chained(c, k_fit, gc, kR, 0, w, s);
        c.clock.end(c.stream, t0, KernelClock::kFit, 0.0);
        t0 = c.clock.begin(c.stream);
        if (tree)
            launch_chained(c, k_resid_tree, gt, kT, 0, w, s);
        else
            launch_chained(c, k_resid, gw, kT, 0, w, s);
        c.clock.end(c.stream, t0, KernelClock::kResid, 0.0);
        t0 = c.clock.begin(c.stream);
        launch_chained(c, k_update, gc, kR, 0, w, s);
        c.clock.end(c.stream, t0, KernelClock::kUpdate, 0.0);
    }
}

} // namespace

void icp_all(Ctx &c, const Model &m, const IcpScene &sc, const IcpParams &p, const float *cands,
             int ncand, int *status, float *score, float *pose, float *trace) {
    if (ncand <= 0)
        return;
    Work w;
    w.pos    = sc.pos;
    w.nrm    = sc.nrm;
    w.maxSrc = std::max(std::max(m.ns, m.nr), 1);
    w.maxDst = std::max(std::max(sc.sampled.m, sc.resampled.m), 1);
    w.cand   = c.arena.get<Cand>("icp.cand", ncand);
    w.nnId   = c.arena.get<int>("icp.nnId", (size_t)ncand * w.maxSrc);
    w.nnR    = c.arena.get<int>("icp.nnR", (size_t)ncand * w.maxSrc);
    w.nnPrev = c.arena.get<int>("icp.nnPrev", (size_t)ncand * w.maxSrc);
    w.x4     = c.arena.get<float4>("icp.x4", (size_t)ncand * w.maxSrc);
    w.n4     = c.arena.get<float4>("icp.n4", (size_t)ncand * w.maxSrc);
    w.resid  = c.arena.get<float>("icp.resid", (size_t)ncand * w.maxSrc);
    w.win    = c.arena.get<unsigned long long>("icp.win", (size_t)ncand * w.maxDst);
    w.trace  = trace;
    w.live   = nullptr;
    if (c.clock.on) {
        w.live = c.arena.get<unsigned long long>("icp.live", 1);
        SM_CUDA(cudaMemsetAsync(w.live, 0, sizeof(unsigned long long), c.stream));
    }
    SM_CUDA(cudaMemsetAsync(w.win, 0xff, (size_t)ncand * w.maxDst * 8, c.stream));
    k_init<<<nblocks(ncand, 128), 128, 0, c.stream>>>(w, cands, ncand, p.voteThreshold, p.sparse);
    SM_LAUNCH_CHECK();
    const float rej2 = p.rejectDist * p.rejectDist;
    const float sc2  = p.scoreDist * p.scoreDist;
    const bool tree = sc.tree != nullptr;
    auto inliers = [&](const float4 *src, int n) {
        if (tree)
            launch_chained(c, k_inliers_tree, dim3(std::max(1, nblocks(n, kT)), ncand), kT, 0,
                           w, src, n, sc.tree->view(nullptr, sc.pos, nullptr, sc.tpF), sc2);
        else
            launch_chained(c, k_inliers, dim3(std::max(1, nblocks(n, kW)), ncand), kT, 0, w,
                           src, n, sc.full.view(), sc2);
    };
    if (p.sparse) {
        Stage s{m.sp, m.sn, m.ns, nblocks(m.ns, kT), sc.sampled.view(), sc.posS, sc.nrmS, sc.sampled.m, 5,
                p.sampleStep * 0.5f, p.sampleStep, rej2, 0};
        if (tree) {
            s.tree   = sc.tree->view(sc.ioiS, sc.pos, sc.neS, sc.tpS);
            s.rankOf = sc.rankS;
        }
        run_stage(c, w, s, ncand);
        launch_chained(c, k_stage_end, nblocks(ncand, 128), 128, 0, w, ncand, 2);
        inliers(m.sp, m.ns);
        launch_chained(c, k_score, nblocks(ncand, 128), 128, 0, w, ncand, m.ns, p.minScore, 3,
                       0);
        if (p.dense) {
            Stage d{m.rp, m.rn, m.nr, nblocks(m.nr, kT), sc.resampled.view(), sc.posR, sc.nrmR,
                    sc.resampled.m, p.denseSteps, p.reSampleStep * 0.5f, p.sampleStep, rej2, 1};
            if (tree) {
                d.tree   = sc.tree->view(sc.ioiR, sc.pos, sc.neR, sc.tpR);
                d.rankOf = sc.rankR;
            }
            run_stage(c, w, d, ncand);
            launch_chained(c, k_stage_end, nblocks(ncand, 128), 128, 0, w, ncand, 4);
            inliers(m.rp, m.nr);
            launch_chained(c, k_score, nblocks(ncand, 128), 128, 0, w, ncand, m.nr, p.minScore,
                           5, 1);
        }
    }
    launch_chained(c, k_finish, nblocks(ncand, 128), 128, 0, w, ncand,
                   (p.sparse || p.dense) ? 1 : 0, p.minScore, status, score, pose);
}

} // namespace sm
