// icp.cu - pose refinement and scoring of matchScene (ppf.cpp:422-495): ICP::regist
// (icp.cpp:214-278) with findCorresponds (icp.cpp:123-167), the symmetric point-to-plane
// step (icp.cpp:39-121) and inliner (util.cpp:628-641).
//
// Every candidate is independent, so all of them are refined at once: one CTA of
// kIcpThreads threads per candidate. Per iteration: grid nearest neighbour of each moved
// model point; per scene point the closest model point wins a 64-bit atomicMin of
// (distance bits, model index), which reproduces the reference's "first minimum in model
// order" without its O(n*m) grouping scan; FP32 Kahan sums in a fixed strided layout and
// tree; FP64 solve on thread 0. The selection walk over the candidates (numMatches) runs
// on the host afterwards and only reads the per-candidate results.
#include <cfloat>

#include "sm_icp.h"
#include "sm_stages.h"

namespace sm {
using namespace smd;

namespace {

constexpr int kT = smi::kIcpThreads;
constexpr int kW = kT / 32;

struct IcpArgs {
    const float4 *sp, *sn, *rp, *rn;
    int           ns, nr;
    const float4 *pos, *nrm;
    GridView      gS, gR, gF;
    const int    *rankS, *rankR; // point id -> index in the sampled / resampled subset
    int           nS, nR;
    IcpParams     p;
    const float  *cands; // ncand x 18
    int           wave0, ncand;
    // per-CTA scratch (indexed by blockIdx.x)
    int                *nnId;  // maxSrc: scene point id of the pair, -1 none
    int                *nnR;   // maxSrc: subset rank of that point
    float4             *x4;    // maxSrc: moved source point, w = squared distance
    float4             *n4;    // maxSrc: rotated source normal
    unsigned long long *winS;  // nS
    unsigned long long *winR;  // nR
    int                 maxSrc;
    int                *status;
    float              *score, *pose;
};

struct Shared {
    float       red[kW][smi::kNumSystem][2];
    smi::Pose34 M, step;
    float       Pm[3], Qm[3];
    float       mse;
    int         ired[kW];
    int         cnt;
};

// Fixed-layout reduction of W Kahan partials (one per thread): warp shfl_down tree, then
// warp 0 over the kW warp partials. Result valid on thread 0. Matches the oracle's
// StridedSum::result.
template <int W> __device__ void kahan_reduce(smi::KahanF (&v)[W], Shared &S) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
#pragma unroll
        for (int k = 0; k < W; k++) {
            smi::KahanF o;
            o.s = __shfl_down_sync(0xffffffffu, v[k].s, off);
            o.c = __shfl_down_sync(0xffffffffu, v[k].c, off);
            v[k].merge(o);
        }
    }
    if (lane == 0)
        for (int k = 0; k < W; k++) {
            S.red[w][k][0] = v[k].s;
            S.red[w][k][1] = v[k].c;
        }
    __syncthreads();
    if (w == 0) {
        for (int k = 0; k < W; k++) {
            v[k].s = lane < kW ? S.red[lane][k][0] : 0.f;
            v[k].c = lane < kW ? S.red[lane][k][1] : 0.f;
        }
#pragma unroll
        for (int off = kW / 2; off >= 1; off >>= 1) {
#pragma unroll
            for (int k = 0; k < W; k++) {
                smi::KahanF o;
                o.s = __shfl_down_sync(0xffffffffu, v[k].s, off);
                o.c = __shfl_down_sync(0xffffffffu, v[k].c, off);
                v[k].merge(o);
            }
        }
    }
    __syncthreads();
}

__device__ int block_sum_int(int v, Shared &S) {
    v = __reduce_add_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0)
        S.ired[threadIdx.x >> 5] = v;
    __syncthreads();
    int t = 0;
    for (int w = 0; w < kW; w++)
        t += S.ired[w];
    __syncthreads();
    return t;
}

__device__ __forceinline__ unsigned long long win_key(float d, int i) {
    return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)i;
}

// ICP::regist of source (src, srcN, n) against the scene subset of grid G, starting from
// S.M; returns converged, leaves the refined pose in S.M.
__device__ bool regist(const IcpArgs &a, Shared &S, const float4 *src, const float4 *srcN, int n,
                       const GridView &G, const int *rank, unsigned long long *win, int iters,
                       float mseMin, float mseMax) {
    const int   tid  = threadIdx.x;
    int        *nnId = a.nnId + (size_t)blockIdx.x * a.maxSrc;
    int        *nnR  = a.nnR + (size_t)blockIdx.x * a.maxSrc;
    float4     *x4   = a.x4 + (size_t)blockIdx.x * a.maxSrc;
    float4     *n4   = a.n4 + (size_t)blockIdx.x * a.maxSrc;
    const float rej2 = a.p.rejectDist * a.p.rejectDist;
    bool        converged = false;
    float       resMse    = FLT_MAX;
    int         iterations = 0;
    while (iterations < iters) {
        // findCorresponds: nearest scene point, rejection, closest model point per scene point
        for (int i = tid; i < n; i += kT) {
            float4 x, y;
            smi::pose_apply(S.M, src[i].x, src[i].y, src[i].z, x.x, x.y, x.z);
            smi::pose_rotate(S.M, srcN[i].x, srcN[i].y, srcN[i].z, y.x, y.y, y.z);
            float     d;
            const int j  = grid_nn(G, a.pos, x.x, x.y, x.z, rej2, d);
            const bool ok = j >= 0 && d <= rej2;
            x.w     = d;
            x4[i]   = x;
            n4[i]   = y;
            nnId[i] = ok ? j : -1;
            nnR[i]  = ok ? rank[j] : -1;
            if (ok)
                atomicMin(&win[nnR[i]], win_key(d, i));
        }
        __syncthreads();
        smi::KahanF mom[6];
        for (int k = 0; k < 6; k++)
            mom[k].init();
        int cnt = 0;
        for (int i = tid; i < n; i += kT) {
            const int r = nnR[i];
            if (r < 0)
                continue;
            if (win[r] != win_key(x4[i].w, i)) {
                nnId[i] = -1; // not the closest source point of its scene point
                continue;
            }
            const float4 q = a.pos[nnId[i]];
            mom[0].add(x4[i].x);
            mom[1].add(x4[i].y);
            mom[2].add(x4[i].z);
            mom[3].add(q.x);
            mom[4].add(q.y);
            mom[5].add(q.z);
            cnt++;
        }
        cnt = block_sum_int(cnt, S);
        kahan_reduce<6>(mom, S);
        if (tid == 0) {
            const float fc = (float)cnt;
            for (int k = 0; k < 3; k++) {
                S.Pm[k] = smm::fdiv(mom[k].value(), fc);
                S.Qm[k] = smm::fdiv(mom[3 + k].value(), fc);
            }
        }
        __syncthreads();
        float mse = FLT_MAX;
        if (cnt >= 6) {
            smi::KahanF sys[smi::kNumSystem];
            for (int k = 0; k < smi::kNumSystem; k++)
                sys[k].init();
            for (int i = tid; i < n; i += kT) {
                if (nnId[i] < 0)
                    continue;
                const float4 q = a.pos[nnId[i]], qn = a.nrm[nnId[i]];
                float        t[smi::kNumSystem];
                smi::system_terms(x4[i].x - S.Pm[0], x4[i].y - S.Pm[1], x4[i].z - S.Pm[2],
                                  q.x - S.Qm[0], q.y - S.Qm[1], q.z - S.Qm[2], n4[i].x + qn.x,
                                  n4[i].y + qn.y, n4[i].z + qn.z, t);
                for (int k = 0; k < smi::kNumSystem; k++)
                    sys[k].add(t[k]);
            }
            kahan_reduce<smi::kNumSystem>(sys, S);
            if (tid == 0) {
                float v[smi::kNumSystem];
                for (int k = 0; k < smi::kNumSystem; k++)
                    v[k] = sys[k].value();
                S.step = smi::solve_step(v, S.Pm, S.Qm);
            }
            __syncthreads();
            smi::KahanF ms[1];
            ms[0].init();
            for (int i = tid; i < n; i += kT) {
                if (nnId[i] < 0)
                    continue;
                float y0, y1, y2, d;
                smi::pose_apply(S.step, x4[i].x, x4[i].y, x4[i].z, y0, y1, y2);
                grid_nn(G, a.pos, y0, y1, y2, FLT_MAX, d);
                ms[0].add(smm::fsqrt(d));
            }
            kahan_reduce<1>(ms, S);
            if (tid == 0)
                S.mse = smm::fdiv(ms[0].value(), (float)cnt);
            __syncthreads();
            mse = S.mse;
        }
        // reset the winner slots this iteration used
        for (int i = tid; i < n; i += kT)
            if (nnR[i] >= 0)
                win[nnR[i]] = ~0ull;
        __syncthreads();
        // regist loop logic (icp.cpp:233-272), uniform across the CTA
        if (cnt > 6 && mse < mseMax)
            converged = true;
        bool stop = false;
        if (cnt < 6) {
            stop = true;
        } else {
            if (mse < mseMin)
                stop = true;
            const float rate = smm::fdiv(resMse - mse, resMse);
            if (rate < 0.05f)
                stop = true;
            if (iterations++ >= iters)
                stop = true;
            if (rate > 0.0f) {
                resMse = mse;
                if (tid == 0)
                    S.M = smi::pose_mul(S.step, S.M);
            }
        }
        __syncthreads();
        if (stop)
            break;
    }
    return converged;
}

__device__ int inliers(const IcpArgs &a, Shared &S, const float4 *src, int n) {
    const float r2 = a.p.scoreDist * a.p.scoreDist;
    int         c  = 0;
    for (int i = threadIdx.x; i < n; i += kT) {
        float x, y, z;
        smi::pose_apply(S.M, src[i].x, src[i].y, src[i].z, x, y, z);
        if (grid_any_within(a.gF, a.pos, x, y, z, r2))
            c++;
    }
    return block_sum_int(c, S);
}

__global__ void __launch_bounds__(kT) k_icp(IcpArgs a) {
    __shared__ Shared S;
    const int         ci  = a.wave0 + blockIdx.x;
    if (ci >= a.ncand)
        return;
    const float *C = a.cands + (size_t)ci * smi::kPoseFloats;
    if (threadIdx.x == 0)
        for (int e = 0; e < 12; e++)
            S.M.m[e] = C[e];
    __syncthreads();
    float score  = C[17];
    int   status = 0;
    if (score < a.p.voteThreshold)
        status = 1;
    smi::Pose34 keep = S.M; // the pose reported when a refinement does not converge
    if (!status && a.p.sparse) {
        const bool conv = regist(a, S, a.sp, a.sn, a.ns, a.gS, a.rankS,
                                 a.winS + (size_t)blockIdx.x * a.nS, 5, a.p.sampleStep * 0.5f,
                                 a.p.sampleStep);
        if (!conv) {
            status = 2;
        } else {
            keep = S.M;
            const int in = inliers(a, S, a.sp, a.ns);
            score        = fminf(1.0f, smm::fdiv((float)in, (float)a.ns));
            if (score < a.p.minScore)
                status = 3;
        }
    }
    if (!status && a.p.sparse && a.p.dense) {
        const bool conv = regist(a, S, a.rp, a.rn, a.nr, a.gR, a.rankR,
                                 a.winR + (size_t)blockIdx.x * a.nR, a.p.denseSteps,
                                 a.p.reSampleStep * 0.5f, a.p.sampleStep);
        if (!conv) {
            status = 4;
        } else {
            keep = S.M;
            const int in = inliers(a, S, a.rp, a.nr);
            score        = fminf(1.0f, smm::fdiv((float)in, (float)a.nr));
            if (score < a.p.minScore)
                status = 5;
        }
    }
    if (!status && (a.p.sparse || a.p.dense) && score < a.p.minScore)
        status = 5;
    if (threadIdx.x == 0) {
        a.status[ci] = status;
        a.score[ci]  = status ? -1.0f : score;
        for (int e = 0; e < 12; e++)
            a.pose[(size_t)ci * 12 + e] = keep.m[e];
    }
}

__global__ void k_rank(const int *__restrict__ ids, int m, int *__restrict__ rank) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m)
        rank[ids[i]] = i;
}

} // namespace

void icp_all(Ctx &c, const Model &m, const IcpScene &s, const IcpParams &p, const float *cands,
             int ncand, int *status, float *score, float *pose) {
    if (ncand <= 0)
        return;
    IcpArgs a;
    a.sp    = m.sp;
    a.sn    = m.sn;
    a.rp    = m.rp;
    a.rn    = m.rn;
    a.ns    = m.ns;
    a.nr    = m.nr;
    a.pos   = s.pos;
    a.nrm   = s.nrm;
    a.gS    = s.sampled.view();
    a.gR    = s.resampled.view();
    a.gF    = s.full.view();
    a.nS    = std::max(s.sampled.m, 1);
    a.nR    = std::max(s.resampled.m, 1);
    a.p     = p;
    a.cands = cands;
    a.ncand = ncand;
    a.status = status;
    a.score  = score;
    a.pose   = pose;
    // point id -> subset rank (the grids' id lists are cell-major, so rank by subset order)
    a.rankS = s.rankS;
    a.rankR = s.rankR;
    a.maxSrc = std::max(m.ns, m.nr);
    const int wave = std::min(ncand, 2 * 152);
    a.nnId = c.arena.get<int>("icp.nnId", (size_t)wave * a.maxSrc);
    a.nnR  = c.arena.get<int>("icp.nnR", (size_t)wave * a.maxSrc);
    a.x4   = c.arena.get<float4>("icp.x4", (size_t)wave * a.maxSrc);
    a.n4   = c.arena.get<float4>("icp.n4", (size_t)wave * a.maxSrc);
    a.winS = c.arena.get<unsigned long long>("icp.winS", (size_t)wave * a.nS);
    a.winR = c.arena.get<unsigned long long>("icp.winR", (size_t)wave * a.nR);
    SM_CUDA(cudaMemsetAsync(a.winS, 0xff, (size_t)wave * a.nS * 8, c.stream));
    SM_CUDA(cudaMemsetAsync(a.winR, 0xff, (size_t)wave * a.nR * 8, c.stream));
    for (int w0 = 0; w0 < ncand; w0 += wave) {
        a.wave0 = w0;
        k_icp<<<std::min(wave, ncand - w0), kT, 0, c.stream>>>(a);
        SM_LAUNCH_CHECK();
    }
}

void subset_rank(Ctx &c, const int *ids, int m, int *rank) {
    if (m <= 0)
        return;
    k_rank<<<nblocks(m, 256), 256, 0, c.stream>>>(ids, m, rank);
    SM_LAUNCH_CHECK();
}

} // namespace sm
