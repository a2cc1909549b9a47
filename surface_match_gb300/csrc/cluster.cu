// cluster.cu - pose clustering of matchScene (ppf.cpp:414-418): sortPoses, clusterPose,
// avgClusters, sortPoses, clusterPose2 (util.cpp:486-601).
//
// Five kernels. k_cluster_rank (all CTAs): stable rank-by-counting sort on (votes desc,
// list position). k_cluster_bits (all CTAs): the compatibility of every pose with every
// earlier pose, as a bit matrix. k_cluster_a (one CTA): clusterPose, a greedy first-fit
// clustering (a pose joins the first earlier head it is compatible with), resolved from the
// bits (in shared memory) in parallel rounds (a pose compatible with a head is a member,
// one whose compatible earlier poses are all members is a head), which reproduces the
// sequential decisions; a member's cluster is its lowest compatible head - the first in
// creation order. Larger pose lists walk the poses with one warp instead. k_cluster_avg:
// one block per cluster sums its members in pose order (FP32 translation, FP64 quaternion
// moments) and averages them, so the clusters' FP64 work spreads over the SMs. k_cluster_b
// (one CTA): the second sort and clusterPose2. Results are identical to the oracle's
// sequential restatement.
#include <cmath>
#include <cstring>

#include "sm_icp.h"
#include "sm_stages.h"

namespace sm {

namespace {

constexpr int kClBs   = 1024;
constexpr int PF      = smi::kPoseFloats;
constexpr int kClMaxC = 1024; // poses for which the compatibility bits are precomputed

// Shared-memory bytes per pose of k_cluster_a: its sort key (float4).
constexpr int kClPerPose = 16;

struct ClArgs {
    const float *poses;
    int          np;
    float        sqThr, angThr, cx, cy, cz, thr2;
    float       *sorted;    // np x PF
    float       *avg;       // np x PF (cluster creation order)
    float       *avgSorted; // np x PF
    float4      *tr;        // np
    float       *out;       // np x PF
    int         *outCount;
    float4      *gbuf4;     // np float4 when the per-pose state does not fit shared memory
    int         *gbuf;      // 2 np ints, likewise
    float4      *tv, *qv;   // np each: sorted {tx, ty, tz, votes} and quaternions
    int         *clu;       // np: cluster number per sorted pose
    int         *heads;     // np: pose index of each cluster head
    int         *nhOut;     // cluster count
    int          smemState; // per-pose state in shared memory
    int          useBits;   // compatibility bits in shared memory
    uint32_t    *bitsG;     // W x np compatibility words (word-major), filled by k_cluster_bits
};

// out[rank(i)] = in[i] for the stable sort by votes (float 17) descending; `votes` holds
// the n vote counts. With `key`, also the sorted {tx, ty, tz, angle}, {tx, ty, tz, votes}
// and quaternion of each pose.
__device__ void stable_sort_votes(const float *in, const float *votes, int n, float *out,
                                  float4 *key, float4 *tv, float4 *qv) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const float v    = votes[i];
        int         rank = 0;
        for (int j = 0; j < n; j++) {
            const float u = votes[j];
            rank += (u > v || (u == v && j < i)) ? 1 : 0;
        }
        const float *P = in + (size_t)i * PF;
        for (int e = 0; e < PF; e++)
            out[(size_t)rank * PF + e] = P[e];
        if (key) {
            key[rank] = make_float4(P[3], P[7], P[11], P[16]);
            tv[rank]  = make_float4(P[3], P[7], P[11], P[17]);
            qv[rank]  = make_float4(P[12], P[13], P[14], P[15]);
        }
    }
}

// clusterPose compatibility of pose a with head b (util.cpp:499-520); the distance test
// sqrt(v) < distThr is evaluated as v < sqThr (exact: see sqrt_lt_bound).
__device__ __forceinline__ bool compat(const float4 &a, const float4 &b, float sqThr, float angThr) {
    const float x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
    return x * x + (y * y + z * z) < sqThr && smm::fabs_(a.w - b.w) < angThr;
}

// sortPoses (util.cpp:486-491) as a stable rank by votes (float 17) descending, one thread
// per pose over all CTAs: out[rank(i)] = in[i], with the sorted {tx, ty, tz, angle} keys
// (gbuf4), {tx, ty, tz, votes} and quaternions. The votes are staged per CTA in shared
// memory (all lanes read the same one at a time: a broadcast).
__global__ void k_cluster_rank(ClArgs a) {
    smd::chain_enter(); // launched chained
    constexpr int kStage = 8192; // votes staged in shared memory (the rest read from L1/L2)
    __shared__ float sv[kStage];
    const int        np = a.np, ns = min(np, kStage);
    for (int j = threadIdx.x; j < ns; j += blockDim.x)
        sv[j] = a.poses[(size_t)j * PF + 17];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np)
        return;
    const float v    = i < ns ? sv[i] : __ldg(&a.poses[(size_t)i * PF + 17]);
    int         rank = 0;
    for (int j = 0; j < np; j++) {
        const float u = j < ns ? sv[j] : __ldg(&a.poses[(size_t)j * PF + 17]);
        rank += (u > v || (u == v && j < i)) ? 1 : 0;
    }
    const float *P = a.poses + (size_t)i * PF;
    for (int e = 0; e < PF; e++)
        a.sorted[(size_t)rank * PF + e] = P[e];
    a.gbuf4[rank] = make_float4(P[3], P[7], P[11], P[16]);
    a.tv[rank]    = make_float4(P[3], P[7], P[11], P[17]);
    a.qv[rank]    = make_float4(P[12], P[13], P[14], P[15]);
}

// Compatibility bits over all CTAs: word w of row i (bitsG[w * np + i]), bit b set when
// sorted pose i is compatible with the earlier sorted pose 32 w + b.
__global__ void k_cluster_bits(ClArgs a) {
    smd::chain_enter(); // launched chained
    const int  np = a.np, W = (np + 31) >> 5;
    const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long)np * W)
        return;
    const int    w = (int)(idx / np), i = (int)(idx % np);
    const float4 P = a.gbuf4[i];
    uint32_t     m = 0;
    if (w * 32 < i) {
        for (int b = 0; b < 32; b++) {
            const int j = w * 32 + b;
            if (j < i && compat(P, a.gbuf4[j], a.sqThr, a.angThr))
                m |= 1u << b;
        }
    }
    a.bitsG[idx] = m;
}

__global__ void __launch_bounds__(kClBs) k_cluster_a(ClArgs a) {
    smd::chain_enter(); // launched chained
    extern __shared__ float4 dsm4[];
    __shared__ int sNh;
    const int      tid = threadIdx.x, lane = tid & 31;
    const int      np  = a.np;
    float4        *key   = a.smemState ? dsm4 : a.gbuf4;
    const int      W     = (np + 31) >> 5;
    uint32_t      *bits  = (uint32_t *)(dsm4 + np); // W x np (word-major), when useBits
    uint32_t      *headB = bits + (size_t)W * np;     // W
    uint32_t      *unkB  = headB + W;                 // W
    uint32_t      *newH  = unkB + W;                  // W
    uint32_t      *newM  = newH + W;                  // W
    int           *hpre  = (int *)(newM + W);         // W + 1
    // the sorted keys (k_cluster_rank, in gbuf4) into shared memory
    if (a.smemState)
        for (int i = tid; i < np; i += kClBs)
            key[i] = a.gbuf4[i];
    __syncthreads();
    if (a.useBits) {
        // the compatibility words of k_cluster_bits (bits[w * np + i], bit b: pose i is
        // compatible with the earlier pose 32 w + b)
        for (int idx = tid; idx < np * W; idx += kClBs)
            bits[idx] = a.bitsG[idx];
        for (int w = tid; w < W; w += kClBs) {
            headB[w] = 0u;
            const int rem = np - w * 32;
            unkB[w]       = rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);
        }
        __syncthreads();
        // Heads by rounds: an undecided pose compatible with a head is a member; one whose
        // compatible earlier poses are all decided members is a head. The smallest undecided
        // pose is decided in every round, and each decision is the sequential one.
        for (;;) {
            for (int w = tid; w < W; w += kClBs) {
                newH[w] = 0u;
                newM[w] = 0u;
            }
            __syncthreads();
            bool any = false;
            for (int i = tid; i < np; i += kClBs) {
                if (!((unkB[i >> 5] >> (i & 31)) & 1u))
                    continue;
                any            = true;
                bool hitHead   = false, hitUnk = false;
                const int wmax = i >> 5;
                for (int w = 0; w <= wmax; w++) {
                    const uint32_t r = bits[(size_t)w * np + i];
                    hitHead          = hitHead || (r & headB[w]) != 0u;
                    hitUnk           = hitUnk || (r & unkB[w]) != 0u;
                }
                if (hitHead)
                    atomicOr(&newM[i >> 5], 1u << (i & 31));
                else if (!hitUnk)
                    atomicOr(&newH[i >> 5], 1u << (i & 31));
            }
            if (!__syncthreads_or(any))
                break;
            for (int w = tid; w < W; w += kClBs) {
                headB[w] |= newH[w];
                unkB[w] &= ~(newH[w] | newM[w]);
            }
            __syncthreads();
        }
        // cluster numbers: heads in pose order; a member joins its lowest compatible head
        if (tid == 0) {
            int s = 0;
            for (int w = 0; w < W; w++) {
                hpre[w] = s;
                s += __popc(headB[w]);
            }
            hpre[W] = s;
            sNh     = s;
        }
        __syncthreads();
        for (int i = tid; i < np; i += kClBs) {
            const uint32_t hb = headB[i >> 5];
            if ((hb >> (i & 31)) & 1u) {
                const int h = hpre[i >> 5] + __popc(hb & ((1u << (i & 31)) - 1u));
                a.clu[i]    = h;
                a.heads[h]  = i;
                continue;
            }
            for (int w = 0; w <= (i >> 5); w++) {
                const uint32_t r = bits[(size_t)w * np + i] & headB[w];
                if (r) {
                    const int b = __ffs(r) - 1;
                    a.clu[i]    = hpre[w] + __popc(headB[w] & ((1u << b) - 1u));
                    break;
                }
            }
        }
    } else if (tid < 32) {
        // clusterPose: warp 0 walks the poses in sorted order, 32 heads per step
        int nh = 0;
        for (int i = 0; i < np; i++) {
            const float4 P     = key[i];
            int          found = -1;
            for (int h0 = 0; h0 < nh && found < 0; h0 += 32) {
                const int      h  = h0 + lane;
                const bool     ok = h < nh && compat(P, key[a.heads[h]], a.sqThr, a.angThr);
                const unsigned m  = __ballot_sync(0xffffffffu, ok);
                if (m)
                    found = h0 + __ffs(m) - 1;
            }
            if (lane == 0) {
                if (found < 0) {
                    a.heads[nh] = i;
                    a.clu[i]    = nh;
                } else {
                    a.clu[i] = found;
                }
            }
            if (found < 0)
                nh++;
            __syncwarp();
        }
        if (lane == 0)
            sNh = nh;
    }
    __syncthreads();
    if (tid == 0)
        *a.nhOut = sNh;
}

// avgClusters: one block per cluster (grid-stride); the warp finds the members in pose
// order (cluster numbers read 256 poses ahead) and sums them in that order, one sum per lane:
// lane e < 10 the FP64 quaternion moment e, lanes 10..13 the FP32 translation and votes (the
// same additions in the same order as one thread summing all of them); then the Markley
// quaternion average in FP64.
__global__ void k_cluster_avg(ClArgs a) {
    smd::chain_enter(); // launched chained
    const int lane = threadIdx.x & 31;
    const int nh   = *a.nhOut;
    // moment e of lane e: q[r] * q[s] over the upper triangle in row order
    int er = 0, es = 0;
    for (int r = 0, e = 0; r < 4; r++)
        for (int s2 = r; s2 < 4; s2++, e++)
            if (e == lane) {
                er = r;
                es = s2;
            }
    for (int h = blockIdx.x; h < nh; h += gridDim.x) {
        const int head = a.heads[h];
        double    Sd   = 0.0; // lane e < 10: moment e
        float     Pf   = 0.0f; // lanes 10..13: tx, ty, tz, votes
        int       cnt  = 0;
        for (int base = head; base < a.np; base += 32 * 8) {
            int cl[8];
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int i = base + u * 32 + lane;
                cl[u]       = i < a.np ? a.clu[i] : -1;
            }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int      i   = base + u * 32 + lane;
                const bool     mem = cl[u] == h;
                const uint32_t m   = __ballot_sync(0xffffffffu, mem);
                if (!m)
                    continue;
                float4 t = make_float4(0.f, 0.f, 0.f, 0.f), q4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (mem) {
                    t  = a.tv[i];
                    q4 = a.qv[i];
                }
                for (uint32_t r = m; r; r &= r - 1) {
                    const int   src = __ffs(r) - 1;
                    const float tv[4] = {__shfl_sync(0xffffffffu, t.x, src),
                                         __shfl_sync(0xffffffffu, t.y, src),
                                         __shfl_sync(0xffffffffu, t.z, src),
                                         __shfl_sync(0xffffffffu, t.w, src)};
                    const float qv[4] = {__shfl_sync(0xffffffffu, q4.x, src),
                                         __shfl_sync(0xffffffffu, q4.y, src),
                                         __shfl_sync(0xffffffffu, q4.z, src),
                                         __shfl_sync(0xffffffffu, q4.w, src)};
                    if (lane < 10)
                        Sd += (double)qv[er] * (double)qv[es];
                    else if (lane < 14)
                        Pf = Pf + tv[lane - 10];
                    cnt++;
                }
            }
        }
        double S[10];
#pragma unroll
        for (int e = 0; e < 10; e++)
            S[e] = __shfl_sync(0xffffffffu, Sd, e);
        const float px = __shfl_sync(0xffffffffu, Pf, 10), py = __shfl_sync(0xffffffffu, Pf, 11),
                    pz = __shfl_sync(0xffffffffu, Pf, 12), vs = __shfl_sync(0xffffffffu, Pf, 13);
        if (lane != 0)
            continue;
        double q[4], R[9];
        sml::quat_average_from_sum(S, cnt, q);
        sml::quat_to_mat(q, R);
        float *O = a.avg + (size_t)h * PF;
        for (int r = 0; r < 3; r++)
            for (int s = 0; s < 3; s++)
                O[r * 4 + s] = (float)R[r * 3 + s];
        const float fc = (float)cnt;
        O[3]           = smm::fdiv(px, fc);
        O[7]           = smm::fdiv(py, fc);
        O[11]          = smm::fdiv(pz, fc);
        for (int r = 0; r < 4; r++)
            O[12 + r] = (float)q[r];
        O[16] = sml::quat_angle(q);
        O[17] = vs;
    }
}

// sortPoses of the averaged clusters and clusterPose2 (overlap of the transformed model-box
// centres, util.cpp:522-551); one block. The greedy walk runs on one warp with the centres,
// the leader list and the leaders' vote sums in shared memory (global memory beyond
// kClMaxC clusters); the vote sums keep the sequential order of the walk, and the output
// records are written by all threads afterwards.
__global__ void __launch_bounds__(kClBs) k_cluster_b(ClArgs a) {
    smd::chain_enter(); // launched chained
    __shared__ int    sNout;
    __shared__ float4 sTr[kClMaxC];
    __shared__ float  sVote[kClMaxC], sSum[kClMaxC];
    __shared__ int    sLead[kClMaxC];
    const int         tid = threadIdx.x, lane = tid & 31;
    const int         nh  = *a.nhOut;
    float            *votes = (float *)a.gbuf;
    for (int h = tid; h < nh; h += kClBs)
        votes[h] = a.avg[(size_t)h * PF + 17];
    __syncthreads();
    stable_sort_votes(a.avg, votes, nh, a.avgSorted, nullptr, nullptr, nullptr);
    __syncthreads();
    const bool inSm = nh <= kClMaxC;
    float4    *tr   = inSm ? sTr : a.tr;
    float     *vote = inSm ? sVote : votes; // votes of the sorted clusters
    float     *sum  = inSm ? sSum : votes + nh;
    int       *lead = inSm ? sLead : a.heads;
    for (int h = tid; h < nh; h += kClBs) {
        smi::Pose34 T;
        for (int e = 0; e < 12; e++)
            T.m[e] = a.avgSorted[(size_t)h * PF + e];
        float x, y, z;
        smi::pose_apply(T, a.cx, a.cy, a.cz, x, y, z);
        tr[h]   = make_float4(x, y, z, 0.f);
        vote[h] = a.avgSorted[(size_t)h * PF + 17];
    }
    __syncthreads();
    if (tid < 32) {
        int nl = 0;
        for (int i = 0; i < nh; i++) {
            const float4 ti    = tr[i];
            int          found = -1;
            for (int h0 = 0; h0 < nl && found < 0; h0 += 32) {
                const int h  = h0 + lane;
                bool      ok = false;
                if (h < nl) {
                    const float4 th = tr[lead[h]];
                    const float  dx = th.x - ti.x, dy = th.y - ti.y, dz = th.z - ti.z;
                    ok              = dx * dx + (dy * dy + dz * dz) < a.thr2;
                }
                const unsigned m = __ballot_sync(0xffffffffu, ok);
                if (m)
                    found = h0 + __ffs(m) - 1;
            }
            if (lane == 0) {
                if (found < 0) {
                    lead[nl] = i;
                    sum[nl]  = vote[i];
                } else {
                    sum[found] = sum[found] + vote[i];
                }
            }
            if (found < 0)
                nl++;
            __syncwarp();
        }
        if (lane == 0)
            sNout = nl;
    }
    __syncthreads();
    const int nl = sNout;
    for (int idx = tid; idx < nl * PF; idx += kClBs) {
        const int l = idx / PF, e = idx - l * PF;
        a.out[idx]  = e == 17 ? sum[l] : a.avgSorted[(size_t)lead[l] * PF + e];
    }
    if (tid == 0)
        *a.outCount = nl;
}

// Smallest float v >= 0 with sqrtf(v) >= t (IEEE square root is correctly rounded and
// monotone, so sqrtf(v) < t <=> v < this bound, NaN included).
float sqrt_lt_bound(float t) {
    if (!(t > 0.0f))
        return 0.0f;
    uint32_t lo = 0, hi = 0x7f800000u; // +0 .. +inf
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        float          v;
        memcpy(&v, &mid, 4);
        if (std::sqrt(v) >= t)
            hi = mid;
        else
            lo = mid + 1;
    }
    float r;
    memcpy(&r, &lo, 4);
    return r;
}

} // namespace

int cluster(Ctx &c, const float *poses, int np, float distThr, float angThr, const float center[3],
            float maxOverlap, float *outCands, const std::string &tag) {
    if (np <= 0)
        return 0;
    ClArgs a;
    a.poses     = poses;
    a.np        = np;
    a.sqThr     = sqrt_lt_bound(distThr);
    a.angThr    = angThr;
    a.cx        = center[0];
    a.cy        = center[1];
    a.cz        = center[2];
    a.thr2      = maxOverlap * maxOverlap;
    a.sorted    = c.arena.get<float>(tag + ".sorted", (size_t)np * PF);
    a.avg       = c.arena.get<float>(tag + ".avg", (size_t)np * PF);
    a.avgSorted = c.arena.get<float>(tag + ".avgs", (size_t)np * PF);
    a.tr        = c.arena.get<float4>(tag + ".tr", np);
    a.out       = outCands;
    a.outCount  = c.arena.get<int>(tag + ".count", 1);
    a.gbuf4     = c.arena.get<float4>(tag + ".g4", np);
    a.gbuf      = c.arena.get<int>(tag + ".gi", (size_t)np * 2);
    a.tv        = c.arena.get<float4>(tag + ".tv", np);
    a.qv        = c.arena.get<float4>(tag + ".qv", np);
    int *ints   = c.arena.get<int>(tag + ".ints", (size_t)np * 2 + 1);
    a.clu       = ints;
    a.heads     = ints + np;
    a.nhOut     = ints + 2 * (size_t)np;
    int optin = 0;
    SM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    const size_t W     = ((size_t)np + 31) / 32;
    const size_t state = (size_t)np * kClPerPose;
    const size_t bitsB = ((size_t)np * W + 6 * W + 1) * 4;
    a.smemState        = state + 1024 <= (size_t)optin ? 1 : 0;
    a.useBits          = a.smemState && np <= kClMaxC && state + bitsB + 1024 <= (size_t)optin ? 1 : 0;
    const size_t smem  = a.smemState ? state + (a.useBits ? bitsB : 0) : 0;
    if (smem > allow_dynamic_smem((const void *)k_cluster_a, c.device))
        throw Error(SM_ERR_CAPACITY, "shared-memory request above the device limit");
    launch_chained(c, k_cluster_rank, nblocks(np, 128), 128, 0, a);
    a.bitsG = nullptr;
    if (a.useBits) {
        a.bitsG = c.arena.get<uint32_t>(tag + ".bits", (size_t)np * W);
        launch_chained(c, k_cluster_bits, nblocks((long long)np * W, 256), 256, 0, a);
    }
    launch_chained(c, k_cluster_a, 1, kClBs, smem, a);
    launch_chained(c, k_cluster_avg, std::min(np, 152 * 8), 32, 0, a);
    launch_chained(c, k_cluster_b, 1, kClBs, 0, a);
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, a.outCount, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    return c.hostCounts[0];
}

} // namespace sm
