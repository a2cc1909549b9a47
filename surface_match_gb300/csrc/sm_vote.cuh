// sm_vote.cuh - device pieces of the voting stage shared by the multi-kernel pipeline
// (vote_pipe.cu) and the single-kernel variant (vote.cu): model table probe, the
// shared-memory vote loop, peak extraction and the per-keypoint result (ppf.cpp:247-409).
#pragma once

#include <algorithm>
#include <climits>

#include "sm_device.cuh"
#include "sm_icp.h"

namespace sm {
namespace vt {

using namespace smd;

constexpr int kVoteU     = 8;           // bucket entries each lane has in flight
constexpr int kItem      = 32 * kVoteU; // bucket entries per warp work item
constexpr int kNarrowMax = 65535;       // 16-bit counters are exact up to this many votes

// Everything a voting kernel reads or writes.
struct VoteArgs {
    // model
    const float4 *sp, *sn;
    int           ns;
    const uint4  *htab;
    uint32_t      hmask;
    const uint2  *entries;
    int           A;
    float         angleStep, distStep, smax, sqDiam, voteThreshold;
    // scene
    const float4 *pos, *nrm;
    const int    *kp;
    int           K;
    const int    *nbrOff, *nbrIds; // CSR neighbour lists, or
    const int    *cand;            // radius mode: candidate point ids (ascending)
    int           ncand;
    // accumulator sizing
    int refChunk;     // reference points per accumulator pass with 16-bit counters
    int refChunkWide; // the same with 32-bit counters
    // outputs
    long long *stats; // K x 8
    float     *cands, *poses;
    int       *poseOk;
    int       *acc;
    int        dumpK;
    int        forceWide;   // 32-bit counters for every keypoint (a test switch)
    int        fingerprint; // fold the accumulators into stats column 4 (a test switch)
};

struct Cand {
    float v;
    int   r, j;
};

__device__ __forceinline__ bool before(const Cand &a, const Cand &b) {
    return a.v > b.v || (a.v == b.v && a.r < b.r);
}

__device__ __forceinline__ void top3_insert(Cand t[3], const Cand &c) {
    if (!before(c, t[2]))
        return;
    if (before(c, t[1])) {
        t[2] = t[1];
        if (before(c, t[0])) {
            t[1] = t[0];
            t[0] = c;
        } else {
            t[1] = c;
        }
    } else {
        t[2] = c;
    }
}

// Open-addressed model table of uint4 {key, first entry, entry count, 0}; count 0 = empty.
__device__ __forceinline__ uint32_t probe(const uint4 *__restrict__ tab, uint32_t mask, uint32_t key,
                                          uint32_t &off, uint32_t &mult) {
    uint32_t i = key & mask;
    for (uint32_t n = 0; n <= mask; n++) {
        const uint4 s = tab[i];
        if (s.z == 0)
            return 0;
        if (s.x == key) {
            off  = s.y;
            mult = s.w;
            return s.z;
        }
        i = (i + 1) & mask;
    }
    return 0;
}

// Votes of the hits hOff/hCnt/hAs/hAsT[0..nHits) into the shared accumulator of reference
// points [r0, r1). A hit's bucket is cut into items of kItem consecutive entries (cPre:
// prefix of items per hit, T in all) and each warp takes a contiguous range of items.
// Within an item the hit's values are warp-uniform registers, lane l owns entries l, l+32,
// ... and issues all its kVoteU loads before the first use, so one L2 latency covers 256
// votes and the loads coalesce. `narrow`: two 16-bit counters per 32-bit word.
__device__ __forceinline__ void cast_votes(const VoteArgs &a, uint32_t *acc, const int *hOff,
                                           const int *hCnt, const float *hAs, const float *hAsT,
                                           const int *cPre, int nHits, int T, int r0, int r1,
                                           bool narrow) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int i0 = (int)((long long)T * w / nw), i1 = (int)((long long)T * (w + 1) / nw);
    if (i0 >= i1)
        return;
    int lo = 0, hi = nHits - 1; // the hit holding item i0: last h with cPre[h] <= i0
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (cPre[mid] <= i0)
            lo = mid;
        else
            hi = mid - 1;
    }
    int        h       = lo;
    const bool allRefs = r0 == 0 && r1 == a.ns; // one pass holds every reference point
    for (int item = i0; item < i1; item++) {
        while (cPre[h + 1] <= item)
            h++;
        const int    B    = hCnt[h];
        const float  as   = hAs[h];
        const float  asT  = hAsT[h];
        const int    e0   = (item - cPre[h]) * kItem;
        const int    eEnd = min(B, e0 + kItem);
        const int    vecB = B - B % smm::kLanes;
        const uint2 *src  = a.entries + hOff[h];
        uint2        ent[kVoteU];
#pragma unroll
        for (int u = 0; u < kVoteU; u++) {
            const int e = e0 + u * 32 + lane;
            ent[u]      = e < eEnd ? src[e] : make_uint2(0xffffffffu, 0u);
        }
#pragma unroll
        for (int u = 0; u < kVoteU; u++) {
            const int  e   = e0 + u * 32 + lane;
            const int  ref = (int)ent[u].x;
            const bool ok  = !(e >= eEnd || (!allRefs && (ref < r0 || ref >= r1)));
            if (!ok)
                continue;
            const float am = __uint_as_float(ent[u].y);
            uint32_t    bin;
            if (e0 + u * 32 + 32 <= vecB) // warp-uniform: the round lies in the 8-lane blocks
                bin = smm::vote_bin(true, am, as, asT, a.smax);
            else
                bin = smm::vote_bin(e < vecB, am, as, asT, a.smax);
            bin         = min(bin, (uint32_t)(a.A - 1)); // unreachable; keeps the index in range
            const int c = (ref - r0) * a.A + (int)bin;
            // one increment per vote: a warp's votes rarely share a cell (a bucket's
            // entries are different pairs), so aggregating them first measured 2.8x
            // slower on the large scene
            if (narrow)
                atomicAdd(&acc[c >> 1], 1u << ((c & 1) * 16));
            else
                atomicAdd(&acc[c], 1u);
        }
    }
}

__device__ __forceinline__ int acc_get(const uint32_t *acc, int e, bool narrow) {
    return narrow ? (int)((acc[e >> 1] >> ((e & 1) * 16)) & 0xffffu) : (int)acc[e];
}

// Peaks of the accumulator rows of reference points [r0, r1) (ppf.cpp:363-389): first
// argmax, both circular neighbours added; rows whose total or maximum is below half the
// vote threshold are skipped. A thread per row; 16-bit rows of an even length are read two
// counters per 32-bit word. With FP, every non-zero cell is also folded into the
// fingerprint (a check of the whole accumulator, for tests).
template <bool FP>
__device__ __forceinline__ void peaks_rows(const VoteArgs &a, const uint32_t *acc, bool narrow,
                                           int r0, int r1, Cand top[3],
                                           unsigned long long &myHash) {
    const int   A     = a.A;
    const float thre  = a.voteThreshold / 2.0f;
    const bool  pairs = narrow && (A & 1) == 0;
    for (int i = r0 + (int)threadIdx.x; i < r1; i += blockDim.x) {
        const int e0    = (i - r0) * A;
        int       total = 0, j = 0, best = -1;
        auto      cell  = [&](int t, int v) {
            total += v;
            if (v > best) {
                best = v;
                j    = t;
            }
            if (FP && v)
                myHash += smm::mix64(((unsigned long long)(i * A + t) << 32) | (uint32_t)v);
        };
        if (pairs) {
            const uint32_t *w = acc + (e0 >> 1);
            for (int t = 0; t < A; t += 2) {
                const uint32_t x = w[t >> 1];
                cell(t, (int)(x & 0xffffu));
                cell(t + 1, (int)(x >> 16));
            }
        } else {
            for (int t = 0; t < A; t++)
                cell(t, acc_get(acc, e0 + t, narrow));
        }
        if ((float)total < thre || (float)best < thre)
            continue;
        int vote = best;
        vote += acc_get(acc, e0 + ((j == 0) ? A - 1 : j - 1), narrow);
        vote += acc_get(acc, e0 + ((j == A - 1) ? 0 : j + 1), narrow);
        top3_insert(top, Cand{(float)vote, i, j});
    }
}

__device__ __forceinline__ void peaks_chunk(const VoteArgs &a, const uint32_t *acc, bool narrow,
                                            int r0, int r1, Cand top[3],
                                            unsigned long long &myHash) {
    if (a.fingerprint)
        peaks_rows<true>(a, acc, narrow, r0, r1, top, myHash);
    else
        peaks_rows<false>(a, acc, narrow, r0, r1, top, myHash);
}

__device__ __forceinline__ void dump_chunk(const VoteArgs &a, int c, const uint32_t *acc,
                                           bool narrow, int r0, int r1) {
    if (c >= a.dumpK)
        return;
    int      *d     = a.acc + ((size_t)c * a.ns + r0) * a.A;
    const int nElem = (r1 - r0) * a.A;
    for (int i = threadIdx.x; i < nElem; i += blockDim.x)
        d[i] = acc_get(acc, i, narrow);
}

// The keypoint's result: the block's top-3 candidates by (votes desc, reference asc), the
// poses of those within 95% of the best (ppf.cpp:391-409) and its statistics row
// {searched, 0, hits, votes, fingerprint, candidates, poses, counter bound}. wc needs
// blockDim/32 x 3 Cand, shash one zeroed word; both in shared memory.
__device__ __forceinline__ void finish_keypoint(const VoteArgs &a, int c, const smm::RT &rt,
                                                Cand top[3], unsigned long long myHash,
                                                long long searched, long long nHits,
                                                long long V, long long bound, Cand (*wc)[3],
                                                unsigned long long *shash) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        Cand other[3];
        for (int t = 0; t < 3; t++) {
            other[t].v = __shfl_xor_sync(0xffffffffu, top[t].v, o);
            other[t].r = __shfl_xor_sync(0xffffffffu, top[t].r, o);
            other[t].j = __shfl_xor_sync(0xffffffffu, top[t].j, o);
        }
        for (int t = 0; t < 3; t++)
            top3_insert(top, other[t]);
        myHash += __shfl_xor_sync(0xffffffffu, myHash, o);
    }
    if (lane == 0) {
        for (int t = 0; t < 3; t++)
            wc[w][t] = top[t];
        atomicAdd(shash, myHash);
    }
    __syncthreads();
    if (tid != 0)
        return;
    Cand t3[3];
    for (int t = 0; t < 3; t++)
        t3[t] = Cand{-1.0f, INT_MAX, 0};
    for (int ww = 0; ww < nw; ww++)
        for (int t = 0; t < 3; t++)
            if (wc[ww][t].r != INT_MAX)
                top3_insert(t3, wc[ww][t]);
    int nc = 0;
    for (int t = 0; t < 3; t++)
        nc += t3[t].r != INT_MAX ? 1 : 0;
    for (int t = 0; t < 3; t++) {
        float *cc = a.cands + (size_t)c * 9 + t * 3;
        cc[0]     = t < nc ? t3[t].v : -1.0f;
        cc[1]     = t < nc ? (float)t3[t].r : -1.0f;
        cc[2]     = t < nc ? (float)t3[t].j : -1.0f;
    }
    int npose = 0;
    if (nc > 0) {
        const float thr2 = (float)((double)t3[0].v * 0.95);
        for (int t = 0; t < nc; t++) {
            if (t3[t].v < thr2)
                continue;
            const float4  pm = a.sp[t3[t].r], nm = a.sn[t3[t].r];
            const smm::RT rm = smm::transform_rt(pm.x, pm.y, pm.z, nm.x, nm.y, nm.z);
            const float   al = smm::candidate_angle(t3[t].j, a.A - 1);
            smi::candidate_pose(rt, rm, al, t3[t].v,
                                a.poses + ((size_t)c * 3 + npose) * smi::kPoseFloats);
            npose++;
        }
    }
    for (int t = 0; t < 3; t++)
        a.poseOk[(size_t)c * 3 + t] = t < npose ? 1 : 0;
    long long *st = a.stats + (size_t)c * 8;
    st[0]         = searched;
    st[1]         = 0;
    st[2]         = nHits;
    st[3]         = V;
    st[4]         = (long long)*shash;
    st[5]         = nc;
    st[6]         = npose;
    st[7]         = bound;
}

// A keypoint that casts no votes: its normal is not finite (flag 1) or fewer neighbours
// than the vote threshold were found (flag 2).
__device__ __forceinline__ void skip_keypoint(const VoteArgs &a, int c, long long searched,
                                              bool nanN) {
    const int tid = threadIdx.x;
    long long *st = a.stats + (size_t)c * 8;
    if (tid < 8)
        st[tid] = tid == 0 ? searched : (tid == 1 ? (nanN ? 1 : 2) : 0);
    if (tid < 3) {
        a.poseOk[(size_t)c * 3 + tid] = 0;
        for (int e = 0; e < 3; e++)
            a.cands[(size_t)c * 9 + tid * 3 + e] = -1.0f;
    }
}

// Shared-memory sizing of the accumulator (host): 16-bit counters for all reference points
// when two CTAs of `staticBytes` then fit an SM, else as many reference points per pass as
// one CTA can hold; the 32-bit passes reuse the same bytes. Returns the dynamic bytes.
inline size_t acc_sizing(int ns, int A, long long staticBytes, int optin, int perSM,
                         int *refChunk, int *refChunkWide) {
    const long long narrowAll = ((long long)ns * A + 1) / 2 * 4;
    const long long cap       = optin - staticBytes;
    long long dyn = narrowAll + staticBytes + 1024 <= perSM / 2 ? narrowAll : std::min(narrowAll, cap);
    dyn           = std::max<long long>(dyn, (long long)A * 4) & ~3ll;
    if (dyn > cap)
        return 0;
    *refChunk     = (int)std::max<long long>(1, std::min<long long>(ns, dyn / 4 * 2 / A));
    *refChunkWide = (int)std::max<long long>(1, std::min<long long>(ns, dyn / 4 / A));
    return (size_t)dyn;
}

} // namespace vt
} // namespace sm
