// vote.cu - the voting hot loop of matchScene (ppf.cpp:247-409) and the model pair
// features of trainModel (ppf.cpp:105-143).
//
// One CTA per keypoint. For each neighbour row: the quantised PPF key and scene alpha
// (sm_math.h, with the reference's 8-lane block / scalar tail rule chosen by the row's
// position), one probe of the open-addressed model table, then the matched bucket's
// entries are spread over the whole CTA (flattened by a prefix sum over the hit buckets of
// the tile) and binned into a shared-memory (reference point x angle bin) accumulator
// with shared atomics. Peaks (first argmax + both circular neighbours), the top three
// candidates by (votes desc, reference asc) and their poses are produced in the same
// kernel.
#include <climits>

#include "sm_icp.h"
#include "sm_stages.h"

namespace sm {
using namespace smd;

namespace {

constexpr int kVoteBs = 512;

struct VoteArgs {
    const float4 *sp, *sn;
    int           ns;
    const uint4  *htab;
    uint32_t      hmask;
    const uint2  *entries;
    int           A;
    float         angleStep, distStep, smax, sqDiam, voteThreshold;
    const float4 *pos, *nrm;
    const int    *kp;
    const int    *nbrOff, *nbrIds; // CSR mode
    const int    *cand;            // radius mode: candidate point ids (ascending)
    int           ncand;
    int           refChunk;
    long long    *stats;
    float        *cands, *poses;
    int          *poseOk;
    int          *acc;
    int           dumpK;
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

__device__ __forceinline__ uint32_t probe(const uint4 *__restrict__ tab, uint32_t mask, uint32_t key,
                                          uint32_t &off) {
    uint32_t i = key & mask;
    for (uint32_t n = 0; n <= mask; n++) {
        const uint4 s = tab[i];
        if (s.z == 0)
            return 0;
        if (s.x == key) {
            off = s.y;
            return s.z;
        }
        i = (i + 1) & mask;
    }
    return 0;
}

constexpr int kRowBuf = 2048; // rows buffered per processing round

// Votes of the hits hOff/hCnt/hAs/hAsT[0..nHits) (prefix hPre, total V) into the shared
// accumulator. Each warp takes a contiguous range of votes and walks the hit list forward,
// so a lane finds its hit in a step or two instead of a binary search per vote.
__device__ __forceinline__ void cast_votes(const VoteArgs &a, uint32_t *acc, const int *hOff,
                                           const int *hCnt, const float *hAs, const float *hAsT,
                                           const int *hPre, int nHits, int V, int r0, int r1) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = kVoteBs / 32;
    const int per  = (V + nw - 1) / nw;
    const int v0 = w * per, v1 = min(V, v0 + per);
    if (v0 >= v1)
        return;
    int lo = 0, hi = nHits - 1; // last hit with hPre <= v0
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (hPre[mid] <= v0)
            lo = mid;
        else
            hi = mid - 1;
    }
    int h = lo;
    for (int base = v0; base < v1; base += 32) {
        const int v = base + lane;
        int       hv = h;
        if (v < v1) {
            while (hPre[hv + 1] <= v)
                hv++;
            const int   e   = v - hPre[hv];
            const int   B   = hCnt[hv];
            const uint2 ent = a.entries[hOff[hv] + e];
            const int   ref = (int)ent.x;
            if (ref >= r0 && ref < r1) {
                uint32_t bin = smm::vote_bin(e < B - B % smm::kLanes, __uint_as_float(ent.y),
                                             hAs[hv], hAsT[hv], a.smax);
                if (bin > (uint32_t)(a.A - 1))
                    bin = a.A - 1; // unreachable; keeps the index in range
                atomicAdd(&acc[(ref - r0) * a.A + bin], 1u);
            }
        }
        h = __shfl_sync(0xffffffffu, hv, 31);
    }
}

template <bool CSR> __global__ void __launch_bounds__(kVoteBs) k_vote(VoteArgs a) {
    extern __shared__ uint32_t acc[];
    __shared__ int       rows[kRowBuf];
    __shared__ int       hOff[kRowBuf], hCnt[kRowBuf], hPre[kRowBuf + 1];
    __shared__ float     hAs[kRowBuf], hAsT[kRowBuf];
    __shared__ int       sh[33];
    __shared__ smm::RT   rt;
    __shared__ Cand      wc[kVoteBs / 32][3];
    __shared__ long long sstat[4];
    __shared__ unsigned long long shash;
    __shared__ int       sRows, sSearched, sHits;

    const int c   = blockIdx.x;
    const int tid = threadIdx.x;
    const int pid = a.kp[c];
    const float4 p1 = a.pos[pid];
    const float4 n1 = a.nrm[pid];
    int listBeg = 0, listLen = 0;
    if (CSR) {
        listBeg = a.nbrOff[c];
        listLen = a.nbrOff[c + 1] - listBeg;
    } else {
        listLen = a.ncand;
    }
    // neighbour count (self included, as the reference's radius search returns it) and
    // the number of rows (self excluded)
    int myS = 0, myR = 0;
    for (int i = tid; i < listLen; i += kVoteBs) {
        const int id = CSR ? a.nbrIds[listBeg + i] : a.cand[i];
        bool      in = true;
        if (!CSR) {
            const float4 q = a.pos[id];
            in             = smm::dist2(p1.x, p1.y, p1.z, q.x, q.y, q.z) < a.sqDiam;
        }
        myS += in ? 1 : 0;
        myR += (in && id != pid) ? 1 : 0;
    }
    {
        int tS, tR;
        block_excl_scan(myS, sh, &tS);
        block_excl_scan(myR, sh, &tR);
        if (tid == 0) {
            sSearched = tS;
            sRows     = tR;
        }
    }
    if (tid == 0) {
        sstat[0] = sstat[1] = sstat[2] = sstat[3] = 0;
        shash                                     = 0;
        rt = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
    }
    __syncthreads();
    const int searched = sSearched;
    const int R        = sRows;
    long long *st      = a.stats + (size_t)c * 8;
    const bool nanN    = !(isfinite(n1.x) && isfinite(n1.y) && isfinite(n1.z));
    if (nanN || (float)searched < a.voteThreshold) {
        if (tid < 8)
            st[tid] = tid == 0 ? searched : (tid == 1 ? (nanN ? 1 : 2) : 0);
        if (tid < 3) {
            a.poseOk[(size_t)c * 3 + tid] = 0;
            for (int e = 0; e < 3; e++)
                a.cands[(size_t)c * 9 + tid * 3 + e] = -1.0f;
        }
        return;
    }
    const int vecR = R - R % smm::kLanes;
    const int A    = a.A;
    Cand      top[3];
    for (int t = 0; t < 3; t++)
        top[t] = Cand{-1.0f, INT_MAX, 0};
    unsigned long long myHash = 0;

    for (int r0 = 0; r0 < a.ns; r0 += a.refChunk) {
        const int r1 = min(r0 + a.refChunk, a.ns);
        const int nb = (r1 - r0) * A;
        for (int i = tid; i < nb; i += kVoteBs)
            acc[i] = 0u;
        int rowBase = 0, nBuf = 0;
        for (int base = 0; base < listLen || nBuf > 0; base += kVoteBs) {
            // gather the next tile's rows (in list order) into the buffer
            if (base < listLen) {
                const int i   = base + tid;
                int       id  = -1;
                bool      row = false;
                if (i < listLen) {
                    id = CSR ? a.nbrIds[listBeg + i] : a.cand[i];
                    if (id != pid) {
                        if (CSR) {
                            row = true;
                        } else {
                            const float4 q = a.pos[id];
                            row = smm::dist2(p1.x, p1.y, p1.z, q.x, q.y, q.z) < a.sqDiam;
                        }
                    }
                }
                int       nRows;
                const int rp = block_excl_scan(row ? 1 : 0, sh, &nRows);
                if (row)
                    rows[nBuf + rp] = id;
                nBuf += nRows;
            }
            const bool last = base + kVoteBs >= listLen;
            if (nBuf + kVoteBs <= kRowBuf && !last)
                continue;
            // process the buffered rows: keys, alphas, probes; hits in any order
            if (tid == 0)
                sHits = 0;
            __syncthreads();
            for (int k = tid; k < nBuf; k += kVoteBs) {
                const int    id  = rows[k];
                const int    rpos = rowBase + k;
                const bool   blk = rpos < vecR;
                const float4 q   = a.pos[id];
                const float4 n2  = a.nrm[id];
                const uint32_t key = smm::ppf_key(blk, p1.x, p1.y, p1.z, n1.x, n1.y, n1.z, q.x, q.y,
                                                  q.z, n2.x, n2.y, n2.z, a.angleStep, a.distStep);
                const float as = smm::alpha_of(blk, rt, q.x, q.y, q.z);
                if (smm::fisnan(as))
                    continue;
                uint32_t  off = 0;
                const int cnt = (int)probe(a.htab, a.hmask, key, off);
                if (cnt > 0) {
                    const int hp = atomicAdd(&sHits, 1);
                    hOff[hp]     = (int)off;
                    hCnt[hp]     = cnt;
                    hAs[hp]      = as;
                    hAsT[hp]     = smm::alpha_tail_shift(as);
                }
            }
            __syncthreads();
            const int nHits = sHits;
            int       V     = 0;
            for (int h0 = 0; h0 < nHits; h0 += kVoteBs) {
                int       tot;
                const int pre = block_excl_scan(h0 + tid < nHits ? hCnt[h0 + tid] : 0, sh, &tot);
                if (h0 + tid < nHits)
                    hPre[h0 + tid] = V + pre;
                V += tot;
            }
            if (tid == 0) {
                hPre[nHits] = V;
                if (r0 == 0) {
                    sstat[2] += nHits;
                    sstat[3] += V;
                }
            }
            __syncthreads();
            if (nHits > 0)
                cast_votes(a, acc, hOff, hCnt, hAs, hAsT, hPre, nHits, V, r0, r1);
            __syncthreads();
            rowBase += nBuf;
            nBuf = 0;
        }
        // peaks of this reference-point chunk (ppf.cpp:363-389)
        const float thre = a.voteThreshold / 2.0f;
        for (int i = r0 + tid; i < r1; i += kVoteBs) {
            const uint32_t *b     = acc + (i - r0) * A;
            int             total = 0, j = 0;
            int             best  = (int)b[0];
            for (int t = 0; t < A; t++) {
                const int v = (int)b[t];
                total += v;
                if (v > best) {
                    best = v;
                    j    = t;
                }
                if (v)
                    myHash += smm::mix64(((unsigned long long)(i * A + t) << 32) | (uint32_t)v);
            }
            if ((float)total < thre || (float)best < thre)
                continue;
            int vote = best;
            vote += (j == 0) ? (int)b[A - 1] : (int)b[j - 1];
            vote += (j == A - 1) ? (int)b[0] : (int)b[j + 1];
            top3_insert(top, Cand{(float)vote, i, j});
        }
        if (c < a.dumpK) {
            int *d = a.acc + ((size_t)c * a.ns + r0) * A;
            for (int i = tid; i < nb; i += kVoteBs)
                d[i] = (int)acc[i];
        }
        __syncthreads();
    }
    // reduce top-3 lists and the fingerprint over the block
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
    const int w = tid >> 5, lane = tid & 31;
    if (lane == 0) {
        for (int t = 0; t < 3; t++)
            wc[w][t] = top[t];
        atomicAdd(&shash, myHash);
    }
    __syncthreads();
    if (tid == 0) {
        Cand t3[3];
        for (int t = 0; t < 3; t++)
            t3[t] = Cand{-1.0f, INT_MAX, 0};
        for (int ww = 0; ww < kVoteBs / 32; ww++)
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
                const float   al = smm::candidate_angle(t3[t].j, A - 1);
                smi::candidate_pose(rt, rm, al, t3[t].v,
                                    a.poses + ((size_t)c * 3 + npose) * smi::kPoseFloats);
                npose++;
            }
        }
        for (int t = 0; t < 3; t++)
            a.poseOk[(size_t)c * 3 + t] = t < npose ? 1 : 0;
        st[0] = searched;
        st[1] = 0;
        st[2] = sstat[2];
        st[3] = sstat[3];
        st[4] = (long long)shash;
        st[5] = nc;
        st[6] = npose;
        st[7] = 0;
    }
}

// trainModel pair rows: for reference point i and column j, key and alpha with the
// column's lane rule (ppf.cpp:126-143: computePPF/computeAlpha over all N columns).
__global__ void k_model_pairs(const float4 *__restrict__ sp, const float4 *__restrict__ sn, int ns,
                              float angleStep, float distStep, uint32_t *__restrict__ keys,
                              float *__restrict__ alphas, int *__restrict__ valid) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)ns * ns)
        return;
    const int    i = (int)(t / ns), j = (int)(t % ns);
    const float4 p1 = sp[i], n1 = sn[i], p2 = sp[j], n2 = sn[j];
    const int    vec = ns - ns % smm::kLanes;
    const bool   blk = j < vec;
    const bool   ok1 = isfinite(n1.x) && isfinite(n1.y) && isfinite(n1.z);
    if (!ok1 || i == j) {
        valid[t] = 0;
        return;
    }
    const smm::RT rt = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
    const float   al = smm::alpha_of(blk, rt, p2.x, p2.y, p2.z);
    keys[t]   = smm::ppf_key(blk, p1.x, p1.y, p1.z, n1.x, n1.y, n1.z, p2.x, p2.y, p2.z, n2.x, n2.y,
                             n2.z, angleStep, distStep);
    alphas[t] = al;
    valid[t]  = smm::fisnan(al) ? 0 : 1;
}

} // namespace

void vote(Ctx &c, const Model &m, const float4 *pos, const float4 *nrm, const int *kp, int K,
          const int *nbrOff, const int *nbrIds, const int *cand, int ncand, float minScore,
          const VoteOut &out, int dumpK) {
    if (K <= 0)
        return;
    VoteArgs a;
    a.sp            = m.sp;
    a.sn            = m.sn;
    a.ns            = m.ns;
    a.htab          = (const uint4 *)m.hkeys;
    a.hmask         = m.hmask;
    a.entries       = m.entries;
    a.A             = m.tp.featAngleResolution;
    a.angleStep     = smm::k2PiF / (float)a.A;
    a.distStep      = m.box.diameter() * m.tp.featDistanceStepRel;
    a.smax          = (float)(a.A - 1) / smm::k2PiF;
    const float d   = m.box.diameter();
    a.sqDiam        = d * d;
    a.voteThreshold = (float)m.ns * minScore;
    a.pos           = pos;
    a.nrm           = nrm;
    a.kp            = kp;
    a.nbrOff        = nbrOff;
    a.nbrIds        = nbrIds;
    a.cand          = cand;
    a.ncand         = ncand;
    a.stats         = out.stats;
    a.cands         = out.cands;
    a.poses         = out.poses;
    a.poseOk        = out.poseOk;
    a.acc           = out.acc;
    a.dumpK         = out.acc ? dumpK : 0;
    int maxSmem = 0;
    SM_CUDA(cudaDeviceGetAttribute(&maxSmem, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    const int staticSmem = 24 * (int)kRowBuf + 8 * 1024;
    int       budget     = maxSmem - staticSmem;
    a.refChunk = std::max(1, std::min(m.ns, budget / (int)(a.A * sizeof(uint32_t))));
    const size_t smem = (size_t)a.refChunk * a.A * sizeof(uint32_t);
    if (nbrOff) {
        SM_CUDA(cudaFuncSetAttribute(k_vote<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_vote<true><<<K, kVoteBs, smem, c.stream>>>(a);
    } else {
        SM_CUDA(cudaFuncSetAttribute(k_vote<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_vote<false><<<K, kVoteBs, smem, c.stream>>>(a);
    }
    SM_LAUNCH_CHECK();
}

void model_pairs(Ctx &c, const float4 *sp, const float4 *sn, int ns, float angleStep,
                 float distStep, uint32_t *keys, float *alphas, int *valid) {
    const long long n = (long long)ns * ns;
    if (n == 0)
        return;
    k_model_pairs<<<nblocks(n, 256), 256, 0, c.stream>>>(sp, sn, ns, angleStep, distStep, keys,
                                                         alphas, valid);
    SM_LAUNCH_CHECK();
}

} // namespace sm
