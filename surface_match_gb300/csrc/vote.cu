// vote.cu - the voting stage in one kernel, for callers that give no workspace (the
// allocation-free entry), and the model pair features of trainModel (ppf.cpp:105-143).
//
// One CTA per keypoint over caller-given CSR neighbour lists. The list is read in windows:
// the window's rows (the reference's 8-lane block / scalar tail rule chosen by the row's
// list position) are compacted, each row's quantised PPF key and scene alpha computed and
// the model table probed; the hit buckets are then voted into a shared-memory (reference
// point x angle bin) accumulator with shared atomics. Peaks, the top three candidates and
// their poses come out of the same kernel. The multi-kernel pipeline in vote_pipe.cu
// produces the same results with more parallelism when a workspace is available.
#include <cstdlib>
#include "sm_stages.h"
#include "sm_vote.cuh"

namespace sm {
using namespace smd;
using namespace vt;

namespace {

constexpr int kVoteBs = 512;
constexpr int kWin    = 2048; // list entries per window: rows and hits of a window fit

__global__ void __launch_bounds__(kVoteBs, 2) k_vote_fused(VoteArgs a) {
    extern __shared__ uint32_t acc[];
    __shared__ int       rows[kWin];
    __shared__ int       hOff[kWin], hCnt[kWin], cPre[kWin + 1];
    __shared__ float     hAs[kWin], hAsT[kWin];
    __shared__ int       sh[33];
    __shared__ smm::RT   rt;
    __shared__ Cand      wc[kVoteBs / 32][3];
    __shared__ long long sHitsTot, sVotesTot, sBoundTot;
    __shared__ unsigned long long shash;
    __shared__ int       sRows, sHits, sVotes, sBound, sTail;

    const int    c       = blockIdx.x;
    const int    tid     = threadIdx.x;
    const int    lane    = tid & 31;
    const int    pid     = a.kp[c];
    const float4 p1      = a.pos[pid];
    const float4 n1      = a.nrm[pid];
    const int    listBeg = a.nbrOff[c];
    const int    listLen = a.nbrOff[c + 1] - listBeg;
    const int   *list    = a.nbrIds + listBeg;
    // rows: the list without the keypoint itself (the reference's radius search returns it)
    int myR = 0;
    for (int i = tid; i < listLen; i += kVoteBs)
        myR += list[i] != pid ? 1 : 0;
    int R;
    block_excl_scan(myR, sh, &R);
    if (tid == 0) {
        sHitsTot = sVotesTot = sBoundTot = 0;
        shash                = 0;
        rt                   = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
    }
    const bool nanN = !(isfinite(n1.x) && isfinite(n1.y) && isfinite(n1.z));
    if (nanN || (float)listLen < a.voteThreshold) {
        skip_keypoint(a, c, listLen, nanN);
        return;
    }
    // The reference computes a keypoint's rows in 8-lane blocks and the last R % 8 one by
    // one (different float rounding): the list position of the first of those tail rows.
    if (tid < 32) {
        int need = R % smm::kLanes, found = listLen;
        for (int end = listLen; end > 0 && need > 0; end -= 32) {
            const int i = end - 1 - lane;
            uint32_t  b = __ballot_sync(0xffffffffu, i >= 0 && list[i] != pid);
            const int k = __popc(b);
            if (k >= need) {
                for (int t = 1; t < need; t++)
                    b &= b - 1;
                found = end - 1 - (__ffs(b) - 1);
                need  = 0;
            } else {
                need -= k;
            }
        }
        if (lane == 0)
            sTail = found;
    }
    __syncthreads();
    const int tailIdx = sTail;
    Cand      top[3];
    for (int t = 0; t < 3; t++)
        top[t] = Cand{-1.0f, INT_MAX, 0};
    unsigned long long myHash = 0;

    bool narrow    = !a.forceWide;
    int  chunk     = narrow ? a.refChunk : a.refChunkWide;
    bool statsDone = false;
    for (int r0 = 0; r0 < a.ns;) {
        const int r1     = min(r0 + chunk, a.ns);
        const int nElem  = (r1 - r0) * a.A;
        const int nWords = narrow ? (nElem + 1) >> 1 : nElem;
        for (int i = tid; i < nWords; i += kVoteBs)
            acc[i] = 0u;
        for (int w0 = 0; w0 < listLen; w0 += kWin) {
            const int w1 = min(listLen, w0 + kWin);
            if (tid == 0) {
                sRows  = 0;
                sHits  = 0;
                sVotes = 0;
                sBound = 0;
            }
            __syncthreads();
            // the window's rows, compacted (any order: votes are counts); bit 0 = block lane
            for (int i0 = w0; i0 < w1; i0 += kVoteBs) {
                const int      i     = i0 + tid;
                const int      id    = i < w1 ? list[i] : -1;
                const bool     row   = i < w1 && id != pid;
                const uint32_t b     = __ballot_sync(0xffffffffu, row);
                int            wbase = 0;
                if (lane == 0 && b)
                    wbase = atomicAdd(&sRows, __popc(b));
                wbase = __shfl_sync(0xffffffffu, wbase, 0);
                if (row)
                    rows[wbase + __popc(b & ((1u << lane) - 1u))] = id * 2 + (i < tailIdx ? 1 : 0);
            }
            __syncthreads();
            const int nRows = sRows;
            for (int k = tid; k < nRows; k += kVoteBs) {
                const int      v   = rows[k];
                const int      id  = v >> 1;
                const bool     blk = (v & 1) != 0;
                const float4   q   = a.pos[id];
                const float4   n2  = a.nrm[id];
                const uint32_t key = smm::ppf_key(blk, p1.x, p1.y, p1.z, n1.x, n1.y, n1.z, q.x,
                                                  q.y, q.z, n2.x, n2.y, n2.z, a.angleStep,
                                                  a.distStep);
                const float as = smm::alpha_of(blk, rt, q.x, q.y, q.z);
                if (smm::fisnan(as))
                    continue;
                uint32_t  off = 0, mult = 0;
                const int cnt = (int)probe(a.htab, a.hmask, key, off, mult);
                if (cnt > 0) {
                    const int hp = atomicAdd(&sHits, 1);
                    atomicAdd(&sVotes, cnt);
                    atomicAdd(&sBound, (int)mult);
                    hOff[hp] = (int)off;
                    hCnt[hp] = cnt;
                    hAs[hp]  = as;
                    hAsT[hp] = smm::alpha_tail_shift(as);
                }
            }
            __syncthreads();
            const int nHits = sHits;
            int       T     = 0;
            for (int h0 = 0; h0 < nHits; h0 += kVoteBs) {
                int       tot;
                const int nit = h0 + tid < nHits ? (hCnt[h0 + tid] + kItem - 1) / kItem : 0;
                const int pre = block_excl_scan(nit, sh, &tot);
                if (h0 + tid < nHits)
                    cPre[h0 + tid] = T + pre;
                T += tot;
            }
            if (tid == 0) {
                cPre[nHits] = T;
                if (!statsDone) {
                    sHitsTot += nHits;
                    sVotesTot += sVotes;
                    sBoundTot += sBound;
                }
            }
            __syncthreads();
            if (nHits > 0)
                cast_votes(a, acc, hOff, hCnt, hAs, hAsT, cPre, nHits, T, r0, r1, narrow);
            __syncthreads();
        }
        statsDone = true;
        if (narrow && sBoundTot > kNarrowMax) {
            // a counter may have overflowed 16 bits: vote again with 32-bit counters
            narrow = false;
            chunk  = a.refChunkWide;
            r0     = 0;
            continue;
        }
        peaks_chunk(a, acc, narrow, r0, r1, top, myHash);
        dump_chunk(a, c, acc, narrow, r0, r1);
        __syncthreads();
        r0 = r1;
    }
    finish_keypoint(a, c, rt, top, myHash, listLen, sHitsTot, sVotesTot, sBoundTot, wc, &shash);
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

// ---- the model table on the device ----------------------------------------------------
__global__ void k_pair_compact(const uint32_t *__restrict__ keys, const int *__restrict__ valid,
                               const int *__restrict__ pre, long long n, uint32_t *__restrict__ ck,
                               uint32_t *__restrict__ cv) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n || !valid[t])
        return;
    ck[pre[t]] = keys[t];
    cv[pre[t]] = (uint32_t)t;
}

__global__ void k_bucket_heads(const uint32_t *__restrict__ ck, int e, int *__restrict__ head) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > e)
        return;
    head[i] = (i < e && (i == 0 || ck[i] != ck[i - 1])) ? 1 : 0;
}

// Entry e of the sorted pairs: bucket key and offset at a bucket's first entry, and the
// (reference point, alpha bits) record.
__global__ void k_bucket_fill(const uint32_t *__restrict__ ck, const uint32_t *__restrict__ cv,
                              int e, const int *__restrict__ head, const int *__restrict__ bidx,
                              const float *__restrict__ alphas, int n1, uint32_t *__restrict__ dkeys,
                              uint32_t *__restrict__ doffs, uint2 *__restrict__ ent, int nkeys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e) {
        if (i == e)
            doffs[nkeys] = (uint32_t)e;
        return;
    }
    if (head[i]) {
        dkeys[bidx[i]] = ck[i];
        doffs[bidx[i]] = (uint32_t)i;
    }
    const uint32_t t = cv[i];
    ent[i]           = make_uint2(t / (uint32_t)n1, __float_as_uint(alphas[t]));
}

// Bucket b into the open-addressed table (linear probing from key & mask; slots are claimed
// by compare-and-swap, so placement depends on timing but every key sits after an unbroken
// run of occupied slots from its home slot, which is all a probe needs). The slot's last
// word is the bucket's largest number of entries of one reference point: entries are in
// pair order, so a reference point's entries are consecutive.
__global__ void k_bucket_insert(const uint32_t *__restrict__ dkeys, const uint32_t *__restrict__ doffs,
                                const uint2 *__restrict__ ent, int nkeys, uint32_t mask,
                                int *__restrict__ claim, uint4 *__restrict__ tab) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nkeys)
        return;
    const uint32_t k = dkeys[b], o0 = doffs[b], o1 = doffs[b + 1];
    uint32_t       best = 0, run = 0, prev = 0xffffffffu;
    for (uint32_t e = o0; e < o1; e++) {
        const uint32_t r = ent[e].x;
        run              = r == prev ? run + 1 : 1;
        prev             = r;
        best             = run > best ? run : best;
    }
    uint32_t i = k & mask;
    for (uint32_t n = 0; n <= mask; n++) {
        if (atomicCAS(&claim[i], -1, b) == -1) {
            tab[i] = make_uint4(k, o0, o1 - o0, best);
            return;
        }
        i = (i + 1) & mask;
    }
}

} // namespace

void build_model_table(Ctx &c, Model &m, const uint32_t *keys, const float *alphas,
                       const int *valid, int n1) {
    const long long npair = (long long)n1 * n1;
    int *pre = c.arena.get<int>("t.tab.pre", (size_t)npair + 1);
    int  E   = 0;
    if (npair > 0) {
        // valid flags of npair entries, exclusive scan with the total (pre[npair])
        scan_excl(c, valid, pre, npair, "t.tab.s1", false);
        SM_CUDA(cudaMemcpyAsync(c.hostCounts, pre + npair - 1, sizeof(int), cudaMemcpyDeviceToHost,
                                c.stream));
        SM_CUDA(cudaMemcpyAsync(c.hostCounts + 1, valid + npair - 1, sizeof(int),
                                cudaMemcpyDeviceToHost, c.stream));
        c.sync_checked();
        E = c.hostCounts[0] + c.hostCounts[1];
    }
    uint32_t *ck = c.arena.get<uint32_t>("t.tab.ck", std::max(E, 1));
    uint32_t *cv = c.arena.get<uint32_t>("t.tab.cv", std::max(E, 1));
    if (E > 0) {
        k_pair_compact<<<nblocks(npair, 256), 256, 0, c.stream>>>(keys, valid, pre, npair, ck, cv);
        SM_LAUNCH_CHECK();
        radix_sort_pairs(c, ck, cv, E, 32, "t.tab");
    }
    int *head = c.arena.get<int>("t.tab.head", (size_t)E + 1);
    int *bidx = c.arena.get<int>("t.tab.bidx", (size_t)E + 1);
    k_bucket_heads<<<nblocks((long long)E + 1, 256), 256, 0, c.stream>>>(ck, E, head);
    SM_LAUNCH_CHECK();
    const int nkeys = scan_excl(c, head, bidx, (long long)E + 1, "t.tab.s2", true);
    m.nkeys    = nkeys;
    m.nentries = E;
    SM_CUDA(cudaMalloc((void **)&m.dkeys, (size_t)std::max(nkeys, 1) * 4));
    SM_CUDA(cudaMalloc((void **)&m.doffs, ((size_t)nkeys + 1) * 4));
    SM_CUDA(cudaMalloc((void **)&m.entries, (size_t)std::max(E, 1) * sizeof(uint2)));
    k_bucket_fill<<<nblocks((long long)E + 1, 256), 256, 0, c.stream>>>(
        ck, cv, E, head, bidx, alphas, n1, m.dkeys, m.doffs, m.entries, nkeys);
    SM_LAUNCH_CHECK();
    uint32_t size = 16;
    while (size < 2u * (uint32_t)nkeys)
        size <<= 1;
    m.hmask    = size - 1;
    int *claim = c.arena.get<int>("t.tab.claim", size);
    SM_CUDA(cudaMalloc((void **)&m.hkeys, (size_t)size * sizeof(uint4)));
    SM_CUDA(cudaMemsetAsync(claim, 0xff, (size_t)size * 4, c.stream));
    SM_CUDA(cudaMemsetAsync(m.hkeys, 0, (size_t)size * sizeof(uint4), c.stream));
    if (nkeys > 0) {
        k_bucket_insert<<<nblocks(nkeys, 128), 128, 0, c.stream>>>(m.dkeys, m.doffs, m.entries, nkeys,
                                                                  m.hmask, claim, (uint4 *)m.hkeys);
        SM_LAUNCH_CHECK();
    }
    c.sync_checked();
}

void fill_vote_model(const Model &m, float minScore, VoteArgs &a) {
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
}

void vote_fused(Ctx &c, const Model &m, const float4 *pos, const float4 *nrm, const int *kp,
                int K, const int *nbrOff, const int *nbrIds, float minScore, const VoteOut &out,
                int dumpK) {
    if (K <= 0)
        return;
    VoteArgs a{};
    fill_vote_model(m, minScore, a);
    a.pos    = pos;
    a.nrm    = nrm;
    a.kp     = kp;
    a.K      = K;
    a.nbrOff = nbrOff;
    a.nbrIds = nbrIds;
    a.stats  = out.stats;
    a.cands  = out.cands;
    a.poses  = out.poses;
    a.poseOk = out.poseOk;
    a.acc    = out.acc;
    a.dumpK  = out.acc ? dumpK : 0;
    // the same test switch as the pipelined stage: 32-bit counters for every keypoint
    const char *fw = std::getenv("SM_VOTE_FORCE_WIDE");
    a.forceWide    = (fw && fw[0] == '1') ? 1 : 0;
    // SM_VOTE_FINGERPRINT=1 folds every accumulator into stats column 4 (checked by tests
    // against the oracle); without it the column is 0 and the peak scan skips the work
    const char *fp = std::getenv("SM_VOTE_FINGERPRINT");
    a.fingerprint  = (fp && fp[0] == '1') ? 1 : 0;

    int optin = 0, perSM = 0;
    SM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    SM_CUDA(cudaDeviceGetAttribute(&perSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c.device));
    cudaFuncAttributes fa;
    SM_CUDA(cudaFuncGetAttributes(&fa, k_vote_fused));
    const size_t smem = acc_sizing(a.ns, a.A, (long long)fa.sharedSizeBytes, optin, perSM,
                                   &a.refChunk, &a.refChunkWide);
    if (!smem)
        throw Error(SM_ERR_CAPACITY, "featAngleResolution too large for the vote accumulator");
    if (smem > allow_dynamic_smem((const void *)k_vote_fused, c.device))
        throw Error(SM_ERR_CAPACITY, "shared-memory request above the device limit");
    k_vote_fused<<<K, kVoteBs, smem, c.stream>>>(a);
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
