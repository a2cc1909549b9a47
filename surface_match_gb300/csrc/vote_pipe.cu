// vote_pipe.cu - the voting stage of matchScene (ppf.cpp:247-409) as a pipeline of
// kernels, each shaped for what it spends its time on.
//
//  1. k_kp_radius / k_kp_csr: per keypoint its neighbour count, its rows (neighbours other
//     than itself) and the list position of its first "tail" row - the reference computes
//     a keypoint's rows in 8-lane blocks and the last (rows mod 8) one by one, with
//     different float rounding. In radius mode (all candidates within the model diameter,
//     in ascending order) the rows are kept as a bitmask over the candidate list, computed
//     from candidate tiles staged in shared memory and shared by eight keypoints.
//  2. A prefix sum over the rows gives every keypoint a segment of the row list.
//  3. k_rows_fill writes (keypoint, point, lane rule) per row into its segment.
//  4. k_ppf: one thread per row at full occupancy - quantised PPF key, scene alpha, model
//     table probe; a hit (bucket, count, alpha) is appended to the keypoint's segment.
//  5. k_lpt: keypoints ordered by their vote count, largest first, so the heaviest
//     accumulators start first and the tail of the next kernel stays short.
//  6. k_vote_acc: one CTA per keypoint votes its hits into a shared-memory (reference
//     point x angle bin) accumulator - 16-bit counters when the keypoint's vote count
//     allows - then extracts peaks, the top three candidates and their poses.
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "sm_stages.h"
#include "sm_vote.cuh"

namespace sm {
using namespace smd;
using namespace vt;

void fill_vote_model(const Model &m, float minScore, VoteArgs &a);

namespace {

constexpr int kKpWarps   = 8;    // keypoints per CTA of the radius kernel
constexpr int kTile      = 1024; // candidates per shared-memory tile
// vote accumulation launch shapes the launch tuner chooses between - CTA size, and one CTA per
// keypoint or a persistent grid that takes keypoints from a device counter in LPT order;
// every one computes the same accumulators, peaks and candidates
constexpr int kAccBs[3]  = {256, 512, 1024};
constexpr int kAccShapes = 6; // shape s: CTA size kAccBs[s % 3], persistent when s >= 3
constexpr int kHitChunk  = 1024; // hits staged in shared memory per round
constexpr int kLptBins   = 40;

struct PipeBufs {
    int4               *info;    // K: {searched, rows voted (0 when skipped), first tail row, flags}
    smm::RT            *rt;      // K: transform of the keypoint
    uint32_t           *mask;    // K x words: row bits over the candidate list (radius mode)
    int                 words;
    int                *rowOff;  // K + 1
    int2               *rows;    // rows: {keypoint, point * 2 + block lane}
    int4               *hits;    // per row segment: {bucket offset, count, alpha bits, 0}
    int                *hitCnt;  // K
    unsigned long long *votes;   // K
    unsigned long long *bound;   // K: sum of the hits' bucket multiplicities (cell bound)
    int                *order;   // K
    int                *next;    // persistent accumulation: the next place in `order` to take
};

// flags: bit 0 = keypoint votes, bit 1 = its normal is not finite
__device__ __forceinline__ int4 kp_info(const VoteArgs &a, int searched, int R, int tail,
                                        const float4 &n1) {
    const bool nanN   = !(isfinite(n1.x) && isfinite(n1.y) && isfinite(n1.z));
    const bool active = !nanN && !((float)searched < a.voteThreshold);
    return make_int4(searched, active ? R : 0, tail, (active ? 1 : 0) | (nanN ? 2 : 0));
}

// Position of the first of the last `need` set bits of the warp's mask words [0, nw) (the
// first tail row); `n` when need == 0. All lanes return the same value.
__device__ __forceinline__ int tail_from_mask(const uint32_t *m, int nw, int need, int n) {
    const int lane  = threadIdx.x & 31;
    int       found = n;
    for (int base = nw - 1; base >= 0 && need > 0; base -= 32) {
        const int      wi = base - lane; // lane 0 = last word
        const uint32_t wv = wi >= 0 ? m[wi] : 0u;
        const int      k  = __popc(wv);
        // rows in words after this lane's word (lanes before it in this round)
        int incl = k;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
                incl += t;
        }
        const int      excl = incl - k;
        const bool     mine = excl < need && incl >= need;
        const uint32_t who  = __ballot_sync(0xffffffffu, mine);
        if (who) {
            const int src = __ffs(who) - 1;
            int       pos = 0;
            if (lane == src) {
                uint32_t b = wv; // the (need - excl)-th highest set bit of wv
                for (int t = 1; t < need - excl; t++)
                    b &= ~(0x80000000u >> __clz(b));
                pos = wi * 32 + (31 - __clz(b));
            }
            found = __shfl_sync(0xffffffffu, pos, src);
            need  = 0;
        } else {
            need -= __shfl_sync(0xffffffffu, incl, 31);
        }
    }
    return found;
}

// Radius mode: eight keypoints per CTA, one per warp, over shared-memory tiles of the
// candidates' positions.
__global__ void __launch_bounds__(kKpWarps * 32) k_kp_radius(VoteArgs a, PipeBufs b) {
    smd::chain_enter(); // launched chained
    __shared__ float4 tp[kTile];
    __shared__ int    tid_[kTile];
    const int   lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int   c    = blockIdx.x * kKpWarps + w;
    const bool  live = c < a.K;
    const int   pid  = live ? a.kp[c] : -1;
    float4      p1   = make_float4(0.f, 0.f, 0.f, 0.f);
    if (live)
        p1 = a.pos[pid];
    uint32_t *mrow = b.mask + (size_t)(live ? c : 0) * b.words;
    int       S = 0, R = 0;
    for (int t0 = 0; t0 < a.ncand; t0 += kTile) {
        const int tn = min(kTile, a.ncand - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < tn; i += blockDim.x) {
            const int id = a.cand[t0 + i];
            tid_[i]      = id;
            tp[i]        = a.pos[id];
        }
        __syncthreads();
        if (!live)
            continue;
        for (int j = 0; j < tn; j += 32) {
            const int  i   = j + lane;
            bool       in  = false;
            bool       row = false;
            if (i < tn) {
                const float4 q = tp[i];
                in             = smm::dist2(p1.x, p1.y, p1.z, q.x, q.y, q.z) < a.sqDiam;
                row            = in && tid_[i] != pid;
            }
            const uint32_t bi = __ballot_sync(0xffffffffu, in);
            const uint32_t br = __ballot_sync(0xffffffffu, row);
            S += __popc(bi);
            R += __popc(br);
            if (lane == 0)
                mrow[(t0 + j) >> 5] = br;
        }
    }
    if (!live)
        return;
    __syncwarp();
    const int tail = tail_from_mask(mrow, b.words, R % smm::kLanes, a.ncand);
    if (lane == 0) {
        const float4 n1 = a.nrm[pid];
        b.info[c]       = kp_info(a, S, R, tail, n1);
        b.rt[c]         = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
    }
}

// CSR mode: one warp per keypoint over its list.
__global__ void k_kp_csr(VoteArgs a, PipeBufs b) {
    smd::chain_enter(); // launched chained
    const int lane = threadIdx.x & 31;
    const int c    = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= a.K)
        return;
    const int  pid = a.kp[c];
    const int  beg = a.nbrOff[c], len = a.nbrOff[c + 1] - beg;
    const int *L   = a.nbrIds + beg;
    int        R   = 0;
    for (int i = lane; i < len; i += 32)
        R += L[i] != pid ? 1 : 0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1)
        R += __shfl_xor_sync(0xffffffffu, R, o);
    int need = R % smm::kLanes, found = len;
    for (int end = len; end > 0 && need > 0; end -= 32) {
        const int i = end - 1 - lane;
        uint32_t  m = __ballot_sync(0xffffffffu, i >= 0 && L[i] != pid);
        const int k = __popc(m);
        if (k >= need) {
            for (int t = 1; t < need; t++)
                m &= m - 1;
            found = end - 1 - (__ffs(m) - 1);
            need  = 0;
        } else {
            need -= k;
        }
    }
    if (lane == 0) {
        const float4 p1 = a.pos[pid], n1 = a.nrm[pid];
        b.info[c]       = kp_info(a, len, R, found, n1);
        b.rt[c]         = smm::transform_rt(p1.x, p1.y, p1.z, n1.x, n1.y, n1.z);
    }
}

// Row counts per keypoint (cnt[K] = 0 closes the scan's input), and the per-keypoint hit
// counters and vote totals cleared for k_ppf.
__global__ void k_rows_count(const int4 *__restrict__ info, int K, int *__restrict__ cnt,
                             PipeBufs b) {
    smd::chain_enter(); // launched chained
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0)
        cnt[K] = 0;
    if (c < K) {
        cnt[c]      = info[c].y;
        b.hitCnt[c] = 0;
        b.votes[c]  = 0ull;
        b.bound[c]  = 0ull;
    }
}

// The rows of keypoint blockIdx.x into its segment (any order within it).
__global__ void k_rows_fill(VoteArgs a, PipeBufs b, int csr) {
    smd::chain_enter(); // launched chained
    __shared__ int sN;
    const int  c    = blockIdx.x;
    const int4 info = b.info[c];
    if (info.y == 0)
        return;
    if (threadIdx.x == 0)
        sN = 0;
    __syncthreads();
    int2     *out  = b.rows + b.rowOff[c];
    const int pid  = a.kp[c];
    const int lane = threadIdx.x & 31;
    if (!csr) {
        const uint32_t *m = b.mask + (size_t)c * b.words;
        for (int wi = threadIdx.x; wi < b.words; wi += blockDim.x) {
            uint32_t wv = m[wi];
            if (!wv)
                continue;
            int p = atomicAdd(&sN, __popc(wv));
            while (wv) {
                const int bit = __ffs(wv) - 1;
                wv &= wv - 1;
                const int i = wi * 32 + bit;
                out[p++]    = make_int2(c, a.cand[i] * 2 + (i < info.z ? 1 : 0));
            }
        }
        return;
    }
    const int  beg = a.nbrOff[c], len = a.nbrOff[c + 1] - beg;
    const int *L   = a.nbrIds + beg;
    for (int i0 = 0; i0 < len; i0 += blockDim.x) {
        const int      i     = i0 + threadIdx.x;
        const int      id    = i < len ? L[i] : -1;
        const bool     row   = i < len && id != pid;
        const uint32_t m     = __ballot_sync(0xffffffffu, row);
        int            wbase = 0;
        if (lane == 0 && m)
            wbase = atomicAdd(&sN, __popc(m));
        wbase = __shfl_sync(0xffffffffu, wbase, 0);
        if (row)
            out[wbase + __popc(m & ((1u << lane) - 1u))] = make_int2(c, id * 2 + (i < info.z ? 1 : 0));
    }
}

// One thread per row: PPF key and scene alpha with the row's lane rule, then the model
// table probe; hits go to the keypoint's segment.
__global__ void k_ppf(VoteArgs a, PipeBufs b, const int *__restrict__ total) {
    smd::chain_enter(); // launched chained
    const int n = *total;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int2     row = b.rows[r];
        const int      c   = row.x;
        const int      id  = row.y >> 1;
        const bool     blk = (row.y & 1) != 0;
        const int      pid = a.kp[c];
        const float4   p1 = a.pos[pid], n1 = a.nrm[pid];
        const float4   q = a.pos[id], n2 = a.nrm[id];
        const smm::RT  rt  = b.rt[c];
        const uint32_t key = smm::ppf_key(blk, p1.x, p1.y, p1.z, n1.x, n1.y, n1.z, q.x, q.y, q.z,
                                          n2.x, n2.y, n2.z, a.angleStep, a.distStep);
        const float as = smm::alpha_of(blk, rt, q.x, q.y, q.z);
        if (smm::fisnan(as))
            continue;
        uint32_t  off = 0, mult = 0;
        const int cnt = (int)probe(a.htab, a.hmask, key, off, mult);
        if (cnt > 0) {
            const int slot               = atomicAdd(&b.hitCnt[c], 1);
            b.hits[b.rowOff[c] + slot]   = make_int4((int)off, cnt, __float_as_int(as), 0);
            atomicAdd(&b.votes[c], (unsigned long long)cnt);
            atomicAdd(&b.bound[c], (unsigned long long)mult);
        }
    }
}

__device__ __forceinline__ int lpt_bin(unsigned long long v) {
    return v == 0 ? 0 : min(kLptBins - 1, 64 - __clzll((long long)v));
}

// Keypoints by vote count, largest first (binned by powers of two).
__global__ void k_lpt(const unsigned long long *__restrict__ votes, int K, int *__restrict__ order,
                      int *__restrict__ next) {
    smd::chain_enter(); // launched chained
    __shared__ int hist[kLptBins], start[kLptBins];
    if (threadIdx.x == 0)
        *next = 0; // the persistent vote grid's work counter
    if (threadIdx.x < kLptBins)
        hist[threadIdx.x] = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < K; c += blockDim.x)
        atomicAdd(&hist[lpt_bin(votes[c])], 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        int s = 0;
        for (int k = kLptBins - 1; k >= 0; k--) {
            start[k] = s;
            s += hist[k];
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < K; c += blockDim.x)
        order[atomicAdd(&start[lpt_bin(votes[c])], 1)] = c;
}

// One CTA per keypoint (in LPT order by block index), or with PERSIST a resident grid whose
// CTAs take the next keypoint of the LPT order from a device counter until none is left.
template <int BS, bool PERSIST>
__global__ void __launch_bounds__(BS, BS >= 1024 ? 1 : 2) k_vote_acc(VoteArgs a, PipeBufs b) {
    smd::chain_enter(); // launched chained
    extern __shared__ uint32_t acc[];
    __shared__ int       hOff[kHitChunk], hCnt[kHitChunk], cPre[kHitChunk + 1];
    __shared__ float     hAs[kHitChunk], hAsT[kHitChunk];
    __shared__ int       sh[33];
    __shared__ Cand      wc[BS / 32][3];
    __shared__ unsigned long long shash;
    __shared__ int       sNext;

    const int tid = threadIdx.x;
    for (int it = 0;; it++) {
        int idx = blockIdx.x;
        if (PERSIST) {
            if (tid == 0)
                sNext = atomicAdd(b.next, 1);
            __syncthreads();
            idx = sNext;
            __syncthreads();
            if (idx >= a.K)
                return;
        } else if (it > 0) {
            return;
        }
        const int  c    = b.order[idx];
        const int4 info = b.info[c];
        if (!(info.w & 1)) {
            skip_keypoint(a, c, info.x, (info.w & 2) != 0);
            continue;
        }
        if (tid == 0)
            shash = 0;
        const long long V      = (long long)b.votes[c];
        const long long bound  = (long long)b.bound[c];
        const int       nH     = b.hitCnt[c];
        const int4     *H      = b.hits + b.rowOff[c];
        const bool      narrow = bound <= kNarrowMax && !a.forceWide; // no cell can pass 65535
        const int       chunk  = narrow ? a.refChunk : a.refChunkWide;
        Cand            top[3];
        for (int t = 0; t < 3; t++)
            top[t] = Cand{-1.0f, INT_MAX, 0};
        unsigned long long myHash = 0;
        for (int r0 = 0; r0 < a.ns; r0 += chunk) {
            const int r1     = min(r0 + chunk, a.ns);
            const int nElem  = (r1 - r0) * a.A;
            const int nWords = narrow ? (nElem + 1) >> 1 : nElem;
            for (int i = tid; i < nWords; i += BS)
                acc[i] = 0u;
            for (int h0 = 0; h0 < nH; h0 += kHitChunk) {
                const int n = min(kHitChunk, nH - h0);
                __syncthreads();
                int T = 0;
                for (int j0 = 0; j0 < n; j0 += BS) {
                    const int j   = j0 + tid;
                    int       nit = 0;
                    if (j < n) {
                        const int4 hv = H[h0 + j];
                        hOff[j]       = hv.x;
                        hCnt[j]       = hv.y;
                        hAs[j]        = __int_as_float(hv.z);
                        hAsT[j]       = smm::alpha_tail_shift(__int_as_float(hv.z));
                        nit           = (hv.y + kItem - 1) / kItem;
                    }
                    int       tot;
                    const int pre = block_excl_scan(nit, sh, &tot);
                    if (j < n)
                        cPre[j] = T + pre;
                    T += tot;
                }
                if (tid == 0)
                    cPre[n] = T;
                __syncthreads();
                cast_votes(a, acc, hOff, hCnt, hAs, hAsT, cPre, n, T, r0, r1, narrow);
            }
            __syncthreads();
            peaks_chunk(a, acc, narrow, r0, r1, top, myHash);
            dump_chunk(a, c, acc, narrow, r0, r1);
            __syncthreads();
        }
        finish_keypoint(a, c, b.rt[c], top, myHash, info.x, nH, V, bound, wc, &shash);
        __syncthreads(); // the shared buffers serve the CTA's next keypoint
    }
}

const void *vote_acc_fn(int shape) {
    switch (shape) {
    case 0: return (const void *)k_vote_acc<kAccBs[0], false>;
    case 1: return (const void *)k_vote_acc<kAccBs[1], false>;
    case 2: return (const void *)k_vote_acc<kAccBs[2], false>;
    case 3: return (const void *)k_vote_acc<kAccBs[0], true>;
    case 4: return (const void *)k_vote_acc<kAccBs[1], true>;
    default: return (const void *)k_vote_acc<kAccBs[2], true>;
    }
}

// Dynamic shared memory of the accumulator for launch shape `shape` (its static shared
// memory differs a little by CTA size); 0 when it does not fit.
size_t vote_acc_smem(int shape, const Ctx &c, VoteArgs &a) {
    int optin = 0, perSM = 0;
    SM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    SM_CUDA(cudaDeviceGetAttribute(&perSM, cudaDevAttrMaxSharedMemoryPerMultiprocessor, c.device));
    cudaFuncAttributes fa;
    SM_CUDA(cudaFuncGetAttributes(&fa, vote_acc_fn(shape)));
    const size_t smem = acc_sizing(a.ns, a.A, (long long)fa.sharedSizeBytes, optin, perSM,
                                   &a.refChunk, &a.refChunkWide);
    if (smem && smem > allow_dynamic_smem(vote_acc_fn(shape), c.device))
        return 0;
    return smem;
}

// counterClear: the persistent grid's work counter is zero already (k_lpt clears it; each
// of the tuner's timed launches uses it up).
void launch_vote_acc(int shape, const Ctx &c, const VoteArgs &a, const PipeBufs &b, int K,
                     size_t smem, bool counterClear) {
    const int bs = kAccBs[shape % 3];
    int       g  = K;
    if (shape >= 3) {
        // one resident wave, keypoints from the counter
        int per = 0, nsm = 0;
        SM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, vote_acc_fn(shape), bs, smem));
        SM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
        g = std::max(1, std::min(K, std::max(per, 1) * nsm));
        if (!counterClear)
            SM_CUDA(cudaMemsetAsync(b.next, 0, sizeof(int), c.stream));
    }
    switch (shape) {
    case 0: launch_chained(c, k_vote_acc<kAccBs[0], false>, g, bs, smem, a, b); break;
    case 1: launch_chained(c, k_vote_acc<kAccBs[1], false>, g, bs, smem, a, b); break;
    case 2: launch_chained(c, k_vote_acc<kAccBs[2], false>, g, bs, smem, a, b); break;
    case 3: launch_chained(c, k_vote_acc<kAccBs[0], true>, g, bs, smem, a, b); break;
    case 4: launch_chained(c, k_vote_acc<kAccBs[1], true>, g, bs, smem, a, b); break;
    default: launch_chained(c, k_vote_acc<kAccBs[2], true>, g, bs, smem, a, b); break;
    }
}

// The launch tuner: per device, the vote accumulation shape measured fastest on the first
// call with at least kTuneMinK keypoints (each shape timed twice with CUDA events on the
// call's own data, the faster of the two runs kept), then used for every later call.
// SM_VOTE_SHAPE=256|512|1024, with a trailing 'p' for the persistent grid, in the
// environment fixes the shape instead (tests).
constexpr int    kTuneMinK = 512;
std::atomic<int> g_voteShape[64] = {};     // 0 untuned, else 1 + shape index
std::mutex       g_tuneMu;

int forced_vote_shape() {
    const char *e = std::getenv("SM_VOTE_SHAPE");
    if (!e)
        return -1;
    const int  v       = std::atoi(e);
    const bool persist = std::strchr(e, 'p') != nullptr;
    for (int s = 0; s < 3; s++)
        if (kAccBs[s] == v)
            return s + (persist ? 3 : 0);
    return -1;
}

} // namespace

int vote_tuned_shape(int device, int *persistent) {
    *persistent = 0;
    if (device < 0 || device >= 64)
        return 0;
    const int t = g_voteShape[device].load();
    if (t <= 0)
        return 0;
    *persistent = t - 1 >= 3 ? 1 : 0;
    return kAccBs[(t - 1) % 3];
}

void vote(Ctx &c, const Model &m, const float4 *pos, const float4 *nrm, const int *kp, int K,
          const int *nbrOff, const int *nbrIds, const int *cand, int ncand, float minScore,
          const VoteOut &out, int dumpK) {
    if (K <= 0)
        return;
    // rows (keypoint, neighbour) are counted and offset in 32-bit ints: at most K x ncand in
    // radius mode (every candidate a neighbour of every keypoint)
    if (!nbrOff && (long long)K * (long long)ncand > 0x7fffffffll)
        throw Error(SM_ERR_CAPACITY, "too many keypoint x sampled point pairs for one call");
    VoteArgs a{};
    fill_vote_model(m, minScore, a);
    a.pos    = pos;
    a.nrm    = nrm;
    a.kp     = kp;
    a.K      = K;
    a.nbrOff = nbrOff;
    a.nbrIds = nbrIds;
    a.cand   = cand;
    a.ncand  = ncand;
    a.stats  = out.stats;
    a.cands  = out.cands;
    a.poses  = out.poses;
    a.poseOk = out.poseOk;
    a.acc    = out.acc;
    a.dumpK  = out.acc ? dumpK : 0;
    // SM_VOTE_FORCE_WIDE=1 runs every keypoint on 32-bit counters, a regime that the cell
    // bound otherwise reserves for extreme inputs, so that tests reach it
    const char *fw = std::getenv("SM_VOTE_FORCE_WIDE");
    a.forceWide    = (fw && fw[0] == '1') ? 1 : 0;
    // SM_VOTE_FINGERPRINT=1 folds every accumulator into stats column 4 (checked by tests
    // against the oracle); without it the column is 0 and the peak scan skips the work
    const char *fp = std::getenv("SM_VOTE_FINGERPRINT");
    a.fingerprint  = (fp && fp[0] == '1') ? 1 : 0;

    const bool csr = nbrOff != nullptr;

    // the accumulation's launch shape: forced, tuned on this device, or the default (512)
    const int dev    = c.device >= 0 && c.device < 64 ? c.device : 0;
    const int forced = forced_vote_shape();
    int       shape  = forced >= 0 ? forced : (g_voteShape[dev].load() > 0 ? g_voteShape[dev].load() - 1 : 1);
    const bool tune  = forced < 0 && g_voteShape[dev].load() == 0 && K >= kTuneMinK;
    size_t     smem  = vote_acc_smem(shape, c, a);
    if (!smem)
        throw Error(SM_ERR_CAPACITY, "featAngleResolution too large for the vote accumulator");

    PipeBufs b{};
    b.info   = c.arena.get<int4>("v.info", K);
    b.rt     = c.arena.get<smm::RT>("v.rt", K);
    b.words  = csr ? 0 : (ncand + 31) / 32;
    b.mask   = csr ? nullptr : c.arena.get<uint32_t>("v.mask", (size_t)K * std::max(b.words, 1));
    b.rowOff = c.arena.get<int>("v.rowoff", (size_t)K + 1);
    b.hitCnt = c.arena.get<int>("v.hitcnt", K);
    b.votes  = c.arena.get<unsigned long long>("v.votes", K);
    b.bound  = c.arena.get<unsigned long long>("v.bound", K);
    b.order  = c.arena.get<int>("v.order", K);
    b.next   = c.arena.get<int>("v.next", 1);
    int *cnt = c.arena.get<int>("v.rowcnt", (size_t)K + 1);
    if (csr)
        launch_chained(c, k_kp_csr, nblocks((long long)K * 32, 256), 256, 0, a, b);
    else
        launch_chained(c, k_kp_radius, nblocks(K, kKpWarps), kKpWarps * 32, 0, a, b);
    launch_chained(c, k_rows_count, nblocks(K, 256), 256, 0, b.info, K, cnt, b);
    const int rtot = scan_excl(c, cnt, b.rowOff, (long long)K + 1, "v.scan", true);
    b.rows = c.arena.get<int2>("v.rows", std::max(rtot, 1));
    b.hits = c.arena.get<int4>("v.hits", std::max(rtot, 1));
    launch_chained(c, k_rows_fill, K, 256, 0, a, b, csr ? 1 : 0);
    SM_CUDA(cudaEventRecord(c.ev[10], c.stream));
    if (rtot > 0) {
        const int g = (int)std::min<long long>(nblocks(rtot, 256), 152LL * 8);
        launch_chained(c, k_ppf, g, 256, 0, a, b, b.rowOff + K);
    }
    SM_CUDA(cudaEventRecord(c.ev[11], c.stream));
    launch_chained(c, k_lpt, 1, 1024, 0, b.votes, K, b.order, b.next);
    if (tune) {
        // every shape computes the same outputs: time each on this call's keypoints, keep
        // the fastest for the device (one process-wide decision, taken once)
        std::lock_guard<std::mutex> lk(g_tuneMu);
        if (g_voteShape[dev].load() == 0) {
            cudaEvent_t e0, e1;
            SM_CUDA(cudaEventCreate(&e0));
            SM_CUDA(cudaEventCreate(&e1));
            float best[kAccShapes];
            for (int sh = 0; sh < kAccShapes; sh++)
                best[sh] = 1e30f;
            for (int rep = 0; rep < 2; rep++)
                for (int sh = 0; sh < kAccShapes; sh++) {
                    VoteArgs     at = a;
                    const size_t sm = vote_acc_smem(sh, c, at);
                    if (!sm)
                        continue;
                    SM_CUDA(cudaEventRecord(e0, c.stream));
                    launch_vote_acc(sh, c, at, b, K, sm, false);
                    SM_CUDA(cudaEventRecord(e1, c.stream));
                    SM_CUDA(cudaEventSynchronize(e1));
                    float ms = 0.0f;
                    SM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                    best[sh] = std::min(best[sh], ms);
                }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            int pick = 1;
            for (int sh = 0; sh < kAccShapes; sh++)
                if (best[sh] < best[pick])
                    pick = sh;
            g_voteShape[dev].store(1 + pick);
        }
        shape = g_voteShape[dev].load() - 1;
        smem  = vote_acc_smem(shape, c, a);
    }
    SM_CUDA(cudaEventRecord(c.ev[12], c.stream));
    launch_vote_acc(shape, c, a, b, K, smem, !tune);
    SM_CUDA(cudaEventRecord(c.ev[13], c.stream));
}

} // namespace sm
