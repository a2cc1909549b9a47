// prep.cu - point preparation, scans and compaction, uniform grids, greedy sampling and
// normal estimation of the matching path.
//
// Reference counterparts: removeNan / computeBoundingBox (util.cpp:86-105, 178-207), the
// k-d tree (kdtree/kdtree.h) replaced by uniform grids, samplePointCloud (util.cpp:107-139),
// estimateNormal / computeNormal (util.cpp:234-334), normalizeNormal (util.cpp:163-176).
#include <atomic>
#include <climits>
#include <cmath>

#include "sm_icp.h"
#include "sm_linalg.h"
#include "sm_stages.h"

namespace sm {
using namespace smd;

namespace {

constexpr int kScanBs   = 512;
constexpr int kScanIpt  = 8;
constexpr int kScanTile = kScanBs * kScanIpt;
constexpr int kNoEq     = INT_MIN; // scan raw values instead of (value == eq)

struct GridParams {
    float org[3], g;
    int   dim[3];
};

GridParams grid_params(const Box &b, float g, int dim[3]) {
    GridParams p;
    for (int a = 0; a < 3; a++) {
        p.org[a] = b.mn[a];
        p.dim[a] = dim[a];
    }
    p.g = g;
    return p;
}

__device__ __forceinline__ float4 nan4() {
    const float q = __int_as_float(0x7fc00000);
    return make_float4(q, q, q, 0.0f);
}

__device__ __forceinline__ bool finite3(float x, float y, float z) {
    return isfinite(x) && isfinite(y) && isfinite(z);
}

// ---------------------------------------------------------------------------------------
__global__ void k_prep(const float *__restrict__ xyz, const float *__restrict__ nin, int n,
                       float4 *__restrict__ pos, float4 *__restrict__ nrm, int *__restrict__ valid,
                       int *__restrict__ bbox, int *__restrict__ nvalid) {
    __shared__ int smn[3], smx[3], scnt;
    if (threadIdx.x < 3) {
        smn[threadIdx.x] = INT_MAX;
        smx[threadIdx.x] = INT_MIN;
    }
    if (threadIdx.x == 0)
        scnt = 0;
    __syncthreads();
    int lmn[3] = {INT_MAX, INT_MAX, INT_MAX}, lmx[3] = {INT_MIN, INT_MIN, INT_MIN}, lc = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = xyz[3 * (size_t)i], y = xyz[3 * (size_t)i + 1], z = xyz[3 * (size_t)i + 2];
        bool        ok = finite3(x, y, z);
        float4      nn = nan4();
        if (nin) {
            float a = nin[3 * (size_t)i], b = nin[3 * (size_t)i + 1], c = nin[3 * (size_t)i + 2];
            ok      = ok && finite3(a, b, c);
            const float sq = a * a + (b * b + c * c);
            if (sq > 0.0f) {
                const float s = smm::fsqrt(sq);
                a             = smm::fdiv(a, s);
                b             = smm::fdiv(b, s);
                c             = smm::fdiv(c, s);
            }
            nn = make_float4(a, b, c, 0.0f);
        }
        pos[i]   = make_float4(x, y, z, 0.0f);
        nrm[i]   = nn;
        valid[i] = ok ? 1 : 0;
        if (ok) {
            const int o[3] = {f2ord(x), f2ord(y), f2ord(z)};
            for (int a = 0; a < 3; a++) {
                lmn[a] = min(lmn[a], o[a]);
                lmx[a] = max(lmx[a], o[a]);
            }
            lc++;
        }
    }
    for (int a = 0; a < 3; a++) {
        lmn[a] = __reduce_min_sync(0xffffffffu, lmn[a]);
        lmx[a] = __reduce_max_sync(0xffffffffu, lmx[a]);
    }
    lc = __reduce_add_sync(0xffffffffu, lc);
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; a++) {
            atomicMin(&smn[a], lmn[a]);
            atomicMax(&smx[a], lmx[a]);
        }
        atomicAdd(&scnt, lc);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int a = 0; a < 3; a++) {
            atomicMin(&bbox[a], smn[a]);
            atomicMax(&bbox[3 + a], smx[a]);
        }
        atomicAdd(nvalid, scnt);
    }
}

__global__ void k_init_bbox(int *bbox, int *nvalid) {
    if (threadIdx.x < 3) {
        bbox[threadIdx.x]     = INT_MAX;
        bbox[3 + threadIdx.x] = INT_MIN;
    }
    if (threadIdx.x == 0)
        *nvalid = 0;
}

// Up to four buffers of 32-bit words, each set to its value, in one chained launch (a
// cudaMemsetAsync per buffer would be one stream operation each and break the launch chain).
struct FillSet {
    uint32_t *p[4];
    long long n[4]; // words
    uint32_t  v[4];
    int       k = 0;
    void add(void *ptr, size_t bytes, uint32_t value) {
        if (k == 4)
            throw Error(SM_ERR_RUNTIME, "buffer clear: more than four buffers in one launch");
        p[k]   = (uint32_t *)ptr;
        n[k]   = (long long)(bytes / 4);
        v[k++] = value;
    }
};

__global__ void k_fill(FillSet f) {
    chain_enter(); // launched chained
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (int s = 0; s < f.k; s++) {
        uint32_t       *p = f.p[s];
        const long long n = f.n[s];
        const uint32_t  v = f.v[s];
        // 16-byte stores over an aligned buffer's body, 4-byte stores for the rest
        const long long n4 = ((uintptr_t)p & 15) == 0 ? n / 4 : 0;
        uint4          *q  = reinterpret_cast<uint4 *>(p);
        for (long long i = t0; i < n4; i += st)
            q[i] = make_uint4(v, v, v, v);
        for (long long i = n4 * 4 + t0; i < n; i += st)
            p[i] = v;
    }
}

static void fill(Ctx &c, const FillSet &f) {
    long long words = 0;
    for (int s = 0; s < f.k; s++)
        words += f.n[s];
    if (words == 0)
        return;
    int nsm = 0;
    SM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
    const int g = (int)std::min<long long>(nblocks((words + 3) / 4, 256), 8LL * std::max(nsm, 1));
    launch_chained(c, k_fill, g, 256, 0, f);
}

// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int scan_val(const int *in, long long i, long long n, int eq) {
    if (i >= n)
        return 0;
    const int v = in[i];
    return eq == kNoEq ? v : (v == eq ? 1 : 0);
}

// Single-pass exclusive scan with decoupled look-back (Merrill & Garland, "Single-pass
// Parallel Prefix Scan with Decoupled Look-back", 2016). Tiles of kScanTile values take a
// ticket in launch order; a tile publishes its aggregate, then warp 0 walks back over the
// tiles before it, 32 at a time, summing aggregates until it meets a tile whose inclusive
// prefix is published, and publishes its own inclusive prefix. A tile waits only on tiles
// that took earlier tickets (already running or done), so every wait ends; each is bounded
// all the same and sets *err when its limit passes. Status words: epoch (30 bits, new per
// scan, so the array needs no reset) | flag (2 bits: 1 aggregate, 2 inclusive) | value.
constexpr unsigned long long kLbAgg = 1ull << 32, kLbIncl = 2ull << 32;

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__global__ void __launch_bounds__(kScanBs)
    k_scan_lookback(const int *__restrict__ in, int *__restrict__ out, long long n, int eq,
                    unsigned long long *__restrict__ status, int *__restrict__ ticket,
                    int nparts, unsigned epoch, int *__restrict__ total) {
    chain_enter(); // launched chained
    __shared__ int sh[33];
    __shared__ int sTile, sExcl;
    if (threadIdx.x == 0) {
        const int t = atomicAdd(ticket, 1);
        if (t == nparts - 1)
            ticket[0] = 0; // every ticket of this launch is taken: ready for the next scan
        sTile = t;
    }
    __syncthreads();
    const int       tile = sTile;
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanIpt;
    int             v[kScanIpt], s = 0;
#pragma unroll
    for (int k = 0; k < kScanIpt; k++) {
        v[k] = scan_val(in, base + k, n, eq);
        s += v[k];
    }
    int       agg;
    const int ex  = block_excl_scan(s, sh, &agg);
    const unsigned long long tag = (unsigned long long)epoch << 34;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int       excl = 0;
        if (tile == 0) {
            if (lane == 0)
                st_relaxed_u64(&status[0], tag | kLbIncl | (unsigned)agg);
        } else {
            if (lane == 0)
                st_relaxed_u64(&status[tile], tag | kLbAgg | (unsigned)agg);
            for (int top = tile - 1;; top -= 32) {
                const int          p = top - lane; // lane 0: the nearest predecessor
                unsigned long long w = tag | kLbIncl; // lanes before tile 0: inclusive 0
                for (int it = 0;; it++) {
                    if (p >= 0)
                        w = ld_relaxed_u64(&status[p]);
                    const bool ready = (w >> 34) == epoch && ((w >> 32) & 3ull) != 0;
                    if (__all_sync(0xffffffffu, ready))
                        break;
                    if (it > (1 << 22)) {
                        if (lane == 0)
                            atomicExch(ticket + 1, 1);
                        w = tag | kLbIncl;
                        break;
                    }
                    __nanosleep(32);
                }
                const bool     isIncl = ((w >> 32) & 3ull) == 2ull;
                const unsigned incl   = __ballot_sync(0xffffffffu, isIncl);
                int            val    = (int)(unsigned)(w & 0xffffffffull);
                if (incl) {
                    const int first = __ffs(incl) - 1;
                    excl += __reduce_add_sync(0xffffffffu, lane <= first ? val : 0);
                    break;
                }
                excl += __reduce_add_sync(0xffffffffu, val);
            }
            if (lane == 0)
                st_relaxed_u64(&status[tile], tag | kLbIncl | (unsigned)(excl + agg));
        }
        if (lane == 0) {
            sExcl = excl;
            if (tile == nparts - 1 && total)
                *total = excl + agg;
        }
    }
    __syncthreads();
    int o = ex + sExcl;
#pragma unroll
    for (int k = 0; k < kScanIpt; k++) {
        if (base + k < n)
            out[base + k] = o;
        o += v[k];
    }
}

__global__ void k_scatter_flags(const int *__restrict__ flags, const int *__restrict__ pre, int n,
                                int eq, int *__restrict__ out) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int v = flags[i];
    if (eq == kNoEq ? v != 0 : v == eq)
        out[pre[i]] = i;
}

// ---------------------------------------------------------------------------------------
constexpr int kSpHeavy = 128; // sampler cells with more points are taken by a whole CTA

// The sampler's cells keep their side just above the step whatever the scene's extent
// (the work per point is then bounded by the packing of kept points, not by how coarse a
// capped grid would have to be). Their table is dense (slot = cell key) when the cell box is
// small against the points (see sample_points), else hashed: keys[slot] holds the cell key
// (open addressing, ~0 = empty), so only occupied cells are stored. A cell's points are
// contiguous in pts from start[slot] (an empty dense slot has start[slot + 1] == start[slot]);
// rankCnt[slot] = {the cell's kept-point record (its place in the phase lists), kept count},
// written for occupied cells only.
struct ThinView {
    float                     org[3];
    float                     g;
    int                       dim[3];
    const unsigned long long *keys; // nullptr: dense table
    uint32_t                  mask;
    const int                *start; // table slots + 1
    const float4             *pts;
    // the table slot of the cell with key `key`, -1 when the cell holds no point
    __device__ __forceinline__ int find(unsigned long long key) const {
        if (!keys)
            return start[key + 1] > start[key] ? (int)key : -1;
        uint32_t h = (uint32_t)smm::mix64(key) & mask;
        for (uint32_t p = 0; p <= mask; p++) {
            const unsigned long long k = keys[h];
            if (k == key)
                return (int)h;
            if (k == ~0ull)
                return -1;
            h = (h + 1) & mask;
        }
        return -1;
    }
};

__device__ __forceinline__ unsigned long long cell_key(int x, int y, int z, int dim0, int dim1) {
    return ((unsigned long long)z * (unsigned)dim1 + (unsigned)y) * (unsigned)dim0 + (unsigned)x;
}

// Counting pass: the point's cell enters the table (slotOf) and the point takes its place
// within the cell (sub); the point that opens a cell also counts the cell in its phase
// (ph[0..7]). A hashed table has at least twice as many slots as points, so every cell
// finds one; a dense one (keys == nullptr) files the cell under its key.
__global__ void k_thin_insert(const float4 *__restrict__ pos, const int *__restrict__ ids, int m,
                              GridParams gp, unsigned long long *__restrict__ keys, uint32_t mask,
                              int *__restrict__ slotOf, int *__restrict__ sub,
                              int *__restrict__ cnt, int *__restrict__ ph) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const float4             p   = pos[ids[i]];
    const int                cx  = smg::coord(p.x, gp.org[0], gp.g, gp.dim[0]);
    const int                cy  = smg::coord(p.y, gp.org[1], gp.g, gp.dim[1]);
    const int                cz  = smg::coord(p.z, gp.org[2], gp.g, gp.dim[2]);
    const unsigned long long key = cell_key(cx, cy, cz, gp.dim[0], gp.dim[1]);
    uint32_t                 h   = keys ? (uint32_t)smm::mix64(key) & mask : (uint32_t)key;
    for (uint32_t q = 0; q <= mask; q++) {
        const unsigned long long prev = keys ? atomicCAS(&keys[h], ~0ull, key) : key;
        if (prev == ~0ull || prev == key) {
            slotOf[i]   = (int)h;
            const int k = atomicAdd(&cnt[h], 1);
            sub[i]      = k;
            if (k == 0)
                atomicAdd(&ph[smg::phase_of(cx, cy, cz)], 1);
            return;
        }
        h = (h + 1) & mask;
    }
}

// ph[0..7] = occupied cells per phase; this sets ph[8..15] = the phases' list offsets and
// ph[16..23] = their front fill pointers (ph[24..31] count heavy cells placed from the
// back, ph[32..39] hand heavy cells to CTAs; both start at 0).
__global__ void k_phase_offsets(int *__restrict__ ph) {
    chain_enter(); // launched chained
    if (threadIdx.x != 0)
        return;
    int o = 0;
    for (int p = 0; p < 8; p++) {
        ph[8 + p]  = o;
        ph[16 + p] = o;
        o += ph[p];
    }
}

// Placing pass: the point's position (its place i in the ascending id list in w: list order
// is index order) at its place in the cell; the point with place 0 lists the cell's slot in
// its phase (any order: cells of one phase do not interact) and records
// rankCnt[slot] = {its list place (the index of the cell's kept-point record), 0 kept}.
__global__ void k_thin_scatter(const float4 *__restrict__ pos, const int *__restrict__ ids, int m,
                               const int *__restrict__ slotOf, const int *__restrict__ sub,
                               const int *__restrict__ start,
                               const unsigned long long *__restrict__ keys, int dim0, int dim1,
                               float4 *__restrict__ pts, int *__restrict__ ph,
                               int *__restrict__ lists, int2 *__restrict__ rankCnt,
                               int *__restrict__ keptFlag) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    keptFlag[i] = 0; // the phases' kept flags (and, at m, the overflow word) start clear
    if (i == 0)
        keptFlag[m] = 0;
    const int    h = slotOf[i];
    const int    k = sub[i];
    const float4 p = pos[ids[i]];
    pts[start[h] + k] = make_float4(p.x, p.y, p.z, __int_as_float(i));
    if (k == 0) {
        const unsigned long long key = keys ? keys[h] : (unsigned long long)h;
        const unsigned long long xy  = (unsigned long long)dim0 * (unsigned)dim1;
        const int cx = (int)(key % (unsigned)dim0), cy = (int)((key / (unsigned)dim0) % (unsigned)dim1);
        const int cz    = (int)(key / xy);
        const int phase = smg::phase_of(cx, cy, cz);
        // light cells fill the phase's list region from the front, heavy ones (more than
        // kSpHeavy points, taken by whole CTAs) from the back
        const int slot = start[h + 1] - start[h] > kSpHeavy
                             ? ph[8 + phase] + ph[phase] - 1 - atomicAdd(&ph[24 + phase], 1)
                             : atomicAdd(&ph[16 + phase], 1);
        lists[slot]    = h;
        rankCnt[h]     = make_int2(slot, 0);
    }
}

// ---------------------------------------------------------------------------------------
constexpr int kSpWarps  = 8;   // warps per CTA of the phase kernel (a warp per light cell)
constexpr int kSpReg    = kSpHeavy / 32; // light cell: points per lane, held in registers
constexpr int kSpHStage = 448; // heavy cell: neighbours' kept points staged (26 x 16 + 32)
constexpr int kSpStage  = 128; // light cell: neighbours' kept points staged per warp
constexpr int kSpBuf    = kSpWarps * kSpStage > kSpHStage ? kSpWarps * kSpStage : kSpHStage;
constexpr int kSpPh     = 40;  // ph[]: counts, offsets, light fill, heavy fill, heavy take

// The 26 neighbours of cell (cx, cy, cz) without its centre, lane l < 26 taking one:
// the neighbour's kept-point record and kept count (cells of later phases have none yet,
// empty cells have no record: -1, 0).
__device__ __forceinline__ void sp_neighbour(const ThinView &G, const int2 *__restrict__ rankCnt,
                                             int cx, int cy, int cz, int l, int &nr, int &cnt) {
    nr  = -1;
    cnt = 0;
    const int o = l < 13 ? l : l + 1;
    const int x = cx + o % 3 - 1, y = cy + (o / 3) % 3 - 1, z = cz + o / 9 - 1;
    if (x >= 0 && y >= 0 && z >= 0 && x < G.dim[0] && y < G.dim[1] && z < G.dim[2]) {
        const int t = G.find(cell_key(x, y, z, G.dim[0], G.dim[1]));
        if (t >= 0) {
            const int2 v = rankCnt[t];
            nr           = v.x;
            cnt          = nr >= 0 ? v.y : 0;
        }
    }
}

__device__ __forceinline__ void cell_coords(const ThinView &G, int cell, int &cx, int &cy, int &cz) {
    const unsigned long long key = G.keys ? G.keys[cell] : (unsigned long long)cell;
    cx = (int)(key % (unsigned)G.dim[0]);
    cy = (int)((key / (unsigned)G.dim[0]) % (unsigned)G.dim[1]);
    cz = (int)(key / ((unsigned long long)G.dim[0] * (unsigned)G.dim[1]));
}

// One warp per light cell, one CTA per heavy cell of the current phase. The sequential
// greedy visits the cell's points by ascending index and keeps a point unless a kept point
// lies within the step; the kept points of the 26 neighbour cells (earlier phases) are
// fixed, so the cell first drops every point within the step of one of them (order-free),
// then repeats "keep the smallest surviving index, drop the survivors within the step of
// it" - the same kept set as the sequential visit, at (kept points x cell size / threads)
// work and without sorting. Kept points are recorded as positions (keptPos, `cap` per cell)
// and their number in rankCnt[slot].y, next to the cell's record index (one load per
// neighbour). Points are named by their place in the ascending id list (same order as the
// index), and keptFlag is over those places. A light cell's points sit in its warp's
// registers (kSpReg per lane) and the neighbours' kept points are read once each by the
// warp; heavy cells (more than kSpHeavy points) spread each step over the CTA, which takes
// them first, one at a time from a per-phase counter (neighbours' kept points staged in
// shared memory when they fit, `alive` flags in aliveTmp).
__global__ void __launch_bounds__(kSpWarps * 32)
    k_sample_phase(ThinView G, const int *__restrict__ lists, int *__restrict__ ph, int phase,
                   int2 *__restrict__ rankCnt, float4 *__restrict__ keptPos, int cap, float r2,
                   int *__restrict__ keptFlag, int *__restrict__ overflow,
                   int *__restrict__ aliveTmp) {
    smd::chain_enter(); // phases are chained launches: the previous phase's flags are final
    __shared__ float4 stageBuf[kSpBuf]; // heavy cell: [0, kSpHStage); light warp w: its slice
    __shared__ int    snr[26], scnt[26];
    __shared__ int    sCell, sMin[kSpWarps];
    __shared__ float4 sKeep;
    const int  wl    = threadIdx.x >> 5;
    const int  lane  = threadIdx.x & 31;
    const int  tid   = threadIdx.x;
    const int  off   = ph[8 + phase];
    const int  total = ph[phase];
    const int  nl    = ph[16 + phase] - off; // light cells: list front
    const int  nh    = ph[24 + phase];       // heavy cells: list back
    const int *cells = lists + off;

    // ---- heavy cells: the whole CTA on one cell
    for (; nh > 0;) {
        if (tid == 0)
            sCell = atomicAdd(&ph[32 + phase], 1);
        __syncthreads();
        const int hc = sCell;
        __syncthreads(); // every thread has read sCell before it is taken again
        if (hc >= nh)
            break;
        const int cell = cells[total - 1 - hc];
        const int rk   = rankCnt[cell].x;
        int       cx, cy, cz;
        cell_coords(G, cell, cx, cy, cz);
        const int s = G.start[cell], n = G.start[cell + 1] - s;
        if (wl == 0) {
            int nr = -1, cnt = 0;
            if (lane < 26)
                sp_neighbour(G, rankCnt, cx, cy, cz, lane, nr, cnt);
            const int incl = warp_incl_scan(cnt);
            if (lane < 26) {
                snr[lane]  = nr;
                scnt[lane] = incl - cnt; // exclusive prefix
            }
            if (lane == 31)
                sMin[0] = incl; // NK
        }
        __syncthreads();
        const int  NK      = sMin[0];
        const bool stageNb = NK <= kSpHStage;
        if (stageNb) {
            for (int t = tid; t < NK; t += kSpWarps * 32) {
                int j = 0;
                while (j < 25 && scnt[j + 1] <= t)
                    j++;
                stageBuf[t] = keptPos[(size_t)snr[j] * cap + (t - scnt[j])];
            }
        }
        __syncthreads();
        int *alive = aliveTmp + s;
        for (int i = tid; i < n; i += kSpWarps * 32) {
            const float4 q  = G.pts[s + i];
            bool         ok = true;
            if (stageNb) {
                for (int k = 0; k < NK && ok; k++) {
                    const float4 o = stageBuf[k];
                    if (smm::dist2(o.x, o.y, o.z, q.x, q.y, q.z) < r2)
                        ok = false;
                }
            } else {
                for (int j = 0; j < 26 && ok; j++) {
                    const int nj = snr[j];
                    const int cj = (j < 25 ? scnt[j + 1] : NK) - scnt[j];
                    for (int k = 0; k < cj && ok; k++) {
                        const float4 o = keptPos[(size_t)nj * cap + k];
                        if (smm::dist2(o.x, o.y, o.z, q.x, q.y, q.z) < r2)
                            ok = false;
                    }
                }
            }
            alive[i] = ok ? 1 : 0;
        }
        __syncthreads();
        float4 *mine = keptPos + (size_t)rk * cap;
        int     nk   = 0;
        for (;;) {
            int    myMin = INT_MAX;
            float4 myP   = make_float4(0.f, 0.f, 0.f, 0.f);
            for (int i = tid; i < n; i += kSpWarps * 32)
                if (alive[i]) {
                    const float4 q  = G.pts[s + i];
                    const int    id = __float_as_int(q.w);
                    if (id < myMin) {
                        myMin = id;
                        myP   = q;
                    }
                }
            const int wm = __reduce_min_sync(0xffffffffu, myMin);
            if (lane == 0)
                sMin[wl] = wm;
            __syncthreads();
            int m = INT_MAX;
            for (int k = 0; k < kSpWarps; k++)
                m = min(m, sMin[k]);
            if (m == INT_MAX)
                break; // (uniform: every thread read the same minima)
            if (myMin == m)
                sKeep = make_float4(myP.x, myP.y, myP.z, 0.0f); // the unique holder
            __syncthreads();
            const float4 kp = sKeep;
            if (tid == 0) {
                keptFlag[m] = 1;
                if (nk < cap)
                    mine[nk] = kp;
                else
                    atomicExch(overflow, 1);
            }
            nk = min(nk + 1, cap);
            for (int i = tid; i < n; i += kSpWarps * 32) {
                if (!alive[i])
                    continue;
                const float4 q = G.pts[s + i];
                if (__float_as_int(q.w) == m || smm::dist2(kp.x, kp.y, kp.z, q.x, q.y, q.z) < r2)
                    alive[i] = 0;
            }
            __syncthreads(); // drops done and sMin / sKeep read before the next round
        }
        if (tid == 0)
            rankCnt[cell].y = nk;
        __syncthreads(); // the buffers are reused by the next cell
    }

    // ---- light cells: a warp each, the cell's points in registers (kSpReg per lane)
    for (int w = blockIdx.x * kSpWarps + wl; w < nl; w += gridDim.x * kSpWarps) {
        const int cell = cells[w];
        const int rk   = rankCnt[cell].x;
        int       cx, cy, cz;
        cell_coords(G, cell, cx, cy, cz);
        const int s = G.start[cell], n = G.start[cell + 1] - s; // n <= kSpHeavy
        float4    q[kSpReg];
        unsigned  alive = 0u; // bit j: point lane + 32 j is still a candidate
#pragma unroll
        for (int j = 0; j < kSpReg; j++) {
            const int i = lane + 32 * j;
            q[j]        = i < n ? G.pts[s + i] : make_float4(0.f, 0.f, 0.f, 0.f);
            alive |= (i < n ? 1u : 0u) << j;
        }
        int nr = -1, cnt = 0;
        if (lane < 26)
            sp_neighbour(G, rankCnt, cx, cy, cz, lane, nr, cnt);
        // survivors of the neighbours' kept points, each tested against every point the lane
        // holds: staged in shared memory by the whole warp at once when they fit, else the
        // neighbours one by one, each kept point read once by the warp (a broadcast)
        const int incl = warp_incl_scan(cnt);
        const int excl = incl - cnt;
        const int NK   = __shfl_sync(0xffffffffu, incl, 31);
        unsigned  nz   = __ballot_sync(0xffffffffu, cnt > 0);
        if (NK <= kSpStage) {
            float4 *st = stageBuf + wl * kSpStage;
            for (int base = 0; base < NK; base += 32) {
                const int t  = base + lane;
                int       lo = 0; // the neighbour holding kept point t: last with excl <= t
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int mid = lo + step;
                    const int ev  = __shfl_sync(0xffffffffu, excl, mid & 31);
                    if (mid < 26 && ev <= t)
                        lo = mid;
                }
                const int nj = __shfl_sync(0xffffffffu, nr, lo);
                const int ej = __shfl_sync(0xffffffffu, excl, lo);
                if (t < NK)
                    st[t] = keptPos[(size_t)nj * cap + (t - ej)];
            }
            __syncwarp();
            for (int kk = 0; kk < NK; kk++) {
                const float4 o = st[kk];
#pragma unroll
                for (int j = 0; j < kSpReg; j++)
                    if (smm::dist2(o.x, o.y, o.z, q[j].x, q[j].y, q[j].z) < r2)
                        alive &= ~(1u << j);
            }
            __syncwarp(); // the slice is refilled by the warp's next cell
            nz = 0u;
        }
        while (nz && __any_sync(0xffffffffu, alive != 0u)) {
            const int jn = __ffs(nz) - 1;
            nz &= nz - 1u;
            const int     nj = __shfl_sync(0xffffffffu, nr, jn);
            const int     cj = __shfl_sync(0xffffffffu, cnt, jn);
            const float4 *kn = keptPos + (size_t)nj * cap;
            for (int k = 0; k < cj; k++) {
                const float4 o = kn[k];
#pragma unroll
                for (int j = 0; j < kSpReg; j++)
                    if (smm::dist2(o.x, o.y, o.z, q[j].x, q[j].y, q[j].z) < r2)
                        alive &= ~(1u << j);
            }
        }
        // keep the smallest surviving index, drop the survivors within the step, repeat; the
        // lane that holds the kept point hands its position to the warp
        float4 *mine = keptPos + (size_t)rk * cap;
        int     nk   = 0;
        for (;;) {
            int    myMin = INT_MAX;
            float4 myP   = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
            for (int j = 0; j < kSpReg; j++) {
                const int id = __float_as_int(q[j].w);
                if (((alive >> j) & 1u) && id < myMin) {
                    myMin = id;
                    myP   = q[j];
                }
            }
            const int m = __reduce_min_sync(0xffffffffu, myMin);
            if (m == INT_MAX)
                break;
            const int    src = __ffs(__ballot_sync(0xffffffffu, myMin == m)) - 1;
            const float4 kp  = make_float4(__shfl_sync(0xffffffffu, myP.x, src),
                                           __shfl_sync(0xffffffffu, myP.y, src),
                                           __shfl_sync(0xffffffffu, myP.z, src), 0.0f);
            if (lane == 0) {
                keptFlag[m] = 1;
                if (nk < cap)
                    mine[nk] = kp;
                else
                    atomicExch(overflow, 1);
            }
            nk = min(nk + 1, cap);
#pragma unroll
            for (int j = 0; j < kSpReg; j++)
                if (__float_as_int(q[j].w) == m ||
                    smm::dist2(kp.x, kp.y, kp.z, q[j].x, q[j].y, q[j].z) < r2)
                    alive &= ~(1u << j);
        }
        if (lane == 0)
            rankCnt[cell].y = nk;
    }
}

// ---------------------------------------------------------------------------------------
__global__ void k_mark_todo(const int *__restrict__ ids, int m, const float4 *__restrict__ nrm,
                            int *__restrict__ need) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const int id = ids[i];
    if (!finite3(nrm[id].x, nrm[id].y, nrm[id].z))
        need[id] = 2;
}

// One warp per query (exact k nearest neighbours, sm_device.cuh warp_knn_sorted); lane j
// writes the j-th neighbour, and with smoothing marks it when it still needs a normal.
__global__ void __launch_bounds__(256, 6)
    k_knn(const int *__restrict__ list, const int *__restrict__ nlp, HGridView G, const float4 *__restrict__ pos,
                      int k, int *__restrict__ nbr, int *__restrict__ nbrCnt, int markNeighbours,
                      const float4 *__restrict__ nrm, int *__restrict__ need) {
    chain_enter(); // launched chained
    const int nl = *nlp; // device-side count of the list
    const int lane = threadIdx.x & 31;
    const int t    = (int)(((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (t >= nl)
        return;
    const float4 q = pos[list[t]];
    int          id;
    float        d;
    const int    n = warp_knn_sorted(G, q.x, q.y, q.z, k, &id, &d);
    if (lane < k)
        nbr[(size_t)t * k + lane] = lane < n ? id : -1;
    if (lane == 0)
        nbrCnt[t] = n;
    if (markNeighbours && lane < n && need[id] == 0 && !finite3(nrm[id].x, nrm[id].y, nrm[id].z))
        need[id] = 1;
}

// list[0 .. *nlp) on the device; nlMax bounds it for the launch.
void launch_knn(const Ctx &c, const int *list, const int *nlp, int nlMax, const HGridView &G,
                const float4 *pos, int k, int *nbr, int *cnt, int mark, const float4 *nrm,
                int *need) {
    if (nlMax <= 0)
        return;
    launch_chained(c, k_knn, nblocks((long long)nlMax * 32, 256), 256, 0, list, nlp, G, pos, k, nbr,
                   cnt, mark, nrm, need);
}

// ---- hashed grid build -----------------------------------------------------------------
__device__ __forceinline__ unsigned long long hkey(const float4 &p, const GridParams &gp) {
    const int cx = smg::coord(p.x, gp.org[0], gp.g, gp.dim[0]);
    const int cy = smg::coord(p.y, gp.org[1], gp.g, gp.dim[1]);
    const int cz = smg::coord(p.z, gp.org[2], gp.g, gp.dim[2]);
    return ((unsigned long long)cz * (unsigned)gp.dim[1] + (unsigned)cy) * (unsigned)gp.dim[0] +
           (unsigned)cx;
}

__global__ void k_hg_insert(const float4 *__restrict__ pos, const int *__restrict__ ids, int m,
                            GridParams gp, unsigned long long *__restrict__ keys, uint32_t mask,
                            int *__restrict__ slotOf, int *__restrict__ cnt) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const unsigned long long key = hkey(pos[ids[i]], gp);
    uint32_t                 h   = (uint32_t)smm::mix64(key) & mask;
    for (uint32_t p = 0; p <= mask; p++) {
        const unsigned long long prev = atomicCAS(&keys[h], ~0ull, key);
        if (prev == ~0ull || prev == key) {
            slotOf[i] = (int)h;
            atomicAdd(&cnt[h], 1);
            return;
        }
        h = (h + 1) & mask;
    }
}

__global__ void k_hg_scatter(const float4 *__restrict__ pos, const int *__restrict__ ids,
                             const int *__restrict__ slotOf, int m, int *__restrict__ fill,
                             int *__restrict__ gids, float4 *__restrict__ pts, int wIsRank) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const int    id = ids[i];
    const float4 p  = pos[id];
    const int    k  = atomicAdd(&fill[slotOf[i]], 1);
    gids[k]         = id;
    pts[k]          = make_float4(p.x, p.y, p.z, __int_as_float(wIsRank ? i : id));
}

// Rank-ordered copies of a subset's positions and normals: out[r] = in[ids[r]].
__global__ void k_gather_subset(const float4 *__restrict__ pos, const float4 *__restrict__ nrm,
                                const int *__restrict__ ids, int m, float4 *__restrict__ subPos,
                                float4 *__restrict__ subNrm) {
    chain_enter(); // launched chained
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m)
        return;
    const int id = ids[r];
    subPos[r]    = pos[id];
    subNrm[r]    = nrm[id];
}

__global__ void k_hg_pack_from_start(const unsigned long long *__restrict__ keys,
                                     const int *__restrict__ start, uint32_t T,
                                     uint4 *__restrict__ slot, uint32_t *__restrict__ occ,
                                     int2 *__restrict__ dense) {
    chain_enter(); // launched chained
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T)
        return;
    const unsigned long long k   = keys[t];
    const uint32_t           cnt = (uint32_t)(start[t + 1] - start[t]);
    slot[t] = make_uint4((uint32_t)k, (uint32_t)(k >> 32), (uint32_t)start[t], cnt);
    if (occ && cnt)
        atomicOr(&occ[k >> 5], 1u << (k & 31));
    if (dense && cnt)
        dense[k] = make_int2(start[t], (int)cnt);
}

// Query lists in the query grid's cell order: a warp then searches 32 neighbouring queries
// (similar cells, shared cache lines, little divergence). flags[k] = need[gids[k]] == eq.
__global__ void k_flags_grid_order(const int *__restrict__ gids, int m, const int *__restrict__ need,
                                   int eq, int *__restrict__ flags) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m)
        flags[i] = need[gids[i]] == eq ? 1 : 0;
}

__global__ void k_scatter_ids(const int *__restrict__ flags, const int *__restrict__ pre, int n,
                              const int *__restrict__ gids, int *__restrict__ out) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flags[i])
        out[pre[i]] = gids[i];
}

// Phase A: centroid and FP32-Kahan covariance of the neighbourhood, FP64 eigensolve.
__global__ void k_pca(const int *__restrict__ list, const int *__restrict__ nlp, const int *__restrict__ nbr,
                      const int *__restrict__ nbrCnt, int k, const float4 *__restrict__ pos,
                      float4 *__restrict__ cen, float4 *__restrict__ nout) {
    chain_enter(); // launched chained
    const int nl = *nlp; // device-side count of the list
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl)
        return;
    const int  m = nbrCnt[t];
    const int *L = nbr + (size_t)t * k;
    if (m < 3) {
        cen[t]  = make_float4(0.f, 0.f, 0.f, -1.0f); // w < 0: no estimate
        nout[t] = make_float4(0.f, 0.f, 0.f, -1.0f);
        return;
    }
    smi::KahanF sx, sy, sz;
    sx.init();
    sy.init();
    sz.init();
    for (int j = 0; j < m; j++) {
        const float4 p = pos[L[j]];
        sx.add(p.x);
        sy.add(p.y);
        sz.add(p.z);
    }
    const float cx = smm::fdiv(sx.value(), (float)m), cy = smm::fdiv(sy.value(), (float)m),
                cz = smm::fdiv(sz.value(), (float)m);
    smi::KahanF a[6];
    for (int e = 0; e < 6; e++)
        a[e].init();
    for (int j = 0; j < m; j++) {
        const float4 p  = pos[L[j]];
        const float  dx = p.x - cx, dy = p.y - cy, dz = p.z - cz;
        a[0].add(dx * dx);
        a[1].add(dx * dy);
        a[2].add(dx * dz);
        a[3].add(dy * dy);
        a[4].add(dy * dz);
        a[5].add(dz * dz);
    }
    double C[6];
    for (int e = 0; e < 6; e++)
        C[e] = (double)a[e].value();
    float n3[3];
    sml::normal_from_cov(C, n3);
    cen[t]  = make_float4(cx, cy, cz, 1.0f);
    nout[t] = make_float4(n3[0], n3[1], n3[2], 1.0f);
}

__global__ void k_pca_write(const int *__restrict__ list, const int *__restrict__ nlp, const float4 *__restrict__ cen,
                            const float4 *__restrict__ nin, float4 *__restrict__ pos,
                            float4 *__restrict__ nrm) {
    chain_enter(); // launched chained
    const int nl = *nlp; // device-side count of the list
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl || cen[t].w < 0.0f)
        return;
    const int id = list[t];
    pos[id]      = make_float4(cen[t].x, cen[t].y, cen[t].z, 0.0f);
    nrm[id]      = make_float4(nin[t].x, nin[t].y, nin[t].z, 0.0f);
}

// Phase B: sign-aligned sum of the raw neighbourhood normals (util.cpp:292-306).
__global__ void k_smooth(const int *__restrict__ list, const int *__restrict__ nlp, const int *__restrict__ nbr,
                         const int *__restrict__ nbrCnt, int k, const float4 *__restrict__ nrm,
                         float4 *__restrict__ out) {
    chain_enter(); // launched chained
    const int nl = *nlp; // device-side count of the list
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl)
        return;
    const int m = nbrCnt[t];
    if (m < 3) {
        out[t] = make_float4(0.f, 0.f, 0.f, -1.0f);
        return;
    }
    const float4 n0 = nrm[list[t]];
    float        sx = 0.f, sy = 0.f, sz = 0.f;
    for (int j = 0; j < m; j++) {
        const float4 n = nrm[nbr[(size_t)t * k + j]];
        const float  d = n.x * n0.x + (n.y * n0.y + n.z * n0.z);
        if (d > 0.0f) {
            sx = sx + n.x;
            sy = sy + n.y;
            sz = sz + n.z;
        } else {
            sx = sx - n.x;
            sy = sy - n.y;
            sz = sz - n.z;
        }
    }
    const float sq = sx * sx + (sy * sy + sz * sz);
    if (sq > 0.0f) {
        const float s = smm::fsqrt(sq);
        sx            = smm::fdiv(sx, s);
        sy            = smm::fdiv(sy, s);
        sz            = smm::fdiv(sz, s);
    }
    out[t] = make_float4(sx, sy, sz, 1.0f);
}

__global__ void k_smooth_write(const int *__restrict__ list, const int *__restrict__ nlp, const float4 *__restrict__ sm,
                               float4 *__restrict__ nrm) {
    chain_enter(); // launched chained
    const int nl = *nlp; // device-side count of the list
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nl || sm[t].w < 0.0f)
        return;
    nrm[list[t]] = make_float4(sm[t].x, sm[t].y, sm[t].z, 0.0f);
}

// Phase C: orientation toward the viewpoint, or +z (util.cpp:309-333).
__global__ void k_orient(const int *__restrict__ ids, int m, const float4 *__restrict__ pos,
                         float4 *__restrict__ nrm, int hasVp, float vx, float vy, float vz,
                         int invert) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    const int id = ids[i];
    float4    n  = nrm[id];
    float     d;
    if (hasVp) {
        const float4 p = pos[id];
        const float  ax = vx - p.x, ay = vy - p.y, az = vz - p.z;
        d               = n.x * ax + (n.y * ay + n.z * az);
    } else {
        d = n.x * 0.0f + (n.y * 0.0f + n.z * 1.0f);
    }
    const bool flip = invert ? (d > 0.0f) : (d < 0.0f);
    if (flip)
        nrm[id] = make_float4(-n.x, -n.y, -n.z, 0.0f);
}

__global__ void k_normalize(float4 *__restrict__ nrm, int n) {
    chain_enter(); // launched chained
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float4      v  = nrm[i];
    const float sq = v.x * v.x + (v.y * v.y + v.z * v.z);
    if (sq > 0.0f) {
        const float s = smm::fsqrt(sq);
        nrm[i]        = make_float4(smm::fdiv(v.x, s), smm::fdiv(v.y, s), smm::fdiv(v.z, s), 0.0f);
    }
}

} // namespace

// =======================================================================================
int prep_points(Ctx &c, const float *xyz, const float *nin, int n, float4 *pos, float4 *nrm,
                int *validFlag, Box &box) {
    int *dev = c.arena.get<int>("prep.bbox", 8);
    k_init_bbox<<<1, 32, 0, c.stream>>>(dev, dev + 6);
    SM_LAUNCH_CHECK();
    const int bs = 256;
    int       nb = std::min(nblocks(n, bs), 152 * 16);
    if (nb < 1)
        nb = 1;
    k_prep<<<nb, bs, 0, c.stream>>>(xyz, nin, n, pos, nrm, validFlag, dev, dev + 6);
    SM_LAUNCH_CHECK();
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, dev, 7 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    for (int a = 0; a < 3; a++) {
        box.mn[a] = ord2f(c.hostCounts[a]);
        box.mx[a] = ord2f(c.hostCounts[3 + a]);
    }
    return c.hostCounts[6];
}

// The context's look-back state, grown to at least nparts tiles (zeroed when allocated);
// returns the next scan epoch.
static unsigned scan_state(Ctx &c, int nparts) {
    Ctx::ScanState &S = c.scan;
    if (nparts > S.cap || S.epoch >= (1u << 30) - 1) {
        const int cap = std::max(nparts, std::max(S.cap, 1024));
        S.status      = c.arena.get<unsigned long long>("scan.status", cap);
        S.ticket      = c.arena.get<int>("scan.ticket", 2);
        SM_CUDA(cudaMemsetAsync(S.status, 0, (size_t)cap * 8, c.stream));
        SM_CUDA(cudaMemsetAsync(S.ticket, 0, 2 * sizeof(int), c.stream));
        S.cap   = cap;
        S.epoch = 0;
    }
    return ++S.epoch;
}

// Exclusive scan of n values (or of value == eq flags) into out; the total goes to *total
// (device) when given.
static void scan_into(Ctx &c, const int *in, int *out, long long n, int eq, int *total) {
    const int nparts = (int)((n + kScanTile - 1) / kScanTile);
    if (nparts == 0) {
        if (total)
            SM_CUDA(cudaMemsetAsync(total, 0, sizeof(int), c.stream));
        return;
    }
    const unsigned epoch = scan_state(c, nparts);
    cudaEvent_t    t0    = c.clock.begin(c.stream);
    launch_chained(c, k_scan_lookback, nparts, kScanBs, 0, in, out, n, eq, c.scan.status,
                   c.scan.ticket, nparts, epoch, total);
    c.clock.end(c.stream, t0, KernelClock::kScan, 8.0 * (double)n); // 4-byte value in, 4 out
}

static int scan_impl(Ctx &c, const int *in, int *out, long long n, int eq, const std::string &tag,
                     bool wantTotal) {
    int *total = c.arena.get<int>(tag + ".scantot", 1);
    scan_into(c, in, out, n, eq, total);
    if (!wantTotal)
        return -1;
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, total, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync_checked();
    return c.hostCounts[0];
}

// Exclusive scan of 0/1 flags without a host round trip; returns the device address of the
// total.
static int *scan_flags_total(Ctx &c, const int *flags, int *pre, int n, const std::string &tag) {
    int *total = c.arena.get<int>(tag + ".scantot", 1);
    scan_into(c, flags, pre, n, kNoEq, total);
    return total;
}

int scan_excl(Ctx &c, const int *in, int *out, long long n, const std::string &tag, bool wantTotal) {
    return scan_impl(c, in, out, n, kNoEq, tag, wantTotal);
}

static int compact_eq(Ctx &c, const int *flags, int n, int eq, int *outIds, const std::string &tag) {
    if (n <= 0)
        return 0;
    int      *pre   = c.arena.get<int>(tag + ".pre", n);
    const int total = scan_impl(c, flags, pre, n, eq, tag, true);
    launch_chained(c, k_scatter_flags, nblocks(n, 256), 256, 0, flags, pre, n, eq, outIds);
    return total;
}

int compact(Ctx &c, const int *flags, int n, int *outIds, const std::string &tag) {
    return compact_eq(c, flags, n, kNoEq, outIds, tag);
}

void compact_known(Ctx &c, const int *flags, int n, int *outIds, const std::string &tag) {
    if (n <= 0)
        return;
    int *pre = c.arena.get<int>(tag + ".pre", n);
    scan_impl(c, flags, pre, n, kNoEq, tag, false);
    launch_chained(c, k_scatter_flags, nblocks(n, 256), 256, 0, flags, pre, n, kNoEq, outIds);
}

// The points p of grid H with need[p] == eq, in H's cell order, into out; returns the device
// address of their count (no host round trip).
static int *compact_grid_order(Ctx &c, const HGrid &H, const int *need, int eq, int *out,
                               const std::string &tag) {
    int *flags = c.arena.get<int>(tag + ".gf", std::max(H.m, 1));
    int *pre   = c.arena.get<int>(tag + ".gp", std::max(H.m, 1));
    if (H.m <= 0) {
        int *z = c.arena.get<int>(tag + ".gz", 1);
        SM_CUDA(cudaMemsetAsync(z, 0, sizeof(int), c.stream));
        return z;
    }
    launch_chained(c, k_flags_grid_order, nblocks(H.m, 256), 256, 0, H.ids, H.m, need, eq,
                   flags);
    int *total = scan_flags_total(c, flags, pre, H.m, tag + ".gc");
    launch_chained(c, k_scatter_ids, nblocks(H.m, 256), 256, 0, flags, pre, H.m, H.ids, out);
    return total;
}

void build_hgrid(Ctx &c, const float4 *pos, const int *ids, int m, const Box &box, float g,
                 HGrid &H, const std::string &tag, bool wIsRank) {
    // cells per axis stay below 2^20 so that cell keys fit 60 bits (coarser cells if needed)
    while (smg::dim_of(box.ext(0), g) >= (1 << 20) || smg::dim_of(box.ext(1), g) >= (1 << 20) ||
           smg::dim_of(box.ext(2), g) >= (1 << 20))
        g = g * 2.0f;
    H.g = g;
    for (int a = 0; a < 3; a++) {
        H.org[a] = box.mn[a];
        H.dim[a] = smg::dim_of(box.ext(a), g);
    }
    uint32_t T = 1024;
    while (T < 2u * (uint32_t)std::max(m, 1))
        T <<= 1;
    H.mask = T - 1;
    H.m    = m;
    auto *keys   = c.arena.get<unsigned long long>(tag + ".keys", T);
    int  *cnt    = c.arena.get<int>(tag + ".cnt", T + 1);
    int  *start  = c.arena.get<int>(tag + ".start", T + 1);
    int  *slotOf = c.arena.get<int>(tag + ".slotOf", std::max(m, 1));
    H.ids        = c.arena.get<int>(tag + ".ids", std::max(m, 1));
    H.pts        = c.arena.get<float4>(tag + ".pts", std::max(m, 1));
    H.slot       = c.arena.get<uint4>(tag + ".slot", T);
    // occupancy bits over the cell box, when it has at most 2^28 cells (32 MB), and a direct
    // {first, count} table too when it has at most 2^22 cells (32 MB); all cleared with the
    // key and count tables in one launch
    const unsigned long long ncell = (unsigned long long)H.dim[0] * H.dim[1] * H.dim[2];
    const size_t             words = (size_t)((ncell + 31) / 32);
    H.occ   = ncell <= (1ull << 28) ? c.arena.get<uint32_t>(tag + ".occ", words) : nullptr;
    H.dense = ncell <= (1ull << 22) ? c.arena.get<int2>(tag + ".dense", (size_t)ncell) : nullptr;
    FillSet clear;
    clear.add(keys, (size_t)T * 8, 0xffffffffu);
    clear.add(cnt, (size_t)(T + 1) * 4, 0u);
    if (H.occ)
        clear.add(H.occ, words * 4, 0u);
    if (H.dense)
        clear.add(H.dense, (size_t)ncell * sizeof(int2), 0u);
    fill(c, clear);
    GridParams gp = grid_params(box, g, H.dim);
    if (m > 0) {
        launch_chained(c, k_hg_insert, nblocks(m, 256), 256, 0, pos, ids, m, gp, keys, H.mask,
                       slotOf, cnt);
    }
    scan_excl(c, cnt, start, (long long)T + 1, tag, false);
    int *fill = cnt;
    SM_CUDA(cudaMemcpyAsync(fill, start, (size_t)T * 4, cudaMemcpyDeviceToDevice, c.stream));
    if (m > 0) {
        launch_chained(c, k_hg_scatter, nblocks(m, 256), 256, 0, pos, ids, slotOf, m, fill,
                       H.ids, H.pts, wIsRank ? 1 : 0);
    }
    // counts again for the packed table: start[t+1] - start[t]
    launch_chained(c, k_hg_pack_from_start, nblocks(T, 256), 256, 0, keys, start, T, H.slot,
                   H.occ, H.dense);
}

void gather_subset(Ctx &c, const float4 *pos, const float4 *nrm, const int *ids, int m,
                   float4 *subPos, float4 *subNrm) {
    if (m <= 0)
        return;
    launch_chained(c, k_gather_subset, nblocks(m, 256), 256, 0, pos, nrm, ids, m, subPos,
                   subNrm);
}

int sample_points(Ctx &c, const float4 *pos, int npoints, const int *ids, int m, const Box &box,
                  float step, int *outIds, const std::string &tag) {
    if (m <= 0)
        return 0;
    if (!(step > 0.0f)) {
        // no point lies at a squared distance below zero: every point is kept (the list is
        // ascending already)
        SM_CUDA(cudaMemcpyAsync(outIds, ids, (size_t)m * sizeof(int), cudaMemcpyDeviceToDevice,
                                c.stream));
        return m;
    }
    float ext[3] = {box.ext(0), box.ext(1), box.ext(2)};
    const float g = smg::thin_cell(step, ext);
    // the cell table over the points (dense or hashed, see ThinView), its occupied cells
    // listed per phase on the device (no host round trip; at most m of them)
    int dim[3];
    for (int a = 0; a < 3; a++)
        dim[a] = smg::dim_of(ext[a], g);
    uint32_t T = 1024;
    while (T < 2u * (uint32_t)m)
        T <<= 1;
    // dense table (slot = cell key) when the cell box has at most 2^22 cells or 16 per
    // point (its counts and their scan move 12 bytes a cell, the hashed table's key claims
    // and scattered placing cost more a point), never above 2^27 cells
    const unsigned long long ncell = (unsigned long long)dim[0] * dim[1] * dim[2];
    const unsigned long long dmax  = std::max<unsigned long long>(1ull << 22, 16ull * (unsigned)m);
    const bool               dense = ncell <= std::min<unsigned long long>(dmax, 1ull << 27);
    if (dense)
        T = (uint32_t)ncell;
    const long long maxOcc = m;
    auto *keys = dense ? nullptr : c.arena.get<unsigned long long>(tag + ".g.keys", T);
    int   *cnt     = c.arena.get<int>(tag + ".g.cnt", (size_t)T + 1);
    int   *start   = c.arena.get<int>(tag + ".g.start", (size_t)T + 1);
    float4 *pts    = c.arena.get<float4>(tag + ".g.pts", m);
    int   *slotOf  = c.arena.get<int>(tag + ".g.slotOf", m);
    int   *sub     = c.arena.get<int>(tag + ".g.sub", m);
    int   *ph      = c.arena.get<int>(tag + ".ph", kSpPh);
    int2  *rankCnt = c.arena.get<int2>(tag + ".rank", T);
    int   *lists   = c.arena.get<int>(tag + ".phl", maxOcc);
    int   *keptFlag = c.arena.get<int>(tag + ".kf", (size_t)m + 1); // over the list places
    int   *overflow = keptFlag + m;
    FillSet clear;
    if (!dense)
        clear.add(keys, (size_t)T * 8, 0xffffffffu);
    clear.add(cnt, ((size_t)T + 1) * sizeof(int), 0u);
    clear.add(ph, kSpPh * sizeof(int), 0u);
    fill(c, clear);
    const GridParams gpar = grid_params(box, g, dim);
    launch_chained(c, k_thin_insert, nblocks(m, 256), 256, 0, pos, ids, m, gpar, keys,
                   dense ? 0u : T - 1, slotOf, sub, cnt, ph);
    scan_excl(c, cnt, start, (long long)T + 1, tag + ".g", false);
    launch_chained(c, k_phase_offsets, 1, 32, 0, ph);
    launch_chained(c, k_thin_scatter, nblocks(m, 256), 256, 0, pos, ids, m, slotOf, sub,
                   start, keys, dim[0], dim[1], pts, ph, lists, rankCnt, keptFlag);
    ThinView V;
    for (int a = 0; a < 3; a++) {
        V.org[a] = box.mn[a];
        V.dim[a] = dim[a];
    }
    V.g     = g;
    V.keys  = keys;
    V.mask  = dense ? 0u : T - 1;
    V.start = start;
    V.pts   = pts;
    // kept-list capacity: points at pairwise distance >= step inside a cube of side g fit
    // disjoint balls of radius step/2 inside the cube grown by step/2.
    const double s   = (double)g / (double)step;
    const int    cap = (int)std::floor((s + 1.0) * (s + 1.0) * (s + 1.0) / (3.14159265358979 / 6.0)) + 1;
    float4 *keptPos  = c.arena.get<float4>(tag + ".kp", (size_t)maxOcc * cap);
    int    *aliveTmp = c.arena.get<int>(tag + ".al", std::max(m, 1));
    const float r2 = step * step;
    // one resident wave: heavy cells are handed out by a counter, light cells by stride
    static std::atomic<int> resident[64];
    const int               dev = c.device >= 0 && c.device < 64 ? c.device : 0;
    int                     per = resident[dev].load();
    if (per <= 0) {
        SM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sample_phase, kSpWarps * 32, 0));
        per = std::max(per, 1);
        resident[dev].store(per);
    }
    int nsm = 0;
    SM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
    const int gp = (int)std::min<long long>((maxOcc + kSpWarps - 1) / kSpWarps, (long long)nsm * per);
    for (int p = 0; p < 8; p++) {
        cudaEvent_t t0 = c.clock.begin(c.stream);
        launch_chained(c, k_sample_phase, gp, kSpWarps * 32, 0, V, lists, ph, p, rankCnt,
                       keptPos, cap, r2, keptFlag, overflow, aliveTmp);
        // algorithmic bytes of a sampling: each point's position read and its flag written
        // once (16 + 4 bytes), spread over the 8 phases
        c.clock.end(c.stream, t0, KernelClock::kSamplePhase, 20.0 * (double)m / 8.0);
    }
    // the kept points in index order (list order), and the overflow flag, in one round trip
    int *pre   = c.arena.get<int>(tag + ".out.pre", std::max(m, 1));
    int *total = scan_flags_total(c, keptFlag, pre, m, tag + ".out");
    launch_chained(c, k_scatter_ids, nblocks(m, 256), 256, 0, keptFlag, pre, m, ids, outIds);
    SM_CUDA(cudaMemcpyAsync(c.hostCounts, total, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    SM_CUDA(cudaMemcpyAsync(c.hostCounts + 1, overflow, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    c.sync();
    if (c.hostCounts[1])
        throw Error(SM_ERR_CAPACITY, "sampler: kept-point capacity per cell exceeded");
    return c.hostCounts[0];
}

// The points p < n with need[p] == eq, ascending, into out; returns the device address of
// their count (no host round trip).
static int *compact_need(Ctx &c, const int *need, int n, int eq, int *out, const std::string &tag) {
    int *total = c.arena.get<int>(tag + ".scantot", 1);
    int *pre   = c.arena.get<int>(tag + ".pre", std::max(n, 1));
    scan_into(c, need, pre, n, eq, total);
    if (n > 0) {
        launch_chained(c, k_scatter_flags, nblocks(n, 256), 256, 0, need, pre, n, eq, out);
    }
    return total;
}

void estimate_normals(Ctx &c, float4 *pos, float4 *nrm, int npoints, const int *ids, int m,
                      const HGrid &query, int k, bool smooth, bool invert, const float *vp,
                      const std::string &tag, const KdTree *tree) {
    if (m <= 0)
        return;
    if (k < 3)
        k = 3;
    if (k > kMaxKnn)
        throw Error(SM_ERR_RANGE, "knnNormal larger than " + std::to_string(kMaxKnn) + " is not supported");
    int *need = c.arena.get<int>(tag + ".need", npoints);
    FillSet clear;
    clear.add(need, (size_t)npoints * sizeof(int), 0u);
    fill(c, clear);
    launch_chained(c, k_mark_todo, nblocks(m, 256), 256, 0, ids, m, nrm, need);
    // the query lists and their counts stay on the device; launches are sized by bounds
    // with the reference's k-d tree the k nearest come from its depth-first search (ties:
    // first found); the lists are then in index order (the results do not depend on it)
    int       *todo   = c.arena.get<int>(tag + ".todo", std::max(tree ? npoints : m, 1));
    const int *ntodo  = tree ? compact_need(c, need, npoints, 2, todo, tag + ".ct")
                             : compact_grid_order(c, query, need, 2, todo, tag + ".ct");
    int       *nbrT   = c.arena.get<int>(tag + ".nbrT", (size_t)m * k);
    int       *cntT   = c.arena.get<int>(tag + ".cntT", m);
    if (tree)
        kd_knn(c, *tree, nullptr, pos, nullptr, todo, ntodo, m, k, nbrT, nullptr, cntT, nrm,
               smooth ? need : nullptr);
    else
        launch_knn(c, todo, ntodo, m, query.view(), pos, k, nbrT, cntT, smooth ? 1 : 0, nrm, need);
    const int  extraMax = smooth ? (int)std::min<long long>(npoints, (long long)m * k) : 0;
    int       *extra = nullptr, *nbrE = nullptr, *cntE = nullptr;
    const int *nextra = nullptr;
    if (extraMax > 0) {
        extra  = c.arena.get<int>(tag + ".extra", std::max(tree ? npoints : extraMax, 1));
        nextra = tree ? compact_need(c, need, npoints, 1, extra, tag + ".ce")
                      : compact_grid_order(c, query, need, 1, extra, tag + ".ce");
        nbrE   = c.arena.get<int>(tag + ".nbrE", (size_t)extraMax * k);
        cntE   = c.arena.get<int>(tag + ".cntE", extraMax);
        if (tree)
            kd_knn(c, *tree, nullptr, pos, nullptr, extra, nextra, extraMax, k, nbrE, nullptr, cntE);
        else
            launch_knn(c, extra, nextra, extraMax, query.view(), pos, k, nbrE, cntE, 0, nrm, need);
    }
    const int nmax = std::max(m, extraMax);
    float4   *cen  = c.arena.get<float4>(tag + ".cen", 2 * (size_t)nmax);
    float4   *nn   = c.arena.get<float4>(tag + ".nn", 2 * (size_t)nmax);
    launch_chained(c, k_pca, nblocks(m, 128), 128, 0, todo, ntodo, nbrT, cntT, k, pos, cen,
                   nn);
    if (extraMax > 0) {
        launch_chained(c, k_pca, nblocks(extraMax, 128), 128, 0, extra, nextra, nbrE, cntE, k,
                       pos, cen + nmax, nn + nmax);
    }
    launch_chained(c, k_pca_write, nblocks(m, 256), 256, 0, todo, ntodo, cen, nn, pos, nrm);
    if (extraMax > 0) {
        launch_chained(c, k_pca_write, nblocks(extraMax, 256), 256, 0, extra, nextra,
                       cen + nmax, nn + nmax, pos, nrm);
    }
    if (smooth) {
        launch_chained(c, k_smooth, nblocks(m, 256), 256, 0, todo, ntodo, nbrT, cntT, k, nrm,
                       cen);
        launch_chained(c, k_smooth_write, nblocks(m, 256), 256, 0, todo, ntodo, cen, nrm);
    }
    const bool hasVp = vp && std::isfinite(vp[0]) && std::isfinite(vp[1]) && std::isfinite(vp[2]);
    launch_chained(c, k_orient, nblocks(m, 256), 256, 0, ids, m, pos, nrm, hasVp ? 1 : 0,
                   hasVp ? vp[0] : 0.f, hasVp ? vp[1] : 0.f, hasVp ? vp[2] : 0.f, invert ? 1 : 0);
}

void normalize_normals(Ctx &c, float4 *nrm, int n) {
    if (n <= 0)
        return;
    launch_chained(c, k_normalize, nblocks(n, 256), 256, 0, nrm, n);
}

} // namespace sm
