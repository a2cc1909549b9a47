// sm_device.cuh - device-side building blocks of the matching path: grid views and exact
// grid searches, ordered float atomics, warp/block helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sm_grid.h"
#include "sm_math.h"

namespace smd {

constexpr int kMaxKnn = 32; // largest supported knnNormal

// Device view of a dense uniform grid over a subset of points: cells are stored cell-major
// as a CSR (start[cell] .. start[cell+1] into ids). Used where per-cell state is needed
// (the sampler).
struct GridView {
    float      org[3];
    float      g;
    int        dim[3];
    const int *start;
    const int *ids;
    __device__ __forceinline__ void range(int x, int y, int z, int &s, int &e) const {
        const int c = (z * dim[1] + y) * dim[0] + x;
        s           = start[c];
        e           = start[c + 1];
    }
};

// Device view of a hashed uniform grid: only occupied cells are stored, in an
// open-addressed table of uint4 {key low, key high, first point, point count} (count 0 =
// empty slot), so cells can be as fine as the queries want whatever the scene's extent,
// and the table stays small enough to live in L2. The points of a cell are contiguous in
// `pts` (position, point index in w), so a search reads them without an indirection, and
// an occupancy bitmap over the cell box lets searches skip empty cells without a probe.
struct HGridView {
    float         org[3];
    float         g;
    int           dim[3];
    const uint4  *slot;
    uint32_t      mask;
    const int    *ids;
    const float4 *pts;
    const uint32_t *occ; // one bit per cell of the dim box (nullptr: not built)
    __device__ __forceinline__ void range(int x, int y, int z, int &s, int &e) const {
        const unsigned long long key =
            ((unsigned long long)z * (unsigned)dim[1] + (unsigned)y) * (unsigned)dim[0] + (unsigned)x;
        if (occ && !((occ[key >> 5] >> (key & 31)) & 1u)) {
            s = e = 0; // empty cell: no table probe
            return;
        }
        uint32_t h = (uint32_t)smm::mix64(key) & mask;
        for (uint32_t p = 0; p <= mask; p++) {
            const uint4 v = slot[h];
            if (v.w == 0u)
                break;
            if (v.x == (uint32_t)key && v.y == (uint32_t)(key >> 32)) {
                s = (int)v.z;
                e = (int)(v.z + v.w);
                return;
            }
            h = (h + 1) & mask;
        }
        s = e = 0;
    }
};

template <class G> __device__ __forceinline__ void grid_cc(const G &g, float x, float y, float z, int c[3]) {
    c[0] = smg::coord(x, g.org[0], g.g, g.dim[0]);
    c[1] = smg::coord(y, g.org[1], g.g, g.dim[1]);
    c[2] = smg::coord(z, g.org[2], g.g, g.dim[2]);
}

__device__ __forceinline__ int grid_cell(const GridView &G, int x, int y, int z) {
    return (z * G.dim[1] + y) * G.dim[0] + x;
}

template <class G> __device__ __forceinline__ int grid_max_shell(const G &g, const int c[3]) {
    int m = 0;
    for (int a = 0; a < 3; a++) {
        const int lo = c[a], hi = g.dim[a] - 1 - c[a];
        m          = max(m, max(lo, hi));
    }
    return m;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o)
            v += t;
    }
    return v;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v                          = t < v ? t : v;
    }
    return v;
}

// Ascending bitonic sort of one 64-bit key per lane across the warp.
__device__ __forceinline__ unsigned long long warp_bitonic_sort(unsigned long long key) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            const unsigned long long o  = __shfl_xor_sync(0xffffffffu, key, j);
            const bool               up = (lane & k) == 0, lower = (lane & j) == 0;
            key = (lower == up) ? (o < key ? o : key) : (o > key ? o : key);
        }
    }
    return key;
}

// The 32 smallest of two ascending warp-wide lists (one key per lane), ascending.
__device__ __forceinline__ unsigned long long warp_merge_low(unsigned long long r,
                                                             unsigned long long sorted) {
    const int                lane = threadIdx.x & 31;
    const unsigned long long rev  = __shfl_sync(0xffffffffu, sorted, 31 - lane);
    unsigned long long       m    = rev < r ? rev : r; // bitonic, holds the 32 smallest
#pragma unroll
    for (int j = 16; j > 0; j >>= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, m, j);
        m                          = (lane & j) == 0 ? (o < m ? o : m) : (o > m ? o : m);
    }
    return m;
}

// Warp-cooperative walk over the points around q, shell by shell (shells 0 and 1 together:
// the 3x3x3 block; no search can stop after shell 0, whose ring bound is 0). The lanes probe
// 32 cells at a time (occupancy bit, table), a prefix sum flattens the probed cells' points,
// and visit(p, valid) is called by all lanes for each round of 32 points (p = position with
// the point index in w; valid false on idle lanes). After each shell, stop(s) - evaluated by
// all lanes, warp-uniform - ends the walk. Every point of shells 1..s is visited exactly once
// before stop(s), so a search written on it sees the same points as one that walks the
// cells one by one.
template <class G, class V, class S>
__device__ __forceinline__ void warp_walk(const G &g, float qx, float qy, float qz, V &&visit,
                                          S &&stop) {
    const int lane = threadIdx.x & 31;
    int       c[3];
    grid_cc(g, qx, qy, qz, c);
    const int ms = max(grid_max_shell(g, c), 1);
    for (int s = 1; s <= ms; s++) {
        const int lo = s == 1 ? 0 : s, w = 2 * s + 1, cube = w * w * w;
        for (int t0 = 0; t0 < cube; t0 += 32) {
            const int t = t0 + lane;
            int       b = 0, e = 0;
            if (t < cube) {
                const int dx = t % w - s, dy = (t / w) % w - s, dz = t / (w * w) - s;
                const int r  = max(abs(dx), max(abs(dy), abs(dz)));
                const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                if (r >= lo && x >= 0 && y >= 0 && z >= 0 && x < g.dim[0] && y < g.dim[1] &&
                    z < g.dim[2])
                    g.range(x, y, z, b, e);
            }
            const int cnt  = e - b;
            const int incl = warp_incl_scan(cnt);
            const int excl = incl - cnt;
            const int T    = __shfl_sync(0xffffffffu, incl, 31);
            for (int base = 0; base < T; base += 32) {
                const int r   = base + lane;
                int       own = 0; // the lane whose cell holds point r: last lane with excl <= r
#pragma unroll
                for (int step = 16; step >= 1; step >>= 1) {
                    const int mid = own + step;
                    if (__shfl_sync(0xffffffffu, excl, mid) <= r)
                        own = mid;
                }
                const int bj = __shfl_sync(0xffffffffu, b, own);
                const int ej = __shfl_sync(0xffffffffu, excl, own);
                const bool   valid = r < T;
                const float4 p     = valid ? g.pts[bj + (r - ej)] : make_float4(0.f, 0.f, 0.f, 0.f);
                visit(p, valid);
            }
        }
        if (stop(s))
            return;
    }
}

// Exact k nearest neighbours (k <= 32) of q by (squared distance, index), one warp per
// query, on warp_walk: each round of 32 points is sorted across the lanes and merged into
// the running 32 best (lane j holds the j-th smallest key: distance bits, index); rounds with
// no point below the current k-th best are skipped. The search ends after shell s once k
// points were seen and the k-th distance is below the ring bound of s (every unvisited point
// is farther), so the result is the exact k nearest. Returns the number found (<= k); lane
// j < that count gets the j-th neighbour's index in *id and squared distance in *d.
template <class G>
__device__ __forceinline__ int warp_knn_sorted(const G &g, float qx, float qy, float qz, int k,
                                               int *id, float *d) {
    unsigned long long best = ~0ull; // lane j: j-th smallest so far
    int                seen = 0;
    warp_walk(
        g, qx, qy, qz,
        [&](const float4 &p, bool valid) {
            seen += __popc(__ballot_sync(0xffffffffu, valid));
            unsigned long long key = ~0ull;
            if (valid) {
                const float dd = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
                key = ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)__float_as_int(p.w);
            }
            const unsigned long long kth = __shfl_sync(0xffffffffu, best, k - 1);
            if (__any_sync(0xffffffffu, key < kth))
                best = warp_merge_low(best, warp_bitonic_sort(key));
        },
        [&](int s) {
            if (seen < k)
                return false;
            const unsigned long long kth = __shfl_sync(0xffffffffu, best, k - 1);
            const float              bnd = smg::ring_bound(s, g.g);
            return __uint_as_float((unsigned)(kth >> 32)) < bnd * bnd;
        });
    const int n = min(seen, k);
    *id         = (int)(unsigned)(best & 0xffffffffu);
    *d          = __uint_as_float((unsigned)(best >> 32));
    return n;
}

// Nearest point by (squared distance, index) on warp_walk, searched until the nearest is
// below the ring bound or the ring bound passes limit2; -1 when none was found. All lanes
// return the result.
template <class G>
__device__ __forceinline__ int warp_nn_walk(const G &g, float qx, float qy, float qz,
                                            float limit2, float &outd) {
    unsigned long long best = ~0ull;
    warp_walk(
        g, qx, qy, qz,
        [&](const float4 &p, bool valid) {
            if (valid) {
                const float dd = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
                const unsigned long long key =
                    ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)__float_as_int(p.w);
                best = key < best ? key : best;
            }
        },
        [&](int s) {
            best          = warp_min_u64(best);
            const float b = smg::ring_bound(s, g.g);
            return (best != ~0ull && __uint_as_float((unsigned)(best >> 32)) < b * b) ||
                   b * b > limit2;
        });
    best = warp_min_u64(best);
    if (best == ~0ull) {
        outd = 3.402823466e+38f;
        return -1;
    }
    outd = __uint_as_float((unsigned)(best >> 32));
    return (int)(unsigned)(best & 0xffffffffu);
}

// Whether any point lies closer than sqrt(r2) to q, by a warp: stops at a hit or after the
// shell whose ring bound reaches sqrt(r2).
template <class G>
__device__ __forceinline__ bool warp_any_within(const G &g, float qx, float qy, float qz, float r2) {
    bool hit = false;
    warp_walk(
        g, qx, qy, qz,
        [&](const float4 &p, bool valid) {
            const bool h = valid && smm::dist2(qx, qy, qz, p.x, p.y, p.z) < r2;
            hit          = hit || __any_sync(0xffffffffu, h);
        },
        [&](int s) {
            const float b = smg::ring_bound(s, g.g);
            return hit || b * b >= r2;
        });
    return hit;
}

// Order-preserving float <-> int mapping for atomicMin/atomicMax on floats.
__device__ __forceinline__ int f2ord(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__host__ __device__ __forceinline__ float ord2f(int i) {
#if defined(__CUDA_ARCH__)
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
#else
    int   j = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    memcpy(&f, &j, 4);
    return f;
#endif
}


// Block-wide exclusive scan of one int per thread (blockDim.x <= 1024, multiple of 32).
// `sh` needs 33 ints. Returns the exclusive prefix; *total gets the block sum.
__device__ __forceinline__ int block_excl_scan(int v, int *sh, int *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int inc  = warp_incl_scan(v);
    if (lane == 31)
        sh[w] = inc;
    __syncthreads();
    if (w == 0) {
        int s  = lane < nw ? sh[lane] : 0;
        int si = warp_incl_scan(s);
        if (lane < nw)
            sh[lane] = si - s;
        if (lane == 31)
            sh[32] = si;
    }
    __syncthreads();
    const int r = sh[w] + inc - v;
    if (total)
        *total = sh[32];
    __syncthreads();
    return r;
}

} // namespace smd
