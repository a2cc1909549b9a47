// sm_device.cuh - device-side building blocks of the matching path: grid views and exact
// grid searches, ordered float atomics, warp/block helpers.
#pragma once

#include <climits>

#include <cuda_runtime.h>
#include <stdint.h>

#include "sm_grid.h"
#include "sm_math.h"

namespace smd {

constexpr int kMaxKnn      = 32; // largest supported knnNormal
constexpr int kKnnMaxShell = 24; // shells a k-nearest walk visits before it scans every point

// Device view of a hashed uniform grid: only occupied cells are stored, in an
// open-addressed table of uint4 {key low, key high, first point, point count} (count 0 =
// empty slot), so cells can be as fine as the queries want whatever the scene's extent,
// and the table stays small enough to live in L2. The points of a cell are contiguous in
// `pts` (position, point index in w), so a search reads them without an indirection, and
// an occupancy bitmap over the cell box lets searches skip empty cells without a probe.
// Small cell boxes also get a direct table of {first, count} per cell, read in one load.
struct HGridView {
    float         org[3];
    float         g;
    int           dim[3];
    const uint4  *slot;
    uint32_t      mask;
    const int    *ids;
    const float4 *pts;
    const uint32_t *occ;   // one bit per cell of the dim box (nullptr: not built)
    const int2     *dense; // {first, count} per cell of the dim box (nullptr: not built)
    int             m;     // points in pts
    __device__ __forceinline__ unsigned long long key_of(int x, int y, int z) const {
        return ((unsigned long long)z * (unsigned)dim[1] + (unsigned)y) * (unsigned)dim[0] +
               (unsigned)x;
    }
    // the table entry of an occupied cell (s = e = 0 when the cell holds no point)
    __device__ __forceinline__ void lookup(unsigned long long key, int &s, int &e) const {
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
    __device__ __forceinline__ void range(int x, int y, int z, int &s, int &e) const {
        const unsigned long long key = key_of(x, y, z);
        if (dense) {
            const int2 v = __ldg(&dense[key]);
            s            = v.x;
            e            = v.x + v.y;
            return;
        }
        if (occ && !((occ[key >> 5] >> (key & 31)) & 1u)) {
            s = e = 0; // empty cell: no table probe
            return;
        }
        lookup(key, s, e);
    }
};

template <class G> __device__ __forceinline__ void grid_cc(const G &g, float x, float y, float z, int c[3]) {
    c[0] = smg::coord(x, g.org[0], g.g, g.dim[0]);
    c[1] = smg::coord(y, g.org[1], g.g, g.dim[1]);
    c[2] = smg::coord(z, g.org[2], g.g, g.dim[2]);
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

// Warp minimum of a 64-bit key: the high words' minimum, then the low words' minimum among
// the lanes that hold it (two single-instruction warp reductions).
__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
    const unsigned hi = (unsigned)(v >> 32), lo = (unsigned)v;
    const unsigned mh = __reduce_min_sync(0xffffffffu, hi);
    const unsigned ml = __reduce_min_sync(0xffffffffu, hi == mh ? lo : 0xffffffffu);
    return ((unsigned long long)mh << 32) | ml;
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

// The points of the cells the lanes hold (lane: cell points [b, e) of g.pts), flattened
// over the warp by a prefix sum: visit(p, valid) is called by all lanes for each round of 32
// points (p = position with the point index in w; valid false on idle lanes) and returns a
// warp-uniform "done" that ends the rounds early.
template <class G, class V>
__device__ __forceinline__ bool warp_visit_cells(const G &g, int b, int e, V &&visit) {
    const int lane = threadIdx.x & 31;
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
        const int    bj    = __shfl_sync(0xffffffffu, b, own);
        const int    ej    = __shfl_sync(0xffffffffu, excl, own);
        const bool   valid = r < T;
        const float4 p     = valid ? g.pts[bj + (r - ej)] : make_float4(0.f, 0.f, 0.f, 0.f);
        if (visit(p, valid))
            return true;
    }
    return false;
}

// Warp-cooperative walk over the points around q, shell by shell (shells 0 and 1 together:
// the 3x3x3 block; no search can stop after shell 0, whose ring bound is 0). The lanes probe
// 32 cells at a time (occupancy bit, table) and warp_visit_cells visits their points. After
// each shell, stop(s) - evaluated by all lanes, warp-uniform - ends the walk. Every point of
// shells s0..s is visited exactly once before stop(s), so a search written on it sees the
// same points as one that walks the cells one by one. Returns false when it stopped at
// shell smax before stop() or the grid's last shell ended it.
template <class G, class V, class S>
__device__ __forceinline__ bool warp_walk(const G &g, float qx, float qy, float qz, V &&visit,
                                          S &&stop, int s0 = 1, int smax = INT_MAX) {
    const int lane = threadIdx.x & 31;
    int       c[3];
    grid_cc(g, qx, qy, qz, c);
    const int ms = max(grid_max_shell(g, c), 1);
    for (int s = s0; s <= ms; s++) {
        if (s > smax)
            return false; // the walk gave up before stop() ended it
        // shell 1 is the whole 3x3x3 block; a later shell s is its ring of 24 s^2 + 2 cells:
        // the two z faces, then the square perimeters (8 s cells) of the 2 s - 1 layers between
        const int w = 2 * s + 1, F = w * w;
        const int N = s == 1 ? 27 : 24 * s * s + 2;
        for (int t0 = 0; t0 < N; t0 += 32) {
            const int t = t0 + lane;
            int       b = 0, e = 0;
            if (t < N) {
                int dx, dy, dz;
                if (s == 1) {
                    dx = t % 3 - 1;
                    dy = (t / 3) % 3 - 1;
                    dz = t / 9 - 1;
                } else if (t < 2 * F) {
                    const int u = t < F ? t : t - F;
                    dz          = t < F ? -s : s;
                    dx          = u % w - s;
                    dy          = u / w - s;
                } else {
                    const int u = t - 2 * F, per = 8 * s;
                    dz          = u / per - (s - 1);
                    const int p = u % per, side = p / (2 * s), q = p % (2 * s);
                    dx          = side == 0 ? -s + q : side == 1 ? s : side == 2 ? s - q : -s;
                    dy          = side == 0 ? -s : side == 1 ? -s + q : side == 2 ? s : s - q;
                }
                const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                if (x >= 0 && y >= 0 && z >= 0 && x < g.dim[0] && y < g.dim[1] && z < g.dim[2])
                    g.range(x, y, z, b, e);
            }
            warp_visit_cells(g, b, e, [&](const float4 &p, bool valid) {
                visit(p, valid);
                return false;
            });
        }
        if (stop(s))
            return true;
    }
    return true; // every shell of the grid visited
}

// Lower bound of the squared distance from q to any point filed under cell (x, y, z): the
// distance to the cell's box grown by the 1% cell margin that covers the rounding of cell
// coordinates (as in ring_bound).
__device__ __forceinline__ float cell_lb2(const HGridView &g, float qx, float qy, float qz, int x,
                                          int y, int z) {
    const float q[3] = {qx, qy, qz};
    const int   k[3] = {x, y, z};
    float       s    = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float lo  = g.org[a] + ((float)k[a] - 0.01f) * g.g;
        const float hi  = g.org[a] + ((float)k[a] + 1.01f) * g.g;
        const float gap = fmaxf(0.0f, fmaxf(lo - q[a], q[a] - hi));
        s += gap * gap;
    }
    return s;
}

// Shells 0 and 1 (the 3x3x3 block around c) in one round of cell probes, cells whose lower
// bound exceeds b2 skipped. Returns visit's "done".
template <class V>
__device__ __forceinline__ bool warp_block27(const HGridView &g, float qx, float qy, float qz,
                                             const int c[3], float b2, V &&visit) {
    const int lane = threadIdx.x & 31;
    int       b = 0, e = 0;
    if (lane < 27) {
        const int x = c[0] + lane % 3 - 1, y = c[1] + (lane / 3) % 3 - 1, z = c[2] + lane / 9 - 1;
        if (x >= 0 && y >= 0 && z >= 0 && x < g.dim[0] && y < g.dim[1] && z < g.dim[2] &&
            cell_lb2(g, qx, qy, qz, x, y, z) <= b2)
            g.range(x, y, z, b, e);
    }
    return warp_visit_cells(g, b, e, visit);
}

// The cells of Chebyshev rings lo..hi around c whose lower bound does not exceed bound()
// (warp-uniform, re-read every 256 cells), visited through warp_visit_cells. The ring cube is
// screened 256 cells at a time - each lane computes 8 cells' bounds and issues their 8
// occupancy-bit loads together - and only the occupied survivors, compacted over the warp,
// are looked up in the table: a deep search costs a few rounds of independent loads instead
// of one dependent probe round per 32 cells. Returns visit's "done".
template <class B, class V>
__device__ __forceinline__ bool warp_band(const HGridView &g, float qx, float qy, float qz,
                                          const int c[3], int lo, int hi, B &&bound, V &&visit) {
    const int lane = threadIdx.x & 31;
    const int w = 2 * hi + 1, w2 = w * w, N = w2 * w;
    for (int base = 0; base < N; base += 256) {
        const float b2 = bound();
        // candidates of this lane (bit j: cell base + 32 j + lane), then their occupancy
        // (direct-table counts or bitmap bits), 8 loads in flight (both exist only for grids
        // of <= 2^28 cells, so their keys fit 32 bits)
        uint32_t m = 0, key[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const int t = base + j * 32 + lane;
            key[j]      = 0u;
            if (t < N) {
                const int tz = t / w2, ty = (t - tz * w2) / w, tx = t - tz * w2 - ty * w;
                const int dx = tx - hi, dy = ty - hi, dz = tz - hi;
                const int r  = max(abs(dx), max(abs(dy), abs(dz)));
                const int x = c[0] + dx, y = c[1] + dy, z = c[2] + dz;
                if (r >= lo && x >= 0 && y >= 0 && z >= 0 && x < g.dim[0] && y < g.dim[1] &&
                    z < g.dim[2] && cell_lb2(g, qx, qy, qz, x, y, z) <= b2) {
                    m |= 1u << j;
                    key[j] = (uint32_t)g.key_of(x, y, z);
                }
            }
        }
        if (g.dense) {
            int cnt8[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                cnt8[j] = (m >> j) & 1u ? __ldg(&g.dense[key[j]]).y : 0;
#pragma unroll
            for (int j = 0; j < 8; j++)
                m &= ~((cnt8[j] > 0 ? 0u : 1u) << j);
        } else if (g.occ) {
            uint32_t word[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                word[j] = (m >> j) & 1u ? __ldg(&g.occ[key[j] >> 5]) : 0u;
#pragma unroll
            for (int j = 0; j < 8; j++)
                m &= ~((((word[j] >> (key[j] & 31u)) & 1u) ^ 1u) << j);
        }
        const int cnt  = __popc(m);
        const int incl = warp_incl_scan(cnt);
        const int excl = incl - cnt;
        const int T    = __shfl_sync(0xffffffffu, incl, 31);
        for (int r0 = 0; r0 < T; r0 += 32) {
            const int r   = r0 + lane;
            int       own = 0; // the lane holding occupied cell r: last lane with excl <= r
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                const int mid = own + step;
                if (__shfl_sync(0xffffffffu, excl, mid) <= r)
                    own = mid;
            }
            uint32_t  om = __shfl_sync(0xffffffffu, m, own);
            const int oe = __shfl_sync(0xffffffffu, excl, own);
            int       b = 0, e = 0;
            if (r < T) {
                for (int k = r - oe; k > 0; k--)
                    om &= om - 1u;
                const int j  = __ffs(om) - 1;
                const int t  = base + j * 32 + own;
                const int tz = t / w2, ty = (t - tz * w2) / w, tx = t - tz * w2 - ty * w;
                const unsigned long long k = g.key_of(c[0] + tx - hi, c[1] + ty - hi, c[2] + tz - hi);
                if (g.dense) {
                    const int2 v = __ldg(&g.dense[k]);
                    b            = v.x;
                    e            = v.x + v.y;
                } else {
                    g.lookup(k, b, e);
                }
            }
            if (warp_visit_cells(g, b, e, visit))
                return true;
        }
    }
    return false;
}

// The last ring of the next band after ring `done`: the first ring whose bound passes b2
// (rings beyond it cannot hold a point within b2), at most 3 rings on and never past ms.
__device__ __forceinline__ int band_end(int done, int ms, float b2, float g) {
    int hi = done + 1;
    while (hi < ms && hi < done + 3) {
        const float rb = smg::ring_bound(hi, g);
        if (rb * rb > b2)
            break;
        hi++;
    }
    return hi;
}

// k nearest by a scan of every point of g, for a query whose shell walk gave up (a point
// far from the others would walk shells up to the grid's extent). The scan starts over
// (best and seen reset: each point is visited once, so the result is the same exact k
// nearest) and keeps only points within a bound on the k-th distance: the walk's k-th when
// it saw k points, else the k-th of a strided sample of the points; a merge runs only for a
// round with a point below the current k-th. It runs for few queries and is kept lean (two
// loads in flight per lane) so that the walk's register count stays as it is.
static __device__ __noinline__ void knn_scan_all(const HGridView &g, float qx, float qy, float qz, int k,
                                          unsigned long long &best, int &seen) {
    const int lane  = threadIdx.x & 31;
    unsigned  bound = 0xffffffffu; // distance bits
    auto      key_of = [&](const float4 &p) {
        const float dd = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
        return ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)__float_as_int(p.w);
    };
    if (seen >= k) {
        bound = (unsigned)(__shfl_sync(0xffffffffu, best, k - 1) >> 32);
    } else {
        const int          stride = max(1, g.m / 4096);
        unsigned long long sb     = ~0ull;
        int                ss     = 0;
        for (long long base = 0; base < g.m; base += 32ll * stride) {
            const long long          r   = base + (long long)lane * stride;
            const unsigned long long key = r < g.m ? key_of(g.pts[r]) : ~0ull;
            ss += __popc(__ballot_sync(0xffffffffu, r < g.m));
            if (__any_sync(0xffffffffu, key < __shfl_sync(0xffffffffu, sb, k - 1)))
                sb = warp_merge_low(sb, warp_bitonic_sort(key));
        }
        if (ss >= k)
            bound = (unsigned)(__shfl_sync(0xffffffffu, sb, k - 1) >> 32);
    }
    best = ~0ull;
    seen = 0;
    for (int base = 0; base < g.m; base += 64) {
        const int    r0 = base + lane, r1 = base + 32 + lane;
        const float4 p0 = r0 < g.m ? g.pts[r0] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 p1 = r1 < g.m ? g.pts[r1] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int          r   = j ? r1 : r0;
            unsigned long long key = r < g.m ? key_of(j ? p1 : p0) : ~0ull;
            if ((unsigned)(key >> 32) > bound)
                key = ~0ull;
            seen += __popc(__ballot_sync(0xffffffffu, r < g.m));
            if (__any_sync(0xffffffffu, key < __shfl_sync(0xffffffffu, best, k - 1)))
                best = warp_merge_low(best, warp_bitonic_sort(key));
        }
    }
}

// Exact k nearest neighbours (k <= 32) of q by (squared distance, index), one warp per
// query. Each round of 32 points is sorted across the lanes and merged into the running 32
// best (lane j holds the j-th smallest key: distance bits, index); rounds with no point
// below the current k-th best are skipped. The 3x3x3 block is visited in ascending cell
// lower bound, and its rounds end once the next cell's bound exceeds the k-th distance
// (no point there can enter the list, not even by the index tie-break). The search ends
// after shell s once k points were seen and the k-th distance is below the ring bound of s
// (every unvisited point is farther); further shells are walked one by one. Returns the
// number found (<= k); lane j < that count gets the j-th neighbour's index in *id and
// squared distance in *d.
__device__ __forceinline__ int warp_knn_sorted(const HGridView &g, float qx, float qy, float qz,
                                               int k, int *id, float *d) {
    const int          lane = threadIdx.x & 31;
    unsigned long long best = ~0ull; // lane j: j-th smallest so far
    int                seen = 0;
    auto               kth  = [&]() { return __shfl_sync(0xffffffffu, best, k - 1); };
    auto visit = [&](const float4 &p, bool valid) {
        seen += __popc(__ballot_sync(0xffffffffu, valid));
        unsigned long long key = ~0ull;
        if (valid) {
            const float dd = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
            key = ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)__float_as_int(p.w);
        }
        if (__any_sync(0xffffffffu, key < kth()))
            best = warp_merge_low(best, warp_bitonic_sort(key));
    };
    int c[3];
    grid_cc(g, qx, qy, qz, c);
    const int ms = max(grid_max_shell(g, c), 1);
    {
        // the block's occupied cells, sorted by lower bound (ties by lane)
        int   b = 0, e = 0;
        float lb = __int_as_float(0x7f800000);
        if (lane < 27) {
            const int x = c[0] + lane % 3 - 1, y = c[1] + (lane / 3) % 3 - 1, z = c[2] + lane / 9 - 1;
            if (x >= 0 && y >= 0 && z >= 0 && x < g.dim[0] && y < g.dim[1] && z < g.dim[2]) {
                g.range(x, y, z, b, e);
                if (e > b)
                    lb = cell_lb2(g, qx, qy, qz, x, y, z);
            }
        }
        const unsigned long long sk =
            warp_bitonic_sort(((unsigned long long)__float_as_uint(lb) << 32) | (unsigned)lane);
        const int src = (int)(sk & 31u);
        b             = __shfl_sync(0xffffffffu, b, src);
        e             = __shfl_sync(0xffffffffu, e, src);
        lb            = __uint_as_float((unsigned)(sk >> 32));
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
            const float lbr = __shfl_sync(0xffffffffu, lb, __shfl_sync(0xffffffffu, own, 0));
            if (seen >= k && lbr > __uint_as_float((unsigned)(kth() >> 32)))
                break;
            const int    bj    = __shfl_sync(0xffffffffu, b, own);
            const int    ej    = __shfl_sync(0xffffffffu, excl, own);
            const bool   valid = r < T;
            const float4 p     = valid ? g.pts[bj + (r - ej)] : make_float4(0.f, 0.f, 0.f, 0.f);
            visit(p, valid);
        }
    }
    auto done = [&](int s) {
        if (seen < k)
            return false;
        const float bnd = smg::ring_bound(s, g.g);
        return __uint_as_float((unsigned)(kth() >> 32)) < bnd * bnd;
    };
    if (!done(1) && ms >= 2 && !warp_walk(g, qx, qy, qz, visit, done, 2, kKnnMaxShell))
        knn_scan_all(g, qx, qy, qz, k, best, seen);
    const int n = min(seen, k);
    *id         = (int)(unsigned)(best & 0xffffffffu);
    *d          = __uint_as_float((unsigned)(best >> 32));
    return n;
}

// Nearest point by (squared distance, index), one warp per query: the 3x3x3 block first,
// then bands of rings (warp_band), cells screened against min(best, limit2) throughout,
// until the nearest is below the ring bound or the ring bound passes limit2. A point
// farther than limit2 may be returned (callers test the distance); -1 when none was found.
// A caller that knows a point of the grid at squared distance u from q may pass limit2 <= u:
// the nearest is then found exactly with fewer cells visited. All lanes return the result.
__device__ __forceinline__ int warp_nn_walk(const HGridView &g, float qx, float qy, float qz,
                                            float limit2, float &outd) {
    unsigned long long best  = ~0ull;
    auto               visit = [&](const float4 &p, bool valid) {
        if (valid) {
            const float dd = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
            const unsigned long long key =
                ((unsigned long long)__float_as_uint(dd) << 32) | (unsigned)__float_as_int(p.w);
            best = key < best ? key : best;
        }
        return false;
    };
    const float kInf = __int_as_float(0x7f800000);
    auto        bd   = [&]() {
        best = warp_min_u64(best);
        return best == ~0ull ? kInf : __uint_as_float((unsigned)(best >> 32));
    };
    int c[3];
    grid_cc(g, qx, qy, qz, c);
    const int ms = max(grid_max_shell(g, c), 1);
    warp_block27(g, qx, qy, qz, c, limit2, visit);
    for (int done = 1;;) {
        const float d  = bd();
        const float rb = smg::ring_bound(done, g.g);
        if (d < rb * rb || rb * rb > limit2 || done >= ms)
            break;
        const int hi = band_end(done, ms, fminf(d, limit2), g.g);
        warp_band(g, qx, qy, qz, c, done + 1, hi, [&]() { return fminf(bd(), limit2); }, visit);
        done = hi;
    }
    best = warp_min_u64(best);
    if (best == ~0ull) {
        outd = 3.402823466e+38f;
        return -1;
    }
    outd = __uint_as_float((unsigned)(best >> 32));
    return (int)(unsigned)(best & 0xffffffffu);
}

// Whether any point lies closer than sqrt(r2) to q, by a warp: cells whose lower bound
// reaches r2 are skipped, and the search ends at the first round with a hit or after the
// ring whose bound reaches sqrt(r2).
__device__ __forceinline__ bool warp_any_within(const HGridView &g, float qx, float qy, float qz,
                                                float r2) {
    bool hit   = false;
    auto visit = [&](const float4 &p, bool valid) {
        const bool h = valid && smm::dist2(qx, qy, qz, p.x, p.y, p.z) < r2;
        hit          = hit || __any_sync(0xffffffffu, h);
        return hit;
    };
    int c[3];
    grid_cc(g, qx, qy, qz, c);
    const int ms = max(grid_max_shell(g, c), 1);
    warp_block27(g, qx, qy, qz, c, r2, visit);
    for (int done = 1;;) {
        const float rb = smg::ring_bound(done, g.g);
        if (hit || rb * rb >= r2 || done >= ms)
            break;
        const int hi = band_end(done, ms, r2, g.g);
        warp_band(g, qx, qy, qz, c, done + 1, hi, [&]() { return r2; }, visit);
        done = hi;
    }
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

// Programmatic dependent launch. A kernel launched chained to the previous kernel of its
// stream (sm::launch_chained) may be scheduled while that kernel is still running; it calls
// chain_enter() before it touches memory: griddepcontrol.wait returns once the previous
// kernel has completed and its writes are visible (for an ordinary launch it returns at
// once), then launch_dependents lets the next chained kernel be scheduled. Since every
// chained kernel waits before it releases its successor, a kernel that has entered sees the
// writes of every kernel before it on the stream.
__device__ __forceinline__ void chain_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

} // namespace smd
