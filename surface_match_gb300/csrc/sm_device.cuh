// sm_device.cuh - device-side building blocks of the matching path: grid views and exact
// grid searches, ordered float atomics, warp/block helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sm_grid.h"
#include "sm_math.h"

namespace smd {

constexpr int kMaxKnn = 32; // largest supported knnNormal

// Device view of a uniform grid over a subset of points: cells are stored cell-major as a
// CSR (start[cell] .. start[cell+1] into ids).
struct GridView {
    float      org[3];
    float      g;
    int        dim[3];
    const int *start;
    const int *ids;
};

__device__ __forceinline__ void grid_cc(const GridView &G, float x, float y, float z, int c[3]) {
    c[0] = smg::coord(x, G.org[0], G.g, G.dim[0]);
    c[1] = smg::coord(y, G.org[1], G.g, G.dim[1]);
    c[2] = smg::coord(z, G.org[2], G.g, G.dim[2]);
}

__device__ __forceinline__ int grid_cell(const GridView &G, int x, int y, int z) {
    return (z * G.dim[1] + y) * G.dim[0] + x;
}

__device__ __forceinline__ int grid_max_shell(const GridView &G, const int c[3]) {
    int m = 0;
    for (int a = 0; a < 3; a++) {
        const int lo = c[a], hi = G.dim[a] - 1 - c[a];
        m          = max(m, max(lo, hi));
    }
    return m;
}

// Visit every point of the cells at Chebyshev distance exactly s from cell c.
template <class F>
__device__ __forceinline__ void grid_shell(const GridView &G, const int c[3], int s, F &&f) {
    const int z0 = max(c[2] - s, 0), z1 = min(c[2] + s, G.dim[2] - 1);
    const int y0 = max(c[1] - s, 0), y1 = min(c[1] + s, G.dim[1] - 1);
    for (int z = z0; z <= z1; z++) {
        for (int y = y0; y <= y1; y++) {
            const bool face = (z == c[2] - s || z == c[2] + s || y == c[1] - s || y == c[1] + s);
            const int  step = face ? 1 : 2 * s;
            for (int x = c[0] - s; x <= c[0] + s; x += (step > 0 ? step : 1)) {
                if (x < 0 || x >= G.dim[0])
                    continue;
                const int cell = grid_cell(G, x, y, z);
                const int e    = G.start[cell + 1];
                for (int k = G.start[cell]; k < e; k++)
                    f(G.ids[k]);
            }
        }
    }
}

// k nearest neighbours of q by (squared distance, index); returns how many were found.
__device__ __forceinline__ int grid_knn(const GridView &G, const float4 *__restrict__ pos,
                                        float qx, float qy, float qz, int k, int *oi,
                                        float *od) {
    int c[3];
    grid_cc(G, qx, qy, qz, c);
    int       n  = 0;
    const int ms = grid_max_shell(G, c);
    for (int s = 0; s <= ms; s++) {
        grid_shell(G, c, s, [&](int id) {
            const float4 p = pos[id];
            const float  d = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
            if (n == k && !(d < od[k - 1] || (d == od[k - 1] && id < oi[k - 1])))
                return;
            int i = (n < k) ? n++ : k - 1;
            while (i > 0 && (od[i - 1] > d || (od[i - 1] == d && oi[i - 1] > id))) {
                od[i] = od[i - 1];
                oi[i] = oi[i - 1];
                i--;
            }
            od[i] = d;
            oi[i] = id;
        });
        const float b = smg::ring_bound(s, G.g);
        if (n == k && od[k - 1] < b * b)
            break;
    }
    return n;
}

// Nearest neighbour by (squared distance, index), searched until the ring bound passes
// `limit2`; returns -1 when the grid is empty.
__device__ __forceinline__ int grid_nn(const GridView &G, const float4 *__restrict__ pos,
                                       float qx, float qy, float qz, float limit2, float &outd) {
    int c[3];
    grid_cc(G, qx, qy, qz, c);
    int       best = -1;
    float     bd   = 3.402823466e+38f;
    const int ms   = grid_max_shell(G, c);
    for (int s = 0; s <= ms; s++) {
        grid_shell(G, c, s, [&](int id) {
            const float4 p = pos[id];
            const float  d = smm::dist2(qx, qy, qz, p.x, p.y, p.z);
            if (d < bd || (d == bd && id < best)) {
                bd   = d;
                best = id;
            }
        });
        const float b = smg::ring_bound(s, G.g);
        if (best >= 0 && bd < b * b)
            break;
        if (b * b > limit2)
            break;
    }
    outd = bd;
    return best;
}

__device__ __forceinline__ bool grid_any_within(const GridView &G, const float4 *__restrict__ pos,
                                                float qx, float qy, float qz, float r2) {
    int c[3];
    grid_cc(G, qx, qy, qz, c);
    const int ms = grid_max_shell(G, c);
    for (int s = 0; s <= ms; s++) {
        bool hit = false;
        grid_shell(G, c, s, [&](int id) {
            if (hit)
                return;
            const float4 p = pos[id];
            if (smm::dist2(qx, qy, qz, p.x, p.y, p.z) < r2)
                hit = true;
        });
        if (hit)
            return true;
        const float b = smg::ring_bound(s, G.g);
        if (b * b >= r2)
            break;
    }
    return false;
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
