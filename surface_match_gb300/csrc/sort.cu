// sort.cu - stable LSD radix sort of (u32 key, u32 value) pairs on the device.
//
// Used where the reference's order has to be reproduced from a parallel build: the model
// table is grouped by key in pair order (trainModel's insertion order, ppf.cpp:125-143),
// and the reference-order sampler lists each grid cell's points in k-d-tree order. Both
// need a sort that keeps equal keys in input order.
//
// Each pass sorts by one 8-bit digit: per tile of 2048 keys a digit histogram (digit-major,
// so one exclusive scan over all tiles gives every (digit, tile) its output offset), then
// a scatter that ranks the tile's keys stably - by round, warp and lane - with
// __match_any_sync groups and per-warp digit counts in shared memory.
#include "sm_stages.h"

namespace sm {
namespace {

constexpr int kRsBs   = 256;
constexpr int kRsIpt  = 8;
constexpr int kRsTile = kRsBs * kRsIpt;
constexpr int kRsBins = 256; // == kRsBs: one digit per thread in the per-digit steps
constexpr int kRsW    = kRsBs / 32;

__global__ void __launch_bounds__(kRsBs)
    k_rs_hist(const uint32_t *__restrict__ keys, int n, int shift, int ntiles, int *__restrict__ hist) {
    __shared__ int h[kRsBins];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * kRsTile;
#pragma unroll
    for (int k = 0; k < kRsIpt; k++) {
        const int i = base + k * kRsBs + threadIdx.x;
        if (i < n)
            atomicAdd(&h[(keys[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kRsBs)
    k_rs_scatter(const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin, int n,
                 int shift, int ntiles, const int *__restrict__ off, uint32_t *__restrict__ kout,
                 uint32_t *__restrict__ vout) {
    __shared__ int run[kRsBins];       // next output slot per digit for this tile
    __shared__ int wc[kRsW][kRsBins];  // per-warp digit counts of the current round
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int base = blockIdx.x * kRsTile;
    run[tid]       = off[tid * ntiles + blockIdx.x];
    for (int k = 0; k < kRsIpt; k++) {
#pragma unroll
        for (int ww = 0; ww < kRsW; ww++)
            wc[ww][tid] = 0;
        __syncthreads();
        const int      i   = base + k * kRsBs + tid;
        const bool     ok  = i < n;
        const uint32_t key = ok ? kin[i] : 0u;
        const int      d   = (int)((key >> shift) & 255u);
        // lanes past the end form groups of their own and write nothing
        const unsigned peers = __match_any_sync(0xffffffffu, ok ? d : 0x1000 + lane);
        const int      rank  = __popc(peers & ((1u << lane) - 1u));
        if (ok && rank == 0)
            wc[w][d] = __popc(peers);
        __syncthreads();
        int pos = 0;
        if (ok) {
            int before = 0;
            for (int ww = 0; ww < w; ww++)
                before += wc[ww][d];
            pos = run[d] + before + rank;
        }
        __syncthreads();
        int s = 0;
#pragma unroll
        for (int ww = 0; ww < kRsW; ww++)
            s += wc[ww][tid];
        run[tid] += s;
        if (ok) {
            kout[pos] = key;
            vout[pos] = vin[i];
        }
        __syncthreads();
    }
}

} // namespace

void radix_sort_pairs(Ctx &c, uint32_t *keys, uint32_t *vals, int n, int bits,
                      const std::string &tag) {
    if (n <= 1 || bits <= 0)
        return;
    const int ntiles = (n + kRsTile - 1) / kRsTile;
    int      *hist   = c.arena.get<int>(tag + ".rs.hist", (size_t)kRsBins * ntiles + 1);
    int      *off    = c.arena.get<int>(tag + ".rs.off", (size_t)kRsBins * ntiles + 1);
    uint32_t *k2     = c.arena.get<uint32_t>(tag + ".rs.k", n);
    uint32_t *v2     = c.arena.get<uint32_t>(tag + ".rs.v", n);
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    for (int shift = 0; shift < bits; shift += 8) {
        k_rs_hist<<<ntiles, kRsBs, 0, c.stream>>>(ka, n, shift, ntiles, hist);
        SM_LAUNCH_CHECK();
        scan_excl(c, hist, off, (long long)kRsBins * ntiles, tag + ".rs", false);
        k_rs_scatter<<<ntiles, kRsBs, 0, c.stream>>>(ka, va, n, shift, ntiles, off, kb, vb);
        SM_LAUNCH_CHECK();
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    if (ka != keys) {
        SM_CUDA(cudaMemcpyAsync(keys, ka, (size_t)n * 4, cudaMemcpyDeviceToDevice, c.stream));
        SM_CUDA(cudaMemcpyAsync(vals, va, (size_t)n * 4, cudaMemcpyDeviceToDevice, c.stream));
    }
}

} // namespace sm
