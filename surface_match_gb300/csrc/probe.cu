// probe.cu - a measured device rate that the vote stage's roofline is quoted against.
//
// The vote accumulation (ppf.cpp:342-346 on the CPU) is bound by shared-memory atomic
// increments at data-dependent cells, a rate no vendor figure gives for this access
// pattern. It is measured here with a kernel shaped like the vote kernel: 512-thread CTAs,
// two per SM, a 48 KB accumulator of 16-bit counters (two per 32-bit word), one atomic
// increment per vote at a pseudo-random cell, several waves of CTAs.
#include "sm_stages.h"

namespace sm {
namespace {

constexpr int kPbBs    = 512;
constexpr int kPbIters = 2048; // increments per thread
constexpr int kPbCells = 24576; // 48 KB of 16-bit counters

__global__ void __launch_bounds__(kPbBs, 2) k_probe_vote_atomics(uint32_t seed, unsigned *sink) {
    extern __shared__ uint32_t acc[];
    constexpr int words = kPbCells / 2;
    for (int i = threadIdx.x; i < words; i += blockDim.x)
        acc[i] = 0u;
    __syncthreads();
    uint32_t x = seed ^ (blockIdx.x * 0x9E3779B9u) ^ (threadIdx.x * 0x85EBCA6Bu);
    for (int it = 0; it < kPbIters; it += 8) {
#pragma unroll
        for (int u = 0; u < 8; u++) {
            x                = x * 1664525u + 1013904223u; // LCG (Numerical Recipes constants)
            const uint32_t c = (uint32_t)(((unsigned long long)(x >> 8) * kPbCells) >> 24);
            atomicAdd(&acc[c >> 1], 1u << ((c & 1u) * 16u));
        }
    }
    __syncthreads();
    unsigned s = 0; // keeps the increments observable
    for (int i = threadIdx.x; i < words; i += blockDim.x)
        s += acc[i];
    if (s == 0x9E3779B9u)
        sink[0] = s;
}

} // namespace
} // namespace sm

using namespace sm;

extern "C" SM_API int sm_probe_vote_atomics(int device, double *atomics_per_second) {
    return run_guarded([&] {
        if (!atomics_per_second)
            throw Error(SM_ERR_ARG, "NULL output");
        SM_CUDA(cudaSetDevice(device));
        int sms = 0;
        SM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        const size_t smem = (size_t)kPbCells / 2 * sizeof(uint32_t);
        SM_CUDA(cudaFuncSetAttribute(k_probe_vote_atomics,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        cudaStream_t st;
        SM_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        unsigned   *sink = nullptr;
        cudaEvent_t e0, e1;
        SM_CUDA(cudaMalloc(&sink, sizeof(unsigned)));
        SM_CUDA(cudaEventCreate(&e0));
        SM_CUDA(cudaEventCreate(&e1));
        const int grid = sms * 2 * 8; // eight waves of two CTAs per SM
        float     best = 0.0f;
        for (int rep = 0; rep < 4; rep++) { // the first run warms up; the fastest counts
            SM_CUDA(cudaEventRecord(e0, st));
            k_probe_vote_atomics<<<grid, kPbBs, smem, st>>>(0x2545F491u + rep, sink);
            SM_LAUNCH_CHECK();
            SM_CUDA(cudaEventRecord(e1, st));
            SM_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            SM_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0 && (best == 0.0f || ms < best))
                best = ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(sink);
        cudaStreamDestroy(st);
        *atomics_per_second = (double)grid * kPbBs * kPbIters / (best * 1e-3);
    });
}
