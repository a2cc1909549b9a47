// noalloc.cu - sm_vote_stage_noalloc: the voting stage for callers that cannot allocate
// device memory.
//
// Some callers may not call cudaMalloc on their execution path: a plugin inside a host
// framework that owns and hands out all device memory itself and forbids allocation while
// its work runs, or a latency-critical loop that cannot afford cudaMalloc's implicit
// device synchronisation and unbounded latency. They can still pass their own device
// buffers for inputs and outputs. The staging this stage needs beyond those buffers
// (float4 copies of the points and normals, per-candidate pose flags, a validation flag)
// lives in one file-scope __device__ array of fixed size instead of the context's arena,
// so the call allocates nothing.
//
// The array is part of the library image: every GPU that loads the library holds its
// kScratchBytes until the process exits. All calls share it and it keeps the previous
// call's contents; everything read is rewritten (or cleared) by the call itself. Two calls
// whose GPU work overlaps (e.g. on different streams) race on it.
#include <cuda.h>

#include <mutex>

#include "sm_icp.h"
#include "sm_stages.h"

namespace sm {
namespace {

constexpr int64_t kMaxPoints    = 131072; // points per call
constexpr int64_t kMaxKeypoints = 65536;  // keypoints per call
constexpr size_t  kPosBytes     = (size_t)kMaxPoints * sizeof(float4);
constexpr size_t  kOkBytes      = (size_t)kMaxKeypoints * 3 * sizeof(int);
constexpr size_t  kScratchBytes = 2 * kPosBytes + kOkBytes + 256; // + validation words

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch, resolved with the device current and cached per device and
// CUDA context: a context created anew on the device (after cudaDeviceReset) reloads the
// module, so the address is resolved again there.
using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using MemRangeFn      = CUresult (*)(CUdeviceptr *, size_t *, CUdeviceptr);

template <class F> F driver_fn(const char *name) {
    void                           *fn = nullptr;
    cudaDriverEntryPointQueryResult q  = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion(name, &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (F)fn;
}

std::mutex g_mu;
struct ScratchAddr {
    CUcontext ctx  = nullptr;
    void     *addr = nullptr;
};
ScratchAddr g_addr[256];

void *scratch_address(int device) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (device < 0 || device >= 256)
        throw Error(SM_ERR_ARG, "device ordinal out of range");
    static CtxGetCurrentFn ctxCurrent = driver_fn<CtxGetCurrentFn>("cuCtxGetCurrent");
    CUcontext              cur        = nullptr;
    if (ctxCurrent)
        ctxCurrent(&cur);
    ScratchAddr &a = g_addr[device];
    if (!a.addr || a.ctx != cur) {
        void       *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess)
            throw Error(SM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                         cudaGetErrorString(e));
        a.addr = p;
        a.ctx  = cur;
    }
    return a.addr;
}

// Bytes from p to the end of the device allocation that holds it, or -1 when the driver
// cannot tell (the check is then skipped).
long long bytes_to_allocation_end(const void *p) {
    static MemRangeFn range = driver_fn<MemRangeFn>("cuMemGetAddressRange");
    if (!range)
        return -1;
    CUdeviceptr base = 0;
    size_t      size = 0;
    if (range(&base, &size, (CUdeviceptr)p) != CUDA_SUCCESS)
        return -1;
    return (long long)(base + size - (CUdeviceptr)p);
}

__global__ void k_stage_points(const float *__restrict__ p, const float *__restrict__ q, int n,
                               float4 *__restrict__ P, float4 *__restrict__ Q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    P[i] = make_float4(p[3 * (size_t)i], p[3 * (size_t)i + 1], p[3 * (size_t)i + 2], 0.0f);
    Q[i] = make_float4(q[3 * (size_t)i], q[3 * (size_t)i + 1], q[3 * (size_t)i + 2], 0.0f);
}

// Validation of the caller's index arrays before anything reads points through them.
// Step 1: keypoints in range, off[0] == 0, offsets non-decreasing, no list longer than n
// (a radius search lists a point at most once); bad[1] receives off[K] for the host.
// `bad` is cleared by the host before the launch.
__global__ void k_check_indices(const int *__restrict__ kp, int K, const int *__restrict__ off,
                                int n, int *__restrict__ bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t == 0) {
        if (off[0] != 0)
            atomicExch(bad, 1);
        bad[1] = off[K];
    }
    for (int c = t; c < K; c += gridDim.x * blockDim.x) {
        const int len = off[c + 1] - off[c];
        if (kp[c] < 0 || kp[c] >= n || len < 0 || len > n)
            atomicExch(bad, 1);
    }
}

// Step 2, launched only after the host has seen step 1 pass and checked `total` = off[K]
// against the ids allocation: every listed id in range.
__global__ void k_check_ids(int total, const int *__restrict__ ids, int n, int *__restrict__ bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        if (ids[i] < 0 || ids[i] >= n)
            atomicExch(bad, 1);
}

// Zero the pose slots the stage did not emit (the layout sm_vote_stage returns).
__global__ void k_clear_unemitted(const int *__restrict__ ok, int slots, float *__restrict__ poses) {
    const int i = blockIdx.x;
    if (i >= slots || ok[i])
        return;
    for (int e = threadIdx.x; e < smi::kPoseFloats; e += blockDim.x)
        poses[(size_t)i * smi::kPoseFloats + e] = 0.0f;
}

} // namespace
} // namespace sm

extern "C" SM_API int sm_vote_stage_noalloc(sm_model m, const float *points, const float *normals,
                                            int64_t n, const int32_t *kp, int64_t K,
                                            const int32_t *nbrOff, const int32_t *nbrIds,
                                            float minScore, int64_t *outStats, float *outCands,
                                            float *outPoses, int dumpK, int32_t *outAcc) {
    using namespace sm;
    return run_guarded([&] {
        if (!m || !points || !normals || !kp || !nbrOff || !nbrIds || !outStats || !outCands ||
            !outPoses)
            throw Error(SM_ERR_ARG, "NULL argument");
        if (n < 1 || n > kMaxPoints)
            throw Error(SM_ERR_CAPACITY, "sm_vote_stage_noalloc: n = " + std::to_string(n) +
                                             " points, the fixed scratch holds 1.." +
                                             std::to_string(kMaxPoints));
        if (K < 1 || K > kMaxKeypoints)
            throw Error(SM_ERR_CAPACITY, "sm_vote_stage_noalloc: K = " + std::to_string(K) +
                                             " keypoints, the fixed scratch holds 1.." +
                                             std::to_string(kMaxKeypoints));
        Model &M = *model_core(m);
        Ctx   &c = *model_ctx(m);
        if (!M.trained)
            throw Error(SM_ERR_RUNTIME, "No trained model in matchScene");
        if (dumpK > 0 && !outAcc)
            throw Error(SM_ERR_ARG, "dump_k > 0 needs out_acc");
        SM_CUDA(cudaSetDevice(M.device));
        unsigned char *base = (unsigned char *)scratch_address(M.device);
        float4        *P    = (float4 *)base;
        float4        *N    = (float4 *)(base + kPosBytes);
        int           *ok   = (int *)(base + 2 * kPosBytes);
        int           *bad  = (int *)(base + 2 * kPosBytes + kOkBytes);
        const int      ni = (int)n, Ki = (int)K;
        int *hostBad = c.hostCounts + 48; // pinned scratch of the context
        SM_CUDA(cudaMemsetAsync(bad, 0, 2 * sizeof(int), c.stream));
        k_check_indices<<<nblocks(Ki, 256), 256, 0, c.stream>>>(kp, Ki, nbrOff, ni, bad);
        SM_LAUNCH_CHECK();
        SM_CUDA(cudaMemcpyAsync(hostBad, bad, 2 * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
        SM_CUDA(cudaStreamSynchronize(c.stream));
        if (hostBad[0])
            throw Error(SM_ERR_ARG, "keypoint index out of range, or neighbour offsets not starting "
                                    "at 0, decreasing or listing more than n points");
        const int       total = hostBad[1];
        const long long room  = bytes_to_allocation_end(nbrIds);
        if (room >= 0 && (long long)total * (long long)sizeof(int32_t) > room)
            throw Error(SM_ERR_ARG, "nbr_off[K] = " + std::to_string(total) +
                                        " entries run past the end of the allocation holding nbr_ids");
        if (total > 0) {
            k_check_ids<<<152 * 4, 256, 0, c.stream>>>(total, nbrIds, ni, bad);
            SM_LAUNCH_CHECK();
            SM_CUDA(cudaMemcpyAsync(hostBad, bad, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            SM_CUDA(cudaStreamSynchronize(c.stream));
            if (hostBad[0])
                throw Error(SM_ERR_ARG, "neighbour index out of range");
        }
        k_stage_points<<<nblocks(ni, 256), 256, 0, c.stream>>>(points, normals, ni, P, N);
        SM_LAUNCH_CHECK();
        const int dk = std::max(0, std::min(dumpK, Ki));
        if (dk)
            SM_CUDA(cudaMemsetAsync(outAcc, 0,
                                    (size_t)dk * M.ns * M.tp.featAngleResolution * sizeof(int),
                                    c.stream));
        VoteOut vo;
        vo.stats  = (long long *)outStats;
        vo.cands  = outCands;
        vo.poses  = outPoses;
        vo.poseOk = ok;
        vo.acc    = dk ? outAcc : nullptr;
        vote_fused(c, M, P, N, kp, Ki, nbrOff, nbrIds, minScore, vo, dk);
        k_clear_unemitted<<<Ki * 3, 32, 0, c.stream>>>(ok, Ki * 3, outPoses);
        SM_LAUNCH_CHECK();
        SM_CUDA(cudaStreamSynchronize(c.stream));
    });
}
