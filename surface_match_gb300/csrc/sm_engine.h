// sm_engine.h - host-side engine types shared by the CUDA translation units: errors,
// the device arena, grids, the model and the per-context match state.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/surface_match.h"
#include "sm_device.cuh"

namespace sm {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define SM_CUDA(x)                                                                             \
    do {                                                                                       \
        cudaError_t e_ = (x);                                                                  \
        if (e_ != cudaSuccess)                                                                 \
            throw ::sm::Error(SM_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_));   \
    } while (0)

// Kernel launches issued by the library (all contexts); read by sm_launch_count().
extern long long g_launches;
#define SM_LAUNCH_CHECK()                                                                      \
    do {                                                                                       \
        __atomic_add_fetch(&::sm::g_launches, 1, __ATOMIC_RELAXED);                            \
        SM_CUDA(cudaGetLastError());                                                           \
    } while (0)

inline int nblocks(long long n, int bs) { return (int)((n + bs - 1) / bs); }

// Device buffers by name, grown on demand and reused across calls. With a stream set, a
// buffer grows by stream-ordered free + allocation on that stream (the device's default
// memory pool, which keeps freed memory for reuse), so that growing one context's
// workspace never waits for the work of other contexts on the device.
class Arena {
public:
    ~Arena() { release(); }
    void set_stream(cudaStream_t s, int device) {
        stream_ = s;
        keep_pool_memory(device);
    }
    void *get(const std::string &name, size_t bytes) {
        if (bytes == 0)
            bytes = 16;
        auto it = slots_.find(name);
        if (it != slots_.end() && it->second.second >= bytes)
            return it->second.first;
        if (it != slots_.end()) {
            if (stream_)
                cudaFreeAsync(it->second.first, stream_);
            else
                cudaFree(it->second.first);
            slots_.erase(it);
        }
        size_t      cap = bytes + bytes / 4;
        void       *p   = nullptr;
        cudaError_t e   = stream_ ? cudaMallocAsync(&p, cap, stream_) : cudaMalloc(&p, cap);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(SM_ERR_NOMEM, "device allocation of " + std::to_string(cap) +
                                          " bytes failed for " + name);
        }
        slots_[name] = {p, cap};
        return p;
    }
    template <class T> T *get(const std::string &name, size_t count) {
        return (T *)get(name, count * sizeof(T));
    }
    size_t bytes() const {
        size_t s = 0;
        for (auto &kv : slots_)
            s += kv.second.second;
        return s;
    }
    // frees everything (synchronising: the stream may be gone by then)
    void release() {
        for (auto &kv : slots_)
            cudaFree(kv.second.first);
        slots_.clear();
    }

private:
    static void keep_pool_memory(int device) {
        static std::mutex mu;
        static std::vector<int> done;
        std::lock_guard<std::mutex> lk(mu);
        for (int d : done)
            if (d == device)
                return;
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t keep = ~0ull;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
        done.push_back(device);
    }
    cudaStream_t                                     stream_ = nullptr;
    std::map<std::string, std::pair<void *, size_t>> slots_;
};

// A hashed grid built on the device over a subset of points (see smd::HGridView).
struct HGrid {
    float     org[3] = {0, 0, 0};
    float     g      = 1;
    int       dim[3] = {1, 1, 1};
    uint4    *slot   = nullptr;
    uint32_t  mask   = 0;
    int      *ids    = nullptr;
    float4   *pts    = nullptr; // positions in cell order, point index in w (bit pattern)
    uint32_t *occ    = nullptr; // occupancy bit per cell (nullptr when the cell box is too large)
    int2     *dense  = nullptr; // {first, count} per cell (nullptr unless the cell box is small)
    int       m      = 0;
    smd::HGridView view() const {
        smd::HGridView v;
        for (int a = 0; a < 3; a++) {
            v.org[a] = org[a];
            v.dim[a] = dim[a];
        }
        v.g    = g;
        v.slot = slot;
        v.mask = mask;
        v.ids  = ids;
        v.pts  = pts;
        v.occ   = occ;
        v.dense = dense;
        v.m     = m;
        return v;
    }
};

struct Box {
    float mn[3], mx[3];
    float ext(int a) const { return mx[a] - mn[a]; }
    // Eigen norm order of the box size: x*x + (y*y + z*z)
    float diameter() const {
        const float x = ext(0), y = ext(1), z = ext(2);
        return smm::fsqrt(x * x + (y * y + z * z));
    }
};

// A trained model resident on the device.
struct Model {
    int            device = 0;
    bool           trained = false;
    int            order   = SM_ORDER_GRID; // search order of train and match
    float          sdRel   = 0.04f;
    sm_train_param tp{};
    Box            box{};
    int            ns = 0, nr = 0, nkeys = 0;
    long long      nentries = 0;
    // device copies
    float4   *sp = nullptr, *sn = nullptr, *rp = nullptr, *rn = nullptr;
    uint32_t *hkeys = nullptr;  // open-addressed table keys (EMPTY = 0xffffffff sentinel slot)
    uint32_t *hslot = nullptr;  // bucket index per table slot
    uint32_t  hmask = 0;        // table size - 1 (power of two)
    uint32_t  emptyKeySlot = 0xffffffffu; // bucket of key 0xffffffff if present
    uint32_t *boff  = nullptr;  // bucket offsets (nkeys + 1)
    uint2    *entries = nullptr; // (ref, alpha bits) in bucket order
    uint32_t *dkeys   = nullptr; // bucket keys, ascending (nkeys)
    uint32_t *doffs   = nullptr; // bucket offsets (nkeys + 1)
    // host copies for download / save, fetched from the device on first use after a train
    bool                  hostValid = false;
    std::vector<float>    h_sp, h_sn, h_rp, h_rn;
    std::vector<uint32_t> h_keys, h_offs, h_refs;
    std::vector<float>    h_alphas;
    void free_device();
    void ensure_host();
};

} // namespace sm
