// server.cu - serving loop for matchScene requests: resident models, admission by an HBM
// budget, continuous batching.
//
// Requests are queued in arrival order. `slots` worker threads, each with its own
// context (CUDA stream + workspace), take the oldest request as soon as a slot is free and
// the request's estimated device footprint fits the budget next to those in flight; the
// work of all admitted requests overlaps on the GPU. A request arriving while others run
// is admitted as soon as a slot and memory free up - there is no batch boundary to wait
// for. Models stay resident in their sm_model handles; a request only carries its scene.
// Each request's result is exactly what sm_match returns for it alone (same kernels, same
// arithmetic, private workspace).
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <vector>

#include "sm_stages.h"

namespace sm {
namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t             id;
    sm_model            model;
    std::vector<float>  xyz, nrm;
    const float        *devXyz = nullptr, *devNrm = nullptr; // caller-owned device inputs
    int64_t             n;
    bool                hasNrm, hasVp;
    float               vp[3];
    float               sdRel, kpFrac, minScore;
    sm_match_param      mp;
    int64_t             bytes;
    Clock::time_point   tSubmit;
};

struct Done {
    int64_t            id;
    int                status;
    std::vector<float> pose, score;
    double             queueMs, serviceMs, totalMs;
};

} // namespace
} // namespace sm

struct sm_server_s {
    int                      device;
    int                      slots;
    int64_t                  budget;
    int64_t                  inFlightBytes = 0, peakBytes = 0;
    int64_t                  running = 0, completed = 0;
    std::mutex               mu;
    std::condition_variable  cvWork, cvDone;
    std::deque<sm::Req>      pending;
    std::deque<sm::Done>     done;
    std::vector<std::thread> workers;
    bool                     stop   = false;
    int64_t                  nextId = 1;
};

namespace sm {
namespace {

// Device footprint estimate of a scene of n points: the match workspace (point arrays,
// grids, neighbour lists, refinement scratch) grows about linearly in n.
constexpr int64_t kBytesPerPoint = 512;
constexpr int64_t kBytesFixed    = 64ll << 20;

int64_t estimate_bytes(int64_t n) { return kBytesFixed + kBytesPerPoint * n; }

void worker(sm_server_s *s) {
    std::unique_ptr<Ctx> c;
    try {
        SM_CUDA(cudaSetDevice(s->device));
        c = acquire_worker(s->device);
    } catch (const std::exception &) {
        return;
    }
    for (;;) {
        Req r;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cvWork.wait(lk, [&] {
                if (s->stop)
                    return true;
                if (s->pending.empty())
                    return false;
                const int64_t b = s->pending.front().bytes;
                return s->inFlightBytes + b <= s->budget || s->running == 0;
            });
            if (s->stop && s->pending.empty())
                break;
            if (s->pending.empty())
                continue;
            r = std::move(s->pending.front());
            s->pending.pop_front();
            s->inFlightBytes += r.bytes;
            s->peakBytes = std::max(s->peakBytes, s->inFlightBytes);
            s->running++;
        }
        const Clock::time_point t0 = Clock::now();
        Done d;
        d.id     = r.id;
        d.status = SM_OK;
        try {
            match_into(*c, *model_core(r.model), r.devXyz ? r.devXyz : r.xyz.data(),
                       r.devNrm ? r.devNrm : (r.hasNrm ? r.nrm.data() : nullptr), r.n,
                       r.hasVp ? r.vp : nullptr, r.sdRel, r.kpFrac, r.minScore, r.mp, d.pose,
                       d.score, nullptr);
        } catch (const Error &e) {
            d.status = e.code;
        } catch (const std::exception &) {
            d.status = SM_ERR_RUNTIME;
        }
        const Clock::time_point t1 = Clock::now();
        d.queueMs   = std::chrono::duration<double, std::milli>(t0 - r.tSubmit).count();
        d.serviceMs = std::chrono::duration<double, std::milli>(t1 - t0).count();
        d.totalMs   = std::chrono::duration<double, std::milli>(t1 - r.tSubmit).count();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->inFlightBytes -= r.bytes;
            s->running--;
            s->completed++;
            s->done.push_back(std::move(d));
        }
        s->cvWork.notify_all();
        s->cvDone.notify_all();
    }
    release_worker(s->device, std::move(c));
}

bool device_pointer(const void *p) {
    if (!p)
        return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

} // namespace
} // namespace sm

using namespace sm;

extern "C" {

SM_API int sm_server_create(int device, int slots, int64_t budget, sm_server *out) {
    return run_guarded([&] {
        if (!out || slots < 1 || budget <= 0)
            throw Error(SM_ERR_ARG, "invalid server arguments");
        int ndev = 0;
        SM_CUDA(cudaGetDeviceCount(&ndev));
        if (device < 0 || device >= ndev || device >= 64)
            throw Error(SM_ERR_ARG, "no CUDA device " + std::to_string(device));
        auto *s   = new sm_server_s();
        s->device = device;
        s->slots  = slots;
        s->budget = budget;
        for (int i = 0; i < slots; i++)
            s->workers.emplace_back(worker, s);
        *out = s;
    });
}

SM_API int sm_server_destroy(sm_server s) {
    return run_guarded([&] {
        if (!s)
            return;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stop = true;
        }
        s->cvWork.notify_all();
        for (auto &t : s->workers)
            t.join();
        delete s;
    });
}

SM_API int sm_server_submit(sm_server s, sm_model model, const float *xyz, const float *normal,
                            int64_t n, const float *viewpoint, float sdRel, float kpFrac,
                            float minScore, const sm_match_param *param, int64_t *outId) {
    return run_guarded([&] {
        if (!s || !model || !xyz || n <= 0)
            throw Error(SM_ERR_ARG, "invalid request");
        if (model_core(model)->device != s->device)
            throw Error(SM_ERR_ARG, "model and server live on different devices");
        Req r;
        r.model = model;
        r.n     = n;
        // each input on its own: device arrays are read in place when the request runs (the
        // caller keeps them alive until it is polled), host arrays are copied now
        if (device_pointer(xyz))
            r.devXyz = xyz;
        else
            r.xyz.assign(xyz, xyz + n * 3);
        if (normal && device_pointer(normal))
            r.devNrm = normal;
        else if (normal)
            r.nrm.assign(normal, normal + n * 3);
        r.hasNrm = normal != nullptr;
        r.hasVp  = viewpoint != nullptr;
        if (viewpoint)
            memcpy(r.vp, viewpoint, sizeof(r.vp));
        r.sdRel    = sdRel;
        r.kpFrac   = kpFrac;
        r.minScore = minScore;
        sm_match_param_default(&r.mp);
        if (param)
            r.mp = *param;
        r.bytes   = estimate_bytes(n);
        r.tSubmit = Clock::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            r.id = s->nextId++;
            if (outId)
                *outId = r.id;
            s->pending.push_back(std::move(r));
        }
        s->cvWork.notify_one();
    });
}

SM_API int sm_server_poll(sm_server s, int maxRequests, int maxResults, int waitMs, int64_t *ids,
                          int *status, int *counts, float *poses, float *scores, double *timesMs,
                          int *nOut) {
    return run_guarded([&] {
        if (!s || !nOut || maxRequests < 0 || maxResults < 0)
            throw Error(SM_ERR_ARG, "invalid poll arguments");
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->done.empty() && waitMs > 0)
            s->cvDone.wait_for(lk, std::chrono::milliseconds(waitMs),
                               [&] { return !s->done.empty(); });
        int k = 0;
        while (k < maxRequests && !s->done.empty()) {
            Done d = std::move(s->done.front());
            s->done.pop_front();
            if (ids)
                ids[k] = d.id;
            if (status)
                status[k] = d.status;
            const int nres = (int)d.score.size();
            if (counts)
                counts[k] = nres;
            for (int i = 0; i < nres && i < maxResults; i++) {
                if (poses) {
                    float *P = poses + ((size_t)k * maxResults + i) * 16;
                    for (int e = 0; e < 12; e++)
                        P[e] = d.pose[(size_t)i * 12 + e];
                    P[12] = P[13] = P[14] = 0.0f;
                    P[15]                 = 1.0f;
                }
                if (scores)
                    scores[(size_t)k * maxResults + i] = d.score[i];
            }
            if (timesMs) {
                timesMs[3 * k]     = d.queueMs;
                timesMs[3 * k + 1] = d.serviceMs;
                timesMs[3 * k + 2] = d.totalMs;
            }
            k++;
        }
        *nOut = k;
    });
}

SM_API int sm_server_status(sm_server s, int64_t *out6) {
    return run_guarded([&] {
        if (!s || !out6)
            throw Error(SM_ERR_ARG, "NULL argument");
        std::lock_guard<std::mutex> lk(s->mu);
        out6[0] = (int64_t)s->pending.size();
        out6[1] = s->running;
        out6[2] = s->completed;
        out6[3] = s->inFlightBytes;
        out6[4] = s->peakBytes;
        out6[5] = s->budget;
    });
}

} // extern "C"
