// batch.cu - sm_match_batch: many (scene, model) matching jobs of uneven size at once.
//
// Each job is the same matchScene as sm_match. A pool of worker contexts per device (each
// its own non-blocking CUDA stream and workspace, reused across calls) pulls jobs from a
// shared counter; every worker drives its job's launches on its stream from its own host
// thread, so the kernels of different scenes overlap on the GPU and a worker that finishes
// a small scene immediately takes the next one. Models are read-only device tables shared
// by all workers. Results per job are the ones sm_match returns for it.
#include <atomic>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "sm_stages.h"

namespace sm {

namespace {

struct Pool {
    std::mutex                        mu;
    std::vector<std::unique_ptr<Ctx>> free;
};
// Worker contexts stay alive for the process (never destroyed at exit, where the CUDA
// runtime may already be torn down).
Pool *const g_pools = new Pool[64];

} // namespace

std::unique_ptr<Ctx> acquire_worker(int device) {
    Pool &p = g_pools[device];
    {
        std::lock_guard<std::mutex> lk(p.mu);
        if (!p.free.empty()) {
            auto c = std::move(p.free.back());
            p.free.pop_back();
            return c;
        }
    }
    std::unique_ptr<Ctx> c(new Ctx());
    c->device = device;
    SM_CUDA(cudaSetDevice(device));
    SM_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    c->ownStream = true;
    SM_CUDA(cudaMallocHost((void **)&c->hostCounts, 64 * sizeof(int)));
    for (auto &e : c->ev)
        SM_CUDA(cudaEventCreate(&e));
    c->arena.set_stream(c->stream, device);
    c->chain = false; // many workers share the device (see launch_chained)
    return c;
}

void release_worker(int device, std::unique_ptr<Ctx> c) {
    Pool                       &p = g_pools[device];
    std::lock_guard<std::mutex> lk(p.mu);
    p.free.push_back(std::move(c));
}

} // namespace sm

using namespace sm;

extern "C" SM_API int sm_match_batch(int njobs, const sm_model *models, const float *const *xyz,
                                     const float *const *normals, const int64_t *n,
                                     const float *viewpoints, float sdRel, float kpFrac,
                                     float minScore, const sm_match_param *param, int maxResults,
                                     float *outPose, float *outScore, int *outCount,
                                     int *outStatus, int concurrency, sm_match_stats *stats) {
    return run_guarded([&] {
        if (njobs < 0 || (njobs > 0 && (!models || !xyz || !n || !outCount)) || maxResults < 0)
            throw Error(SM_ERR_ARG, "invalid batch arguments");
        if (njobs == 0)
            return;
        sm_match_param mp;
        sm_match_param_default(&mp);
        if (param)
            mp = *param;
        for (int j = 0; j < njobs; j++)
            if (!models[j])
                throw Error(SM_ERR_ARG, "NULL model in batch");
        const int device = model_core(models[0])->device;
        for (int j = 0; j < njobs; j++)
            if (model_core(models[j])->device != device)
                throw Error(SM_ERR_ARG, "all models of a batch must live on one device");
        if (device < 0 || device >= 64)
            throw Error(SM_ERR_ARG, "device ordinal out of range");
        const int         workers = std::max(1, std::min(concurrency, njobs));
        std::atomic<int>  next{0};
        std::vector<int>  status(njobs, SM_OK);
        std::vector<std::string> errors(njobs);
        std::vector<std::thread> threads;
        auto body = [&]() {
            std::unique_ptr<Ctx> c;
            try {
                SM_CUDA(cudaSetDevice(device));
                c = acquire_worker(device);
            } catch (const std::exception &) {
                // no context: the remaining jobs go to the threads that have one (or are
                // reported as never taken below); nothing may escape the thread
                return;
            }
            for (int j = next++; j < njobs; j = next++) {
                try {
                    std::vector<float> pose, score;
                    match_into(*c, *model_core(models[j]), xyz[j], normals ? normals[j] : nullptr,
                               n[j], viewpoints ? viewpoints + 3 * (size_t)j : nullptr, sdRel,
                               kpFrac, minScore, mp, pose, score, stats ? stats + j : nullptr);
                    const int k = (int)score.size();
                    outCount[j] = k;
                    for (int i = 0; i < k && i < maxResults; i++) {
                        if (outPose) {
                            float *P = outPose + ((size_t)j * maxResults + i) * 16;
                            for (int e = 0; e < 12; e++)
                                P[e] = pose[(size_t)i * 12 + e];
                            P[12] = P[13] = P[14] = 0.0f;
                            P[15]                 = 1.0f;
                        }
                        if (outScore)
                            outScore[(size_t)j * maxResults + i] = score[i];
                    }
                    if (k > maxResults) {
                        status[j] = SM_ERR_CAPACITY;
                        errors[j] = "more results than max_results";
                    }
                } catch (const Error &e) {
                    status[j] = e.code;
                    errors[j] = e.what();
                    outCount[j] = 0;
                } catch (const std::exception &e) {
                    status[j] = SM_ERR_RUNTIME;
                    errors[j] = e.what();
                    outCount[j] = 0;
                }
            }
            release_worker(device, std::move(c));
        };
        for (int w = 0; w < workers; w++)
            threads.emplace_back(body);
        for (auto &t : threads)
            t.join();
        int first = SM_OK;
        std::string msg;
        for (int j = 0; j < njobs; j++) {
            if (next.load() <= j && status[j] == SM_OK) { // never taken: no worker context
                status[j] = SM_ERR_NOMEM;
                errors[j] = "no worker context could be created";
            }
            if (outStatus)
                outStatus[j] = status[j];
            if (status[j] != SM_OK && first == SM_OK) {
                first = status[j];
                msg   = "job " + std::to_string(j) + ": " + errors[j];
            }
        }
        if (first != SM_OK)
            throw Error(first, msg);
    });
}
