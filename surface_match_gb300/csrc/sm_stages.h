// sm_stages.h - host entry points of the device stages (implemented in prep.cu, vote.cu,
// cluster.cu, icp.cu) and the per-context state they share.
#pragma once

#include <cuda_runtime.h>

#include <condition_variable>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "sm_engine.h"
#include "sm_kdtree.cuh"

namespace sm {

// A host thread kept for the life of a context that runs one task at a time: matchScene
// hands it the dense-refinement preparation (which drives the context's second stream)
// instead of starting a thread per call.
class Helper {
public:
    Helper() : th_([this] { loop(); }) {}
    ~Helper() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        th_.join();
    }
    void post(std::function<void()> f) {
        std::lock_guard<std::mutex> lk(mu_);
        task_ = std::move(f);
        busy_ = true;
        err_  = nullptr;
        cv_.notify_all();
    }
    // waits for the posted task; rethrows its exception
    void wait() {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [this] { return !busy_; });
        if (err_) {
            std::exception_ptr e = err_;
            err_                 = nullptr;
            std::rethrow_exception(e);
        }
    }
    bool busy() {
        std::lock_guard<std::mutex> lk(mu_);
        return busy_;
    }

private:
    void loop() {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
            cv_.wait(lk, [this] { return stop_ || (busy_ && task_); });
            if (stop_ && !busy_)
                return;
            std::function<void()> f = std::move(task_);
            task_                   = nullptr;
            lk.unlock();
            std::exception_ptr e;
            try {
                f();
            } catch (...) {
                e = std::current_exception();
            }
            lk.lock();
            err_  = e;
            busy_ = false;
            cv_.notify_all();
        }
    }
    std::mutex              mu_;
    std::condition_variable cv_;
    std::function<void()>   task_;
    bool                    busy_ = false, stop_ = false;
    std::exception_ptr      err_;
    std::thread             th_;
};

// Opt-in timing of chosen kernels for throughput reports: an event pair around each launch
// on the launching stream, resolved after the call's final synchronisation, with the
// launch's algorithmic bytes (host-known, or added from a device count). Off by default:
// nothing is recorded.
struct KernelClock {
    enum Kind {
        kSamplePhase = 0,
        kScan        = 1,
        kCorr        = 2,
        kFit         = 3, // the refinement's other per-iteration launches: time only
        kResid       = 4,
        kUpdate      = 5,
        kKinds       = 6
    };
    bool      on = false;
    double    ms[kKinds]       = {};
    double    bytes[kKinds]    = {};
    long long launches[kKinds] = {};
    struct Rec {
        int         kind;
        double      bytes;
        cudaEvent_t a, b;
    };
    std::vector<Rec>         open;
    std::vector<cudaEvent_t> pool;
    cudaEvent_t take() {
        if (!pool.empty()) {
            cudaEvent_t e = pool.back();
            pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        SM_CUDA(cudaEventCreate(&e));
        return e;
    }
    // before the launch; nullptr when off
    cudaEvent_t begin(cudaStream_t s) {
        if (!on)
            return nullptr;
        cudaEvent_t a = take();
        SM_CUDA(cudaEventRecord(a, s));
        return a;
    }
    // after the launch
    void end(cudaStream_t s, cudaEvent_t a, int kind, double algBytes) {
        if (!a)
            return;
        cudaEvent_t b = take();
        SM_CUDA(cudaEventRecord(b, s));
        open.push_back({kind, algBytes, a, b});
    }
    // once the stream has synchronised
    void resolve() {
        for (const Rec &r : open) {
            float t = 0.0f;
            SM_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
            ms[r.kind] += t;
            bytes[r.kind] += r.bytes;
            launches[r.kind]++;
            pool.push_back(r.a);
            pool.push_back(r.b);
        }
        open.clear();
    }
    void reset() {
        for (int k = 0; k < kKinds; k++) {
            ms[k]       = 0.0;
            bytes[k]    = 0.0;
            launches[k] = 0;
        }
    }
    ~KernelClock() {
        for (const Rec &r : open) {
            cudaEventDestroy(r.a);
            cudaEventDestroy(r.b);
        }
        for (cudaEvent_t e : pool)
            cudaEventDestroy(e);
    }
};

struct Ctx {
    int          device    = 0;
    cudaStream_t stream    = nullptr;
    bool         ownStream = false;
    Arena        arena;
    int         *hostCounts = nullptr; // pinned scratch for small device->host reads
    cudaEvent_t  ev[14]{}; // stage timing (api.cu), vote-kernel timing 10..13 (vote_pipe.cu)
    // intermediate state of the last match (device pointers into the arena + sizes);
    // `dense` is the context whose workspace holds the refinement scene and the final
    // positions and normals (this one, or `aux`)
    struct Last {
        int  n = 0, ns = 0, nk = 0, nr = 0, np = 0, nc = 0, ncand = 0;
        bool valid = false;
        Ctx *dense = nullptr;
    } last;
    // second stream and workspace of this context (api.cu): matchScene prepares the dense
    // refinement scene there while it votes and clusters here; `fork` orders it after this
    // stream's work. Created on first use, released with the context.
    std::unique_ptr<Ctx>    aux;
    cudaEvent_t             fork = nullptr;
    std::unique_ptr<Helper> helper; // host thread that drives `aux` (created with it)
    // single-pass scan state (prep.cu): per-tile status words, {ticket, wait-expired flag}
    struct ScanState {
        unsigned long long *status = nullptr;
        int                *ticket = nullptr;
        int                 cap    = 0;
        unsigned            epoch  = 0;
    } scan;
    KernelClock clock; // opt-in per-launch timing (sm_context_kernel_clock)
    // launches of this context are chained to the previous kernel of its stream (see
    // launch_chained); off for the batch and serving workers, many of which run at once
    bool chain = true;
    void sync() { SM_CUDA(cudaStreamSynchronize(stream)); }
    // sync, then fail loudly if a bounded device wait of the scans expired
    void sync_checked() {
        if (scan.ticket)
            SM_CUDA(cudaMemcpyAsync(hostCounts + 63, scan.ticket + 1, sizeof(int),
                                    cudaMemcpyDeviceToHost, stream));
        sync();
        if (scan.ticket && hostCounts[63])
            throw Error(SM_ERR_RUNTIME, "device scan: a bounded look-back wait expired");
    }
};

// Launches kernel k (smem bytes of dynamic shared memory) on the context's stream. With
// c.chain the launch is chained to the previous kernel of the stream (programmatic dependent
// launch): it is processed, and the kernel's blocks may be scheduled, while that kernel
// finishes, which hides the launch latency of a dependent chain on an otherwise idle device.
// When many streams share the device, blocks parked in their wait would hold slots that
// other streams' kernels could use, so worker contexts launch ordinarily. Either way the
// kernel calls smd::chain_enter() before it touches memory.
template <typename... P, typename... A>
void launch_chained(const Ctx &c, void (*k)(P...), dim3 grid, dim3 block, size_t smem,
                    A &&...args) {
    cudaLaunchAttribute at[1];
    at[0].id                                         = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg                           = {};
    cfg.gridDim                                      = grid;
    cfg.blockDim                                     = block;
    cfg.dynamicSmemBytes                             = smem;
    cfg.stream                                       = c.stream;
    cfg.attrs                                        = at;
    cfg.numAttrs                                     = c.chain ? 1 : 0;
    SM_CUDA(cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...));
    SM_LAUNCH_CHECK();
}

// ---- prep.cu ------------------------------------------------------------------------
// Convert input xyz (+normals) to float4, mark finite points, reduce the bounding box of
// the valid points. Synchronises; returns the number of valid points.
int prep_points(Ctx &c, const float *xyz, const float *nrm, int n, float4 *pos, float4 *nrmOut,
                int *validFlag, Box &box);
// Exclusive scan of n ints (out may alias nothing); returns the total (synchronises if
// wantTotal).
int scan_excl(Ctx &c, const int *in, int *out, long long n, const std::string &tag,
              bool wantTotal = true);
// Ascending indices i with flags[i] != 0; returns the count (synchronises).
int compact(Ctx &c, const int *flags, int n, int *outIds, const std::string &tag);
// The same when the count is known already (no host round trip).
void compact_known(Ctx &c, const int *flags, int n, int *outIds, const std::string &tag);
// Hashed grid over points ids[0..m) with cell side g (fine cells at any scene extent).
void build_hgrid(Ctx &c, const float4 *pos, const int *ids, int m, const Box &box, float g,
                 HGrid &H, const std::string &tag, bool wIsRank = false);
// subPos[r] = pos[ids[r]], subNrm[r] = nrm[ids[r]] for r < m.
void gather_subset(Ctx &c, const float4 *pos, const float4 *nrm, const int *ids, int m,
                   float4 *subPos, float4 *subNrm);
// Greedy thinning of ids[0..m) (ascending) at `step` in (phase, cell, index) order; writes
// kept ids ascending, returns their count.
int sample_points(Ctx &c, const float4 *pos, int npoints, const int *ids, int m, const Box &box,
                  float step, int *outIds, const std::string &tag);
struct KdTree;
// Two-phase normal estimation of ids[0..m) (estimateNormal, util.cpp:234-334; all
// neighbourhoods from the positions at the start of the call, then smoothing). The k
// nearest come from the grid `query`, or, when `tree` is given, from the reference's k-d
// tree (over all points, searched on the live positions `pos`).
void estimate_normals(Ctx &c, float4 *pos, float4 *nrm, int npoints, const int *ids, int m,
                      const HGrid &query, int k, bool smooth, bool invert, const float *vp,
                      const std::string &tag, const KdTree *tree = nullptr);
// Normalise all normals (normalizeNormal, util.cpp:163-176).
void normalize_normals(Ctx &c, float4 *nrm, int n);

// ---- sort.cu --------------------------------------------------------------------------
// Stable LSD radix sort of n (key, value) pairs by the low `bits` bits of the key, in place.
void radix_sort_pairs(Ctx &c, uint32_t *keys, uint32_t *vals, int n, int bits,
                      const std::string &tag);

// ---- kdtree.cu ------------------------------------------------------------------------
// The reference-order k-d tree over points ids[0..m) (device arrays in the context's
// workspace, named by `tag`).
struct KdTree {
    int     m = 0, npoints = 0, nnodes = 0;
    int4   *nd      = nullptr; // nodes (sm_kdtree.cuh layout), root 0
    float  *box     = nullptr; // per node tight box (lo xyz, hi xyz), build-time positions
    int    *vacc    = nullptr; // per tree position: point id
    int    *leafOf  = nullptr; // per tree position: its leaf
    int    *treePos = nullptr; // per point id: tree position (-1: not in the tree)
    float4 *rec     = nullptr; // build-time positions in tree order (w = point id)
    int    *parent  = nullptr; // per node: its parent (-1 for the root)
    smk::KdView view(const int *vaccActive, const float4 *pos, const int *nonEmpty = nullptr,
                     const float4 *tpos = nullptr) const {
        smk::KdView v;
        v.nd       = nd;
        v.box      = box;
        v.vacc     = vaccActive ? vaccActive : vacc;
        v.pos      = pos;
        v.nonEmpty = nonEmpty;
        v.tpos     = tpos;
        return v;
    }
};
// KDTree construction of the reference (kdtree.h:65-79, nanoflann divideTree): the tree
// over ids[0..m) (the valid points in index order), root box `box`.
void build_kdtree(Ctx &c, const float4 *pos, int npoints, const int *ids, int m, const Box &box,
                  KdTree &T, const std::string &tag);
// samplePointCloud (util.cpp:107-139) on the tree: greedy thinning at `step` in tree
// position order over the positions whose vaccActive entry is >= 0 (the reduce()d tree),
// distances on the live positions `pos`. Writes the kept ids in tree order to outIds and,
// when ioi is given, the reduce() array (kept point id per tree position, else -1).
// Returns the number kept. `box` bounds the grid that buckets the points (points outside
// are clamped into its border cells).
int kd_sample(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos, float step,
              const Box &box, int *outIds, int *ioi, const std::string &tag);
// KNNResultSet searches (nanoflann findNeighbors) on the tree, one per query: query t is at
// qpos[t] (or pos[list[t]] when qpos is null) for t < *nq (a device count, nqMax bounds the
// launch); nbr[t*k + j] / dist[t*k + j] (dist nullable) its j-th nearest, cnt[t] (nullable)
// how many there are.
void kd_knn(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos,
            const float4 *qpos, const int *list, const int *nq, int nqMax, int k, int *nbr,
            float *dist, int *cnt, const float4 *nrm = nullptr, int *need = nullptr);
// flags[v] = 1 when node v's subtree holds a position whose vaccActive entry is >= 0
// (the searches of a reduce()d tree skip the others).
void kd_mark_nonempty(Ctx &c, const KdTree &T, const int *vaccActive, int *flags);
// tpos[i] = pos[id] with w = id bits for the tree positions i whose vaccActive entry id is
// >= 0, else w = -1 bits: the leaf records of the searches (taken after the positions last
// moved).
void kd_tree_positions(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos,
                       float4 *tpos);
// The voting stage's radius searches (ppf.cpp:273-276) in the reduced tree: for each of the
// K keypoints the candidates (cand[0..ncand), the sampled points) its search of radius^2 r2
// returns, as CSR lists (*offOut: K + 1 offsets, *idsOut: ids) whose last (rows mod 8) rows
// other than the keypoint are the search's last ones in depth-first order (the reference's
// scalar-tail rows); the rest in candidate order. Returns the total list length.
int kd_vote_lists(Ctx &c, const KdTree &T, const int *vaccActive, const float4 *pos,
                  const int *kp, int K, const int *cand, int ncand, float r2, int **offOut,
                  int **idsOut, const std::string &tag);

// ---- mls.cu ---------------------------------------------------------------------------
constexpr int kMlsMaxOrder = 4; // largest polynomial order of the MLS fit
// Moving-least-squares normals and projected points of ids[0..m) (estimateNormalMLS,
// util.cpp:336-457) with neighbours among valid[0..nvalid) within |radius|; writes the
// listed points' results into outXyz / outNrm (n x 3 floats, pre-filled by the caller).
void estimate_normals_mls(Ctx &c, const float4 *pos, const int *valid, int nvalid, const Box &box,
                          const int *ids, int m, float radius, int order, bool invert,
                          const float *vp, float *outXyz, float *outNrm);
// x[0..n) = NaN
void fill_nan(Ctx &c, float *x, long long n);

// ---- vote.cu --------------------------------------------------------------------------
struct VoteOut {
    long long *stats;   // K x 8
    float     *cands;   // K x 9
    float     *poses;   // K x 3 x 18
    int       *poseOk;  // K x 3 flags
    int       *acc;     // dumpK x refNum x A (nullable)
};
// Voting for K keypoints with neighbours either given as CSR lists (nbrOff/nbrIds) or, when
// nbrOff == nullptr, all points of `cand[0..ncand)` within the model diameter in ascending
// order.
void vote(Ctx &c, const Model &m, const float4 *pos, const float4 *nrm, const int *kp, int K,
          const int *nbrOff, const int *nbrIds, const int *cand, int ncand, float minScore,
          const VoteOut &out, int dumpK);
// The same from CSR lists in a single kernel that needs no workspace (same results).
void vote_fused(Ctx &c, const Model &m, const float4 *pos, const float4 *nrm, const int *kp,
                int K, const int *nbrOff, const int *nbrIds, float minScore, const VoteOut &out,
                int dumpK);
// All ordered model pairs (trainModel's table rows): key and alpha per (i, j).
void model_pairs(Ctx &c, const float4 *sp, const float4 *sn, int ns, float angleStep,
                 float distStep, uint32_t *keys, float *alphas, int *valid);
// trainModel's hash table (ppf.cpp:125-143) from the n1 x n1 pair rows: the valid pairs
// grouped by key, stable in pair order (reference point i, then column j), into the
// model's device arrays (keys, offsets, entries, open-addressed slot table).
void build_model_table(Ctx &c, Model &m, const uint32_t *keys, const float *alphas,
                       const int *valid, int n1);

// ---- cluster.cu -----------------------------------------------------------------------
// Pose clustering (clusterPose, avgClusters, sortPoses, clusterPose2) of np poses
// (18 floats each, in list order). Writes the ordered candidates (18 floats) and returns
// their count.
int cluster(Ctx &c, const float *poses, int np, float distThr, float angThr,
            const float center[3], float maxOverlap, float *outCands, const std::string &tag);

// ---- icp.cu ---------------------------------------------------------------------------
struct IcpScene {
    const float4 *pos, *nrm;
    HGrid         sampled, resampled, full; // the subset grids carry subset ranks in pts.w
    const float4 *posS, *nrmS, *posR, *nrmR; // the sampled / resampled subsets, rank order
    // reference search order (tree != nullptr): searches in the k-d tree, reduced to the
    // sampled (ioiS) or resampled (ioiR) points, whose ids map to subset ranks by rankS /
    // rankR; the grids are then unused (only their point counts m are read)
    const KdTree *tree = nullptr;
    const int    *ioiS = nullptr, *ioiR = nullptr, *rankS = nullptr, *rankR = nullptr;
    const int    *neS = nullptr, *neR = nullptr;                  // non-empty node flags
    const float4 *tpS = nullptr, *tpR = nullptr, *tpF = nullptr; // leaf records
};
struct IcpParams {
    int   sparse, dense, denseSteps;
    float rejectDist, sampleStep, reSampleStep, scoreDist, voteThreshold, minScore;
};
// Threads per CTA of the vote accumulation chosen by its launch tuner on `device` (0 while
// untuned), and whether it is the persistent grid (vote_pipe.cu).
int vote_tuned_shape(int device, int *persistent);
// ICP refinement + scoring of every candidate in parallel. Outputs per candidate: status,
// score, refined pose (12 floats).
void icp_all(Ctx &c, const Model &m, const IcpScene &s, const IcpParams &p, const float *cands,
             int ncand, int *status, float *score, float *pose, float *trace = nullptr);
constexpr int kIcpTraceFloats = 2 * 32 * 4 + 2; // per candidate, see icp.cu

// matchScene on one context (api.cu), and the per-device pool of worker contexts that the
// batch and serving entry points run jobs on (batch.cu).
void match_into(Ctx &c, const Model &m, const float *xyz, const float *nrm, int64_t n,
                const float *vp, float sdRel, float kpFrac, float minScore,
                const sm_match_param &mp, std::vector<float> &pose, std::vector<float> &score,
                sm_match_stats *stats);
std::unique_ptr<Ctx> acquire_worker(int device);
void                 release_worker(int device, std::unique_ptr<Ctx> c);

// Raise a kernel's dynamic shared-memory limit to the device maximum, once per kernel and
// device (the attribute is per function and process-wide: setting it to each launch's own
// size would race between concurrent worker threads). Returns the usable bytes.
size_t allow_dynamic_smem(const void *kernel, int device);

// Access to a model handle's engine state and the C ABI's error handling, for entry points
// defined outside api.cu.
Model *model_core(sm_model m);
Ctx   *model_ctx(sm_model m);
int    run_guarded(const std::function<void()> &f);

} // namespace sm
