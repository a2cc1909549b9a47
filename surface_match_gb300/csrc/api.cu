// api.cu - the C ABI (include/surface_match.h) and the host orchestration of the
// matching path on one device: ppf::Detector::trainModel / matchScene / save / load
// (ppf.cpp:36-547) over the device stages of prep.cu, vote.cu, cluster.cu and icp.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <exception>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/surface_match.h"
#include "sm_icp.h"
#include "sm_stages.h"

struct sm_context_s {
    sm::Ctx ctx;
};

struct sm_model_s {
    sm_context ctx;
    sm::Model  m;
};

namespace sm {

static thread_local std::string g_lastError;
long long                       g_launches = 0;

void Model::free_device() {
    void *ps[] = {sp, sn, rp, rn, hkeys, boff, entries, dkeys, doffs};
    for (void *p : ps)
        if (p)
            cudaFree(p);
    sp = sn = rp = rn = nullptr;
    hkeys = boff = nullptr;
    entries      = nullptr;
    dkeys = doffs = nullptr;
    hostValid     = false;
}


namespace {

template <class F> int guarded(F &&f) {
    try {
        f();
        g_lastError.clear();
        return SM_OK;
    } catch (const Error &e) {
        g_lastError = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        g_lastError = "host allocation failed";
        return SM_ERR_NOMEM;
    } catch (const std::exception &e) {
        g_lastError = e.what();
        return SM_ERR_RUNTIME;
    }
}

bool is_device_ptr(const void *p) {
    if (!p)
        return false;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Copy n*3 floats to the device unless they already are there.
const float *to_device(Ctx &c, const float *src, int64_t n, const std::string &tag) {
    if (!src)
        return nullptr;
    if (is_device_ptr(src))
        return src;
    float *d = c.arena.get<float>(tag, (size_t)n * 3);
    SM_CUDA(cudaMemcpyAsync(d, src, (size_t)n * 12, cudaMemcpyHostToDevice, c.stream));
    return d;
}

__global__ void k_gather4(const float4 *__restrict__ src, const int *__restrict__ ids, int m,
                          float4 *__restrict__ dst, int renormalize) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m)
        return;
    float4 v = src[ids[i]];
    if (renormalize) {
        const float sq = v.x * v.x + (v.y * v.y + v.z * v.z);
        if (sq > 0.0f) {
            const float s = smm::fsqrt(sq);
            v = make_float4(smm::fdiv(v.x, s), smm::fdiv(v.y, s), smm::fdiv(v.z, s), 0.0f);
        }
    }
    dst[i] = v;
}

__global__ void k_gather_poses(const float *__restrict__ poses, const int *__restrict__ slots,
                               int m, float *__restrict__ out) {
    smd::chain_enter(); // launched chained
    const int i = blockIdx.x;
    if (i >= m)
        return;
    const int s = slots[i];
    for (int e = threadIdx.x; e < smi::kPoseFloats; e += blockDim.x)
        out[(size_t)i * smi::kPoseFloats + e] = poses[(size_t)s * smi::kPoseFloats + e];
}

__global__ void k_rank_of(const int *__restrict__ ids, int m, int *__restrict__ rank) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < m)
        rank[ids[r]] = r;
}

// rank[ids[r]] = r for r < m
void rank_of(Ctx &c, const int *ids, int m, int *rank) {
    if (m <= 0)
        return;
    k_rank_of<<<nblocks(m, 256), 256, 0, c.stream>>>(ids, m, rank);
    SM_LAUNCH_CHECK();
}

__global__ void k_f3_to_f4(const float *__restrict__ a, int n, float4 *__restrict__ o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        o[i] = make_float4(a[3 * (size_t)i], a[3 * (size_t)i + 1], a[3 * (size_t)i + 2], 0.0f);
}

void check_train_param(const sm_train_param &p) {
    if (p.featDistanceStepRel > 1 || p.featDistanceStepRel <= 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: featDistanceStepRel range mismatch in TrainParam()");
    if (p.featAngleResolution <= 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: featAngleResolution range mismatch in TrainParam()");
    if (p.poseRefRelSamplingDistance > 1 || p.poseRefRelSamplingDistance <= 0)
        throw Error(SM_ERR_RANGE,
                    "Invalid Input: poseRefRelSamplingDistance range mismatch in TrainParam()");
}

void check_match_param(const sm_match_param &p) {
    if (p.numMatches < 1)
        throw Error(SM_ERR_RANGE, "Invalid Input: numMatches range mismatch in MatchParam()");
    if (p.maxOverlapDistRel < 0 && p.maxOverlapDistAbs < 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: maxOverlapDist range mismatch in MatchParam()");
    if (!p.densePoseRefinement) {
        if (p.poseRefNumSteps < 1)
            throw Error(SM_ERR_RANGE, "Invalid Input: poseRefNumSteps range mismatch in MatchParam()");
        if (p.poseRefDistThresholdRel < 0 && p.poseRefDistThresholdAbs < 0)
            throw Error(SM_ERR_RANGE,
                        "Invalid Input: poseRefDistThreshold range mismatch in MatchParam()");
        if (p.poseRefScoringDistRel < 0 && p.poseRefScoringDistAbs < 0)
            throw Error(SM_ERR_RANGE, "Invalid Input: poseRefScoringDist range mismatch in MatchParam()");
    }
}

// Upload host arrays of a model and build the open-addressed key table.
void upload_model(Model &m, const std::vector<float> &sp, const std::vector<float> &sn,
                  const std::vector<float> &rp, const std::vector<float> &rn, const float box[6],
                  const std::vector<uint32_t> &keys, const std::vector<uint32_t> &offs,
                  const std::vector<uint32_t> &refs, const std::vector<float> &alphas) {
    m.free_device();
    m.ns       = (int)(sp.size() / 3);
    m.nr       = (int)(rp.size() / 3);
    m.nkeys    = (int)keys.size();
    m.nentries = (long long)refs.size();
    for (int a = 0; a < 3; a++) {
        m.box.mn[a] = box[a];
        m.box.mx[a] = box[3 + a];
    }
    for (size_t b = 0; b + 1 < offs.size(); b++)
        if (offs[b + 1] < offs[b] || offs[b + 1] > refs.size())
            throw Error(SM_ERR_ARG, "model table offsets are not monotone");
    for (uint32_t r : refs)
        if ((int)r >= m.ns)
            throw Error(SM_ERR_ARG, "model table references a point beyond the sampled model");
    auto up4 = [](const std::vector<float> &v, float4 *&d) {
        const size_t n = v.size() / 3;
        std::vector<float4> h(n);
        for (size_t i = 0; i < n; i++)
            h[i] = make_float4(v[3 * i], v[3 * i + 1], v[3 * i + 2], 0.0f);
        SM_CUDA(cudaMalloc(&d, std::max<size_t>(n, 1) * sizeof(float4)));
        if (n)
            SM_CUDA(cudaMemcpy(d, h.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    };
    up4(sp, m.sp);
    up4(sn, m.sn);
    up4(rp, m.rp);
    up4(rn, m.rn);
    uint32_t size = 16;
    while (size < 2u * (uint32_t)m.nkeys)
        size <<= 1;
    std::vector<uint4> tab(size, make_uint4(0, 0, 0, 0));
    for (int b = 0; b < m.nkeys; b++) {
        uint32_t i = keys[b] & (size - 1);
        while (tab[i].z != 0)
            i = (i + 1) & (size - 1);
        tab[i] = make_uint4(keys[b], offs[b], offs[b + 1] - offs[b],
                            smm::bucket_max_ref_multiplicity(refs.data(), offs[b], offs[b + 1]));
    }
    m.hmask = size - 1;
    SM_CUDA(cudaMalloc((void **)&m.hkeys, size * sizeof(uint4)));
    SM_CUDA(cudaMemcpy(m.hkeys, tab.data(), size * sizeof(uint4), cudaMemcpyHostToDevice));
    std::vector<uint2> ent(std::max<size_t>(refs.size(), 1));
    for (size_t e = 0; e < refs.size(); e++) {
        uint32_t ab;
        memcpy(&ab, &alphas[e], 4);
        ent[e] = make_uint2(refs[e], ab);
    }
    SM_CUDA(cudaMalloc((void **)&m.entries, ent.size() * sizeof(uint2)));
    SM_CUDA(cudaMemcpy(m.entries, ent.data(), ent.size() * sizeof(uint2), cudaMemcpyHostToDevice));
    SM_CUDA(cudaMalloc((void **)&m.dkeys, std::max<size_t>(keys.size(), 1) * 4));
    SM_CUDA(cudaMalloc((void **)&m.doffs, offs.size() * 4));
    if (!keys.empty())
        SM_CUDA(cudaMemcpy(m.dkeys, keys.data(), keys.size() * 4, cudaMemcpyHostToDevice));
    SM_CUDA(cudaMemcpy(m.doffs, offs.data(), offs.size() * 4, cudaMemcpyHostToDevice));
    m.hostValid = true;
    m.h_sp     = sp;
    m.h_sn     = sn;
    m.h_rp     = rp;
    m.h_rn     = rn;
    m.h_keys   = keys;
    m.h_offs   = offs;
    m.h_refs   = refs;
    m.h_alphas = alphas;
    m.trained  = true;
}

std::vector<float> download4(const float4 *d, int n) {
    std::vector<float4> h(n);
    if (n)
        SM_CUDA(cudaMemcpy(h.data(), d, n * sizeof(float4), cudaMemcpyDeviceToHost));
    std::vector<float> o(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        o[3 * i]     = h[i].x;
        o[3 * i + 1] = h[i].y;
        o[3 * i + 2] = h[i].z;
    }
    return o;
}

} // namespace

void Model::ensure_host() {
    if (hostValid)
        return;
    h_sp = download4(sp, ns);
    h_sn = download4(sn, ns);
    h_rp = download4(rp, nr);
    h_rn = download4(rn, nr);
    h_keys.resize(nkeys);
    h_offs.resize((size_t)nkeys + 1);
    std::vector<uint2> ent((size_t)nentries);
    if (nkeys)
        SM_CUDA(cudaMemcpy(h_keys.data(), dkeys, (size_t)nkeys * 4, cudaMemcpyDeviceToHost));
    SM_CUDA(cudaMemcpy(h_offs.data(), doffs, ((size_t)nkeys + 1) * 4, cudaMemcpyDeviceToHost));
    if (nentries)
        SM_CUDA(cudaMemcpy(ent.data(), entries, (size_t)nentries * 8, cudaMemcpyDeviceToHost));
    h_refs.resize((size_t)nentries);
    h_alphas.resize((size_t)nentries);
    for (size_t e = 0; e < ent.size(); e++) {
        h_refs[e] = ent[e].x;
        memcpy(&h_alphas[e], &ent[e].y, 4);
    }
    hostValid = true;
}

namespace {

// Query-grid cell for k-nearest-neighbour searches: about 1.6x the expected k-NN radius,
// from the point density the greedy sampling reveals (n_sampled points at `step` cover an
// area of about n_sampled * step^2 / 0.7), so that the query's cell and its 26 neighbours
// decide nearly every query. Results do not depend on it, only run time.
float knn_cell(int nvalid, int nsampled, float step, int k) {
    float g = step * 0.25f;
    if (nvalid > 0 && nsampled > 0) {
        const double area = (double)nsampled * step * step / 0.7;
        const double rk   = std::sqrt((double)std::max(k, 3) * area / (3.14159265 * nvalid));
        g = (float)std::min<double>(std::max<double>(1.6 * rk, step * 0.1), step);
    }
    return g;
}

// trainModel (ppf.cpp:36-147) with the device sampler, normal estimation and pair kernel;
// the table is grouped by key on the host in pair order, i.e. the reference's
// single-threaded insertion order (reference point i, then column j).
void train(Ctx &c, Model &m, const float *xyzIn, const float *nrmIn, int64_t n64, float sdRel,
           const sm_train_param &tp) {
    if (sdRel > 1 || sdRel < 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: samplingDistanceRel range mismatch in trainModel");
    if (n64 <= 0 || !xyzIn)
        throw Error(SM_ERR_RUNTIME, "Invalid Input: empty model in trainModel");
    check_train_param(tp);
    if (n64 > (1ll << 30))
        throw Error(SM_ERR_ARG, "model has too many points");
    const int    n   = (int)n64;
    const float *xyz = to_device(c, xyzIn, n, "t.xyz");
    const float *nin = to_device(c, nrmIn, n, "t.nrm");
    float4      *pos = c.arena.get<float4>("t.pos", n);
    float4      *nrm = c.arena.get<float4>("t.n4", n);
    int         *val = c.arena.get<int>("t.valid", n);
    Box          box;
    const int    nvalid = prep_points(c, xyz, nin, n, pos, nrm, val, box);
    if (nvalid == 0)
        throw Error(SM_ERR_RUNTIME, "Invalid Input: empty model in trainModel");
    int *valid = c.arena.get<int>("t.vids", n);
    compact_known(c, val, n, valid, "t.cv");
    const float diam         = box.diameter();
    const float sampleStep   = diam * sdRel;
    const float reSampleStep = diam * tp.poseRefRelSamplingDistance;
    int        *idx1         = c.arena.get<int>("t.idx1", n);
    int        *idx2         = c.arena.get<int>("t.idx2", n);
    int         n1 = 0, n2 = 0;
    if (m.order == SM_ORDER_REFERENCE) {
        // the reference's tree over the model (ppf.cpp:77-83): both samplings in tree order
        // on the positions as given, then normals from the tree's k nearest
        KdTree T;
        build_kdtree(c, pos, n, valid, nvalid, box, T, "t.tree");
        n1 = kd_sample(c, T, nullptr, pos, sampleStep, box, idx1, nullptr, "t.s1");
        n2 = kd_sample(c, T, nullptr, pos, reSampleStep, box, idx2, nullptr, "t.s2");
        if (!nrmIn) {
            HGrid none;
            estimate_normals(c, pos, nrm, n, idx1, n1, none, tp.knnNormal, tp.smoothNormal != 0,
                             false, nullptr, "t.n1", &T);
            estimate_normals(c, pos, nrm, n, idx2, n2, none, tp.knnNormal, tp.smoothNormal != 0,
                             false, nullptr, "t.n2", &T);
        }
    } else {
        n1 = sample_points(c, pos, n, valid, nvalid, box, sampleStep, idx1, "t.s1");
        n2 = sample_points(c, pos, n, valid, nvalid, box, reSampleStep, idx2, "t.s2");
        if (!nrmIn) {
            HGrid q;
            const float gq = knn_cell(nvalid, n1, sampleStep, tp.knnNormal);
            build_hgrid(c, pos, valid, nvalid, box, gq, q, "t.q");
            estimate_normals(c, pos, nrm, n, idx1, n1, q, tp.knnNormal, tp.smoothNormal != 0, false,
                             nullptr, "t.n1");
            build_hgrid(c, pos, valid, nvalid, box, gq, q, "t.q");
            estimate_normals(c, pos, nrm, n, idx2, n2, q, tp.knnNormal, tp.smoothNormal != 0, false,
                             nullptr, "t.n2");
        }
    }
    float4 *sp = c.arena.get<float4>("t.sp", std::max(n1, 1));
    float4 *sn = c.arena.get<float4>("t.sn", std::max(n1, 1));
    float4 *rp = c.arena.get<float4>("t.rp", std::max(n2, 1));
    float4 *rn = c.arena.get<float4>("t.rn", std::max(n2, 1));
    if (n1) {
        k_gather4<<<nblocks(n1, 256), 256, 0, c.stream>>>(pos, idx1, n1, sp, 0);
        k_gather4<<<nblocks(n1, 256), 256, 0, c.stream>>>(nrm, idx1, n1, sn, 1);
    }
    if (n2) {
        k_gather4<<<nblocks(n2, 256), 256, 0, c.stream>>>(pos, idx2, n2, rp, 0);
        k_gather4<<<nblocks(n2, 256), 256, 0, c.stream>>>(nrm, idx2, n2, rn, 1);
    }
    SM_LAUNCH_CHECK();
    const int   A         = tp.featAngleResolution;
    const float angleStep = smm::k2PiF / (float)A;
    const float distStep  = diam * tp.featDistanceStepRel;
    const long long npair = (long long)n1 * n1;
    uint32_t *keys   = c.arena.get<uint32_t>("t.keys", std::max<long long>(npair, 1));
    float    *alphas = c.arena.get<float>("t.alphas", std::max<long long>(npair, 1));
    int      *pv     = c.arena.get<int>("t.pv", std::max<long long>(npair, 1));
    model_pairs(c, sp, sn, n1, angleStep, distStep, keys, alphas, pv);
    // the table grouped on the device by key in pair order - the reference's single-threaded
    // insertion order (ppf.cpp:125-143) - into model-owned arrays
    m.free_device();
    m.ns = n1;
    m.nr = n2;
    for (int a = 0; a < 3; a++) {
        m.box.mn[a] = box.mn[a];
        m.box.mx[a] = box.mx[a];
    }
    auto own4 = [&](const float4 *src, int cnt, float4 *&dst) {
        SM_CUDA(cudaMalloc((void **)&dst, (size_t)std::max(cnt, 1) * sizeof(float4)));
        if (cnt)
            SM_CUDA(cudaMemcpyAsync(dst, src, (size_t)cnt * sizeof(float4), cudaMemcpyDeviceToDevice,
                                    c.stream));
    };
    own4(sp, n1, m.sp);
    own4(sn, n1, m.sn);
    own4(rp, n2, m.rp);
    own4(rn, n2, m.rn);
    build_model_table(c, m, keys, alphas, pv, n1);
    m.trained   = true;
    m.hostValid = false;
    m.sdRel = sdRel;
    m.tp    = tp;
}

struct MatchOutputs {
    std::vector<float> pose;  // 12 per result
    std::vector<float> score;
};

void record(Ctx &c, int i) { SM_CUDA(cudaEventRecord(c.ev[i], c.stream)); }

// The context's second stream and workspace (created on first use). The dense preparation
// it runs is the longer of the two concurrent chains, so its stream takes the device's
// highest priority: its kernels are scheduled first when both chains have work queued.
Ctx &aux_ctx(Ctx &c) {
    if (!c.aux) {
        std::unique_ptr<Ctx> a(new Ctx());
        a->device = c.device;
        int least = 0, greatest = 0;
        SM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        SM_CUDA(cudaStreamCreateWithPriority(&a->stream, cudaStreamNonBlocking, greatest));
        a->ownStream = true;
        SM_CUDA(cudaMallocHost((void **)&a->hostCounts, 64 * sizeof(int)));
        for (auto &e : a->ev)
            SM_CUDA(cudaEventCreate(&e));
        a->arena.set_stream(a->stream, c.device);
        a->chain = c.chain;
        SM_CUDA(cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming));
        c.aux    = std::move(a);
        c.helper.reset(new Helper());
    }
    return *c.aux;
}

// Release a context's stream, events, pinned scratch and workspace (and its second
// context's).
void release_ctx(Ctx &c) {
    c.helper.reset(); // joins the helper thread (idle: every call waits for its task)
    if (c.aux) {
        release_ctx(*c.aux);
        c.aux.reset();
    }
    cudaStreamSynchronize(c.stream);
    c.arena.release();
    for (auto &e : c.ev)
        if (e)
            cudaEventDestroy(e);
    if (c.fork)
        cudaEventDestroy(c.fork);
    if (c.hostCounts)
        cudaFreeHost(c.hostCounts);
    if (c.ownStream)
        cudaStreamDestroy(c.stream);
}

// matchScene (ppf.cpp:149-510) on the device.
void match(Ctx &c, const Model &m, const float *xyzIn, const float *nrmIn, int64_t n64,
           const float *vp, float sdRel, float kpFrac, float minScore, const sm_match_param &mp,
           MatchOutputs &res, sm_match_stats *stats, bool overlap) {
    if (!m.trained)
        throw Error(SM_ERR_RUNTIME, "No trained model in matchScene");
    if (sdRel > 1 || sdRel < 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: samplingDistanceRel range mismatch in matchScene");
    if (kpFrac > 1 || kpFrac < 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: keyPointFraction range mismatch in matchScene");
    if (minScore > 1 || minScore < 0)
        throw Error(SM_ERR_RANGE, "Invalid Input: minScore range mismatch in matchScene");
    if (n64 <= 0 || !xyzIn)
        throw Error(SM_ERR_RUNTIME, "Invalid Input: empty scene in matchScene");
    check_match_param(mp);
    if (n64 > (1ll << 30))
        throw Error(SM_ERR_ARG, "scene has too many points");
    const int n = (int)n64;
    c.last.valid = false;
    record(c, 0);
    const float *xyz  = to_device(c, xyzIn, n, "m.xyz");
    const float *nin  = to_device(c, nrmIn, n, "m.nrm");
    const bool   hasN = nrmIn != nullptr;
    float4      *pos  = c.arena.get<float4>("m.pos", n);
    float4      *nrm  = c.arena.get<float4>("m.n4", n);
    int         *val  = c.arena.get<int>("m.valid", n);
    Box          box;
    const int    nvalid = prep_points(c, xyz, nin, n, pos, nrm, val, box);
    int         *valid  = c.arena.get<int>("m.vids", n);
    compact_known(c, val, n, valid, "m.cv"); // nvalid points
    record(c, 1);
    if (nvalid == 0) {
        // no finite point: the reference's search structures are empty and it returns no
        // pose; nothing is sampled (there is no bounding box to build grids on)
        c.sync_checked();
        res.pose.clear();
        res.score.clear();
        c.last       = Ctx::Last{};
        c.last.n     = n;
        c.last.dense = &c;
        c.last.valid = true;
        if (stats) {
            memset(stats, 0, sizeof(*stats));
            stats->n_points = n;
        }
        return;
    }
    const float diam         = m.box.diameter();
    const int   A            = m.tp.featAngleResolution;
    const float angleStep    = smm::k2PiF / (float)A;
    const float reSampleStep = diam * m.tp.poseRefRelSamplingDistance;
    const float sampleStep   = diam * sdRel;
    int        *sampled      = c.arena.get<int>("m.sampled", std::max(n, 1));
    const bool  ref          = m.order == SM_ORDER_REFERENCE;
    // reference order: the scene's k-d tree (ppf.cpp:197) over the valid points; `ioi` is
    // its reduce() array of the sampled points (ppf.cpp:201-213)
    KdTree      T;
    int        *ioi = nullptr;
    int         ns  = 0;
    HGrid       q;
    float       gq  = 0.0f;
    if (ref) {
        build_kdtree(c, pos, n, valid, nvalid, box, T, "m.tree");
        ioi = c.arena.get<int>("m.ioi", std::max(nvalid, 1));
        ns  = kd_sample(c, T, nullptr, pos, sampleStep, box, sampled, ioi, "m.s1");
        if (!hasN)
            estimate_normals(c, pos, nrm, n, sampled, ns, q, mp.knnNormal, mp.smoothNormal != 0,
                             mp.invertNormal != 0, vp, "m.n1", &T);
    } else {
        ns = sample_points(c, pos, n, valid, nvalid, box, sampleStep, sampled, "m.s1");
        gq = knn_cell(nvalid, ns, sampleStep, mp.knnNormal);
        if (!hasN) {
            build_hgrid(c, pos, valid, nvalid, box, gq, q, "m.q");
            estimate_normals(c, pos, nrm, n, sampled, ns, q, mp.knnNormal, mp.smoothNormal != 0,
                             mp.invertNormal != 0, vp, "m.n1");
        }
    }
    record(c, 2);
    float maxOverlap = 0;
    if (mp.maxOverlapDistRel > 0)
        maxOverlap = diam * mp.maxOverlapDistRel;
    if (mp.maxOverlapDistAbs > 0)
        maxOverlap = mp.maxOverlapDistAbs;
    float refDist = 0;
    if (mp.poseRefDistThresholdRel > 0)
        refDist = diam * mp.poseRefDistThresholdRel;
    if (mp.poseRefDistThresholdAbs > 0)
        refDist = mp.poseRefDistThresholdAbs;
    float scoreDist = 0;
    if (mp.poseRefScoringDistRel > 0)
        scoreDist = diam * mp.poseRefScoringDistRel;
    if (mp.poseRefScoringDistAbs > 0)
        scoreDist = mp.poseRefScoringDistAbs;
    // The dense refinement scene (ppf.cpp:428-434) and the refinement's search grids depend
    // only on the positions and normals as they are now: keypoint sampling, voting and
    // clustering write neither. With `overlap` a second context builds them from a snapshot
    // on its own stream and host thread while this one votes and clusters, and the
    // refinement reads that context's buffers; otherwise the same steps run here, in place,
    // after clustering. Both give the same values.
    int      nres = 0;
    IcpScene s;
    auto     prepare_dense = [&](Ctx &d) {
        float4 *P = pos, *N = nrm;
        if (&d != &c) {
            SM_CUDA(cudaStreamWaitEvent(d.stream, c.fork, 0));
            P = d.arena.get<float4>("m.pos", n);
            N = d.arena.get<float4>("m.n4", n);
            SM_CUDA(cudaMemcpyAsync(P, pos, (size_t)n * 16, cudaMemcpyDeviceToDevice, d.stream));
            SM_CUDA(cudaMemcpyAsync(N, nrm, (size_t)n * 16, cudaMemcpyDeviceToDevice, d.stream));
        }
        int *resampled = d.arena.get<int>("m.resampled", std::max(n, 1));
        s.pos = P;
        s.nrm = N;
        if (ref) {
            // restore() and resample the whole tree, normals without smoothing (ppf.cpp:428-
            // 434); the refinement searches the tree reduced to each subset, and scores on
            // the whole tree
            int *ioi2 = d.arena.get<int>("m.ioi2", std::max(nvalid, 1));
            if (mp.densePoseRefinement) {
                nres = kd_sample(d, T, nullptr, P, reSampleStep, box, resampled, ioi2, "m.s3");
                if (!hasN) {
                    HGrid none;
                    estimate_normals(d, P, N, n, resampled, nres, none, mp.knnNormal, false,
                                     mp.invertNormal != 0, vp, "m.n2", &T);
                }
            }
            int *rankS = d.arena.get<int>("m.rankS", std::max(n, 1));
            int *rankR = d.arena.get<int>("m.rankR", std::max(n, 1));
            rank_of(d, sampled, ns, rankS);
            rank_of(d, resampled, nres, rankR);
            // the refinement's searches: empty subtrees of the reduced trees are skipped,
            // leaves read tree-ordered records of the positions as they are now
            int    *neS = d.arena.get<int>("m.neS", std::max(T.nnodes, 1));
            int    *neR = d.arena.get<int>("m.neR", std::max(T.nnodes, 1));
            float4 *tpS = d.arena.get<float4>("m.tpS", std::max(T.m, 1));
            float4 *tpR = d.arena.get<float4>("m.tpR", std::max(T.m, 1));
            float4 *tpF = d.arena.get<float4>("m.tpF", std::max(T.m, 1));
            kd_mark_nonempty(d, T, ioi, neS);
            kd_mark_nonempty(d, T, ioi2, neR);
            kd_tree_positions(d, T, ioi, P, tpS);
            kd_tree_positions(d, T, ioi2, P, tpR);
            kd_tree_positions(d, T, nullptr, P, tpF);
            s.neS         = neS;
            s.neR         = neR;
            s.tpS         = tpS;
            s.tpR         = tpR;
            s.tpF         = tpF;
            s.tree        = &T;
            s.ioiS        = ioi;
            s.ioiR        = ioi2;
            s.rankS       = rankS;
            s.rankR       = rankR;
            s.sampled.m   = ns;
            s.resampled.m = nres;
        } else {
            if (mp.densePoseRefinement) {
                nres = sample_points(d, P, n, valid, nvalid, box, reSampleStep, resampled, "m.s3");
                if (!hasN) {
                    HGrid q2;
                    build_hgrid(d, P, valid, nvalid, box, gq, q2, "m.q");
                    estimate_normals(d, P, N, n, resampled, nres, q2, mp.knnNormal, false,
                                     mp.invertNormal != 0, vp, "m.n2");
                }
            }
            // Nearest-neighbour grids of the refinement: cells of about a third of the
            // rejection distance (never finer than the subset's spacing), so three cell
            // shells always cover it. The inlier grid's cell just exceeds the scoring
            // distance, so two shells decide. The subset grids name points by subset rank
            // (the subsets are ascending, so rank order is index order), and the refinement
            // reads rank-ordered copies of the subsets.
            build_hgrid(d, P, sampled, ns, box, std::max(sampleStep, refDist / 2.98f), s.sampled,
                        "m.gS", true);
            build_hgrid(d, P, resampled, nres, box, std::max(2.0f * reSampleStep, refDist / 2.98f),
                        s.resampled, "m.gR", true);
            build_hgrid(d, P, valid, nvalid, box, std::max(scoreDist * 1.02f, gq), s.full, "m.gF");
        }
        float4 *posS = d.arena.get<float4>("m.posS", std::max(ns, 1));
        float4 *nrmS = d.arena.get<float4>("m.nrmS", std::max(ns, 1));
        float4 *posR = d.arena.get<float4>("m.posR", std::max(nres, 1));
        float4 *nrmR = d.arena.get<float4>("m.nrmR", std::max(nres, 1));
        gather_subset(d, P, N, sampled, ns, posS, nrmS);
        gather_subset(d, P, N, resampled, nres, posR, nrmR);
        s.posS = posS;
        s.nrmS = nrmS;
        s.posR = posR;
        s.nrmR = nrmR;
        if (&d != &c)
            d.sync_checked();
    };
    Ctx *dctx = &c;
    // the helper reads this call's buffers: never leave the call while its task runs
    struct Waiter {
        Helper *h = nullptr;
        ~Waiter() {
            if (h) {
                try {
                    h->wait();
                } catch (...) {
                }
            }
        }
    } waiter;
    if (overlap) {
        dctx            = &aux_ctx(c);
        dctx->clock.on  = c.clock.on;
        SM_CUDA(cudaEventRecord(c.fork, c.stream));
        Ctx *d = dctx;
        c.helper->post([&, d] {
            SM_CUDA(cudaSetDevice(c.device));
            prepare_dense(*d);
        });
        waiter.h = c.helper.get();
    }
    const float keyStep = smm::fsqrt(1.f / kpFrac) * sampleStep;
    int        *kp      = c.arena.get<int>("m.kp", std::max(ns, 1));
    // keypoints: the tree reduced to the sampled points (ppf.cpp:213-215)
    const int K = ref ? kd_sample(c, T, ioi, pos, keyStep, box, kp, nullptr, "m.s2")
                      : sample_points(c, pos, n, sampled, ns, box, keyStep, kp, "m.s2");
    record(c, 3);
    // voting
    VoteOut vo;
    vo.stats  = c.arena.get<long long>("m.kstats", (size_t)std::max(K, 1) * 8);
    vo.cands  = c.arena.get<float>("m.kcands", (size_t)std::max(K, 1) * 9);
    vo.poses  = c.arena.get<float>("m.kposes", (size_t)std::max(K, 1) * 3 * smi::kPoseFloats);
    vo.poseOk = c.arena.get<int>("m.kposeok", (size_t)std::max(K, 1) * 3);
    vo.acc    = nullptr;
    record(c, 8);
    if (ref) {
        // the keypoints' radius searches in the reduced tree, tail rows last (ppf.cpp:273-299)
        int        *off = nullptr, *ids = nullptr;
        const float dm  = m.box.diameter();
        kd_vote_lists(c, T, ioi, pos, kp, K, sampled, ns, dm * dm, &off, &ids, "m.rl");
        vote(c, m, pos, nrm, kp, K, off, ids, nullptr, 0, minScore, vo, 0);
    } else {
        vote(c, m, pos, nrm, kp, K, nullptr, nullptr, sampled, ns, minScore, vo, 0);
    }
    record(c, 9);
    int      *slots = c.arena.get<int>("m.slots", (size_t)std::max(K, 1) * 3);
    const int np    = compact(c, vo.poseOk, K * 3, slots, "m.cp");
    float    *plist = c.arena.get<float>("m.plist", (size_t)std::max(np, 1) * smi::kPoseFloats);
    if (np) {
        launch_chained(c, k_gather_poses, np, 32, 0, vo.poses, slots, np, plist);
    }
    record(c, 4);
    const float center[3] = {(m.box.mn[0] + m.box.mx[0]) / 2.f, (m.box.mn[1] + m.box.mx[1]) / 2.f,
                             (m.box.mn[2] + m.box.mx[2]) / 2.f};
    float    *cands = c.arena.get<float>("m.cands", (size_t)std::max(np, 1) * smi::kPoseFloats);
    const int ncand = cluster(c, plist, np, 0.1f * diam, angleStep, center, maxOverlap, cands, "m.cl");
    record(c, 5);
    if (overlap) {
        waiter.h = nullptr;
        c.helper->wait(); // rethrows the preparation's error
    } else if (ncand > 0) {
        // in place: only when a cluster is left to refine (nothing reads the refinement
        // scene otherwise; the resampled count then reads 0)
        prepare_dense(c);
    }
    record(c, 6);
    IcpParams ip;
    ip.sparse        = mp.sparsePoseRefinement;
    ip.dense         = mp.densePoseRefinement;
    ip.denseSteps    = mp.poseRefNumSteps;
    ip.rejectDist    = refDist;
    ip.sampleStep    = sampleStep;
    ip.reSampleStep  = reSampleStep;
    ip.scoreDist     = scoreDist;
    ip.voteThreshold = (float)m.ns * minScore;
    ip.minScore      = minScore;
    int   *cstat  = c.arena.get<int>("m.cstat", std::max(ncand, 1));
    float *cscore = c.arena.get<float>("m.cscore", std::max(ncand, 1));
    float *cpose  = c.arena.get<float>("m.cpose", (size_t)std::max(ncand, 1) * 12);
    float *ctrace = c.arena.get<float>("m.ctrace", (size_t)std::max(ncand, 1) * kIcpTraceFloats);
    icp_all(c, m, s, ip, cands, ncand, cstat, cscore, cpose, ctrace);
    std::vector<int>   hs(ncand);
    std::vector<float> hsc(ncand), hp((size_t)ncand * 12);
    if (ncand) {
        SM_CUDA(cudaMemcpyAsync(hs.data(), cstat, ncand * 4, cudaMemcpyDeviceToHost, c.stream));
        SM_CUDA(cudaMemcpyAsync(hsc.data(), cscore, ncand * 4, cudaMemcpyDeviceToHost, c.stream));
        SM_CUDA(cudaMemcpyAsync(hp.data(), cpose, (size_t)ncand * 48, cudaMemcpyDeviceToHost, c.stream));
    }
    record(c, 7);
    c.sync_checked();
    if (c.clock.on) {
        // the timed launches of this call (the refinement searches' bytes from their count:
        // per (candidate, source point) 16 + 16 bytes read, 16 + 16 + 3 x 4 written, 8 of
        // winner atomic)
        if (ncand > 0) {
            unsigned long long live = 0;
            SM_CUDA(cudaMemcpy(&live, c.arena.get<unsigned long long>("icp.live", 1), sizeof(live),
                               cudaMemcpyDeviceToHost));
            c.clock.bytes[KernelClock::kCorr] += 88.0 * (double)live;
        }
        c.clock.resolve();
        if (c.aux)
            c.aux->clock.resolve();
    }
    // selection walk (ppf.cpp:439-495) and ordering by score (ppf.cpp:498-507)
    std::vector<int> acc;
    for (int i = 0; i < ncand; i++) {
        if (hs[i] != 0)
            continue;
        acc.push_back(i);
        if ((int)acc.size() >= mp.numMatches)
            break;
    }
    std::stable_sort(acc.begin(), acc.end(), [&](int a, int b) { return hsc[a] > hsc[b]; });
    res.pose.clear();
    res.score.clear();
    for (int i : acc) {
        res.pose.insert(res.pose.end(), hp.begin() + (size_t)i * 12, hp.begin() + (size_t)i * 12 + 12);
        res.score.push_back(hsc[i]);
    }
    c.last.n     = n;
    c.last.ns    = ns;
    c.last.nk    = K;
    c.last.nr    = nres;
    c.last.np    = np;
    c.last.ncand = ncand;
    c.last.dense = dctx;
    c.last.valid = true;
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        stats->n_points    = n;
        stats->n_valid     = nvalid;
        stats->n_sampled   = ns;
        stats->n_keypoints = K;
        stats->n_resampled = nres;
        stats->n_poses     = np;
        stats->n_clusters  = ncand;
        std::vector<long long> st((size_t)K * 8);
        if (K)
            SM_CUDA(cudaMemcpy(st.data(), vo.stats, (size_t)K * 64, cudaMemcpyDeviceToHost));
        for (int k = 0; k < K; k++) {
            if (st[(size_t)k * 8 + 1] == 0)
                stats->n_pairs += st[(size_t)k * 8] - 1;
            stats->n_hits += st[(size_t)k * 8 + 2];
            stats->n_votes += st[(size_t)k * 8 + 3];
        }
        const int stage[8][2] = {{0, 1}, {1, 2}, {2, 3}, {8, 9}, {4, 5}, {5, 6}, {6, 7}, {0, 7}};
        for (int i = 0; i < 8; i++)
            SM_CUDA(cudaEventElapsedTime(&stats->ms[i], c.ev[stage[i][0]], c.ev[stage[i][1]]));
        if (K > 0) {
            SM_CUDA(cudaEventElapsedTime(&stats->vote_ms[0], c.ev[10], c.ev[11]));
            SM_CUDA(cudaEventElapsedTime(&stats->vote_ms[1], c.ev[12], c.ev[13]));
        }
    }
}

std::string read_all(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open())
        throw Error(SM_ERR_RUNTIME, "failed to open file:" + path);
    return std::string((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

struct Reader {
    const std::string &s;
    size_t             p = 0;
    template <class T> T get() {
        if (p + sizeof(T) > s.size())
            throw Error(SM_ERR_RUNTIME, "truncated model file");
        T v;
        memcpy(&v, s.data() + p, sizeof(T));
        p += sizeof(T);
        return v;
    }
    std::vector<float> vec3() {
        const uint32_t n = get<uint32_t>();
        if ((size_t)n * 12 > s.size() - p)
            throw Error(SM_ERR_RUNTIME, "truncated model file");
        std::vector<float> v((size_t)n * 3);
        memcpy(v.data(), s.data() + p, (size_t)n * 12);
        p += (size_t)n * 12;
        return v;
    }
};

constexpr int kMagic   = 0x7F27F; // ppf.cpp:22
constexpr int kVersion = 100;     // ppf.cpp:21

template <class T> void put(std::string &o, const T &v) { o.append((const char *)&v, sizeof(T)); }

void put_cloud(std::string &o, const std::vector<float> &p, const std::vector<float> &n,
               const float box[6]) {
    put<uint32_t>(o, (uint32_t)(p.size() / 3));
    o.append((const char *)p.data(), p.size() * 4);
    put<uint32_t>(o, (uint32_t)(n.size() / 3));
    o.append((const char *)n.data(), n.size() * 4);
    for (int i = 0; i < 6; i++)
        put<float>(o, box[i]);
    const float nanv = NAN;
    for (int i = 0; i < 3; i++)
        put<float>(o, nanv); // viewPoint (type.h:28): not set on a model
}

} // namespace

void match_into(Ctx &c, const Model &m, const float *xyz, const float *nrm, int64_t n,
                const float *vp, float sdRel, float kpFrac, float minScore,
                const sm_match_param &mp, std::vector<float> &pose, std::vector<float> &score,
                sm_match_stats *stats) {
    MatchOutputs res;
    match(c, m, xyz, nrm, n, vp, sdRel, kpFrac, minScore, mp, res, stats, false);
    pose  = std::move(res.pose);
    score = std::move(res.score);
}

Model *model_core(sm_model m) { return &m->m; }
Ctx   *model_ctx(sm_model m) { return &m->ctx->ctx; }
int    run_guarded(const std::function<void()> &f) { return guarded(f); }

size_t allow_dynamic_smem(const void *kernel, int device) {
    static std::mutex                                mu;
    static std::map<std::pair<const void *, int>, size_t> done;
    std::lock_guard<std::mutex>                      lk(mu);
    auto                                             it = done.find({kernel, device});
    if (it != done.end())
        return it->second;
    int optin = 0;
    SM_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    cudaFuncAttributes fa;
    SM_CUDA(cudaFuncGetAttributes(&fa, kernel));
    const size_t avail = (size_t)optin - fa.sharedSizeBytes;
    SM_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)avail));
    done[{kernel, device}] = avail;
    return avail;
}

} // namespace sm

using namespace sm;

// =======================================================================================
extern "C" {

SM_API const char *sm_last_error(void) { return g_lastError.c_str(); }
SM_API const char *sm_version(void) { return "surface_match_gb300 0.1 (sm_103a)"; }
SM_API int64_t     sm_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

SM_API int sm_host_alloc(int64_t bytes, void **out) {
    return guarded([&] {
        if (!out || bytes < 0)
            throw Error(SM_ERR_ARG, "invalid host allocation arguments");
        *out = nullptr;
        if (bytes == 0)
            return;
        void *p = nullptr;
        const cudaError_t e = cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocPortable);
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(e == cudaErrorMemoryAllocation ? SM_ERR_NOMEM : SM_ERR_CUDA,
                        std::string("page-locked host allocation failed: ") + cudaGetErrorString(e));
        }
        *out = p;
    });
}

SM_API int sm_vote_tuned_shape(int device, int *threads_per_cta, int *persistent) {
    return guarded([&] {
        if (!threads_per_cta || !persistent)
            throw Error(SM_ERR_ARG, "NULL argument");
        *threads_per_cta = vote_tuned_shape(device, persistent);
    });
}

SM_API int sm_host_free(void *p) {
    return guarded([&] {
        if (p)
            SM_CUDA(cudaFreeHost(p));
    });
}

SM_API void sm_train_param_default(sm_train_param *p) {
    if (p)
        *p = sm_train_param{0.04f, 30, 0.01f, 10, 1};
}
SM_API void sm_match_param_default(sm_match_param *p) {
    if (p)
        *p = sm_match_param{1, 10, 1, 0, 0.5f, 0.0f, 1, 1, 5, 0.1f, 0.0f, 0.01f, 0.0f};
}
SM_API int sm_train_param_check(const sm_train_param *p) {
    return guarded([&] {
        if (!p)
            throw Error(SM_ERR_ARG, "NULL param");
        check_train_param(*p);
    });
}
SM_API int sm_match_param_check(const sm_match_param *p) {
    return guarded([&] {
        if (!p)
            throw Error(SM_ERR_ARG, "NULL param");
        check_match_param(*p);
    });
}

SM_API int sm_context_create(int device, void *stream, sm_context *out) {
    return guarded([&] {
        if (!out)
            throw Error(SM_ERR_ARG, "NULL output handle");
        *out = nullptr;
        int ndev = 0;
        SM_CUDA(cudaGetDeviceCount(&ndev));
        if (device < 0 || device >= ndev)
            throw Error(SM_ERR_ARG, "no CUDA device " + std::to_string(device));
        SM_CUDA(cudaSetDevice(device));
        std::unique_ptr<sm_context_s> c(new sm_context_s());
        c->ctx.device = device;
        if (stream) {
            c->ctx.stream = (cudaStream_t)stream;
        } else {
            SM_CUDA(cudaStreamCreateWithFlags(&c->ctx.stream, cudaStreamNonBlocking));
            c->ctx.ownStream = true;
        }
        SM_CUDA(cudaMallocHost((void **)&c->ctx.hostCounts, 64 * sizeof(int)));
        for (auto &e : c->ctx.ev)
            SM_CUDA(cudaEventCreate(&e));
        c->ctx.arena.set_stream(c->ctx.stream, device);
        *out = c.release();
    });
}

SM_API int sm_context_destroy(sm_context c) {
    return guarded([&] {
        if (!c)
            return;
        cudaSetDevice(c->ctx.device);
        release_ctx(c->ctx);
        delete c;
    });
}

SM_API int sm_context_synchronize(sm_context c) {
    return guarded([&] {
        if (!c)
            throw Error(SM_ERR_ARG, "NULL context");
        c->ctx.sync();
    });
}

SM_API void *sm_context_stream(sm_context c) { return c ? (void *)c->ctx.stream : nullptr; }

SM_API int sm_context_kernel_clock(sm_context c, int on) {
    return guarded([&] {
        if (!c)
            throw Error(SM_ERR_ARG, "NULL argument");
        SM_CUDA(cudaSetDevice(c->ctx.device));
        c->ctx.sync();
        for (Ctx *x : {&c->ctx, c->ctx.aux.get()}) {
            if (!x)
                continue;
            x->clock.resolve();
            if (on)
                x->clock.reset(); // a new count; switching off keeps the totals for reading
            x->clock.on = on != 0;
        }
    });
}

SM_API int sm_context_kernel_report(sm_context c, int kind, double *ms, double *bytes,
                                    int64_t *launches) {
    return guarded([&] {
        if (!c || !ms || !bytes || !launches)
            throw Error(SM_ERR_ARG, "NULL argument");
        if (kind < 0 || kind >= KernelClock::kKinds)
            throw Error(SM_ERR_ARG, "unknown kernel kind");
        *ms       = 0.0;
        *bytes    = 0.0;
        *launches = 0;
        for (Ctx *x : {&c->ctx, c->ctx.aux.get()}) {
            if (!x)
                continue;
            *ms += x->clock.ms[kind];
            *bytes += x->clock.bytes[kind];
            *launches += x->clock.launches[kind];
        }
    });
}

SM_API int sm_context_workspace_bytes(sm_context c, int64_t *bytes) {
    return guarded([&] {
        if (!c || !bytes)
            throw Error(SM_ERR_ARG, "NULL argument");
        int64_t b = (int64_t)c->ctx.arena.bytes();
        if (c->ctx.aux)
            b += (int64_t)c->ctx.aux->arena.bytes();
        *bytes = b;
    });
}

// estimateNormalMLS (util.cpp:336-457): the finite points are the search set (the
// reference's k-d tree over the cloud), the listed points are estimated (mls.cu).
SM_API int sm_estimate_normals_mls(sm_context ctx, const float *xyzIn, const float *nrmIn,
                                   int64_t n64, const int64_t *indices, int64_t nIdx,
                                   float radius, int order, int invert, const float *vp,
                                   float *outXyz, float *outNrm) {
    return guarded([&] {
        if (!ctx || !xyzIn || !outXyz || !outNrm)
            throw Error(SM_ERR_ARG, "NULL argument");
        if (order < 1 || order > kMlsMaxOrder)
            throw Error(SM_ERR_ARG, "MLS order must be in 1.." + std::to_string(kMlsMaxOrder));
        if (!std::isfinite(radius))
            throw Error(SM_ERR_ARG, "MLS radius must be finite");
        if (n64 < 0 || n64 > (1ll << 30))
            throw Error(SM_ERR_ARG, "bad point count");
        if (n64 == 0)
            return;
        const int        n = (int)n64;
        std::vector<int> ids;
        if (indices) {
            if (nIdx < 0 || nIdx > (1ll << 31) - 1)
                throw Error(SM_ERR_ARG, "bad index count");
            ids.resize((size_t)nIdx);
            for (int64_t i = 0; i < nIdx; i++) {
                if (indices[i] < 0 || indices[i] >= n64)
                    throw Error(SM_ERR_ARG, "point index out of range");
                ids[(size_t)i] = (int)indices[i];
            }
        } else {
            ids.resize((size_t)n);
            for (int i = 0; i < n; i++)
                ids[(size_t)i] = i;
        }
        Ctx &c = ctx->ctx;
        SM_CUDA(cudaSetDevice(c.device));
        const float *xyz  = to_device(c, xyzIn, n, "l.xyz");
        const float *nin  = to_device(c, nrmIn, n, "l.nrm");
        float4      *pos  = c.arena.get<float4>("l.pos", n);
        float4      *nrm  = c.arena.get<float4>("l.n4", n);
        int         *val  = c.arena.get<int>("l.valid", n);
        float       *oXyz = c.arena.get<float>("l.oxyz", (size_t)n * 3);
        float       *oNrm = c.arena.get<float>("l.onrm", (size_t)n * 3);
        SM_CUDA(cudaMemcpyAsync(oXyz, xyz, (size_t)n * 12, cudaMemcpyDeviceToDevice, c.stream));
        if (nin)
            SM_CUDA(cudaMemcpyAsync(oNrm, nin, (size_t)n * 12, cudaMemcpyDeviceToDevice, c.stream));
        else
            fill_nan(c, oNrm, (long long)n * 3);
        // validity of the search set by position only: the tree indexes every point
        Box       box;
        const int nvalid = prep_points(c, xyz, nullptr, n, pos, nrm, val, box);
        if (nvalid > 0 && !ids.empty()) {
            int *valid = c.arena.get<int>("l.vids", n);
            compact_known(c, val, n, valid, "l.cv");
            int *dids = c.arena.get<int>("l.ids", ids.size());
            SM_CUDA(cudaMemcpyAsync(dids, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice,
                                    c.stream));
            estimate_normals_mls(c, pos, valid, nvalid, box, dids, (int)ids.size(), radius, order,
                                 invert != 0, vp, oXyz, oNrm);
        }
        SM_CUDA(cudaMemcpyAsync(outXyz, oXyz, (size_t)n * 12, cudaMemcpyDefault, c.stream));
        SM_CUDA(cudaMemcpyAsync(outNrm, oNrm, (size_t)n * 12, cudaMemcpyDefault, c.stream));
        c.sync_checked();
    });
}

// Reference-order k-d tree probe (kdtree.h:65-79, util.cpp:107-139, nanoflann
// findNeighbors): the tree over the finite points with their tight box as root box.
SM_API int sm_kdtree_probe(sm_context ctx, const float *xyzIn, int64_t n64, float step,
                           int32_t *outVacc, int32_t *outSampled, int64_t *outNSampled,
                           const float *queries, int64_t nq64, int k, int32_t *outKnn,
                           float *outKnnDist) {
    return guarded([&] {
        if (!ctx || !xyzIn)
            throw Error(SM_ERR_ARG, "NULL argument");
        if (n64 <= 0 || n64 > (1ll << 30) || nq64 < 0 || nq64 > (1ll << 30))
            throw Error(SM_ERR_ARG, "bad point count");
        if (nq64 > 0 && (!queries || !outKnn || k < 1))
            throw Error(SM_ERR_ARG, "kNN queries need queries, out_knn and k >= 1");
        const int n = (int)n64, nq = (int)nq64;
        Ctx      &c = ctx->ctx;
        SM_CUDA(cudaSetDevice(c.device));
        const float *xyz = to_device(c, xyzIn, n, "kp.xyz");
        float4      *pos = c.arena.get<float4>("kp.pos", n);
        float4      *nrm = c.arena.get<float4>("kp.n4", n);
        int         *val = c.arena.get<int>("kp.valid", n);
        Box          box;
        const int    nvalid = prep_points(c, xyz, nullptr, n, pos, nrm, val, box);
        int         *valid  = c.arena.get<int>("kp.vids", n);
        compact_known(c, val, n, valid, "kp.cv");
        KdTree T;
        build_kdtree(c, pos, n, valid, nvalid, box, T, "kp.tree");
        if (outVacc) {
            std::vector<int> h(n, -1);
            if (nvalid)
                SM_CUDA(cudaMemcpy(h.data(), T.vacc, (size_t)nvalid * 4, cudaMemcpyDeviceToHost));
            memcpy(outVacc, h.data(), (size_t)n * 4);
        }
        if (step > 0 && outSampled) {
            int      *ids = c.arena.get<int>("kp.sampled", n);
            const int ns  = kd_sample(c, T, nullptr, pos, step, box, ids, nullptr, "kp.s");
            if (ns)
                SM_CUDA(cudaMemcpy(outSampled, ids, (size_t)ns * 4, cudaMemcpyDeviceToHost));
            if (outNSampled)
                *outNSampled = ns;
        }
        if (nq > 0) {
            float4 *q4 = c.arena.get<float4>("kp.q4", nq);
            float  *qd = c.arena.get<float>("kp.q", (size_t)nq * 3);
            SM_CUDA(cudaMemcpyAsync(qd, queries, (size_t)nq * 12, cudaMemcpyDefault, c.stream));
            k_f3_to_f4<<<nblocks(nq, 256), 256, 0, c.stream>>>(qd, nq, q4);
            SM_LAUNCH_CHECK();
            int   *cnt = c.arena.get<int>("kp.nq", 1);
            int   *nb  = c.arena.get<int>("kp.nb", (size_t)nq * k);
            float *nd  = c.arena.get<float>("kp.nd", (size_t)nq * k);
            SM_CUDA(cudaMemcpyAsync(cnt, &nq, sizeof(int), cudaMemcpyHostToDevice, c.stream));
            kd_knn(c, T, nullptr, pos, q4, nullptr, cnt, nq, k, nb, nd, nullptr);
            c.sync_checked();
            SM_CUDA(cudaMemcpy(outKnn, nb, (size_t)nq * k * 4, cudaMemcpyDeviceToHost));
            if (outKnnDist)
                SM_CUDA(cudaMemcpy(outKnnDist, nd, (size_t)nq * k * 4, cudaMemcpyDeviceToHost));
        }
        c.sync_checked();
    });
}

SM_API int sm_model_create(sm_context ctx, sm_model *out) {
    return guarded([&] {
        if (!ctx || !out)
            throw Error(SM_ERR_ARG, "NULL handle");
        sm_model m = new sm_model_s();
        m->ctx     = ctx;
        m->m.device = ctx->ctx.device;
        sm_train_param_default(&m->m.tp);
        *out = m;
    });
}

SM_API int sm_model_destroy(sm_model m) {
    return guarded([&] {
        if (!m)
            return;
        cudaSetDevice(m->m.device);
        m->m.free_device();
        delete m;
    });
}

SM_API int sm_model_train(sm_model m, const float *xyz, const float *normal, int64_t n,
                          float sdRel, const sm_train_param *param) {
    return guarded([&] {
        if (!m)
            throw Error(SM_ERR_ARG, "NULL model");
        sm_train_param tp;
        sm_train_param_default(&tp);
        if (param)
            tp = *param;
        SM_CUDA(cudaSetDevice(m->m.device));
        train(m->ctx->ctx, m->m, xyz, normal, n, sdRel, tp);
    });
}

SM_API int sm_model_upload(sm_model m, int64_t ns, const float *sxyz, const float *snrm,
                           int64_t nr, const float *rxyz, const float *rnrm, const float *box6,
                           int64_t nk, const uint32_t *keys, const uint32_t *offs,
                           const uint32_t *refs, const float *alphas, float sdRel,
                           const sm_train_param *param) {
    return guarded([&] {
        if (!m || !box6 || ns < 0 || nr < 0 || nk < 0 || (nk > 0 && (!keys || !offs)))
            throw Error(SM_ERR_ARG, "invalid model arrays");
        sm_train_param tp;
        sm_train_param_default(&tp);
        if (param)
            tp = *param;
        check_train_param(tp);
        SM_CUDA(cudaSetDevice(m->m.device));
        const int64_t ne = nk > 0 ? offs[nk] : 0;
        if ((ns > 0 && (!sxyz || !snrm)) || (nr > 0 && (!rxyz || !rnrm)) ||
            (ne > 0 && (!refs || !alphas)) || (nk > 0 && offs[0] != 0))
            throw Error(SM_ERR_ARG, "invalid model arrays");
        std::vector<float> sp(sxyz, sxyz + ns * 3), sn(snrm, snrm + ns * 3);
        std::vector<float> rp(rxyz, rxyz + nr * 3), rn(rnrm, rnrm + nr * 3);
        std::vector<uint32_t> K(keys, keys + nk), O(offs, offs + nk + 1), R(refs, refs + ne);
        std::vector<float>    AL(alphas, alphas + ne);
        for (int64_t b = 1; b < nk; b++)
            if (K[b] <= K[b - 1])
                throw Error(SM_ERR_ARG, "model keys must be strictly ascending");
        upload_model(m->m, sp, sn, rp, rn, box6, K, O, R, AL);
        m->m.sdRel = sdRel;
        m->m.tp    = tp;
    });
}

SM_API int sm_model_set_search_order(sm_model m, int order) {
    return guarded([&] {
        if (!m)
            throw Error(SM_ERR_ARG, "NULL model");
        if (order != SM_ORDER_GRID && order != SM_ORDER_REFERENCE)
            throw Error(SM_ERR_ARG, "unknown search order " + std::to_string(order));
        m->m.order = order;
    });
}

SM_API int sm_model_search_order(sm_model m) { return m ? m->m.order : -1; }

SM_API int sm_model_sizes(sm_model m, int64_t *sizes) {
    return guarded([&] {
        if (!m || !sizes)
            throw Error(SM_ERR_ARG, "NULL argument");
        sizes[0] = m->m.ns;
        sizes[1] = m->m.nr;
        sizes[2] = m->m.nkeys;
        sizes[3] = m->m.nentries;
    });
}

SM_API int sm_model_download(sm_model m, float *sxyz, float *snrm, float *rxyz, float *rnrm,
                             float *box6, uint32_t *keys, uint32_t *offs, uint32_t *refs,
                             float *alphas, float *sdRel, sm_train_param *param) {
    return guarded([&] {
        if (!m)
            throw Error(SM_ERR_ARG, "NULL model");
        if (!m->m.trained)
            throw Error(SM_ERR_RUNTIME, "No trained model in save");
        SM_CUDA(cudaSetDevice(m->m.device));
        m->m.ensure_host();
        const Model &M = m->m;
        auto cp = [](void *dst, const void *src, size_t b) {
            if (dst && b)
                memcpy(dst, src, b);
        };
        cp(sxyz, M.h_sp.data(), M.h_sp.size() * 4);
        cp(snrm, M.h_sn.data(), M.h_sn.size() * 4);
        cp(rxyz, M.h_rp.data(), M.h_rp.size() * 4);
        cp(rnrm, M.h_rn.data(), M.h_rn.size() * 4);
        if (box6)
            for (int a = 0; a < 3; a++) {
                box6[a]     = M.box.mn[a];
                box6[3 + a] = M.box.mx[a];
            }
        cp(keys, M.h_keys.data(), M.h_keys.size() * 4);
        cp(offs, M.h_offs.data(), M.h_offs.size() * 4);
        cp(refs, M.h_refs.data(), M.h_refs.size() * 4);
        cp(alphas, M.h_alphas.data(), M.h_alphas.size() * 4);
        if (sdRel)
            *sdRel = M.sdRel;
        if (param)
            *param = M.tp;
    });
}

// The reference's model file (ppf.cpp:512-547, serialize.cpp): magic, version,
// samplingDistanceRel, TrainParam field by field, the two clouds, then the hash table as
// (key, refInd[], alphaAngle[]) buckets.
SM_API int sm_model_save(sm_model m, const char *path) {
    return guarded([&] {
        if (!m || !path)
            throw Error(SM_ERR_ARG, "NULL argument");
        std::ofstream f(path, std::ios::out | std::ios::binary);
        if (!f.is_open())
            throw Error(SM_ERR_RUNTIME, std::string("failed to open file:") + path);
        if (!m->m.trained)
            throw Error(SM_ERR_RUNTIME, "No trained model in save");
        SM_CUDA(cudaSetDevice(m->m.device));
        m->m.ensure_host();
        const Model &M = m->m;
        std::string o;
        put<int>(o, kMagic);
        put<int>(o, kVersion);
        put<float>(o, M.sdRel);
        put<float>(o, M.tp.featDistanceStepRel);
        put<int>(o, M.tp.featAngleResolution);
        put<float>(o, M.tp.poseRefRelSamplingDistance);
        put<int>(o, M.tp.knnNormal);
        put<uint8_t>(o, (uint8_t)(M.tp.smoothNormal ? 1 : 0));
        const float b6[6] = {M.box.mn[0], M.box.mn[1], M.box.mn[2], M.box.mx[0], M.box.mx[1], M.box.mx[2]};
        put_cloud(o, M.h_sp, M.h_sn, b6);
        put_cloud(o, M.h_rp, M.h_rn, b6);
        put<uint32_t>(o, (uint32_t)M.h_keys.size());
        for (size_t b = 0; b < M.h_keys.size(); b++) {
            const uint32_t o0 = M.h_offs[b], o1 = M.h_offs[b + 1];
            put<uint32_t>(o, M.h_keys[b]);
            put<uint32_t>(o, o1 - o0);
            o.append((const char *)(M.h_refs.data() + o0), (size_t)(o1 - o0) * 4);
            put<uint32_t>(o, o1 - o0);
            o.append((const char *)(M.h_alphas.data() + o0), (size_t)(o1 - o0) * 4);
        }
        f.write(o.data(), (std::streamsize)o.size());
        if (!f)
            throw Error(SM_ERR_RUNTIME, std::string("failed to write file:") + path);
    });
}

SM_API int sm_model_load(sm_model m, const char *path) {
    return guarded([&] {
        if (!m || !path)
            throw Error(SM_ERR_ARG, "NULL argument");
        const std::string s = read_all(path);
        Reader            r{s};
        if (r.get<int>() != kMagic)
            throw Error(SM_ERR_RUNTIME, std::string("unsupported file format:") + path);
        r.get<int>(); // version
        const float    sdRel = r.get<float>();
        sm_train_param tp;
        tp.featDistanceStepRel        = r.get<float>();
        tp.featAngleResolution        = r.get<int>();
        tp.poseRefRelSamplingDistance = r.get<float>();
        tp.knnNormal                  = r.get<int>();
        tp.smoothNormal               = r.get<uint8_t>() ? 1 : 0;
        check_train_param(tp);
        float              box[6], rbox[6];
        std::vector<float> sp = r.vec3(), sn = r.vec3();
        for (float &b : box)
            b = r.get<float>();
        for (int i = 0; i < 3; i++)
            r.get<float>();
        std::vector<float> rp = r.vec3(), rn = r.vec3();
        for (float &b : rbox)
            b = r.get<float>();
        for (int i = 0; i < 3; i++)
            r.get<float>();
        if (sn.size() != sp.size() || rn.size() != rp.size())
            throw Error(SM_ERR_RUNTIME, std::string("corrupt model file:") + path);
        const uint32_t nb = r.get<uint32_t>();
        if ((size_t)nb * 12 > s.size() - r.p) // key and two counts per bucket at least
            throw Error(SM_ERR_RUNTIME, "truncated model file");
        struct B {
            uint32_t              key;
            std::vector<uint32_t> refs;
            std::vector<float>    al;
        };
        std::vector<B> bk(nb);
        for (uint32_t b = 0; b < nb; b++) {
            bk[b].key        = r.get<uint32_t>();
            const uint32_t n1 = r.get<uint32_t>();
            if ((size_t)n1 * 4 > s.size() - r.p)
                throw Error(SM_ERR_RUNTIME, "truncated model file");
            bk[b].refs.resize(n1);
            memcpy(bk[b].refs.data(), s.data() + r.p, (size_t)n1 * 4);
            r.p += (size_t)n1 * 4;
            const uint32_t n2 = r.get<uint32_t>();
            if (n2 != n1 || (size_t)n2 * 4 > s.size() - r.p)
                throw Error(SM_ERR_RUNTIME, std::string("corrupt model file:") + path);
            bk[b].al.resize(n2);
            memcpy(bk[b].al.data(), s.data() + r.p, (size_t)n2 * 4);
            r.p += (size_t)n2 * 4;
        }
        std::sort(bk.begin(), bk.end(), [](const B &a, const B &b) { return a.key < b.key; });
        std::vector<uint32_t> K, O, R;
        std::vector<float>    AL;
        O.push_back(0);
        for (size_t b = 0; b < bk.size(); b++) {
            if (b && bk[b].key == bk[b - 1].key)
                throw Error(SM_ERR_RUNTIME, std::string("corrupt model file:") + path);
            K.push_back(bk[b].key);
            R.insert(R.end(), bk[b].refs.begin(), bk[b].refs.end());
            AL.insert(AL.end(), bk[b].al.begin(), bk[b].al.end());
            O.push_back((uint32_t)R.size());
        }
        SM_CUDA(cudaSetDevice(m->m.device));
        upload_model(m->m, sp, sn, rp, rn, box, K, O, R, AL);
        m->m.sdRel = sdRel;
        m->m.tp    = tp;
    });
}

SM_API int sm_match(sm_model m, const float *xyz, const float *normal, int64_t n,
                    const float *viewpoint, float sdRel, float kpFrac, float minScore,
                    const sm_match_param *param, float *outPose, float *outScore, int *inoutCount,
                    sm_match_stats *stats) {
    return guarded([&] {
        if (!m || !inoutCount)
            throw Error(SM_ERR_ARG, "NULL argument");
        sm_match_param mp;
        sm_match_param_default(&mp);
        if (param)
            mp = *param;
        SM_CUDA(cudaSetDevice(m->m.device));
        MatchOutputs res;
        match(m->ctx->ctx, m->m, xyz, normal, n, viewpoint, sdRel, kpFrac, minScore, mp, res, stats,
              true);
        const int nres = (int)res.score.size();
        const int cap  = *inoutCount;
        *inoutCount    = nres;
        for (int i = 0; i < nres && i < cap; i++) {
            if (outPose) {
                for (int e = 0; e < 12; e++)
                    outPose[i * 16 + e] = res.pose[(size_t)i * 12 + e];
                outPose[i * 16 + 12] = 0.f;
                outPose[i * 16 + 13] = 0.f;
                outPose[i * 16 + 14] = 0.f;
                outPose[i * 16 + 15] = 1.f;
            }
            if (outScore)
                outScore[i] = res.score[i];
        }
        if (nres > cap)
            throw Error(SM_ERR_CAPACITY, "more results than the output capacity (" +
                                             std::to_string(nres) + " > " + std::to_string(cap) + ")");
    });
}

SM_API int sm_vote_stage(sm_model m, const float *points, const float *normals, int64_t n,
                         const int32_t *kp, int64_t K, const int32_t *nbrOff,
                         const int32_t *nbrIds, float minScore, int64_t *outStats,
                         float *outCands, float *outPoses, int dumpK, int32_t *outAcc) {
    return guarded([&] {
        if (!m || !points || !normals || !kp || !nbrOff || !nbrIds || !outStats || !outCands)
            throw Error(SM_ERR_ARG, "NULL argument");
        if (!m->m.trained)
            throw Error(SM_ERR_RUNTIME, "No trained model in matchScene");
        if (n <= 0 || n > (1ll << 30) || K < 0 || K > (1ll << 30))
            throw Error(SM_ERR_ARG, "bad point or keypoint count");
        // the CSR lists the kernels walk: offsets from 0, never decreasing
        if (nbrOff[0] != 0)
            throw Error(SM_ERR_ARG, "neighbour offsets must start at 0");
        for (int64_t k = 0; k < K; k++)
            if (nbrOff[k + 1] < nbrOff[k])
                throw Error(SM_ERR_ARG, "neighbour offsets must not decrease");
        Ctx &c = m->ctx->ctx;
        SM_CUDA(cudaSetDevice(m->m.device));
        const int    ni = (int)n, Ki = (int)K;
        const float *p3 = to_device(c, points, n, "v.p3");
        const float *n3 = to_device(c, normals, n, "v.n3");
        float4      *pos = c.arena.get<float4>("v.pos", std::max(ni, 1));
        float4      *nrm = c.arena.get<float4>("v.nrm", std::max(ni, 1));
        k_f3_to_f4<<<nblocks(ni, 256), 256, 0, c.stream>>>(p3, ni, pos);
        k_f3_to_f4<<<nblocks(ni, 256), 256, 0, c.stream>>>(n3, ni, nrm);
        SM_LAUNCH_CHECK();
        const int64_t tot  = nbrOff[K];
        int          *dkp  = c.arena.get<int>("v.kp", std::max(Ki, 1));
        int          *doff = c.arena.get<int>("v.off", Ki + 1);
        int          *dids = c.arena.get<int>("v.ids", std::max<int64_t>(tot, 1));
        for (int64_t i = 0; i < tot; i++)
            if (nbrIds[i] < 0 || nbrIds[i] >= n)
                throw Error(SM_ERR_ARG, "neighbour index out of range");
        for (int64_t i = 0; i < K; i++)
            if (kp[i] < 0 || kp[i] >= n)
                throw Error(SM_ERR_ARG, "keypoint index out of range");
        SM_CUDA(cudaMemcpyAsync(dkp, kp, K * 4, cudaMemcpyHostToDevice, c.stream));
        SM_CUDA(cudaMemcpyAsync(doff, nbrOff, (K + 1) * 4, cudaMemcpyHostToDevice, c.stream));
        SM_CUDA(cudaMemcpyAsync(dids, nbrIds, tot * 4, cudaMemcpyHostToDevice, c.stream));
        VoteOut vo;
        vo.stats  = c.arena.get<long long>("v.stats", (size_t)std::max(Ki, 1) * 8);
        vo.cands  = c.arena.get<float>("v.cands", (size_t)std::max(Ki, 1) * 9);
        vo.poses  = c.arena.get<float>("v.poses", (size_t)std::max(Ki, 1) * 3 * smi::kPoseFloats);
        vo.poseOk = c.arena.get<int>("v.poseok", (size_t)std::max(Ki, 1) * 3);
        const int dk = std::max(0, std::min(dumpK, Ki));
        vo.acc = (outAcc && dk) ? c.arena.get<int>("v.acc", (size_t)dk * m->m.ns * m->m.tp.featAngleResolution)
                                : nullptr;
        if (vo.acc)
            SM_CUDA(cudaMemsetAsync(vo.acc, 0, (size_t)dk * m->m.ns * m->m.tp.featAngleResolution * 4, c.stream));
        vote(c, m->m, pos, nrm, dkp, Ki, doff, dids, nullptr, 0, minScore, vo, dk);
        SM_CUDA(cudaMemcpyAsync(outStats, vo.stats, (size_t)K * 64, cudaMemcpyDeviceToHost, c.stream));
        SM_CUDA(cudaMemcpyAsync(outCands, vo.cands, (size_t)K * 36, cudaMemcpyDeviceToHost, c.stream));
        if (outPoses) {
            std::vector<float> ps((size_t)K * 3 * smi::kPoseFloats);
            std::vector<int>   ok((size_t)K * 3);
            SM_CUDA(cudaMemcpyAsync(ps.data(), vo.poses, ps.size() * 4, cudaMemcpyDeviceToHost, c.stream));
            SM_CUDA(cudaMemcpyAsync(ok.data(), vo.poseOk, ok.size() * 4, cudaMemcpyDeviceToHost, c.stream));
            c.sync();
            for (size_t i = 0; i < ok.size(); i++)
                for (int e = 0; e < smi::kPoseFloats; e++)
                    outPoses[i * smi::kPoseFloats + e] = ok[i] ? ps[i * smi::kPoseFloats + e] : 0.f;
        }
        if (vo.acc)
            SM_CUDA(cudaMemcpyAsync(outAcc, vo.acc, (size_t)dk * m->m.ns * m->m.tp.featAngleResolution * 4,
                                    cudaMemcpyDeviceToHost, c.stream));
        c.sync_checked();
    });
}

// Debug fields of the last sm_match (see the header for the field list).
static bool debug_field(sm_model m, int field, const void *&src, int64_t &count, size_t &elem) {
    Ctx &c = m->ctx->ctx;
    if (!c.last.valid)
        return false;
    auto get   = [&](const char *name) { return c.arena.get(name, 1); };
    Ctx &dc    = c.last.dense ? *c.last.dense : c;
    auto dense = [&](const char *name) { return dc.arena.get(name, 1); };
    switch (field) {
        case 0: src = get("m.sampled"); count = c.last.ns; elem = 4; return true;
        case 1: src = get("m.kp"); count = c.last.nk; elem = 4; return true;
        // the refinement scene and the final positions and normals
        case 2: src = dense("m.resampled"); count = c.last.nr; elem = 4; return true;
        case 3: src = dense("m.pos"); count = c.last.n; elem = 16; return true;
        case 4: src = dense("m.n4"); count = c.last.n; elem = 16; return true;
        case 7: src = get("m.kstats"); count = (int64_t)c.last.nk * 8; elem = 8; return true;
        case 8: src = get("m.kcands"); count = (int64_t)c.last.nk * 9; elem = 4; return true;
        case 9: src = get("m.plist"); count = (int64_t)c.last.np * smi::kPoseFloats; elem = 4; return true;
        case 10: src = get("m.cands"); count = (int64_t)c.last.ncand * smi::kPoseFloats; elem = 4; return true;
        case 12: src = get("m.cstat"); count = c.last.ncand; elem = 4; return true;
        case 13: src = get("m.cscore"); count = c.last.ncand; elem = 4; return true;
        case 14: src = get("m.cpose"); count = (int64_t)c.last.ncand * 12; elem = 4; return true;
        case 15: src = get("m.ctrace"); count = (int64_t)c.last.ncand * kIcpTraceFloats; elem = 4; return true;
    }
    return false;
}

SM_API int64_t sm_debug_size(sm_model m, int field) {
    if (!m)
        return -1;
    const void *src;
    int64_t     count;
    size_t      elem;
    if (!debug_field(m, field, src, count, elem))
        return -1;
    return (field == 3 || field == 4) ? count * 3 : count;
}

SM_API int sm_debug_get(sm_model m, int field, void *dst) {
    return guarded([&] {
        if (!m || !dst)
            throw Error(SM_ERR_ARG, "NULL argument");
        const void *src;
        int64_t     count;
        size_t      elem;
        if (!debug_field(m, field, src, count, elem))
            throw Error(SM_ERR_ARG, "no such debug field (or no match yet)");
        SM_CUDA(cudaSetDevice(m->m.device));
        m->ctx->ctx.sync();
        if (field == 3 || field == 4) {
            std::vector<float4> h(count);
            SM_CUDA(cudaMemcpy(h.data(), src, count * 16, cudaMemcpyDeviceToHost));
            float *d = (float *)dst;
            for (int64_t i = 0; i < count; i++) {
                d[3 * i]     = h[i].x;
                d[3 * i + 1] = h[i].y;
                d[3 * i + 2] = h[i].z;
            }
        } else if (count) {
            SM_CUDA(cudaMemcpy(dst, src, count * elem, cudaMemcpyDeviceToHost));
        }
    });
}

} // extern "C"
