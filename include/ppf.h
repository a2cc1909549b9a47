/*
 * ppf.h - drop-in C++ ppf::Detector over the C ABI of libsurface_match.so.
 *
 * Mirrors the reference's public C++ API (ppf.h:10-62, type.h:8-181): the same class,
 * method names, parameter structs, defaults, validation and exception types, so user code
 * written against the reference (main.cpp:6-48, README.md:10-41) compiles unchanged. The
 * work runs on the GPU through surface_match.h. Header-only, so the point and matrix
 * types are whatever the including code uses: Eigen's when <Eigen/Core> is available
 * (as with the reference), otherwise small stand-ins with the members the API needs.
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "surface_match.h"

#if __has_include(<Eigen/Core>) && !defined(PPF_NO_EIGEN)
#include <Eigen/Core>
namespace ppf {
using Vec3f = Eigen::Vector3f;
using Vec3i = Eigen::Vector3i;
using Mat4f = Eigen::Matrix4f;
} // namespace ppf
#define PPF_HAVE_EIGEN 1
#else
namespace ppf {
struct Vec3f {
    float v[3] = {0, 0, 0};
    Vec3f() = default;
    Vec3f(float x, float y, float z) : v{x, y, z} {}
    float       &operator[](int i) { return v[i]; }
    const float &operator[](int i) const { return v[i]; }
    float       &x() { return v[0]; }
    float       &y() { return v[1]; }
    float       &z() { return v[2]; }
    float        x() const { return v[0]; }
    float        y() const { return v[1]; }
    float        z() const { return v[2]; }
    float       *data() { return v; }
    const float *data() const { return v; }
};
struct Vec3i {
    int v[3] = {0, 0, 0};
    Vec3i() = default;
    Vec3i(int a, int b, int c) : v{a, b, c} {}
    int       &operator[](int i) { return v[i]; }
    const int &operator[](int i) const { return v[i]; }
};
struct Mat4f { // row-major storage, (r, c) access like Eigen
    float  m[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
    float &operator()(int r, int c) { return m[r * 4 + c]; }
    float  operator()(int r, int c) const { return m[r * 4 + c]; }
};
} // namespace ppf
#define PPF_HAVE_EIGEN 0
#endif

namespace ppf {

struct BoundingBox {
    Vec3f min, max;
    BoundingBox() : min(0, 0, 0), max(0, 0, 0) {}
    BoundingBox(Vec3f mn, Vec3f mx) : min(mn), max(mx) {}
    Vec3f size() const { return Vec3f(max[0] - min[0], max[1] - min[1], max[2] - min[2]); }
    Vec3f center() const {
        return Vec3f((min[0] + max[0]) / 2.f, (min[1] + max[1]) / 2.f, (min[2] + max[2]) / 2.f);
    }
    float diameter() const {
        const Vec3f s = size();
        return std::sqrt(s[0] * s[0] + (s[1] * s[1] + s[2] * s[2]));
    }
};

struct PointCloud {
    std::vector<Vec3f> point;
    std::vector<Vec3f> normal;
    std::vector<Vec3i> face;
    BoundingBox        box;
    Vec3f              viewPoint = Vec3f(NAN, NAN, NAN);
    bool        hasNormal() const { return !point.empty() && point.size() == normal.size(); }
    std::size_t size() const { return point.size(); }
    bool        empty() const { return point.empty(); }
};

namespace detail {
inline void check(int status) {
    if (status == SM_OK)
        return;
    const std::string msg = sm_last_error();
    if (status == SM_ERR_RANGE)
        throw std::range_error(msg);
    throw std::runtime_error(msg);
}
template <class V> std::vector<float> flat(const std::vector<V> &pts) {
    std::vector<float> f(pts.size() * 3);
    for (std::size_t i = 0; i < pts.size(); i++)
        for (int a = 0; a < 3; a++)
            f[3 * i + a] = pts[i][a];
    return f;
}
} // namespace detail

struct TrainParam {
    float featDistanceStepRel;
    int   featAngleResolution;
    float poseRefRelSamplingDistance;
    int   knnNormal;
    bool  smoothNormal;
    explicit TrainParam(float featDistanceStepRel_ = 0.04f, int featAngleResolution_ = 30,
                        float poseRefRelSamplingDistance_ = 0.01f, int knnNormal_ = 10,
                        bool smoothNormal_ = true)
        : featDistanceStepRel(featDistanceStepRel_), featAngleResolution(featAngleResolution_),
          poseRefRelSamplingDistance(poseRefRelSamplingDistance_), knnNormal(knnNormal_),
          smoothNormal(smoothNormal_) {
        sm_train_param p = c();
        detail::check(sm_train_param_check(&p));
    }
    sm_train_param c() const {
        return sm_train_param{featDistanceStepRel, featAngleResolution, poseRefRelSamplingDistance,
                              knnNormal, smoothNormal ? 1 : 0};
    }
};

struct MatchParam {
    int   numMatches;
    int   knnNormal;
    bool  smoothNormal;
    bool  invertNormal;
    float maxOverlapDistRel;
    float maxOverlapDistAbs;
    bool  sparsePoseRefinement;
    bool  densePoseRefinement;
    int   poseRefNumSteps;
    float poseRefDistThresholdRel;
    float poseRefDistThresholdAbs;
    float poseRefScoringDistRel;
    float poseRefScoringDistAbs;
    explicit MatchParam(int numMatches_ = 1, int knnNormal_ = 10, bool smoothNormal_ = true,
                        bool invertNormal_ = false, float maxOverlapDistRel_ = 0.5f,
                        float maxOverlapDistAbs_ = 0, bool sparsePoseRefinement_ = true,
                        bool densePoseRefinement_ = true, int poseRefNumSteps_ = 5,
                        float poseRefDistThresholdRel_ = 0.1f, float poseRefDistThresholdAbs_ = 0,
                        float poseRefScoringDistRel_ = 0.01f, float poseRefScoringDistAbs_ = 0)
        : numMatches(numMatches_), knnNormal(knnNormal_), smoothNormal(smoothNormal_),
          invertNormal(invertNormal_), maxOverlapDistRel(maxOverlapDistRel_),
          maxOverlapDistAbs(maxOverlapDistAbs_), sparsePoseRefinement(sparsePoseRefinement_),
          densePoseRefinement(densePoseRefinement_), poseRefNumSteps(poseRefNumSteps_),
          poseRefDistThresholdRel(poseRefDistThresholdRel_),
          poseRefDistThresholdAbs(poseRefDistThresholdAbs_),
          poseRefScoringDistRel(poseRefScoringDistRel_),
          poseRefScoringDistAbs(poseRefScoringDistAbs_) {
        sm_match_param p = c();
        detail::check(sm_match_param_check(&p));
    }
    sm_match_param c() const {
        return sm_match_param{numMatches, knnNormal, smoothNormal ? 1 : 0, invertNormal ? 1 : 0,
                              maxOverlapDistRel, maxOverlapDistAbs, sparsePoseRefinement ? 1 : 0,
                              densePoseRefinement ? 1 : 0, poseRefNumSteps,
                              poseRefDistThresholdRel, poseRefDistThresholdAbs,
                              poseRefScoringDistRel, poseRefScoringDistAbs};
    }
};

struct MatchResult {
    PointCloud sampledScene;
    PointCloud keyPoint;
};

// Search order of a Detector (extension; the reference has one order, its k-d tree's).
// Reference: the reference's k-d tree built on the GPU, its sampling order, neighbour order
// and search pruning - results bit-identical to the reference algorithm run single-threaded.
// Grid (default): the same rules in uniform-grid order, several times faster; equally valid
// samples, not the same ones. See sm_model_set_search_order.
enum class SearchOrder { Grid = SM_ORDER_GRID, Reference = SM_ORDER_REFERENCE };

class Detector {
public:
    Detector() = default;
    explicit Detector(SearchOrder order) : order_(order) {}
    ~Detector() {
        if (model_)
            sm_model_destroy(model_);
        if (ctx_)
            sm_context_destroy(ctx_);
    }
    Detector(const Detector &)            = delete;
    Detector &operator=(const Detector &) = delete;

    void trainModel(const PointCloud &model, float samplingDistanceRel = 0.04f,
                    TrainParam param = TrainParam()) {
        if (samplingDistanceRel > 1 || samplingDistanceRel < 0)
            throw std::range_error("Invalid Input: samplingDistanceRel range mismatch in trainModel");
        if (model.point.empty())
            throw std::runtime_error("Invalid Input: empty model in trainModel");
        ensure();
        const std::vector<float> xyz = detail::flat(model.point);
        std::vector<float>       nrm;
        if (model.hasNormal())
            nrm = detail::flat(model.normal);
        const sm_train_param p = param.c();
        detail::check(sm_model_train(model_, xyz.data(), nrm.empty() ? nullptr : nrm.data(),
                                     (int64_t)model.point.size(), samplingDistanceRel, &p));
        trained_ = true;
    }

    void matchScene(const PointCloud &scene, std::vector<Mat4f> &pose, std::vector<float> &score,
                    float samplingDistanceRel = 0.04f, float keyPointFraction = 0.2f,
                    float minScore = 0.2f, MatchParam param = MatchParam(),
                    MatchResult *matchResult = nullptr) {
        if (!trained_)
            throw std::runtime_error("No trained model in matchScene");
        const std::vector<float> xyz = detail::flat(scene.point);
        std::vector<float>       nrm;
        if (scene.hasNormal())
            nrm = detail::flat(scene.normal);
        const float vp[3] = {scene.viewPoint[0], scene.viewPoint[1], scene.viewPoint[2]};
        const bool  hasVp = std::isfinite(vp[0]) && std::isfinite(vp[1]) && std::isfinite(vp[2]);
        const sm_match_param p = param.c();
        int                cap = param.numMatches;
        std::vector<float> P((size_t)cap * 16), S(cap);
        detail::check(sm_match(model_, xyz.empty() ? nullptr : xyz.data(),
                               nrm.empty() ? nullptr : nrm.data(), (int64_t)scene.point.size(),
                               hasVp ? vp : nullptr, samplingDistanceRel, keyPointFraction,
                               minScore, &p, P.data(), S.data(), &cap, nullptr));
        pose.resize(cap);
        score.resize(cap);
        for (int i = 0; i < cap; i++) {
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++)
                    pose[i](r, c) = P[(size_t)i * 16 + r * 4 + c];
            score[i] = S[i];
        }
        if (matchResult)
            fill_result(scene, *matchResult);
    }

    // Applies to later trainModel and matchScene calls.
    void setSearchOrder(SearchOrder order) {
        order_ = order;
        if (model_)
            detail::check(sm_model_set_search_order(model_, (int)order_));
    }
    SearchOrder searchOrder() const { return order_; }

    void save(const std::string &filename) const {
        if (!trained_)
            throw std::runtime_error("No trained model in save");
        detail::check(sm_model_save(model_, filename.c_str()));
    }

    void load(const std::string &filename) {
        ensure();
        detail::check(sm_model_load(model_, filename.c_str()));
        trained_ = true;
    }

private:
    void ensure() {
        if (!ctx_)
            detail::check(sm_context_create(0, nullptr, &ctx_));
        if (!model_) {
            detail::check(sm_model_create(ctx_, &model_));
            detail::check(sm_model_set_search_order(model_, (int)order_));
        }
    }
    void fill_result(const PointCloud &scene, MatchResult &r) {
        auto ids = [&](int field) {
            const int64_t        n = sm_debug_size(model_, field);
            std::vector<int32_t> v(n > 0 ? n : 0);
            if (n > 0)
                detail::check(sm_debug_get(model_, field, v.data()));
            return v;
        };
        const int64_t      np = sm_debug_size(model_, 3);
        std::vector<float> P(np > 0 ? np : 0), N(np > 0 ? np : 0);
        if (np > 0) {
            detail::check(sm_debug_get(model_, 3, P.data()));
            detail::check(sm_debug_get(model_, 4, N.data()));
        }
        auto extract = [&](const std::vector<int32_t> &idx, PointCloud &out) {
            out       = PointCloud();
            out.box   = scene.box;
            for (int32_t i : idx) {
                out.point.emplace_back(P[3 * (size_t)i], P[3 * (size_t)i + 1], P[3 * (size_t)i + 2]);
                Vec3f n(N[3 * (size_t)i], N[3 * (size_t)i + 1], N[3 * (size_t)i + 2]);
                const float s = std::sqrt(n[0] * n[0] + (n[1] * n[1] + n[2] * n[2]));
                if (s > 0)
                    n = Vec3f(n[0] / s, n[1] / s, n[2] / s);
                out.normal.push_back(n);
            }
        };
        extract(ids(1), r.keyPoint);
        extract(ids(0), r.sampledScene);
    }
    sm_context  ctx_     = nullptr;
    sm_model    model_   = nullptr;
    bool        trained_ = false;
    SearchOrder order_   = SearchOrder::Grid;
};

// estimateNormalMLS (privateUtil.h:13, util.cpp:336-457) on the device: moving-least-squares
// normals and projected points of the listed points (all when `indices` is empty), in
// place, oriented toward pc.viewPoint (or +z) and reversed when `invert`; normals are
// created as NaN when the cloud has none. The reference passes the k-d tree to search; the
// device builds its own search structure over the cloud's finite points. `order` is 1..4.
inline void estimateNormalMLS(PointCloud &pc, const std::vector<std::size_t> &indices, float radius,
                              int order, bool invert = false) {
    if (pc.point.empty())
        return;
    const std::size_t        n   = pc.point.size();
    const std::vector<float> xyz = detail::flat(pc.point);
    std::vector<float>       nrm;
    if (pc.hasNormal())
        nrm = detail::flat(pc.normal);
    std::vector<int64_t> idx(indices.begin(), indices.end());
    std::vector<float>   outP(n * 3), outN(n * 3);
    const float vp[3] = {pc.viewPoint[0], pc.viewPoint[1], pc.viewPoint[2]};
    sm_context  ctx   = nullptr;
    detail::check(sm_context_create(0, nullptr, &ctx));
    const int st = sm_estimate_normals_mls(ctx, xyz.data(), nrm.empty() ? nullptr : nrm.data(),
                                           (int64_t)n, idx.empty() ? nullptr : idx.data(),
                                           (int64_t)idx.size(), radius, order, invert ? 1 : 0, vp,
                                           outP.data(), outN.data());
    sm_context_destroy(ctx);
    detail::check(st);
    pc.normal.resize(n);
    for (std::size_t i = 0; i < n; i++) {
        pc.point[i]  = Vec3f(outP[3 * i], outP[3 * i + 1], outP[3 * i + 2]);
        pc.normal[i] = Vec3f(outN[3 * i], outN[3 * i + 1], outN[3 * i + 2]);
    }
}

} // namespace ppf
