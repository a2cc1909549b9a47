// oracle/ref_probe/kd_ref_probe.cpp - TEST INFRASTRUCTURE ONLY.
// Probe of the reference's own k-d tree: compiled against the reference's vendored,
// locally modified nanoflann (kdtree/kdtree.h + kdtree/nanoflann.hpp, included in place
// from the reference tree via -I) into oracle/_ref/, and used only to check that the
// oracle's restatement (oracle/kdtree.h) reproduces its build order, radius-search order
// and kNN results. Same C signatures as the oracle's orc_kd_probe / orc_kd_knn.
#include <array>
#include <cstdint>
#include <cstring>
#include <vector>

#include <kdtree.h>

using Pt   = std::array<float, 3>;
using Tree = KDTreeVectorOfVectorsAdaptor<std::vector<Pt>, float>;

extern "C" int64_t ref_kd_probe(const float *xyz, int64_t n, const float *box, const float *q,
                                float r2, int *vacc, int *found, int64_t maxFound) {
    std::vector<Pt> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    std::vector<Pt>  B = {{box[0], box[1], box[2]}, {box[3], box[4], box[5]}};
    std::vector<int> valid(n);
    for (int64_t i = 0; i < n; i++) valid[i] = (int)i;
    Tree t(P, 10, B, valid);
    for (int64_t i = 0; i < n; i++) vacc[i] = t.index->vAcc_[i];
    std::vector<nanoflann::ResultItem<int, float>> res;
    t.index->radiusSearch(q, r2, res, nanoflann::SearchParameters(0, false));
    for (int64_t i = 0; i < (int64_t)res.size() && i < maxFound; i++) found[i] = res[i].first;
    return (int64_t)res.size();
}

extern "C" void ref_kd_knn(const float *xyz, int64_t n, const float *box, const float *qs,
                           int64_t nq, int k, int *idx, float *dist) {
    std::vector<Pt> P(n);
    for (int64_t i = 0; i < n; i++) P[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    std::vector<Pt>  B = {{box[0], box[1], box[2]}, {box[3], box[4], box[5]}};
    std::vector<int> valid(n);
    for (int64_t i = 0; i < n; i++) valid[i] = (int)i;
    Tree t(P, 10, B, valid);
    for (int64_t j = 0; j < nq; j++)
        t.index->knnSearch(qs + 3 * j, k, idx + (int64_t)k * j, dist + (int64_t)k * j);
}
