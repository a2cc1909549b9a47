/*
 * surface_match.h - C ABI of the GB300 point-pair-feature matcher (libsurface_match.so).
 *
 * This is the drop-in boundary of the reference's ppf::Detector hot path. The reference
 * (SurfaceMan/surface_match) exports a C++ class only and lists a C API as a TODO
 * (TODO.md:4, apiExport.h:17-21 defines an unused API_DEMANGLED extern "C"); the entry
 * points below are that C API: plain pointers and sizes, status codes instead of
 * exceptions, every buffer owned by the caller. Each function names the reference
 * interface it replaces.
 *
 * Pointers to point data may be host or device (CUDA) pointers; the library detects the
 * kind and copies host data to the device itself. Coordinates are float32 xyz triples,
 * normals float32 triples (or NULL when absent).
 *
 * Errors map to the reference's exception types: SM_ERR_RANGE <-> std::range_error,
 * SM_ERR_RUNTIME <-> std::runtime_error (ppf.cpp:39-44,155-168,514-538; type.cpp:79-127).
 * sm_last_error() returns the message of the last failing call of the calling thread,
 * worded as the reference's exception message where one exists.
 */
#ifndef SURFACE_MATCH_H
#define SURFACE_MATCH_H

#include <stdint.h>

#if defined(__GNUC__)
#define SM_API __attribute__((visibility("default")))
#else
#define SM_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SM_OK 0
#define SM_ERR_RANGE 1    /* std::range_error in the reference */
#define SM_ERR_RUNTIME 2  /* std::runtime_error in the reference */
#define SM_ERR_CUDA 3     /* CUDA runtime failure */
#define SM_ERR_ARG 4      /* NULL handle / bad pointer / bad size */
#define SM_ERR_NOMEM 5    /* device allocation failed */
#define SM_ERR_CAPACITY 6 /* an internal capacity was exceeded (reported, never silent) */

/* search orders (sm_model_set_search_order) */
#define SM_ORDER_GRID 0      /* the GPU's grid order (fast; same rules, another visiting order) */
#define SM_ORDER_REFERENCE 1 /* the reference's k-d tree order (bit-exact with the reference's
                                single-threaded sampling, neighbour order and search pruning) */

typedef struct sm_context_s *sm_context; /* one device + one CUDA stream + workspace */
typedef struct sm_model_s *sm_model;     /* a trained model resident on the device */
typedef struct sm_server_s *sm_server;   /* a matchScene serving loop on one device */

/* ppf::TrainParam (type.h:39-74). */
typedef struct {
    float featDistanceStepRel;
    int   featAngleResolution;
    float poseRefRelSamplingDistance;
    int   knnNormal;
    int   smoothNormal;
} sm_train_param;

/* ppf::MatchParam (type.h:80-176). */
typedef struct {
    int   numMatches;
    int   knnNormal;
    int   smoothNormal;
    int   invertNormal;
    float maxOverlapDistRel;
    float maxOverlapDistAbs;
    int   sparsePoseRefinement;
    int   densePoseRefinement;
    int   poseRefNumSteps;
    float poseRefDistThresholdRel;
    float poseRefDistThresholdAbs;
    float poseRefScoringDistRel;
    float poseRefScoringDistAbs;
} sm_match_param;

/* Per-call statistics of sm_match (the reference prints these sizes, ppf.cpp:217-220). */
typedef struct {
    int64_t n_points;     /* input points */
    int64_t n_valid;      /* finite points (removeNan, util.cpp:86-105) */
    int64_t n_sampled;    /* sampled scene points */
    int64_t n_keypoints;  /* reference (key) points */
    int64_t n_resampled;  /* dense-refinement scene points */
    int64_t n_poses;      /* candidate poses from voting */
    int64_t n_clusters;   /* candidates after clustering */
    int64_t n_pairs;      /* point pairs evaluated (keypoint x neighbour) */
    int64_t n_hits;       /* pairs whose key is in the model table */
    int64_t n_votes;      /* votes cast: matched table entries (ppf.cpp:342-346) */
    float   ms[8];        /* stage device times (ms) on the context's stream: prep, sampling +
                             normals, keypoints, voting, clustering, refinement prep,
                             refinement, total. sm_match prepares the refinement on its
                             second stream beside keypoints, voting and clustering, so its
                             refinement-prep entry is the wait for that work */
    float   vote_ms[2];   /* device times (ms) of the voting stage's two main kernels: pair
                             features + table probes, shared-memory accumulation + peaks */
} sm_match_stats;

/* TrainParam / MatchParam defaults and constructor validation (type.cpp:71-127). */
SM_API void sm_train_param_default(sm_train_param *p);
SM_API void sm_match_param_default(sm_match_param *p);
SM_API int  sm_train_param_check(const sm_train_param *p);
SM_API int  sm_match_param_check(const sm_match_param *p);

/* Context: device ordinal, optional external cudaStream_t (NULL = the library creates
 * its own non-blocking stream). sm_match also uses a second stream and workspace of the
 * context (created on its first call, at the device's highest stream priority, released
 * with the context), ordered after the context's stream. A context serves one host thread
 * at a time. Replaces nothing in the reference (its runtime is OpenMP, ppf.cpp:26-31). */
SM_API int sm_context_create(int device, void *cuda_stream, sm_context *out);
SM_API int sm_context_destroy(sm_context ctx);
SM_API int sm_context_synchronize(sm_context ctx);
SM_API void *sm_context_stream(sm_context ctx);
/* Device bytes the context's workspace holds (both of its streams' workspaces). It grows on
 * demand and is reused across calls; no counterpart in the reference. */
SM_API int sm_context_workspace_bytes(sm_context ctx, int64_t *bytes);
/* Opt-in per-launch timing of the matching path's latency-bound kernels, for throughput
 * reports: on != 0 resets the counters and records a CUDA event pair around each launch of
 * them on their stream from then on; 0 stops. No counterpart in the reference. */
SM_API int sm_context_kernel_clock(sm_context ctx, int on);
/* Totals since the clock was switched on for kernel `kind` (SM_KERNEL_*): summed launch
 * durations, algorithmic bytes (per kind: SM_KERNEL_SAMPLE_PHASE 20 per sampled point,
 * SM_KERNEL_SCAN 8 per value, SM_KERNEL_CORR 88 per searched (candidate, source point)) and
 * launches. */
#define SM_KERNEL_SAMPLE_PHASE 0
#define SM_KERNEL_SCAN 1
#define SM_KERNEL_CORR 2
/* the refinement's other per-iteration launches (durations and launches only) */
#define SM_KERNEL_FIT 3
#define SM_KERNEL_RESID 4
#define SM_KERNEL_UPDATE 5
SM_API int sm_context_kernel_report(sm_context ctx, int kind, double *ms, double *bytes,
                                    int64_t *launches);

/* Model handle (ppf::Detector::IMPL, privateType.h:56-66). */
SM_API int sm_model_create(sm_context ctx, sm_model *out);
SM_API int sm_model_destroy(sm_model model);

/* ppf::Detector::trainModel (ppf.h:25-26, ppf.cpp:36-147). xyz/normal: n x 3 floats,
 * normal may be NULL (normals are then estimated). */
SM_API int sm_model_train(sm_model model, const float *xyz, const float *normal, int64_t n,
                          float samplingDistanceRel, const sm_train_param *param);

/* Load a model given as arrays (the state ppf::Detector::load reads, ppf.cpp:529-547):
 * sampled and resampled clouds with normals, the model box (min xyz, max xyz), and the
 * hash table as ascending keys, bucket offsets (nkeys + 1) and per-entry reference index
 * and alpha angle in insertion order. */
SM_API int sm_model_upload(sm_model model, int64_t n_sampled, const float *sampled_xyz,
                           const float *sampled_normal, int64_t n_resampled,
                           const float *resampled_xyz, const float *resampled_normal,
                           const float *box6, int64_t n_keys, const uint32_t *keys,
                           const uint32_t *offsets, const uint32_t *refs, const float *alphas,
                           float samplingDistanceRel, const sm_train_param *param);

/* Search order of the model's subsequent sm_model_train and sm_match calls (and of the
 * batch and serving entries on it). The reference samples clouds greedily in the leaf
 * order of its k-d tree and evaluates each keypoint's neighbours in the tree's depth-first
 * order, which decides which point pairs take its 8-lane SIMD quantisation and which its
 * scalar one (util.cpp:107-139, 765-827; ppf.cpp:273-346). SM_ORDER_REFERENCE builds that
 * tree on the GPU (nanoflann's middle-split rules) and follows its orders and its search
 * pruning in every search of the path: sampling, normals, voting lists, refinement and
 * scoring. SM_ORDER_GRID (default) applies the same rules in the order of uniform grids,
 * which is faster; the results are equally valid but not the same samples. */
SM_API int sm_model_set_search_order(sm_model model, int order);
SM_API int sm_model_search_order(sm_model model);

/* sizes[4] = {n_sampled, n_resampled, n_keys, n_entries} */
SM_API int sm_model_sizes(sm_model model, int64_t *sizes);
/* Copy the model out as arrays (same layout as sm_model_upload; any pointer may be NULL). */
SM_API int sm_model_download(sm_model model, float *sampled_xyz, float *sampled_normal,
                             float *resampled_xyz, float *resampled_normal, float *box6,
                             uint32_t *keys, uint32_t *offsets, uint32_t *refs, float *alphas,
                             float *samplingDistanceRel, sm_train_param *param);

/* ppf::Detector::save / load (ppf.cpp:512-547, serialize.cpp:5-186): the reference's
 * little-endian model file (magic 0x7F27F, version 100). */
SM_API int sm_model_save(sm_model model, const char *path);
SM_API int sm_model_load(sm_model model, const char *path);

/* ppf::Detector::matchScene (ppf.h:39-42, ppf.cpp:149-510).
 * xyz/normal: scene points (normal may be NULL: estimated). viewpoint: 3 floats or NULL
 * (PointCloud::viewPoint, type.h:28; NULL = not set). Results are written sorted by
 * score: out_pose[i*16..] a row-major 4x4 pose, out_score[i]; *inout_count holds the
 * capacity on entry and the number of results on return. stats may be NULL. The call
 * orders after the work already on the context's stream and returns when all of its own
 * work, on both of the context's streams, has finished. */
SM_API int sm_match(sm_model model, const float *xyz, const float *normal, int64_t n,
                    const float *viewpoint, float samplingDistanceRel, float keyPointFraction,
                    float minScore, const sm_match_param *param, float *out_pose,
                    float *out_score, int *inout_count, sm_match_stats *stats);

/* Batched ppf::Detector::matchScene (ppf.cpp:149-510) over njobs (scene, model) jobs of
 * uneven size: job j matches scene xyz[j] (n[j] points; normals[j] or NULL, normals may be
 * NULL as a whole; viewpoints[3*j] or viewpoints NULL) against models[j] (all on one
 * device). Up to `concurrency` jobs run at once, each on its own stream and workspace, so
 * their kernels overlap; results equal sm_match's for the same job. Outputs: out_pose
 * [njobs x max_results x 16], out_score [njobs x max_results], out_count[njobs],
 * out_status[njobs] (nullable, per-job status code), stats[njobs] (nullable). Returns
 * SM_OK, or the first failing job's status with its message in sm_last_error(). */
SM_API int sm_match_batch(int njobs, const sm_model *models, const float *const *xyz,
                          const float *const *normals, const int64_t *n,
                          const float *viewpoints, float samplingDistanceRel,
                          float keyPointFraction, float minScore, const sm_match_param *param,
                          int max_results, float *out_pose, float *out_score, int *out_count,
                          int *out_status, int concurrency, sm_match_stats *stats);

/* Serving (no counterpart in the reference, which matches one scene per call on the host).
 * A server keeps `slots` workers (each a CUDA stream + workspace) over resident models and
 * admits queued requests in arrival order as soon as a slot is free and the request's
 * estimated device footprint (64 MiB + 512 B per point) fits in hbm_budget_bytes next to
 * the requests in flight (a request larger than the budget runs alone). Admitted requests
 * run concurrently; each result equals sm_match's for the same scene and model. */
SM_API int sm_server_create(int device, int slots, int64_t hbm_budget_bytes, sm_server *out);
/* Finishes the queued and running requests, then stops the workers. */
SM_API int sm_server_destroy(sm_server server);
/* Queue a matchScene request; host inputs are copied (the caller may free them on return),
 * device inputs are read when the request runs and must stay valid until it is polled. */
SM_API int sm_server_submit(sm_server server, sm_model model, const float *xyz,
                            const float *normal, int64_t n, const float *viewpoint,
                            float samplingDistanceRel, float keyPointFraction, float minScore,
                            const sm_match_param *param, int64_t *out_request_id);
/* Collect up to max_requests finished requests (waiting up to wait_ms for the first):
 * ids, status codes, result counts, poses [k x max_results x 16], scores [k x max_results],
 * times_ms [k x 3] = queue, service and total milliseconds. *n_out = requests returned. */
SM_API int sm_server_poll(sm_server server, int max_requests, int max_results, int wait_ms,
                          int64_t *ids, int *status, int *counts, float *poses, float *scores,
                          double *times_ms, int *n_out);
/* out6 = {queued, running, completed, estimated bytes in flight, peak, budget} */
SM_API int sm_server_status(sm_server server, int64_t *out6);

/* Stage entry of the voting step (ppf.cpp:247-409) on caller-supplied scene state:
 * points/normals (n x 3), keypoint indices, and per-keypoint neighbour lists in search
 * order (nbr_off: K + 1 offsets into nbr_ids; each list contains the keypoint itself, as
 * the reference's radius search returns it). Outputs per keypoint: out_stats[K x 8] =
 * {neighbours, skipped (0 voted, 1 NaN normal, 2 below threshold), hits, votes,
 * accumulator fingerprint, n candidates, n poses, counter bound (sum over the hits of the
 * bucket's largest entry count of one reference point: a bound on every accumulator cell,
 * which picks 16- or 32-bit counters)}; out_cands[K x 9] = up to 3
 * (vote, ref, angle bin) triples (-1 padded); out_poses[K x 3 x 18] (nullable) = pose
 * 3x4, quaternion wxyz, rotation angle, votes. out_acc (nullable) receives the full
 * refNum x featAngleResolution accumulators of the first dump_k keypoints. */
SM_API int sm_vote_stage(sm_model model, const float *points, const float *normals, int64_t n,
                         const int32_t *keypoints, int64_t K, const int32_t *nbr_off,
                         const int32_t *nbr_ids, float minScore, int64_t *out_stats,
                         float *out_cands, float *out_poses, int dump_k, int32_t *out_acc);

/* sm_vote_stage for callers that cannot allocate device memory: a plugin inside a host
 * framework that owns all device memory and forbids allocation while its work runs, or a
 * latency-critical loop that cannot take cudaMalloc's implicit synchronisation. No
 * counterpart in the reference (its voting loop, ppf.cpp:247-409, allocates per call).
 * Same arguments, meaning and results as sm_vote_stage, except that every pointer is a
 * DEVICE pointer owned by the caller (nbr_ids holding nbr_off[K] entries), and out_poses
 * is required. The call runs on the model context's stream and does not wait for other
 * streams: the caller's device inputs must be complete (e.g. synchronised) before the
 * call. Offsets are validated before any list is read: off[0] must be 0, offsets must not
 * decrease and no list may be longer than n; nbr_off[K] entries must fit in the device
 * allocation that holds nbr_ids (checked with the driver's address range of that pointer);
 * then every id is checked. Violations return SM_ERR_ARG. The call allocates nothing: its
 * staging lives in a fixed array in the library's device image (about 4.8 MiB, held on
 * every GPU that loads the library until the process exits), which limits a call to
 * n <= 131072 points and K <= 65536 keypoints; larger sizes return SM_ERR_CAPACITY. The
 * first call on a device (and the first after the device's context is created anew)
 * resolves that array's address, so make it before any stream capture. All calls share
 * the array: calls whose GPU work overlaps race on it. Returns after the results are
 * written. */
SM_API int sm_vote_stage_noalloc(sm_model model, const float *points, const float *normals,
                                 int64_t n, const int32_t *keypoints, int64_t K,
                                 const int32_t *nbr_off, const int32_t *nbr_ids, float minScore,
                                 int64_t *out_stats, float *out_cands, float *out_poses,
                                 int dump_k, int32_t *out_acc);

/* Intermediate state of the last sm_match on this model's context, for inspection and
 * parity checks. Fields: 0 sampled ids, 1 keypoint ids, 2 resampled ids (int32);
 * 3 positions, 4 normals (float x3, after normal estimation); 7 per-keypoint stats
 * (int64 x8, as sm_vote_stage); 8 candidates (float x9); 9 pose list (float x18);
 * 10 clustered candidates (float x18); 12 candidate ICP status (int32: 0 accepted,
 * 1 votes, 2 sparse not converged, 3 sparse score, 4 dense not converged, 5 dense score);
 * 13 candidate score (float); 14 candidate pose (float x12); 15 ICP trace per candidate
 * (float x258: sparse then dense stage, 32 iterations x {pairs, mean distance, source
 * centroid x, step translation x}, then the sparse and dense inlier counts; -1 unused). */
SM_API int64_t sm_debug_size(sm_model model, int field);
SM_API int     sm_debug_get(sm_model model, int field, void *dst);

/* Reference-order k-d tree probe, for parity checks of the search order the reference
 * uses (KDTreeVectorOfVectorsAdaptor, kdtree/kdtree.h:65-79, over the vendored nanoflann:
 * middle-split build with leaves of 10, depth-first searches). Builds the tree over the
 * finite points of xyz (n x 3, host or device) with their tight box as root box and writes
 * out_vacc[n]: the point ids in tree order (-1 after the finite ones; nullable). With
 * step > 0, out_sampled receives samplePointCloud's result (util.cpp:107-139: greedy
 * thinning at `step` in tree order, the kept ids in that order; capacity n) and
 * *out_n_sampled its count. With nq > 0, out_knn[nq x k] receives the k nearest ids of each
 * query (nq x 3 floats) in the reference's order (distance, then first found) and
 * out_knn_dist (nullable) their squared distances. k <= 32. */
SM_API int sm_kdtree_probe(sm_context ctx, const float *xyz, int64_t n, float step,
                           int32_t *out_vacc, int32_t *out_sampled, int64_t *out_n_sampled,
                           const float *queries, int64_t nq, int k, int32_t *out_knn,
                           float *out_knn_dist);

/* Message of the last failing call on this thread ("" if none). */
SM_API const char *sm_last_error(void);

/* Library version string. */
SM_API const char *sm_version(void);

/* Number of CUDA kernels the library has launched so far in this process. */
SM_API int64_t sm_launch_count(void);

/* Page-locked (pinned) host memory for scene input (filePLY.cpp's reader fills pageable
 * vectors; no counterpart in the reference): a scene read into such a buffer is uploaded by
 * the matching calls as an asynchronous DMA on the context's stream instead of a staged
 * copy. *out = NULL for bytes == 0. Free with sm_host_free. */
SM_API int sm_host_alloc(int64_t bytes, void **out);
SM_API int sm_host_free(void *p);

/* The voting stage's launch tuner: on each device the first call with at least 512
 * keypoints times the vote accumulation kernel in six launch shapes on its own data - 256,
 * 512 or 1024 threads per CTA, one CTA per keypoint or a persistent resident grid taking
 * keypoints from a device work counter in LPT order (every shape computes the same votes,
 * peaks and candidates) - and keeps the fastest for the process. Writes the chosen CTA size
 * (0 while untuned) and whether it is the persistent grid. SM_VOTE_SHAPE=256|512|1024, with a
 * trailing 'p' for the persistent grid, in the environment fixes the shape instead. */
SM_API int sm_vote_tuned_shape(int device, int *threads_per_cta, int *persistent);

/* Measured rate of the vote stage's bounding operation on `device`: shared-memory atomic
 * increments of 16-bit counters at pseudo-random cells of a 48 KB accumulator, 512-thread
 * CTAs, two per SM (the vote kernel's shape). Writes increments per second (whole GPU).
 * Used as the denominator of the vote kernel's roofline; no counterpart in the reference. */
SM_API int sm_probe_vote_atomics(int device, double *atomics_per_second);

/* Moving-least-squares normals and surface projection (estimateNormalMLS,
 * privateUtil.h:13, util.cpp:336-457; the reference declares it privately and builds the
 * k-d tree it takes from the cloud). For each point that `indices` lists (n_indices of
 * them, host int64 in [0, n); NULL: every point) and that has at least 3 finite points
 * closer than |radius|: the PCA plane of those neighbours, a weighted least-squares fit of
 * the polynomial of total degree `order` (1..4) over the plane, and the point moved onto
 * the fit with its normal, oriented toward view_point (3 floats; NULL or non-finite: +z)
 * and reversed when `invert`. out_xyz and out_normal (n x 3, host or device) receive the
 * input points and normals (NaN where `normal` is NULL) with the listed points' results in
 * place; points that stop after the PCA step (order <= 1 with fewer neighbours than
 * coefficients, or a fit that is not positive definite) get the PCA normal and keep their
 * position. Neighbourhoods are read from the input positions (the reference moves points
 * in place while other threads read them). SM_ERR_ARG: order outside 1..4 (the
 * reference's order 0 reads past its coefficient vector), a non-finite radius or an index
 * out of range. */
SM_API int sm_estimate_normals_mls(sm_context ctx, const float *xyz, const float *normal,
                                   int64_t n, const int64_t *indices, int64_t n_indices,
                                   float radius, int order, int invert,
                                   const float *view_point, float *out_xyz,
                                   float *out_normal);

#ifdef __cplusplus
}
#endif

#endif /* SURFACE_MATCH_H */
