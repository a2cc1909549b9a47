"""Python mirror of the reference's ppf::Detector (ppf.h:10-62) over the C ABI.

Same method names, argument meaning, defaults and error behaviour as the reference:
``RangeError`` (a ``ValueError``) where the reference throws std::range_error and
``RuntimeError`` where it throws std::runtime_error. Point clouds are numpy arrays of
shape (n, 3) float32 (host) or device arrays exposing ``data_ptr()``; poses come back as
(k, 4, 4) float32 matrices sorted by score.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import MatchParamC, MatchStatsC, TrainParamC


class RangeError(ValueError):
    """std::range_error of the reference."""


def _check(status):
    if status == _lib.SM_OK:
        return
    msg = _lib.last_error()
    if status == _lib.SM_ERR_RANGE:
        raise RangeError(msg)
    raise RuntimeError(msg)


class _PinnedBlock:
    """Page-locked host memory from sm_host_alloc, freed with the last array that views it."""

    def __init__(self, nbytes: int):
        p = C.c_void_p()
        _check(_lib.load().sm_host_alloc(int(nbytes), C.byref(p)))
        self.ptr = p.value
        self.nbytes = int(nbytes)

    def __del__(self):
        if getattr(self, "ptr", None):
            try:
                _lib.load().sm_host_free(C.c_void_p(self.ptr))
            except Exception:
                pass
            self.ptr = None


def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory (sm_host_alloc): scenes read into it are
    uploaded by matchScene as an asynchronous DMA on the context's stream."""
    dt = np.dtype(dtype)
    n = int(np.prod(shape))
    nbytes = max(n * dt.itemsize, 1)
    blk = _PinnedBlock(nbytes)
    buf = (C.c_char * nbytes).from_address(blk.ptr)
    buf._sm_pinned_block = blk  # the array's buffer keeps the block alive
    return np.frombuffer(buf, dtype=dt, count=n).reshape(shape)


def probe_vote_atomics(device: int = 0) -> float:
    """Measured shared-memory atomic increments per second of the vote kernel's access
    pattern on `device` (include/surface_match.h sm_probe_vote_atomics)."""
    out = C.c_double(0.0)
    _check(_lib.load().sm_probe_vote_atomics(int(device), C.byref(out)))
    return float(out.value)


def estimateNormalMLS(pc: "PointCloud", indices=None, radius: float = 1.0, order: int = 2,
                      invert: bool = False, context: "Context | None" = None) -> "PointCloud":
    """estimateNormalMLS (util.cpp:336-457) on the GPU (sm_estimate_normals_mls): for the
    listed points (None: all) with at least 3 finite neighbours closer than |radius|, a PCA
    plane, a weighted polynomial fit of total degree `order` (1..4) over it, the point moved
    onto the fit and its normal oriented toward ``pc.viewPoint`` (or +z; reversed when
    `invert`). Like the reference it updates ``pc.point`` and ``pc.normal`` in place (normals
    are created as NaN when the cloud has none) and returns `pc`. The reference takes the
    k-d tree to search as an argument; here the search structure is built on the device."""
    L = _lib.load()
    own = context is None
    ctx = Context() if own else context
    try:
        pts = np.ascontiguousarray(pc.point, dtype=np.float32).reshape(-1, 3)
        n = len(pts)
        nrm = None if pc.normal is None else np.ascontiguousarray(pc.normal, dtype=np.float32)
        idx = None if indices is None else np.ascontiguousarray(indices, dtype=np.int64)
        vp = None if pc.viewPoint is None else np.ascontiguousarray(pc.viewPoint, np.float32)
        out_p = np.empty((n, 3), np.float32)
        out_n = np.empty((n, 3), np.float32)
        f32 = C.POINTER(C.c_float)
        _check(L.sm_estimate_normals_mls(
            ctx.handle, pts.ctypes.data_as(f32), None if nrm is None else nrm.ctypes.data_as(f32),
            n, None if idx is None else idx.ctypes.data_as(C.POINTER(C.c_int64)),
            0 if idx is None else len(idx), float(radius), int(order), 1 if invert else 0,
            None if vp is None else vp.ctypes.data_as(f32), out_p.ctypes.data_as(f32),
            out_n.ctypes.data_as(f32)))
    finally:
        if own:
            ctx.close()
    pc.point = out_p
    pc.normal = out_n
    return pc


@dataclass
class TrainParam:
    """ppf::TrainParam (type.h:39-74); validated on construction (type.cpp:71-88)."""
    featDistanceStepRel: float = 0.04
    featAngleResolution: int = 30
    poseRefRelSamplingDistance: float = 0.01
    knnNormal: int = 10
    smoothNormal: bool = True

    def __post_init__(self):
        _check(_lib.load().sm_train_param_check(C.byref(self.c())))

    def c(self):
        return TrainParamC(self.featDistanceStepRel, self.featAngleResolution,
                           self.poseRefRelSamplingDistance, self.knnNormal,
                           int(self.smoothNormal))


@dataclass
class MatchParam:
    """ppf::MatchParam (type.h:80-176); validated on construction (type.cpp:90-127)."""
    numMatches: int = 1
    knnNormal: int = 10
    smoothNormal: bool = True
    invertNormal: bool = False
    maxOverlapDistRel: float = 0.5
    maxOverlapDistAbs: float = 0.0
    sparsePoseRefinement: bool = True
    densePoseRefinement: bool = True
    poseRefNumSteps: int = 5
    poseRefDistThresholdRel: float = 0.1
    poseRefDistThresholdAbs: float = 0.0
    poseRefScoringDistRel: float = 0.01
    poseRefScoringDistAbs: float = 0.0

    def __post_init__(self):
        _check(_lib.load().sm_match_param_check(C.byref(self.c())))

    def c(self):
        return MatchParamC(self.numMatches, self.knnNormal, int(self.smoothNormal),
                           int(self.invertNormal), self.maxOverlapDistRel,
                           self.maxOverlapDistAbs, int(self.sparsePoseRefinement),
                           int(self.densePoseRefinement), self.poseRefNumSteps,
                           self.poseRefDistThresholdRel, self.poseRefDistThresholdAbs,
                           self.poseRefScoringDistRel, self.poseRefScoringDistAbs)


@dataclass
class PointCloud:
    """ppf::PointCloud (type.h:22-33): points, optional normals, optional viewpoint,
    optional triangles (mesh models read from PLY files)."""
    point: object
    normal: object = None
    viewPoint: object = None
    face: object = None


@dataclass
class MatchResult:
    """ppf::MatchResult (type.h:178-181)."""
    sampledScene: PointCloud = None
    keyPoint: PointCloud = None
    stats: dict = field(default_factory=dict)


def _ptr(a):
    """(ctypes float pointer, keepalive) of a numpy array or a device tensor."""
    if a is None:
        return None, None
    if hasattr(a, "data_ptr"):  # device tensor (float32, contiguous, n x 3)
        return C.cast(C.c_void_p(a.data_ptr()), C.POINTER(C.c_float)), a
    arr = np.ascontiguousarray(a, dtype=np.float32)
    return arr.ctypes.data_as(C.POINTER(C.c_float)), arr


def _len(a):
    return int(a.shape[0])


class Context:
    """A device, a CUDA stream and the library's workspace."""

    def __init__(self, device: int = 0, stream: int | None = None):
        L = _lib.load()
        h = C.c_void_p()
        _check(L.sm_context_create(device, C.c_void_p(stream) if stream else None, C.byref(h)))
        self.handle = h
        self.device = device

    @property
    def stream(self) -> int:
        return _lib.load().sm_context_stream(self.handle) or 0

    def synchronize(self):
        _check(_lib.load().sm_context_synchronize(self.handle))

    KERNELS = ("k_sample_phase", "k_scan_lookback", "k_corr", "k_fit", "k_resid", "k_update")

    def kernel_clock(self, on: bool = True):
        """Start (counters reset) or stop per-launch event timing of the latency-bound
        kernels (sm_context_kernel_clock)."""
        _check(_lib.load().sm_context_kernel_clock(self.handle, 1 if on else 0))

    def kernel_report(self) -> dict:
        """{kernel: {"ms", "bytes", "launches"}} since the clock was started."""
        L = _lib.load()
        out = {}
        for kind, name in enumerate(self.KERNELS):
            ms, b, n = C.c_double(), C.c_double(), C.c_int64()
            _check(L.sm_context_kernel_report(self.handle, kind, C.byref(ms), C.byref(b),
                                              C.byref(n)))
            out[name] = {"ms": ms.value, "bytes": b.value, "launches": n.value}
        return out

    def close(self):
        if self.handle:
            _lib.load().sm_context_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Detector:
    """GPU ppf::Detector: trainModel / matchScene / save / load."""

    def __init__(self, context: Context | None = None, device: int = 0,
                 search_order: str = "grid"):
        """search_order: "grid" (the GPU's fast orders) or "reference" (the reference's k-d
        tree orders and search pruning, see sm_model_set_search_order)."""
        self.ctx = context or Context(device)
        self._own_ctx = context is None
        h = C.c_void_p()
        _check(_lib.load().sm_model_create(self.ctx.handle, C.byref(h)))
        self.model = h
        self.trained = False
        self.last_stats = None
        self.set_search_order(search_order)

    def set_search_order(self, order: str):
        codes = {"grid": _lib.SM_ORDER_GRID, "reference": _lib.SM_ORDER_REFERENCE}
        if order not in codes:
            raise ValueError(f"search_order must be one of {sorted(codes)}")
        _check(_lib.load().sm_model_set_search_order(self.model, codes[order]))
        self.search_order = order

    def close(self):
        if getattr(self, "model", None):
            _lib.load().sm_model_destroy(self.model)
            self.model = None
        if self._own_ctx and getattr(self, "ctx", None):
            self.ctx.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- ppf::Detector API ------------------------------------------------------------
    def trainModel(self, model: PointCloud, samplingDistanceRel: float = 0.04,
                   param: TrainParam | None = None):
        param = param or TrainParam()
        p, keep = _ptr(model.point)
        nrm, keep2 = _ptr(model.normal)
        n = _len(model.point) if model.point is not None else 0
        _check(_lib.load().sm_model_train(self.model, p, nrm, n, samplingDistanceRel,
                                          C.byref(param.c())))
        self.trained = True

    def matchScene(self, scene: PointCloud, samplingDistanceRel: float = 0.04,
                   keyPointFraction: float = 0.2, minScore: float = 0.2,
                   param: MatchParam | None = None, matchResult: MatchResult | None = None):
        """Returns (poses (k, 4, 4), scores (k,)), sorted by score."""
        param = param or MatchParam()
        p, keep = _ptr(scene.point)
        nrm, keep2 = _ptr(scene.normal)
        n = _len(scene.point) if scene.point is not None else 0
        vp = None
        if scene.viewPoint is not None:
            vpa = np.ascontiguousarray(scene.viewPoint, np.float32)
            vp = vpa.ctypes.data_as(C.POINTER(C.c_float))
        cap = max(1, param.numMatches)
        poses = np.zeros((cap, 4, 4), np.float32)
        scores = np.zeros(cap, np.float32)
        count = C.c_int(cap)
        st = MatchStatsC()
        _check(_lib.load().sm_match(self.model, p, nrm, n, vp, samplingDistanceRel,
                                    keyPointFraction, minScore, C.byref(param.c()),
                                    poses.ctypes.data_as(C.POINTER(C.c_float)),
                                    scores.ctypes.data_as(C.POINTER(C.c_float)), C.byref(count),
                                    C.byref(st)))
        k = count.value
        self.last_stats = {f: getattr(st, f) for f, _ in MatchStatsC._fields_
                           if f not in ("ms", "vote_ms")}
        self.last_stats["ms"] = list(st.ms)
        self.last_stats["vote_ms"] = list(st.vote_ms)
        if matchResult is not None:
            pos = self.debug(3)
            nrm_ = self.debug(4)
            for name, fid in (("sampledScene", 0), ("keyPoint", 1)):
                ids = self.debug(fid)
                nn = nrm_[ids]
                nn = nn / np.maximum(np.linalg.norm(nn, axis=1, keepdims=True), 1e-30)
                setattr(matchResult, name, PointCloud(pos[ids], nn))
            matchResult.stats = dict(self.last_stats)
        return poses[:k], scores[:k]

    def save(self, filename: str):
        _check(_lib.load().sm_model_save(self.model, str(filename).encode()))

    def load(self, filename: str):
        _check(_lib.load().sm_model_load(self.model, str(filename).encode()))
        self.trained = True

    # snake_case aliases
    train_model = trainModel
    match_scene = matchScene

    # ---- model arrays -------------------------------------------------------------------
    def upload(self, sampled, sampled_normal, resampled, resampled_normal, box, keys, offsets,
               refs, alphas, sd_rel=0.04, param: TrainParam | None = None):
        """Load a model from arrays (e.g. a table built by the reference or the oracle)."""
        param = param or TrainParam()
        a = [np.ascontiguousarray(x, dt) for x, dt in (
            (sampled, np.float32), (sampled_normal, np.float32), (resampled, np.float32),
            (resampled_normal, np.float32), (box, np.float32), (keys, np.uint32),
            (offsets, np.uint32), (refs, np.uint32), (alphas, np.float32))]
        fp = lambda x: x.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
        up = lambda x: x.ctypes.data_as(C.POINTER(C.c_uint32))  # noqa: E731
        _check(_lib.load().sm_model_upload(self.model, len(a[0]), fp(a[0]), fp(a[1]), len(a[2]),
                                           fp(a[2]), fp(a[3]), fp(a[4]), len(a[5]), up(a[5]),
                                           up(a[6]), up(a[7]), fp(a[8]), sd_rel,
                                           C.byref(param.c())))
        self.trained = True

    def download(self):
        L = _lib.load()
        sz = np.zeros(4, np.int64)
        _check(L.sm_model_sizes(self.model, sz.ctypes.data_as(C.POINTER(C.c_int64))))
        ns, nr, nk, ne = (int(v) for v in sz)
        out = dict(sampled=np.zeros((ns, 3), np.float32),
                   sampled_normal=np.zeros((ns, 3), np.float32),
                   resampled=np.zeros((nr, 3), np.float32),
                   resampled_normal=np.zeros((nr, 3), np.float32), box=np.zeros(6, np.float32),
                   keys=np.zeros(nk, np.uint32), offsets=np.zeros(nk + 1, np.uint32),
                   refs=np.zeros(ne, np.uint32), alphas=np.zeros(ne, np.float32))
        sd = C.c_float()
        tp = TrainParamC()
        fp = lambda x: x.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
        up = lambda x: x.ctypes.data_as(C.POINTER(C.c_uint32))  # noqa: E731
        _check(L.sm_model_download(self.model, fp(out["sampled"]), fp(out["sampled_normal"]),
                                   fp(out["resampled"]), fp(out["resampled_normal"]),
                                   fp(out["box"]), up(out["keys"]), up(out["offsets"]),
                                   up(out["refs"]), fp(out["alphas"]), C.byref(sd), C.byref(tp)))
        out["sd_rel"] = sd.value
        return out

    # ---- stage entry and inspection -----------------------------------------------------
    def vote_stage(self, points, normals, keypoints, nbr_off, nbr_ids, min_score, dump_k=0):
        """The voting step on caller-supplied scene state (see sm_vote_stage)."""
        pts = np.ascontiguousarray(points, np.float32)
        nrm = np.ascontiguousarray(normals, np.float32)
        kp = np.ascontiguousarray(keypoints, np.int32)
        off = np.ascontiguousarray(nbr_off, np.int32)
        ids = np.ascontiguousarray(nbr_ids, np.int32)
        K = len(kp)
        stats = np.zeros((K, 8), np.int64)
        cands = np.zeros((K, 9), np.float32)
        poses = np.zeros((K, 3, 18), np.float32)
        acc = None
        if dump_k:
            sz = np.zeros(4, np.int64)
            _lib.load().sm_model_sizes(self.model, sz.ctypes.data_as(C.POINTER(C.c_int64)))
            tp = TrainParamC()
            _lib.load().sm_model_download(self.model, None, None, None, None, None, None, None,
                                          None, None, None, C.byref(tp))
            acc = np.zeros(min(dump_k, K) * int(sz[0]) * tp.featAngleResolution, np.int32)
        i32 = lambda x: x.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
        _check(_lib.load().sm_vote_stage(
            self.model, pts.ctypes.data_as(C.POINTER(C.c_float)),
            nrm.ctypes.data_as(C.POINTER(C.c_float)), len(pts), i32(kp), K, i32(off), i32(ids),
            min_score, stats.ctypes.data_as(C.POINTER(C.c_int64)),
            cands.ctypes.data_as(C.POINTER(C.c_float)),
            poses.ctypes.data_as(C.POINTER(C.c_float)), int(dump_k),
            i32(acc) if acc is not None else None))
        return stats, cands, poses, acc

    _DEBUG = {0: (np.int32, 1), 1: (np.int32, 1), 2: (np.int32, 1), 3: (np.float32, 3),
              4: (np.float32, 3), 7: (np.int64, 8), 8: (np.float32, 9), 9: (np.float32, 18),
              10: (np.float32, 18), 12: (np.int32, 1), 13: (np.float32, 1),
              14: (np.float32, 12), 15: (np.float32, 258)}

    def debug(self, field_id: int):
        """Intermediate state of the last matchScene (field ids as sm_debug_get)."""
        L = _lib.load()
        dt, w = self._DEBUG[field_id]
        n = L.sm_debug_size(self.model, field_id)
        if n < 0:
            raise RuntimeError("no such debug field or no match yet")
        a = np.zeros(n, dt)
        if n:
            _check(L.sm_debug_get(self.model, field_id, a.ctypes.data_as(C.c_void_p)))
        return a.reshape(-1, w) if w > 1 else a


def match_batch(jobs, samplingDistanceRel=0.04, keyPointFraction=0.2, minScore=0.2,
                param: MatchParam | None = None, concurrency=4):
    """Batched matchScene (sm_match_batch). jobs: list of (Detector, PointCloud). Returns a
    list of (poses (k, 4, 4), scores (k,)) per job, in job order, and per-job statistics."""
    param = param or MatchParam()
    L = _lib.load()
    nj = len(jobs)
    maxr = max(1, param.numMatches)
    models = (C.c_void_p * nj)(*[d.model.value for d, _ in jobs])
    keep, xs, ns_ = [], [], []
    nrm_any = any(pc.normal is not None for _, pc in jobs)
    nrms = []
    vps = np.zeros((nj, 3), np.float32)
    have_vp = all(pc.viewPoint is not None for _, pc in jobs)
    for j, (_, pc) in enumerate(jobs):
        p, k = _ptr(pc.point)
        keep.append(k)
        xs.append(C.cast(p, C.c_void_p))
        ns_.append(_len(pc.point))
        if nrm_any:
            q, k2 = _ptr(pc.normal)
            keep.append(k2)
            nrms.append(C.cast(q, C.c_void_p) if q is not None else None)
        if have_vp:
            vps[j] = np.asarray(pc.viewPoint, np.float32)
    xarr = (C.c_void_p * nj)(*xs)
    narr = (C.c_void_p * nj)(*nrms) if nrm_any else None
    n64 = np.asarray(ns_, np.int64)
    poses = np.zeros((nj, maxr, 4, 4), np.float32)
    scores = np.zeros((nj, maxr), np.float32)
    count = np.zeros(nj, np.int32)
    status = np.zeros(nj, np.int32)
    stats = (MatchStatsC * nj)()
    f32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    rc = L.sm_match_batch(nj, C.cast(models, C.c_void_p), C.cast(xarr, C.c_void_p),
                          C.cast(narr, C.c_void_p) if narr is not None else None,
                          n64.ctypes.data_as(C.POINTER(C.c_int64)),
                          f32(vps) if have_vp else None, samplingDistanceRel, keyPointFraction,
                          minScore, C.byref(param.c()), maxr, f32(poses), f32(scores),
                          i32(count), i32(status), concurrency, stats)
    _check(rc)
    out = [(poses[j, :count[j]], scores[j, :count[j]]) for j in range(nj)]
    st = [{f: getattr(s, f) for f, _ in MatchStatsC._fields_ if f not in ("ms", "vote_ms")} |
          {"ms": list(s.ms), "vote_ms": list(s.vote_ms)}
          for s in stats]
    return out, st


class Server:
    """Serving loop over resident models (sm_server_*): submit scenes as they arrive, poll
    finished requests with their queue / service / total latencies."""

    def __init__(self, device=0, slots=4, hbm_budget_bytes=64 << 30):
        h = C.c_void_p()
        _check(_lib.load().sm_server_create(device, slots, hbm_budget_bytes, C.byref(h)))
        self.handle = h

    def submit(self, detector: "Detector", scene: PointCloud, samplingDistanceRel=0.04,
               keyPointFraction=0.2, minScore=0.2, param: MatchParam | None = None) -> int:
        param = param or MatchParam()
        p, k1 = _ptr(scene.point)
        q, k2 = _ptr(scene.normal)
        vp = None
        if scene.viewPoint is not None:
            vpa = np.ascontiguousarray(scene.viewPoint, np.float32)
            vp = vpa.ctypes.data_as(C.POINTER(C.c_float))
        rid = C.c_int64()
        _check(_lib.load().sm_server_submit(self.handle, detector.model, p, q,
                                            _len(scene.point), vp, samplingDistanceRel,
                                            keyPointFraction, minScore, C.byref(param.c()),
                                            C.byref(rid)))
        return rid.value

    def poll(self, max_requests=64, max_results=16, wait_ms=0):
        """Finished requests: list of dicts {id, status, poses, scores, queue_ms, service_ms,
        total_ms}."""
        ids = np.zeros(max_requests, np.int64)
        st = np.zeros(max_requests, np.int32)
        cnt = np.zeros(max_requests, np.int32)
        poses = np.zeros((max_requests, max_results, 4, 4), np.float32)
        scores = np.zeros((max_requests, max_results), np.float32)
        times = np.zeros((max_requests, 3), np.float64)
        n = C.c_int()
        _check(_lib.load().sm_server_poll(
            self.handle, max_requests, max_results, wait_ms,
            ids.ctypes.data_as(C.POINTER(C.c_int64)), st.ctypes.data_as(C.POINTER(C.c_int32)),
            cnt.ctypes.data_as(C.POINTER(C.c_int32)), poses.ctypes.data_as(C.POINTER(C.c_float)),
            scores.ctypes.data_as(C.POINTER(C.c_float)),
            times.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n)))
        out = []
        for i in range(n.value):
            k = min(int(cnt[i]), max_results)
            out.append({"id": int(ids[i]), "status": int(st[i]), "poses": poses[i, :k].copy(),
                        "scores": scores[i, :k].copy(), "queue_ms": float(times[i, 0]),
                        "service_ms": float(times[i, 1]), "total_ms": float(times[i, 2])})
        return out

    def status(self):
        v = np.zeros(6, np.int64)
        _check(_lib.load().sm_server_status(self.handle, v.ctypes.data_as(C.POINTER(C.c_int64))))
        return dict(zip(["queued", "running", "completed", "bytes_in_flight", "peak_bytes",
                         "budget"], (int(x) for x in v)))

    def close(self):
        if getattr(self, "handle", None):
            _lib.load().sm_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

