"""ctypes wrapper and build recipe of the CPU oracle (test infrastructure only)."""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SO = os.path.join(BUILD, "libsm_oracle.so")
SOURCES = [os.path.join(HERE, "sm_oracle.cpp"), os.path.join(HERE, "kdtree.h")] + [
    os.path.join(HERE, "..", "surface_match_gb300", "csrc", f)
    for f in ("sm_math.h", "sm_linalg.h", "sm_icp.h", "sm_grid.h")]

MODE_REF = 0
MODE_GRID = 1

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with the host flags that keep float arithmetic IEEE-exact and
    identical to the device code (no FMA contraction, no fast-math)."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SOURCES)
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= newest:
        return SO
    tmp = SO + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
           "-fPIC", "-shared", "-Wno-array-bounds", "-o", tmp,
           os.path.join(HERE, "sm_oracle.cpp")]
    subprocess.run(cmd, check=True)
    os.replace(tmp, SO)
    return SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(SO)
            vp, f32p, i32p, i64p, u32p = (C.c_void_p, C.POINTER(C.c_float),
                                          C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                          C.POINTER(C.c_uint32))
            L.orc_last_error.restype = C.c_char_p
            L.orc_train.restype = vp
            L.orc_train.argtypes = [f32p, f32p, C.c_int64, C.c_float, vp, C.c_int, C.c_int]
            L.orc_model_free.argtypes = [vp]
            L.orc_model_sizes.argtypes = [vp, i64p]
            L.orc_model_export.argtypes = [vp, f32p, f32p, f32p, f32p, f32p, u32p, u32p,
                                           u32p, f32p]
            L.orc_model_import.restype = vp
            L.orc_model_import.argtypes = [C.c_int64, f32p, f32p, C.c_int64, f32p, f32p, f32p,
                                           C.c_int64, u32p, u32p, u32p, f32p, vp, C.c_float]
            L.orc_match.restype = vp
            L.orc_match.argtypes = [vp, f32p, f32p, C.c_int64, f32p, C.c_float, C.c_float,
                                    C.c_float, vp, C.c_int, C.c_int, C.c_int, C.c_int]
            L.orc_match_free.argtypes = [vp]
            L.orc_res_size.restype = C.c_int64
            L.orc_res_size.argtypes = [vp, C.c_int]
            L.orc_res_get.argtypes = [vp, C.c_int, vp]
            L.orc_vote_stage.argtypes = [vp, f32p, f32p, C.c_int64, i32p, C.c_int64, i32p,
                                         i32p, C.c_float, C.c_int, i64p, f32p, f32p, C.c_int,
                                         i32p]
            for nm in ("orc_atan2f",):
                getattr(L, nm).restype = C.c_float
                getattr(L, nm).argtypes = [C.c_float, C.c_float]
            for nm in ("orc_acosf", "orc_sinf", "orc_cosf"):
                getattr(L, nm).restype = C.c_float
                getattr(L, nm).argtypes = [C.c_float]
            L.orc_murmur4.restype = C.c_uint32
            L.orc_murmur4.argtypes = [u32p]
            L.orc_mls.argtypes = [f32p, C.c_int64, i64p, C.c_int64, C.c_float, C.c_int, C.c_int,
                                  f32p, f32p, f32p, i32p]
            L.orc_kd_probe.restype = C.c_int64
            L.orc_kd_probe.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_float, i32p, i32p,
                                       C.c_int64]
            L.orc_kd_sample.restype = C.c_int64
            L.orc_kd_sample.argtypes = [f32p, C.c_int64, f32p, C.c_float, i32p]
            L.orc_kd_knn.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_int64, C.c_int, i32p, f32p]
            _lib = L
        return _lib


def _p(a, t=C.c_float):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


class _TP(C.Structure):
    _fields_ = [("featDistanceStepRel", C.c_float), ("featAngleResolution", C.c_int),
                ("poseRefRelSamplingDistance", C.c_float), ("knnNormal", C.c_int),
                ("smoothNormal", C.c_int)]


class _MP(C.Structure):
    _fields_ = [("numMatches", C.c_int), ("knnNormal", C.c_int), ("smoothNormal", C.c_int),
                ("invertNormal", C.c_int), ("maxOverlapDistRel", C.c_float),
                ("maxOverlapDistAbs", C.c_float), ("sparsePoseRefinement", C.c_int),
                ("densePoseRefinement", C.c_int), ("poseRefNumSteps", C.c_int),
                ("poseRefDistThresholdRel", C.c_float), ("poseRefDistThresholdAbs", C.c_float),
                ("poseRefScoringDistRel", C.c_float), ("poseRefScoringDistAbs", C.c_float)]


@dataclass
class TrainParam:
    featDistanceStepRel: float = 0.04
    featAngleResolution: int = 30
    poseRefRelSamplingDistance: float = 0.01
    knnNormal: int = 10
    smoothNormal: bool = True

    def c(self):
        return _TP(self.featDistanceStepRel, self.featAngleResolution,
                   self.poseRefRelSamplingDistance, self.knnNormal, int(self.smoothNormal))


@dataclass
class MatchParam:
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

    def c(self):
        return _MP(self.numMatches, self.knnNormal, int(self.smoothNormal),
                   int(self.invertNormal), self.maxOverlapDistRel, self.maxOverlapDistAbs,
                   int(self.sparsePoseRefinement), int(self.densePoseRefinement),
                   self.poseRefNumSteps, self.poseRefDistThresholdRel,
                   self.poseRefDistThresholdAbs, self.poseRefScoringDistRel,
                   self.poseRefScoringDistAbs)


@dataclass
class OracleModel:
    handle: int
    sampled: np.ndarray = field(default=None)
    sampled_normal: np.ndarray = field(default=None)
    resampled: np.ndarray = field(default=None)
    resampled_normal: np.ndarray = field(default=None)
    box: np.ndarray = field(default=None)
    keys: np.ndarray = field(default=None)
    offsets: np.ndarray = field(default=None)
    refs: np.ndarray = field(default=None)
    alphas: np.ndarray = field(default=None)
    train_param: TrainParam = field(default_factory=TrainParam)
    sd_rel: float = 0.04

    def __del__(self):
        if self.handle and _lib is not None:
            _lib.orc_model_free(self.handle)
            self.handle = 0


_FIELDS = {"sampled": (0, np.int32, 1), "keypoints": (1, np.int32, 1),
           "resampled": (2, np.int32, 1), "positions": (3, np.float32, 3),
           "normals": (4, np.float32, 3), "nbr_off": (5, np.int32, 1),
           "nbr_ids": (6, np.int32, 1), "kp_stats": (7, np.int64, 8),
           "kp_cands": (8, np.float32, 9), "pose_list": (9, np.float32, 18),
           "clustered": (10, np.float32, 18), "cluster_sizes": (11, np.int32, 1),
           "cand_status": (12, np.int32, 1), "cand_score": (13, np.float32, 1),
           "cand_pose": (14, np.float32, 12), "results": (15, np.float32, 13),
           "acc_dump": (16, np.int32, 1), "cand_trace": (17, np.float32, 258)}


class MatchResult:
    def __init__(self, handle):
        self.handle = handle
        L = lib()
        for name, (fid, dt, w) in _FIELDS.items():
            n = L.orc_res_size(handle, fid)
            a = np.empty(max(n, 0), dtype=dt)
            if n > 0:
                L.orc_res_get(handle, fid, a.ctypes.data_as(C.c_void_p))
            if w > 1:
                a = a.reshape(-1, w)
            setattr(self, name, a)
        L.orc_match_free(handle)
        self.handle = 0
        r = self.results
        self.poses = r[:, :12].reshape(-1, 3, 4) if len(r) else np.zeros((0, 3, 4), np.float32)
        self.scores = r[:, 12] if len(r) else np.zeros(0, np.float32)


class Oracle:
    """The CPU restatement. ``mode``: MODE_REF (reference search orders) or MODE_GRID
    (the GPU's orders)."""

    def __init__(self, mode=MODE_GRID, threads=1, fp64=False):
        self.mode, self.threads, self.fp64 = mode, threads, fp64
        lib()

    def train(self, xyz, normal=None, sd_rel=0.04, param: TrainParam | None = None):
        param = param or TrainParam()
        xyz = np.ascontiguousarray(xyz, np.float32)
        nrm = None if normal is None else np.ascontiguousarray(normal, np.float32)
        tp = param.c()
        h = lib().orc_train(_p(xyz), _p(nrm), len(xyz), sd_rel, C.addressof(tp), self.mode,
                            self.threads)
        if not h:
            raise RuntimeError(lib().orc_last_error().decode())
        return self._export(h, param, sd_rel)

    @staticmethod
    def _export(h, param, sd_rel):
        L = lib()
        sz = np.zeros(4, np.int64)
        L.orc_model_sizes(h, _p(sz, C.c_int64))
        ns, nr, nk, ne = (int(v) for v in sz)
        m = OracleModel(h, np.zeros((ns, 3), np.float32), np.zeros((ns, 3), np.float32),
                        np.zeros((nr, 3), np.float32), np.zeros((nr, 3), np.float32),
                        np.zeros(6, np.float32), np.zeros(nk, np.uint32),
                        np.zeros(nk + 1, np.uint32), np.zeros(ne, np.uint32),
                        np.zeros(ne, np.float32), param, sd_rel)
        L.orc_model_export(h, _p(m.sampled), _p(m.sampled_normal), _p(m.resampled),
                           _p(m.resampled_normal), _p(m.box), _p(m.keys, C.c_uint32),
                           _p(m.offsets, C.c_uint32), _p(m.refs, C.c_uint32), _p(m.alphas))
        return m

    @staticmethod
    def import_model(sampled, sampled_normal, resampled, resampled_normal, box, keys, offsets,
                     refs, alphas, param: TrainParam, sd_rel=0.04):
        arrs = [np.ascontiguousarray(a, dt) for a, dt in (
            (sampled, np.float32), (sampled_normal, np.float32), (resampled, np.float32),
            (resampled_normal, np.float32), (box, np.float32), (keys, np.uint32),
            (offsets, np.uint32), (refs, np.uint32), (alphas, np.float32))]
        tp = param.c()
        h = lib().orc_model_import(len(arrs[0]), _p(arrs[0]), _p(arrs[1]), len(arrs[2]),
                                   _p(arrs[2]), _p(arrs[3]), _p(arrs[4]), len(arrs[5]),
                                   _p(arrs[5], C.c_uint32), _p(arrs[6], C.c_uint32),
                                   _p(arrs[7], C.c_uint32), _p(arrs[8]), C.addressof(tp),
                                   sd_rel)
        return Oracle._export(h, param, sd_rel)

    def match(self, model: OracleModel, xyz, normal=None, viewpoint=None, sd_rel=0.04,
              kp_frac=0.2, min_score=0.2, param: MatchParam | None = None, dump_k=0):
        param = param or MatchParam()
        xyz = np.ascontiguousarray(xyz, np.float32)
        nrm = None if normal is None else np.ascontiguousarray(normal, np.float32)
        vp = None if viewpoint is None else np.ascontiguousarray(viewpoint, np.float32)
        mp = param.c()
        h = lib().orc_match(model.handle, _p(xyz), _p(nrm), len(xyz), _p(vp), sd_rel, kp_frac,
                            min_score, C.addressof(mp), self.mode, self.threads,
                            int(self.fp64), dump_k)
        if not h:
            raise RuntimeError(lib().orc_last_error().decode())
        return MatchResult(h)

    def vote_stage(self, model: OracleModel, points, normals, keypoints, nbr_off, nbr_ids,
                   min_score, dump_k=0):
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
            A = model.train_param.featAngleResolution
            acc = np.zeros(min(dump_k, K) * len(model.sampled) * A, np.int32)
        lib().orc_vote_stage(model.handle, _p(pts), _p(nrm), len(pts), _p(kp, C.c_int32), K,
                             _p(off, C.c_int32), _p(ids, C.c_int32), min_score, self.threads,
                             _p(stats, C.c_int64), _p(cands), _p(poses), dump_k,
                             _p(acc, C.c_int32))
        return stats, cands, poses, acc


def mls(xyz, normal=None, indices=None, radius=1.0, order=2, invert=False, viewpoint=None):
    """estimateNormalMLS (util.cpp:336-457) by the FP64 restatement: returns the points,
    the normals (inputs, NaN where absent, with the listed points' results in place) and the
    status of each listed point (0 unchanged, 1 PCA normal only, 2 moved onto the fit)."""
    pts = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    n = len(pts)
    idx = np.arange(n, dtype=np.int64) if indices is None else np.ascontiguousarray(indices, np.int64)
    out_p = pts.copy()
    out_n = (np.full((n, 3), np.nan, np.float32) if normal is None
             else np.ascontiguousarray(normal, np.float32).reshape(-1, 3).copy())
    vp = None if viewpoint is None else np.ascontiguousarray(viewpoint, np.float32)
    status = np.zeros(len(idx), np.int32)
    lib().orc_mls(_p(pts), n, _p(idx, C.c_int64), len(idx), float(radius), int(order),
                  1 if invert else 0, _p(vp), _p(out_p), _p(out_n), _p(status, C.c_int32))
    return out_p, out_n, status


def kd_reference(xyz, step=0.0, queries=None, k=10):
    """The oracle's k-d tree over all points of xyz (tight box): vAcc order, the greedy
    sample at `step` in tree order (when step > 0) and the k nearest of each query."""
    L = lib()
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = len(xyz)
    box = np.concatenate([xyz.min(0), xyz.max(0)]).astype(np.float32)
    vacc = np.zeros(n, np.int32)
    q0 = np.zeros(3, np.float32)
    found = np.zeros(1, np.int32)
    L.orc_kd_probe(_p(xyz), n, _p(box), _p(q0), 0.0, _p(vacc, C.c_int32), _p(found, C.c_int32), 0)
    sampled = None
    if step > 0:
        out = np.zeros(n, np.int32)
        ns = L.orc_kd_sample(_p(xyz), n, _p(box), step, _p(out, C.c_int32))
        sampled = out[:ns].copy()
    knn = dist = None
    if queries is not None:
        qs = np.ascontiguousarray(queries, np.float32)
        knn = np.zeros((len(qs), k), np.int32)
        dist = np.zeros((len(qs), k), np.float32)
        L.orc_kd_knn(_p(xyz), n, _p(box), _p(qs), len(qs), k, _p(knn, C.c_int32), _p(dist))
    return vacc, sampled, knn, dist

