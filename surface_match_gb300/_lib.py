"""ctypes binding of libsurface_match.so (the C ABI in include/surface_match.h)."""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsurface_match.so")

SM_OK, SM_ERR_RANGE, SM_ERR_RUNTIME, SM_ERR_CUDA, SM_ERR_ARG, SM_ERR_NOMEM, SM_ERR_CAPACITY = \
    range(7)
SM_ORDER_GRID, SM_ORDER_REFERENCE = 0, 1


class TrainParamC(C.Structure):
    _fields_ = [("featDistanceStepRel", C.c_float), ("featAngleResolution", C.c_int),
                ("poseRefRelSamplingDistance", C.c_float), ("knnNormal", C.c_int),
                ("smoothNormal", C.c_int)]


class MatchParamC(C.Structure):
    _fields_ = [("numMatches", C.c_int), ("knnNormal", C.c_int), ("smoothNormal", C.c_int),
                ("invertNormal", C.c_int), ("maxOverlapDistRel", C.c_float),
                ("maxOverlapDistAbs", C.c_float), ("sparsePoseRefinement", C.c_int),
                ("densePoseRefinement", C.c_int), ("poseRefNumSteps", C.c_int),
                ("poseRefDistThresholdRel", C.c_float), ("poseRefDistThresholdAbs", C.c_float),
                ("poseRefScoringDistRel", C.c_float), ("poseRefScoringDistAbs", C.c_float)]


class MatchStatsC(C.Structure):
    _fields_ = [("n_points", C.c_int64), ("n_valid", C.c_int64), ("n_sampled", C.c_int64),
                ("n_keypoints", C.c_int64), ("n_resampled", C.c_int64),
                ("n_poses", C.c_int64), ("n_clusters", C.c_int64), ("n_pairs", C.c_int64),
                ("n_hits", C.c_int64), ("n_votes", C.c_int64), ("ms", C.c_float * 8),
                ("vote_ms", C.c_float * 2)]


_lock = threading.Lock()
_lib = None

_vp = C.c_void_p
_f32p = C.POINTER(C.c_float)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_u32p = C.POINTER(C.c_uint32)

_SIGNATURES = {
    "sm_train_param_default": (None, [C.POINTER(TrainParamC)]),
    "sm_match_param_default": (None, [C.POINTER(MatchParamC)]),
    "sm_train_param_check": (C.c_int, [C.POINTER(TrainParamC)]),
    "sm_match_param_check": (C.c_int, [C.POINTER(MatchParamC)]),
    "sm_context_create": (C.c_int, [C.c_int, _vp, C.POINTER(_vp)]),
    "sm_context_destroy": (C.c_int, [_vp]),
    "sm_context_synchronize": (C.c_int, [_vp]),
    "sm_context_stream": (_vp, [_vp]),
    "sm_context_workspace_bytes": (C.c_int, [_vp, _i64p]),
    "sm_context_kernel_clock": (C.c_int, [_vp, C.c_int]),
    "sm_context_kernel_report": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double), _i64p]),
    "sm_model_create": (C.c_int, [_vp, C.POINTER(_vp)]),
    "sm_model_destroy": (C.c_int, [_vp]),
    "sm_model_train": (C.c_int, [_vp, _f32p, _f32p, C.c_int64, C.c_float,
                                 C.POINTER(TrainParamC)]),
    "sm_model_upload": (C.c_int, [_vp, C.c_int64, _f32p, _f32p, C.c_int64, _f32p, _f32p, _f32p,
                                  C.c_int64, _u32p, _u32p, _u32p, _f32p, C.c_float,
                                  C.POINTER(TrainParamC)]),
    "sm_model_set_search_order": (C.c_int, [_vp, C.c_int]),
    "sm_model_search_order": (C.c_int, [_vp]),
    "sm_model_sizes": (C.c_int, [_vp, _i64p]),
    "sm_model_download": (C.c_int, [_vp, _f32p, _f32p, _f32p, _f32p, _f32p, _u32p, _u32p,
                                    _u32p, _f32p, _f32p, C.POINTER(TrainParamC)]),
    "sm_model_save": (C.c_int, [_vp, C.c_char_p]),
    "sm_model_load": (C.c_int, [_vp, C.c_char_p]),
    "sm_match": (C.c_int, [_vp, _f32p, _f32p, C.c_int64, _f32p, C.c_float, C.c_float,
                           C.c_float, C.POINTER(MatchParamC), _f32p, _f32p, C.POINTER(C.c_int),
                           C.POINTER(MatchStatsC)]),
    "sm_vote_stage": (C.c_int, [_vp, _f32p, _f32p, C.c_int64, _i32p, C.c_int64, _i32p, _i32p,
                                C.c_float, _i64p, _f32p, _f32p, C.c_int, _i32p]),
    "sm_match_batch": (C.c_int, [C.c_int, _vp, _vp, _vp, _i64p, _f32p, C.c_float, C.c_float,
                                 C.c_float, C.POINTER(MatchParamC), C.c_int, _f32p, _f32p,
                                 _i32p, _i32p, C.c_int, C.POINTER(MatchStatsC)]),
    "sm_server_create": (C.c_int, [C.c_int, C.c_int, C.c_int64, C.POINTER(_vp)]),
    "sm_server_destroy": (C.c_int, [_vp]),
    "sm_server_submit": (C.c_int, [_vp, _vp, _f32p, _f32p, C.c_int64, _f32p, C.c_float,
                                   C.c_float, C.c_float, C.POINTER(MatchParamC), _i64p]),
    "sm_server_poll": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _i64p, _i32p, _i32p, _f32p,
                                 _f32p, C.POINTER(C.c_double), _i32p]),
    "sm_server_status": (C.c_int, [_vp, _i64p]),
    "sm_vote_stage_noalloc": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, C.c_int64, _vp, _vp,
                                        C.c_float, _vp, _vp, _vp, C.c_int, _vp]),
    "sm_kdtree_probe": (C.c_int, [_vp, _f32p, C.c_int64, C.c_float, _i32p, _i32p, _i64p, _f32p,
                                  C.c_int64, C.c_int, _i32p, _f32p]),
    "sm_debug_size": (C.c_int64, [_vp, C.c_int]),
    "sm_debug_get": (C.c_int, [_vp, C.c_int, _vp]),
    "sm_last_error": (C.c_char_p, []),
    "sm_version": (C.c_char_p, []),
    "sm_launch_count": (C.c_int64, []),
    "sm_host_alloc": (C.c_int, [C.c_int64, C.POINTER(_vp)]),
    "sm_host_free": (C.c_int, [_vp]),
    "sm_vote_tuned_shape": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "sm_probe_vote_atomics": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "sm_estimate_normals_mls": (C.c_int, [_vp, _f32p, _f32p, C.c_int64, _i64p, C.c_int64,
                                          C.c_float, C.c_int, C.c_int, _f32p, _f32p, _f32p]),
}


def exported_names():
    return list(_SIGNATURES)


def load():
    """Load the in-tree library. It is built by ``__graft_entry__.build()`` (or
    ``python -m surface_match_gb300.build``); a missing library is an error, never a silent
    fallback."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is not built; run surface_match_gb300.build.build()")
            L = C.CDLL(LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def last_error() -> str:
    return load().sm_last_error().decode()
