"""GB300-native (sm_103a) point-pair-feature surface matching.

A drop-in for the ppf::Detector hot path of SurfaceMan/surface_match: the C ABI lives in
include/surface_match.h (libsurface_match.so, CUDA kernels in csrc/), ``include/ppf.h`` is
the C++ Detector over it, and this package is the Python mirror of the same API.
"""
from .detector import (Context, Detector, MatchParam, MatchResult, PointCloud,  # noqa: F401
                       RangeError, Server, TrainParam, estimateNormalMLS, match_batch,
                       pinned_empty, probe_vote_atomics)
from .ply import read_ply, write_ply  # noqa: F401

__all__ = ["Context", "Detector", "MatchParam", "MatchResult", "PointCloud", "RangeError",
           "Server", "TrainParam", "estimateNormalMLS", "match_batch", "pinned_empty",
           "probe_vote_atomics",
           "read_ply", "write_ply"]
