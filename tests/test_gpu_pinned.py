"""Page-locked scene input (sm_host_alloc / sm_host_free, read_ply(pinned=True)): a PLY scene
read into pinned memory equals the pageable read, and matchScene gives the same poses and
scores from either (the pinned one is uploaded as an asynchronous DMA)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_host_alloc_edge_cases():
    from surface_match_gb300 import _lib
    L = _lib.load()
    p = C.c_void_p(123)
    assert L.sm_host_alloc(0, C.byref(p)) == 0 and p.value is None
    assert L.sm_host_free(None) == 0
    assert L.sm_host_alloc(-1, C.byref(p)) == _lib.SM_ERR_ARG
    assert L.sm_host_alloc(4096, C.byref(p)) == 0 and p.value
    assert L.sm_host_free(p) == 0


def test_pinned_ply_scene_matches_like_pageable(tmp_path):
    from surface_match_gb300 import (Detector, MatchParam, PointCloud, read_ply, synth,
                                     write_ply)
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny(seed=3)
    path = str(tmp_path / "scene.ply")
    assert write_ply(path, PointCloud(sc.cloud.xyz, None))
    a = read_ply(path)
    b = read_ply(path, pinned=True)
    np.testing.assert_array_equal(a.point, b.point)
    assert b.normal is None
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), 0.05)
    pa, sa = det.matchScene(PointCloud(a.point, None, sc.viewpoint), 0.05, 0.2, 0.2,
                            MatchParam(numMatches=8))
    pb, sb = det.matchScene(PointCloud(b.point, None, sc.viewpoint), 0.05, 0.2, 0.2,
                            MatchParam(numMatches=8))
    assert len(sa) > 0
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(pa.view(np.uint32), pb.view(np.uint32))
