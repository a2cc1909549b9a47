"""The reference-order k-d tree on the GPU against the oracle's restatement of the vendored
nanoflann (itself pinned to the real nanoflann in test_oracle_pins): tree order (vAcc),
samplePointCloud's greedy thinning in tree order, and k-nearest searches with the
reference's tie order - on random clouds, clouds with duplicate points and the synthetic
scenes at full size."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _probe(xyz, step=0.0, queries=None, k=10):
    from surface_match_gb300 import _lib
    from surface_match_gb300.detector import Context
    L = _lib.load()
    ctx = Context()
    try:
        xyz = np.ascontiguousarray(xyz, np.float32)
        n = len(xyz)
        vacc = np.zeros(n, np.int32)
        sampled = np.zeros(n, np.int32)
        ns = C.c_int64(0)
        f32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
        i32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
        nq = 0 if queries is None else len(queries)
        qs = np.zeros((max(nq, 1), 3), np.float32) if queries is None else \
            np.ascontiguousarray(queries, np.float32)
        knn = np.zeros((max(nq, 1), k), np.int32)
        dist = np.zeros((max(nq, 1), k), np.float32)
        rc = L.sm_kdtree_probe(ctx.handle, f32(xyz), n, step, i32(vacc), i32(sampled),
                               C.byref(ns), f32(qs), nq, k, i32(knn), f32(dist))
        assert rc == 0, _lib.last_error()
        return vacc, sampled[:ns.value].copy(), knn[:nq], dist[:nq]
    finally:
        ctx.close()


def _compare(xyz, step, nq=300, k=10, seed=0):
    from oracle.pyoracle import kd_reference
    rng = np.random.default_rng(seed)
    qs = xyz[rng.integers(0, len(xyz), nq)] + rng.normal(0, step * 0.1, (nq, 3)).astype(np.float32)
    v, s, kn, kd = _probe(xyz, step, qs, k)
    ov, os_, okn, okd = kd_reference(xyz, step, qs, k)
    np.testing.assert_array_equal(v, ov, err_msg="tree order (vAcc)")
    np.testing.assert_array_equal(s, os_, err_msg="greedy sample in tree order")
    np.testing.assert_array_equal(kn, okn, err_msg="k nearest ids")
    np.testing.assert_array_equal(kd.view(np.uint32), okd.view(np.uint32), err_msg="k nearest distances")
    return len(s)


def test_tree_order_random_clouds():
    rng = np.random.default_rng(4)
    for n in (1, 7, 11, 500, 1024, 1025, 5000, 40000):
        xyz = rng.normal(size=(n, 3)).astype(np.float32) * np.float32(20)
        v, _, _, _ = _probe(xyz)
        from oracle.pyoracle import kd_reference
        ov, _, _, _ = kd_reference(xyz)
        np.testing.assert_array_equal(v, ov, err_msg=f"n={n}")


def test_tree_sample_and_knn_random_and_duplicates():
    rng = np.random.default_rng(5)
    xyz = rng.uniform(-50, 50, (30000, 3)).astype(np.float32)
    assert _compare(xyz, 4.0) > 100
    # duplicates and coordinates on a lattice: equal split values, equal distances
    lat = rng.integers(-20, 20, (20000, 3)).astype(np.float32)
    lat = np.concatenate([lat, lat[:3000]])
    assert _compare(lat, 2.5, k=12) > 100
    # a flat cloud (one axis of zero spread)
    flat = np.concatenate([rng.uniform(-30, 30, (8000, 2)), np.zeros((8000, 1))], 1).astype(np.float32)
    _compare(flat, 1.5)


@pytest.mark.parametrize("which", ["small", "large"])
def test_tree_sample_on_workload_scenes(which):
    """Config-size scenes: the small scene (about 108k points, sampling 0.04 of the gear's
    diameter) and the large one (about 0.92M points, sampling 0.03)."""
    from surface_match_gb300 import synth
    if which == "small":
        sc, rel = synth.scene_small(seed=1), 0.04
    else:
        sc, rel = synth.scene_large(seed=2), 0.03
    xyz = np.ascontiguousarray(sc.cloud.xyz, np.float32)
    mc, _, _ = synth.gear_model(20000, seed=7)
    diam = float(np.linalg.norm(mc.xyz.max(0) - mc.xyz.min(0)))
    assert _compare(xyz, np.float32(diam * rel), nq=500) > 1000
