"""Pins of the CPU oracle against the reference's own code where it compiles here
(vendored nanoflann k-d tree, scalar MurmurHash3) and accuracy of the shared float
transcendental functions against libm."""
import ctypes as C
import math

import numpy as np
import pytest

from conftest import reference_dir

f32p, i32p, u32p = C.POINTER(C.c_float), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)


def _ref_probe():
    if reference_dir() is None:
        pytest.skip("reference source tree not present (probes build only where it is)")
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "build_ref", os.path.join(os.path.dirname(__file__), "..", "oracle", "ref_probe",
                                  "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _clouds():
    from surface_match_gb300 import synth
    rng = np.random.default_rng(0)
    return [rng.uniform(-1, 1, (5000, 3)).astype(np.float32),
            np.round(rng.uniform(-5, 5, (3000, 3))).astype(np.float32),  # many exact ties
            synth.scene_tiny().cloud.xyz]


def test_kdtree_matches_reference_nanoflann(oracle_lib):
    mod = _ref_probe()
    R = C.CDLL(mod.build_kd())
    L = oracle_lib
    for fn in (L.orc_kd_probe, R.ref_kd_probe):
        fn.restype = C.c_int64
        fn.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_float, i32p, i32p, C.c_int64]
    for fn in (L.orc_kd_knn, R.ref_kd_knn):
        fn.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_int64, C.c_int, i32p, f32p]
    rng = np.random.default_rng(1)
    for P in _clouds():
        P = np.ascontiguousarray(P)
        n = len(P)
        box = np.concatenate([P.min(0), P.max(0)]).astype(np.float32)
        r2 = np.float32((np.abs(box[3:] - box[:3]).max() * 0.15) ** 2)
        for _ in range(10):
            q = np.ascontiguousarray(P[rng.integers(n)])
            va, vb = np.zeros(n, np.int32), np.zeros(n, np.int32)
            fa, fb = np.zeros(n, np.int32), np.zeros(n, np.int32)
            args = lambda v, f: (P.ctypes.data_as(f32p), n, box.ctypes.data_as(f32p),
                                 q.ctypes.data_as(f32p), r2, v.ctypes.data_as(i32p),
                                 f.ctypes.data_as(i32p), n)
            na = L.orc_kd_probe(*args(va, fa))
            nb = R.ref_kd_probe(*args(vb, fb))
            assert na == nb
            np.testing.assert_array_equal(va, vb)  # build order (vAcc_)
            np.testing.assert_array_equal(fa[:na], fb[:nb])  # unsorted radius order
        nq, k = 300, 10
        qs = np.ascontiguousarray(P[rng.integers(n, size=nq)] +
                                  rng.normal(0, 0.01, (nq, 3)).astype(np.float32))
        ia, ib = np.zeros((nq, k), np.int32), np.zeros((nq, k), np.int32)
        da, db = np.zeros((nq, k), np.float32), np.zeros((nq, k), np.float32)
        for fn, i, d in ((L.orc_kd_knn, ia, da), (R.ref_kd_knn, ib, db)):
            fn(P.ctypes.data_as(f32p), n, box.ctypes.data_as(f32p), qs.ctypes.data_as(f32p),
               nq, k, i.ctypes.data_as(i32p), d.ctypes.data_as(f32p))
        np.testing.assert_array_equal(ia, ib)
        np.testing.assert_array_equal(da, db)


def test_murmur_matches_reference_scalar_function(oracle_lib):
    mod = _ref_probe()
    M = C.CDLL(mod.build_murmur())
    M.ref_murmur.restype = C.c_uint32
    M.ref_murmur.argtypes = [i32p, C.c_uint32, C.c_uint32]
    L = oracle_lib
    rng = np.random.default_rng(2)
    words = np.concatenate([rng.integers(0, 40, (3000, 4)),
                            rng.integers(0, 2 ** 31, (1000, 4))]).astype(np.int32)
    for w in words:
        a = M.ref_murmur(w.ctypes.data_as(i32p), 16, 42)
        u = w.astype(np.uint32)
        assert a == L.orc_murmur4(u.ctypes.data_as(u32p))


def test_murmur_known_answers(oracle_lib):
    """Known-answer vectors of MurmurHash3_x86_32 (key = four little-endian words, seed
    42), recorded from the reference's own scalar function compiled in the build
    container."""
    from tests_golden import load_json
    kat = load_json("murmur_kat.json")
    for w, h in kat:
        u = np.array(w, np.uint32)
        assert oracle_lib.orc_murmur4(u.ctypes.data_as(u32p)) == h


def _ulp_err(a, b):
    a = np.float32(a)
    b = np.float32(b)
    if a == b:
        return 0
    return abs(int(np.array(a).view(np.int32)) - int(np.array(b).view(np.int32)))


def test_shared_float_math_accuracy(oracle_lib):
    L = oracle_lib
    rng = np.random.default_rng(3)
    worst = {"atan2": 0, "acos": 0, "sin": 0, "cos": 0}
    for _ in range(20000):
        y, x = rng.normal(size=2).astype(np.float32)
        worst["atan2"] = max(worst["atan2"], _ulp_err(L.orc_atan2f(y, x), math.atan2(y, x)))
        c = np.float32(rng.uniform(-1, 1))
        worst["acos"] = max(worst["acos"], _ulp_err(L.orc_acosf(c), math.acos(c)))
        a = np.float32(rng.uniform(-2 * math.pi, 2 * math.pi))
        if abs(math.sin(a)) > 1e-3:
            worst["sin"] = max(worst["sin"], _ulp_err(L.orc_sinf(a), math.sin(a)))
        if abs(math.cos(a)) > 1e-3:
            worst["cos"] = max(worst["cos"], _ulp_err(L.orc_cosf(a), math.cos(a)))
    assert all(v <= 4 for v in worst.values()), worst
    # C99 signed-zero conventions of atan2
    assert L.orc_atan2f(0.0, -1.0) == np.float32(math.pi)
    assert L.orc_atan2f(-0.0, -1.0) == -np.float32(math.pi)
    assert math.copysign(1, L.orc_atan2f(-0.0, 1.0)) < 0
    assert L.orc_atan2f(1.0, 0.0) == np.float32(math.pi / 2)


def test_kdtree_matches_committed_nanoflann_fixture(oracle_lib):
    """Same pin as above, against fixtures recorded from the reference's nanoflann (runs
    where the reference tree is absent)."""
    from tests_golden import load_npz
    g = load_npz("kdtree_ref.npz")
    L = oracle_lib
    L.orc_kd_probe.restype = C.c_int64
    L.orc_kd_probe.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_float, i32p, i32p, C.c_int64]
    L.orc_kd_knn.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_int64, C.c_int, i32p, f32p]
    P = np.ascontiguousarray(g["points"])
    n = len(P)
    box = g["box"]
    for j, qi in enumerate(g["queries"]):
        q = np.ascontiguousarray(P[qi])
        v, f = np.zeros(n, np.int32), np.zeros(n, np.int32)
        k = L.orc_kd_probe(P.ctypes.data_as(f32p), n, box.ctypes.data_as(f32p),
                           q.ctypes.data_as(f32p), g["r2"], v.ctypes.data_as(i32p),
                           f.ctypes.data_as(i32p), n)
        np.testing.assert_array_equal(v, g["vacc"])
        np.testing.assert_array_equal(f[:k], g["found"][g["found_off"][j]:g["found_off"][j + 1]])
    qs = np.ascontiguousarray(g["knn_q"])
    nq, kk = g["knn_idx"].shape
    ki, kd = np.zeros((nq, kk), np.int32), np.zeros((nq, kk), np.float32)
    L.orc_kd_knn(P.ctypes.data_as(f32p), n, box.ctypes.data_as(f32p), qs.ctypes.data_as(f32p),
                 nq, kk, ki.ctypes.data_as(i32p), kd.ctypes.data_as(f32p))
    np.testing.assert_array_equal(ki, g["knn_idx"])
    np.testing.assert_array_equal(kd, g["knn_dist"])


@pytest.mark.parametrize("tag", ["ref", "grid"])
def test_oracle_reproduces_committed_stage_goldens(tag):
    """The restatement is deterministic across machines (x86 build container, Arm GPU machine):
    sampled sets, keypoints, per-keypoint vote statistics, candidates and poses of a
    seeded two-gear scene match the committed fixture bit for bit."""
    import hashlib
    from oracle import MODE_GRID, MODE_REF, MatchParam, Oracle
    from tests_golden import load_npz
    g = load_npz("oracle_tiny.npz")
    o = Oracle(mode=MODE_REF if tag == "ref" else MODE_GRID, threads=1)
    m = o.train(g["model_xyz"], g["model_nrm"], 0.05)
    np.testing.assert_array_equal(m.keys, g[f"{tag}_model_keys"])
    np.testing.assert_array_equal(m.offsets, g[f"{tag}_model_offsets"])
    assert hashlib.sha256(m.refs.tobytes() + m.alphas.tobytes()).hexdigest() == \
        str(g[f"{tag}_model_entries_sha256"])
    r = o.match(m, g["scene_xyz"], None, g["viewpoint"], 0.05, 0.2, 0.2,
                MatchParam(numMatches=8))
    np.testing.assert_array_equal(r.sampled, g[f"{tag}_sampled"])
    np.testing.assert_array_equal(r.keypoints, g[f"{tag}_keypoints"])
    np.testing.assert_array_equal(r.kp_stats, g[f"{tag}_kp_stats"])
    np.testing.assert_array_equal(r.kp_cands, g[f"{tag}_kp_cands"])
    np.testing.assert_array_equal(r.results, g[f"{tag}_results"])


@pytest.mark.parametrize("cell", [0.05, 0.13, 0.5, 2.0])
def test_grid_searches_are_exact_for_any_cell_size(oracle_lib, cell):
    """k nearest (ties by index), nearest within a limit and any-within-radius on the
    uniform grid equal brute force, whatever the cell size (the GPU uses the same
    search-termination rule)."""
    L = oracle_lib
    L.orc_grid_probe.argtypes = [f32p, C.c_int64, f32p, C.c_int64, C.c_float, C.c_int,
                                 C.c_float, C.c_float, i32p, f32p, i32p, f32p, i32p]
    rng = np.random.default_rng(5)
    P = np.ascontiguousarray(np.concatenate([rng.uniform(-1, 1, (3000, 3)),
                                             np.round(rng.uniform(-1, 1, (500, 3)) * 4) / 4])
                             .astype(np.float32))
    Q = np.ascontiguousarray(np.concatenate([P[rng.integers(len(P), size=200)] +
                                             rng.normal(0, 0.05, (200, 3)),
                                             rng.uniform(-1.5, 1.5, (100, 3))])
                             .astype(np.float32))
    k, lim2, r2 = 10, np.float32(0.3 ** 2), np.float32(0.07 ** 2)
    ki, kd = np.zeros((len(Q), k), np.int32), np.zeros((len(Q), k), np.float32)
    ni, nd = np.zeros(len(Q), np.int32), np.zeros(len(Q), np.float32)
    wi = np.zeros(len(Q), np.int32)
    L.orc_grid_probe(P.ctypes.data_as(f32p), len(P), Q.ctypes.data_as(f32p), len(Q), cell, k,
                     lim2, r2, ki.ctypes.data_as(i32p), kd.ctypes.data_as(f32p),
                     ni.ctypes.data_as(i32p), nd.ctypes.data_as(f32p), wi.ctypes.data_as(i32p))
    d = Q[:, None, :] - P[None, :, :]  # same float formula: ((d0^2 + d1^2) + d2^2)
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    order = np.lexsort((np.broadcast_to(np.arange(len(P)), d2.shape), d2), axis=1)
    np.testing.assert_array_equal(ki, order[:, :k])
    np.testing.assert_array_equal(kd, np.take_along_axis(d2, order[:, :k], 1))
    best = order[:, 0]
    bd = d2[np.arange(len(Q)), best]
    inlim = bd <= lim2
    np.testing.assert_array_equal(ni[inlim], best[inlim])
    np.testing.assert_array_equal(wi, (d2 < r2).any(1).astype(np.int32))
