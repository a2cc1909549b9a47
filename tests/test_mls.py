"""Moving-least-squares normals (estimateNormalMLS, util.cpp:336-457).

CPU: the oracle's FP64 restatement against geometry with known answers - a noise-free
tilted plane (exact normal, points unmoved), a noisy sphere (radial normals, noise
reduced by the projection) - and the reference's skip and orientation rules; the C++
mirror in ppf.h compiles. GPU: sm_estimate_normals_mls through the C ABI against the oracle
on the same inputs for every supported order: untouched and skipped points bit-exact,
moved points within 1e-3 degrees (normals) and 1e-4 x radius (positions)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# tolerances of the GPU against the FP64 oracle (FP32 sums on the GPU; an emulation of its
# arithmetic stays below 2e-5 degrees on these surfaces)
NORMAL_TOL_DEG = 1e-3
POINT_TOL_REL = 1e-4


def chord_deg(a, b):
    """Angle between unit vectors from their chord (exact for small angles, unlike arccos
    of a float32 dot product)."""
    return np.degrees(2 * np.arcsin(np.clip(np.linalg.norm(a - b, axis=1) / 2, 0, 1)))


def scene(seed=0):
    """A noisy sphere, a wavy sheet, isolated points and non-finite points."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(6000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    S = d * 20 * (1 + 0.002 * rng.normal(size=(6000, 1))) + [10, -5, 30]
    xy = rng.uniform(-40, 40, size=(6000, 2))
    z = 3 * np.sin(xy[:, 0] / 7) * np.cos(xy[:, 1] / 9) - 30 + 0.05 * rng.normal(size=6000)
    W = np.c_[xy, z]
    iso = np.array([[200, 0, 0], [300, 0, 0], [400, 0, 0], [200, 200, 0], [203, 200, 0]], float)
    bad = np.array([[np.nan, 0, 0], [0, np.inf, 0]])
    return np.concatenate([S, W, iso, bad]).astype(np.float32)


def listed(rng):
    """Sphere and sheet points (sheet away from its rim), the isolated and non-finite
    points, and a repeated index."""
    P = scene()
    sheet = 6000 + np.flatnonzero(np.all(np.abs(P[6000:12000, :2]) < 34, axis=1))
    ids = np.r_[rng.choice(6000, 200, replace=False), rng.choice(sheet, 200, replace=False),
                np.arange(12000, 12007)]
    return np.r_[ids, ids[:3]].astype(np.int64)


# ---------------------------------------------------------------------------- CPU

def test_oracle_plane_is_exact():
    from oracle import pyoracle as po
    rng = np.random.default_rng(1)
    nrm = np.array([0.3, -0.5, 0.81])
    nrm /= np.linalg.norm(nrm)
    a = np.cross(nrm, [1, 0, 0])
    a /= np.linalg.norm(a)
    b = np.cross(nrm, a)
    st = rng.uniform(-30, 30, size=(3000, 2))
    P = (st[:, :1] * a + st[:, 1:] * b + 5 * nrm).astype(np.float32)
    ids = np.flatnonzero(np.all(np.abs(st) < 25, axis=1))[:300]
    for order in (1, 2, 3, 4):
        p, n, s = po.mls(P, None, ids, radius=4.0, order=order)  # no viewpoint: toward +z
        assert np.all(s == 2)
        assert np.all(n[ids, 2] > 0)
        assert chord_deg(n[ids], np.broadcast_to(nrm, (len(ids), 3))).max() < 1e-4
        assert np.abs(p[ids] - P[ids]).max() < 1e-4
        p, n, s = po.mls(P, None, ids, radius=4.0, order=order, invert=True)
        assert np.all(n[ids, 2] < 0)
    # a horizontal plane: the normal along z takes the frame's other branch (x and y both
    # negligible against z)
    H = np.c_[st, np.full(len(st), 5.0)].astype(np.float32)
    for order in (1, 2, 4):
        p, n, s = po.mls(H, None, ids, radius=4.0, order=order)
        assert np.all(s == 2)
        np.testing.assert_allclose(n[ids], np.broadcast_to([0, 0, 1], (len(ids), 3)), atol=1e-6)
        np.testing.assert_allclose(p[ids], H[ids], atol=1e-5)


def test_oracle_sphere_normals_and_projection():
    from oracle import pyoracle as po
    P = scene()
    ctr = np.array([10, -5, 30], np.float32)
    ids = np.arange(0, 6000, 20)
    radial = (P[ids] - ctr) / np.linalg.norm(P[ids] - ctr, axis=1, keepdims=True)
    err0 = np.abs(np.linalg.norm(P[ids] - ctr, axis=1) - 20).mean()
    # a quadric fits the sphere: normals within a degree and most of the noise projected
    # away; a plane (order 1) gives the normal of the weighted neighbourhood and moves
    # points onto its chord; orders 3 and 4 follow the noise of about 30 neighbours
    for order, max_deg in ((1, 3.0), (2, 1.0), (3, 3.0), (4, 3.0)):
        # viewpoint inside: normals face it, so inverted ones face out
        p, n, s = po.mls(P, None, ids, radius=4.0, order=order, invert=True, viewpoint=ctr)
        assert np.all(s == 2)
        assert chord_deg(n[ids], radial).max() < max_deg
        err1 = np.abs(np.linalg.norm(p[ids] - ctr, axis=1) - 20).mean()
        if order == 2:
            assert err1 < 0.4 * err0
        p, n, s = po.mls(P, None, ids, radius=4.0, order=order, viewpoint=ctr)
        assert chord_deg(n[ids], -radial).max() < max_deg


def test_oracle_skip_rules():
    """Fewer than 3 neighbours or a non-finite point: position and normal unchanged (NaN
    normals are created when the cloud has none); unlisted points untouched."""
    from oracle import pyoracle as po
    P = scene()
    ids = np.arange(12000, 12007)
    p, n, s = po.mls(P, None, ids, radius=4.0, order=2)
    assert np.all(s == 0)
    np.testing.assert_array_equal(p, P)
    assert np.all(np.isnan(n))
    N = np.random.default_rng(2).normal(size=P.shape).astype(np.float32)
    p, n, s = po.mls(P, N, np.r_[ids, 5], radius=4.0, order=2)
    assert s.tolist() == [0] * 7 + [2]
    keep = np.ones(len(P), bool)
    keep[5] = False
    np.testing.assert_array_equal(n[keep], N[keep])
    np.testing.assert_array_equal(p[keep], P[keep])


def test_cpp_mirror_compiles(tmp_path):
    src = tmp_path / "m.cpp"
    src.write_text(r'''
#include <ppf.h>
int main() {
    ppf::PointCloud pc;
    pc.point.emplace_back(0.f, 0.f, 0.f);
    ppf::estimateNormalMLS(pc, {0}, 1.0f, 2);
    ppf::estimateNormalMLS(pc, {}, 1.0f, 1, true);
    return 0;
}
''')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-DPPF_NO_EIGEN", "-I",
                        os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


# ---------------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("order,invert,with_vp,with_normals",
                         [(1, False, True, False), (2, False, True, True), (2, True, False, False),
                          (3, True, True, False), (4, False, True, True)])
def test_mls_matches_the_oracle(order, invert, with_vp, with_normals):
    from oracle import pyoracle as po
    from surface_match_gb300 import PointCloud, estimateNormalMLS
    rng = np.random.default_rng(order)
    P = scene()
    ids = listed(rng)
    N = rng.normal(size=P.shape).astype(np.float32) if with_normals else None
    vp = np.array([0, 0, 200], np.float32) if with_vp else None
    radius = 4.0
    op, on, st = po.mls(P, N, ids, radius=radius, order=order, invert=invert, viewpoint=vp)
    pc = estimateNormalMLS(PointCloud(P.copy(), None if N is None else N.copy(), vp), ids, radius,
                           order, invert)
    gp, gn = pc.point, pc.normal
    moved = np.unique(ids[st == 2])
    assert len(moved) >= 390 and set(st.tolist()) <= {0, 2}
    # untouched and skipped points: bit-exact (NaN where the cloud had no normals)
    rest = np.setdiff1d(np.arange(len(P)), moved)
    np.testing.assert_array_equal(gp[rest], op[rest])
    np.testing.assert_array_equal(gn[rest], on[rest])
    # moved points: the fit's point and oriented normal
    ang = chord_deg(gn[moved], on[moved])
    assert ang.max() < NORMAL_TOL_DEG, (ang.max(), moved[np.argmax(ang)])
    dp = np.linalg.norm(gp[moved] - op[moved], axis=1)
    assert dp.max() < POINT_TOL_REL * radius, dp.max()


@pytest.mark.gpu
def test_mls_argument_errors():
    from surface_match_gb300 import PointCloud, estimateNormalMLS
    P = scene()[:100]
    for kw in ({"order": 0}, {"order": 5}, {"radius": float("inf")}):
        args = {"radius": 4.0, "order": 2} | kw
        with pytest.raises(RuntimeError, match="order|radius"):
            estimateNormalMLS(PointCloud(P.copy()), None, **args)
    with pytest.raises(RuntimeError, match="index out of range"):
        estimateNormalMLS(PointCloud(P.copy()), [0, 100], 4.0, 2)
