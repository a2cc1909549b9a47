"""The pose comparison behind the end-to-end agreement checks (bench reference_order_parity
and its vs_truth lists, the GPU pose-tolerance test): the gear's symmetry group really maps
the model onto itself, errors are taken modulo that group, and poses are paired with the
nearest unused reference pose. CPU only."""
import numpy as np
import pytest

from surface_match_gb300 import synth


def rot(axis, deg):
    a = np.radians(deg)
    k = np.asarray(axis, np.float64)
    k /= np.linalg.norm(k)
    K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
    return np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * K @ K


def pose(R, t):
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = t
    return T


def test_gear_symmetries_map_the_model_onto_itself():
    scipy = pytest.importorskip("scipy.spatial")
    P = synth.gear_model(20000, seed=7)[0].xyz.astype(np.float64)
    tree = scipy.cKDTree(P)
    spacing = np.percentile(tree.query(P, k=2)[0][:, 1], 99)  # sample spacing
    syms = synth.gear_symmetries()
    assert len(syms) == 48
    for S in syms:
        assert np.allclose(S @ S.T, np.eye(3)) and np.isclose(abs(np.linalg.det(S)), 1)
        assert np.percentile(tree.query(P @ S.T)[0], 99) < 1.2 * spacing
    # half a tooth pitch is not a symmetry: tips land in gaps
    assert np.percentile(tree.query(P @ rot([0, 0, 1], 7.5).T)[0], 99) > 3 * spacing


def test_pose_error_modulo_symmetry():
    syms = synth.gear_symmetries()
    A = pose(rot([1, 2, 3], 40), [10, -20, 30])
    for S in syms[::7]:
        r, t = synth.pose_error_sym(A, A @ pose(S, [0, 0, 0]), syms)
        assert r < 1e-5 and t < 1e-9
    r, t = synth.pose_error_sym(A, A @ pose(rot([1, 0, 0], 2.0), [0, 0, 0]), syms)
    assert abs(r - 2.0) < 1e-6
    B = pose(A[:3, :3], A[:3, 3] + [0.3, 0.4, 0])
    assert synth.pose_error_sym(A, B, syms)[1] == pytest.approx(0.5)


def test_match_poses_pairs_nearest_unused():
    syms = synth.gear_symmetries()
    rng = np.random.default_rng(3)
    ref = [pose(rot(rng.normal(size=3), rng.uniform(0, 180)), rng.uniform(-200, 200, 3))
           for _ in range(5)]
    # found poses: a slightly perturbed, shuffled subset of the references
    order = [3, 0, 4]
    found = [r @ pose(rot([0, 1, 0], 0.05), [0.01, 0, 0]) for r in (ref[i] for i in order)]
    err = synth.match_poses(found, ref, syms)
    assert len(err) == 3
    for r, t in err:
        assert abs(r - 0.05) < 1e-4 and t < 0.02
    # more found poses than references: pairing stops when the references run out
    assert len(synth.match_poses(found + found, ref[:2], syms)) == 2
