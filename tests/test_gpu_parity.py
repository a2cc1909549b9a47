"""Parity of the GPU path with the CPU oracle (run on a GB300: -m gpu).

Bit-exact: sampling, keypoints, normals, PPF keys / hash hits / per-(reference, bin)
votes, candidates, pose list, clustering and ICP results against the oracle's GPU-order
mode; and the voting kernel against the oracle's reference-order mode (k-d tree neighbour
order, i.e. the reference's lane assignment) on identical inputs.
Tolerance: final poses against the reference-order pipeline within 0.1 degree and
1e-3 * model diameter.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SD = 0.05
KP = 0.2
MS = 0.2


@pytest.fixture(scope="module")
def data():
    from surface_match_gb300 import synth
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny(seed=3)
    return mc, sc


@pytest.fixture(scope="module")
def oracle_grid(data):
    from oracle import MODE_GRID, MatchParam, Oracle
    mc, sc = data
    o = Oracle(mode=MODE_GRID, threads=8)
    m = o.train(mc.xyz, mc.normal, SD)
    r = o.match(m, sc.cloud.xyz, None, sc.viewpoint, SD, KP, MS, MatchParam(numMatches=8))
    return m, r


@pytest.fixture(scope="module")
def oracle_ref(data):
    from oracle import MODE_REF, MatchParam, Oracle
    mc, sc = data
    o = Oracle(mode=MODE_REF, threads=8)
    m = o.train(mc.xyz, mc.normal, SD)
    r = o.match(m, sc.cloud.xyz, None, sc.viewpoint, SD, KP, MS, MatchParam(numMatches=8),
                dump_k=6)
    return m, r


@pytest.fixture(scope="module")
def gpu(data):
    from surface_match_gb300 import Detector, MatchParam, PointCloud
    mc, sc = data
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), SD, KP, MS,
                                   MatchParam(numMatches=8))
    return det, poses, scores


def test_train_matches_oracle_bit_exact(gpu, oracle_grid):
    det = gpu[0]
    m, _ = oracle_grid
    d = det.download()
    for k, v in (("sampled", m.sampled), ("sampled_normal", m.sampled_normal),
                 ("resampled", m.resampled), ("resampled_normal", m.resampled_normal),
                 ("box", m.box), ("keys", m.keys), ("offsets", m.offsets), ("refs", m.refs)):
        np.testing.assert_array_equal(d[k], v, err_msg=k)
    np.testing.assert_array_equal(d["alphas"].view(np.uint32), m.alphas.view(np.uint32))


def test_scene_sampling_and_normals_bit_exact(gpu, oracle_grid):
    det = gpu[0]
    _, r = oracle_grid
    np.testing.assert_array_equal(det.debug(0), r.sampled)
    np.testing.assert_array_equal(det.debug(1), r.keypoints)
    np.testing.assert_array_equal(det.debug(2), r.resampled)
    pos, nrm = det.debug(3), det.debug(4)
    np.testing.assert_array_equal(pos.view(np.uint32), r.positions.view(np.uint32))
    ok = np.isfinite(r.normals).all(1)
    np.testing.assert_array_equal(np.isfinite(nrm).all(1), ok)
    np.testing.assert_array_equal(nrm[ok].view(np.uint32), r.normals[ok].view(np.uint32))


def test_votes_keys_and_candidates_bit_exact(gpu, oracle_grid):
    det = gpu[0]
    _, r = oracle_grid
    st = det.debug(7)
    np.testing.assert_array_equal(st, r.kp_stats)  # neighbours, hits, votes, fingerprint
    np.testing.assert_array_equal(det.debug(8), r.kp_cands)
    np.testing.assert_array_equal(det.debug(9).view(np.uint32), r.pose_list.view(np.uint32))


def test_clustering_and_icp_bit_exact(gpu, oracle_grid):
    det, poses, scores = gpu
    _, r = oracle_grid
    np.testing.assert_array_equal(det.debug(10).view(np.uint32), r.clustered.view(np.uint32))
    n = len(r.cand_status)
    np.testing.assert_array_equal(det.debug(15)[:n], r.cand_trace)  # per-iteration ICP trace
    np.testing.assert_array_equal(det.debug(12)[:n], r.cand_status)
    ok = r.cand_status == 0
    np.testing.assert_array_equal(det.debug(13)[:n][ok], r.cand_score[ok])
    np.testing.assert_array_equal(det.debug(14)[:n][ok], r.cand_pose[ok])
    assert len(scores) == len(r.scores)
    np.testing.assert_array_equal(scores, r.scores)
    np.testing.assert_array_equal(poses[:, :3, :].reshape(len(scores), -1),
                                  r.results[:, :12])


def test_vote_kernel_reference_order_bit_exact(oracle_ref):
    """Voting on the reference-order scene state: the oracle's k-d tree neighbour lists
    (the reference's unsorted radius-search order, which decides each pair's 8-lane block /
    scalar-tail rule) and the reference-order model table, uploaded unchanged."""
    from surface_match_gb300 import Detector, TrainParam
    m, r = oracle_ref
    det = Detector()
    det.upload(m.sampled, m.sampled_normal, m.resampled, m.resampled_normal, m.box, m.keys,
               m.offsets, m.refs, m.alphas, SD, TrainParam())
    stats, cands, poses, acc = det.vote_stage(r.positions, r.normals, r.keypoints, r.nbr_off,
                                              r.nbr_ids, MS, dump_k=6)
    np.testing.assert_array_equal(stats, r.kp_stats)
    np.testing.assert_array_equal(cands, r.kp_cands)
    np.testing.assert_array_equal(acc, r.acc_dump)
    emitted = poses[stats[:, 6][:, None] > np.arange(3)[None, :]]
    np.testing.assert_array_equal(emitted.view(np.uint32), r.pose_list.view(np.uint32))


@pytest.mark.parametrize("dist_rel,angles,wide", [(0.25, 12, False), (0.04, 360, False),
                                                   (0.25, 12, True), (0.04, 360, True)])
def test_vote_kernel_counter_widths_and_passes(data, dist_rel, angles, wide, monkeypatch):
    """The accumulator's other regimes, bit-exact against the oracle: coarse distance
    steps make buckets so large that keypoints cast more than 65535 votes (the per-cell
    bound still keeps them on 16-bit counters), 360 angle bins make the accumulator larger
    than one CTA's shared memory (several reference-point passes), and the 32-bit counters
    that the bound reserves for extreme inputs are forced on (one and several passes)."""
    from oracle import MODE_REF, MatchParam, Oracle, TrainParam as OTP
    from surface_match_gb300 import Detector, TrainParam
    if wide:
        monkeypatch.setenv("SM_VOTE_FORCE_WIDE", "1")
    mc, sc = data
    o = Oracle(mode=MODE_REF, threads=8)
    m = o.train(mc.xyz, mc.normal, SD, OTP(featDistanceStepRel=dist_rel,
                                           featAngleResolution=angles))
    r = o.match(m, sc.cloud.xyz, None, sc.viewpoint, SD, KP, MS, MatchParam(numMatches=8),
                dump_k=4)
    if dist_rel > 0.2:
        assert r.kp_stats[:, 3].max() > 65535
    assert r.kp_stats[:, 7].max() <= 65535  # the bound: 16-bit unless forced
    if angles == 360:
        assert len(m.sampled) * angles * 2 > 200 * 1024
    det = Detector()
    det.upload(m.sampled, m.sampled_normal, m.resampled, m.resampled_normal, m.box, m.keys,
               m.offsets, m.refs, m.alphas, SD,
               TrainParam(featDistanceStepRel=dist_rel, featAngleResolution=angles))
    stats, cands, poses, acc = det.vote_stage(r.positions, r.normals, r.keypoints, r.nbr_off,
                                              r.nbr_ids, MS, dump_k=4)
    np.testing.assert_array_equal(stats, r.kp_stats)
    np.testing.assert_array_equal(cands, r.kp_cands)
    np.testing.assert_array_equal(acc, r.acc_dump)
    emitted = poses[stats[:, 6][:, None] > np.arange(3)[None, :]]
    np.testing.assert_array_equal(emitted.view(np.uint32), r.pose_list.view(np.uint32))


def test_poses_within_tolerance_of_reference_order(gpu, oracle_ref, data):
    """End to end against the reference-order pipeline (k-d tree sampling and neighbour
    order): same instance count; each GPU pose within 0.1 deg / 1e-3 * diameter of the
    reference-order pose it matches, modulo the gear's symmetry group."""
    from surface_match_gb300 import synth
    det, poses, scores = gpu
    m, r = oracle_ref
    diam = float(np.linalg.norm(m.box[3:] - m.box[:3]))
    assert len(scores) == len(r.scores)
    ref = [np.vstack([Q, [0, 0, 0, 1]]) for Q in r.poses]
    for rot, tr in synth.match_poses(poses, ref, synth.gear_symmetries()):
        assert rot < 0.1 and tr < 1e-3 * diam, (rot, tr)


def test_vote_atomic_probe_rate_is_plausible():
    """The measured shared-atomic rate that the vote kernel's roofline is quoted against:
    positive, and between 0.05 and 64 increments per SM per clock at any clock the GPU runs
    (a 32-lane warp instruction per clock is the hard ceiling)."""
    import torch
    from surface_match_gb300 import probe_vote_atomics
    rate = probe_vote_atomics(0)
    props = torch.cuda.get_device_properties(0)
    per_sm = rate / props.multi_processor_count
    assert 0.05 * 0.5e9 < per_sm < 64 * 3.0e9


def test_errors_mirror_reference(data):
    """matchScene's argument checks, in the reference's order and with its exception types
    and messages (ppf.cpp:153-168): untrained model, fractions out of range, empty scene."""
    from surface_match_gb300 import Detector, PointCloud, RangeError
    mc, sc = data
    with pytest.raises(RuntimeError, match="No trained model in matchScene"):
        Detector().matchScene(PointCloud(sc.cloud.xyz), SD, KP, MS)
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    for args, what in (((1.5, KP, MS), "samplingDistanceRel"), ((SD, -0.1, MS), "keyPointFraction"),
                       ((SD, KP, 2.0), "minScore")):
        with pytest.raises(RangeError, match=what):
            det.matchScene(PointCloud(sc.cloud.xyz), *args)
    with pytest.raises(RuntimeError, match="empty scene in matchScene"):
        det.matchScene(PointCloud(np.zeros((0, 3), np.float32)), SD, KP, MS)


def test_nan_points_like_the_oracle(data):
    """Scenes with non-finite coordinates (removeNan, util.cpp:86-105): with 5% of the points
    broken, every stage and the final poses are bit-exact against the oracle on the same
    input; a scene with no finite point returns no pose."""
    from oracle import MODE_GRID, MatchParam as OMP, Oracle
    from surface_match_gb300 import Detector, MatchParam, PointCloud
    mc, sc = data
    xyz = sc.cloud.xyz.copy()
    rng = np.random.default_rng(11)
    bad = rng.choice(len(xyz), len(xyz) // 20, replace=False)
    xyz[bad, rng.integers(0, 3, len(bad))] = np.nan
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    poses, scores = det.matchScene(PointCloud(xyz, None, sc.viewpoint), SD, KP, MS,
                                   MatchParam(numMatches=8))
    o = Oracle(mode=MODE_GRID, threads=8)
    m = o.train(mc.xyz, mc.normal, SD)
    r = o.match(m, xyz, None, sc.viewpoint, SD, KP, MS, OMP(numMatches=8))
    np.testing.assert_array_equal(det.debug(0), r.sampled)
    np.testing.assert_array_equal(det.debug(1), r.keypoints)
    np.testing.assert_array_equal(det.debug(7), r.kp_stats)
    assert len(scores) == len(r.scores) > 0
    np.testing.assert_array_equal(scores, r.scores)
    np.testing.assert_array_equal(poses[:, :3, :].reshape(len(scores), -1), r.results[:, :12])
    none, _ = det.matchScene(PointCloud(np.full((1000, 3), np.nan, np.float32)), SD, KP, MS)
    assert len(none) == 0


def test_workspace_reuse_across_scene_sizes():
    """One detector matching scenes of alternating sizes (its workspace grows and is
    reused, entries of earlier calls stay behind): every result equals a fresh detector's."""
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    mc, _, _ = synth.gear_model(8000, seed=5)
    scenes = [synth.scene_small(seed=1), synth.scene_tiny(seed=3), synth.scene_small(seed=4),
              synth.scene_tiny(seed=5, n_inst=3, pts=4000)]
    param = MatchParam(numMatches=8)
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    for sc in scenes + scenes[::-1]:
        pc = PointCloud(sc.cloud.xyz, None, sc.viewpoint)
        p1, s1 = det.matchScene(pc, SD, KP, MS, param)
        fresh = Detector()
        fresh.trainModel(PointCloud(mc.xyz, mc.normal), SD)
        p2, s2 = fresh.matchScene(pc, SD, KP, MS, param)
        np.testing.assert_array_equal(s1, s2)
        np.testing.assert_array_equal(p1, p2)


def test_sampler_heavy_cells_and_wide_extent_bit_exact(data):
    """The grid-order sampler on a scene that stresses its cell table: a clump of 6000
    points inside one sampling cell (cells above 192 points are thinned by a whole CTA) and
    two far points that stretch the box to ~10^10 cells at the refinement step (only
    occupied cells are stored; the cell side stays at the step). Sampled, keypoint and
    resampled sets equal the oracle's."""
    from oracle import MODE_GRID, MatchParam as OMP, Oracle
    from surface_match_gb300 import Detector, MatchParam, PointCloud
    mc, sc = data
    rng = np.random.default_rng(17)
    diam = float(np.linalg.norm(mc.xyz.max(0) - mc.xyz.min(0)))
    c0 = sc.cloud.xyz[np.isfinite(sc.cloud.xyz).all(1)].mean(0)
    clump = c0 + rng.normal(0, 0.3 * SD * diam, (6000, 3))
    far = np.array([c0 - 120 * diam, c0 + 120 * diam])
    xyz = np.ascontiguousarray(np.vstack([sc.cloud.xyz, clump, far]), np.float32)
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    det.matchScene(PointCloud(xyz, None, sc.viewpoint), SD, KP, MS, MatchParam(numMatches=8))
    o = Oracle(mode=MODE_GRID, threads=8)
    m = o.train(mc.xyz, mc.normal, SD)
    r = o.match(m, xyz, None, sc.viewpoint, SD, KP, MS, OMP(numMatches=8))
    np.testing.assert_array_equal(det.debug(0), r.sampled)
    np.testing.assert_array_equal(det.debug(1), r.keypoints)
    np.testing.assert_array_equal(det.debug(2), r.resampled)


@pytest.mark.parametrize("shape", ["256", "512", "1024", "256p", "512p", "1024p"])
def test_vote_launch_shapes_give_identical_results(data, oracle_grid, monkeypatch, shape):
    """The voting stage's launch tuner picks among CTA sizes that must not change anything:
    with each size forced, per-keypoint statistics (with the accumulator fingerprints),
    candidates, the pose list and the final poses equal the oracle's."""
    from surface_match_gb300 import Detector, MatchParam, PointCloud
    mc, sc = data
    _, r = oracle_grid
    monkeypatch.setenv("SM_VOTE_SHAPE", shape)
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), SD, KP, MS,
                                   MatchParam(numMatches=8))
    np.testing.assert_array_equal(det.debug(7), r.kp_stats)
    np.testing.assert_array_equal(det.debug(8), r.kp_cands)
    np.testing.assert_array_equal(det.debug(9).view(np.uint32), r.pose_list.view(np.uint32))
    np.testing.assert_array_equal(scores, r.scores)


def test_vote_launch_tuner_picks_a_shape_once():
    """On a scene with at least 512 keypoints the tuner times the CTA sizes once per device
    and reports its choice; later calls keep it."""
    import os
    from surface_match_gb300 import Detector, MatchParam, PointCloud, _lib, synth
    if os.environ.get("SM_VOTE_SHAPE"):
        pytest.skip("launch size fixed by the environment")
    model, _, _ = synth.gear_model(20000, seed=7)
    scene = synth.scene_large(seed=2, model=synth.gear_model(20000, seed=7))
    det = Detector()
    det.trainModel(PointCloud(model.xyz, model.normal), 0.03)
    det.matchScene(PointCloud(scene.cloud.xyz, None, scene.viewpoint), 0.03, 0.2, 0.2,
                   MatchParam(numMatches=16))
    assert det.last_stats["n_keypoints"] >= 512
    import ctypes as C
    L = _lib.load()
    t, p = C.c_int(0), C.c_int(0)
    assert L.sm_vote_tuned_shape(0, C.byref(t), C.byref(p)) == 0
    first = (t.value, p.value)
    assert first[0] in (256, 512, 1024) and first[1] in (0, 1)
    det.matchScene(PointCloud(scene.cloud.xyz, None, scene.viewpoint), 0.03, 0.2, 0.2,
                   MatchParam(numMatches=16))
    assert L.sm_vote_tuned_shape(0, C.byref(t), C.byref(p)) == 0
    assert (t.value, p.value) == first
