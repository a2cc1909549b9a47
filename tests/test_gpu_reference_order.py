"""The GPU path in the reference's search order (SM_ORDER_REFERENCE: the k-d tree built on
the GPU, tree-order sampling, depth-first neighbour order and search pruning) against the
oracle's reference-order pipeline, which restates the reference single-threaded on the
vendored nanoflann's orders. Bit-exact stage by stage on the tiny scene; at the full sizes
of the workloads (the small scene of about 108k points and the large scene of about 0.92M
points) the samples, keypoints, per-keypoint vote statistics, candidates and final poses
and scores are bit-exact - in the reference order against the oracle's reference-order mode,
and in the grid order against its grid-order mode."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SD = 0.05
KP = 0.2
MS = 0.2


@pytest.fixture(scope="module")
def tiny():
    from oracle import MODE_REF, MatchParam as OMP, Oracle
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny(seed=3)
    o = Oracle(mode=MODE_REF, threads=8)
    om = o.train(mc.xyz, mc.normal, SD)
    r = o.match(om, sc.cloud.xyz, None, sc.viewpoint, SD, KP, MS, OMP(numMatches=8))
    det = Detector(search_order="reference")
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), SD, KP, MS,
                                   MatchParam(numMatches=8))
    return om, r, det, poses, scores


def test_reference_order_train_bit_exact(tiny):
    om, _, det, _, _ = tiny
    d = det.download()
    for k, v in (("sampled", om.sampled), ("sampled_normal", om.sampled_normal),
                 ("resampled", om.resampled), ("resampled_normal", om.resampled_normal),
                 ("box", om.box), ("keys", om.keys), ("offsets", om.offsets), ("refs", om.refs)):
        np.testing.assert_array_equal(d[k], v, err_msg=k)
    np.testing.assert_array_equal(d["alphas"].view(np.uint32), om.alphas.view(np.uint32))


def test_reference_order_stages_bit_exact(tiny):
    _, r, det, poses, scores = tiny
    np.testing.assert_array_equal(det.debug(0), r.sampled, err_msg="sampled (tree order)")
    np.testing.assert_array_equal(det.debug(1), r.keypoints, err_msg="keypoints")
    np.testing.assert_array_equal(det.debug(2), r.resampled, err_msg="resampled")
    pos, nrm = det.debug(3), det.debug(4)
    np.testing.assert_array_equal(pos.view(np.uint32), r.positions.view(np.uint32))
    ok = np.isfinite(r.normals).all(1)
    np.testing.assert_array_equal(np.isfinite(nrm).all(1), ok)
    np.testing.assert_array_equal(nrm[ok].view(np.uint32), r.normals[ok].view(np.uint32))
    np.testing.assert_array_equal(det.debug(7), r.kp_stats, err_msg="keypoint stats")
    np.testing.assert_array_equal(det.debug(8), r.kp_cands, err_msg="candidates")
    np.testing.assert_array_equal(det.debug(9).view(np.uint32), r.pose_list.view(np.uint32))
    np.testing.assert_array_equal(det.debug(10).view(np.uint32), r.clustered.view(np.uint32))
    n = len(r.cand_status)
    np.testing.assert_array_equal(det.debug(15)[:n], r.cand_trace, err_msg="ICP traces")
    np.testing.assert_array_equal(det.debug(12)[:n], r.cand_status)
    assert len(scores) == len(r.scores) > 0
    np.testing.assert_array_equal(scores, r.scores)
    np.testing.assert_array_equal(poses[:, :3, :].reshape(len(scores), -1), r.results[:, :12])


@pytest.mark.parametrize("order", ["reference", "grid"])
@pytest.mark.parametrize("which", ["small", "large"])
def test_workload_scenes_bit_exact(which, order):
    """The two single-scene workloads at full size, in both search orders against the
    oracle's matching mode: the 3-gear scene (about 108k points, trainModel(0.04),
    matchScene(0.04, 0.1, 0.2)) and the 10-gear scene (about 0.92M points, trainModel(0.03),
    matchScene(0.03, 0.2, 0.2)), numMatches 16."""
    from oracle import MODE_GRID, MODE_REF, MatchParam as OMP, Oracle
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    model = synth.gear_model(20000, seed=7)
    if which == "small":
        sc, sd, kp = synth.scene_small(seed=1, model=model), 0.04, 0.1
    else:
        sc, sd, kp = synth.scene_large(seed=2, model=model), 0.03, 0.2
    mc = model[0]
    o = Oracle(mode=MODE_REF if order == "reference" else MODE_GRID, threads=16)
    om = o.train(mc.xyz, mc.normal, sd)
    r = o.match(om, sc.cloud.xyz, None, sc.viewpoint, sd, kp, MS, OMP(numMatches=16))
    det = Detector(search_order=order)
    det.trainModel(PointCloud(mc.xyz, mc.normal), sd)
    d = det.download()
    np.testing.assert_array_equal(d["keys"], om.keys)
    np.testing.assert_array_equal(d["refs"], om.refs)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), sd, kp, MS,
                                   MatchParam(numMatches=16))
    np.testing.assert_array_equal(det.debug(0), r.sampled, err_msg="sampled")
    np.testing.assert_array_equal(det.debug(1), r.keypoints, err_msg="keypoints")
    np.testing.assert_array_equal(det.debug(2), r.resampled, err_msg="resampled")
    np.testing.assert_array_equal(det.debug(7), r.kp_stats, err_msg="keypoint stats")
    np.testing.assert_array_equal(det.debug(8), r.kp_cands, err_msg="candidates")
    assert len(scores) == len(r.scores) >= 2
    np.testing.assert_array_equal(scores, r.scores)
    np.testing.assert_array_equal(poses[:, :3, :].reshape(len(scores), -1), r.results[:, :12])
