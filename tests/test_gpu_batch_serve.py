"""Batching (sm_match_batch) and serving (sm_server_*) on the GPU: every job's result in
a batch, and every request's result in a concurrent serving mix, equals the same job run
alone through sm_match - bit for bit (the jobs share no state but the read-only models)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SD, KP, MS = 0.05, 0.2, 0.2


@pytest.fixture(scope="module")
def setup():
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    models = {}
    for k, name in enumerate(["gear", "bracket", "torus"]):
        cloud, surf, ctr = synth.model_cloud(name, 6000, 40 + k)
        det = Detector()
        det.trainModel(PointCloud(cloud.xyz, cloud.normal), SD)
        models[name] = (det, surf, ctr)
    rng = np.random.default_rng(5)
    jobs = []
    for i in range(6):
        name = ["gear", "bracket", "torus"][i % 3]
        _, surf, ctr = models[name]
        sc = synth.scene_random(int(rng.integers(1 << 30)), int(rng.integers(15000, 60000)),
                                {name: surf}, {name: ctr}, 0.3, 0.2, int(rng.integers(1, 4)),
                                box=((-120, -120, 0), (120, 120, 120)))
        jobs.append((models[name][0], PointCloud(sc.cloud.xyz, None, sc.viewpoint)))
    param = MatchParam(numMatches=8)
    alone = [det.matchScene(pc, SD, KP, MS, param) for det, pc in jobs]
    return jobs, alone, param


def _same(a, b):
    (pa, sa), (pb, sb) = a, b
    assert len(sa) == len(sb)
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(pa.view(np.uint32), pb.view(np.uint32))


def test_batch_equals_individual_matches(setup):
    from surface_match_gb300 import match_batch
    jobs, alone, param = setup
    assert sum(len(s) for _, s in alone) > 0, "the workload must find instances"
    for conc in (1, 3):
        out, stats = match_batch(jobs, SD, KP, MS, param, concurrency=conc)
        for j in range(len(jobs)):
            _same(out[j], alone[j])
        assert all(st["n_points"] == len(pc.point) for st, (_, pc) in zip(stats, jobs))


def test_serving_mix_equals_alone_and_respects_budget(setup):
    from surface_match_gb300 import Server
    jobs, alone, param = setup
    for slots, budget in ((3, 64 << 30), (2, 1)):  # roomy budget; budget forcing one at a time
        srv = Server(slots=slots, hbm_budget_bytes=budget)
        ids = [srv.submit(det, pc, SD, KP, MS, param) for det, pc in jobs]
        got = {}
        while len(got) < len(ids):
            for r in srv.poll(max_requests=16, max_results=param.numMatches, wait_ms=200):
                got[r["id"]] = r
        st = srv.status()
        srv.close()
        for j, rid in enumerate(ids):
            r = got[rid]
            assert r["status"] == 0
            assert r["total_ms"] >= r["service_ms"] > 0
            _same((r["poses"], r["scores"]), alone[j])
        assert st["completed"] == len(jobs) and st["queued"] == 0
        if budget == 1:  # every request exceeds the budget: admitted only when alone
            assert st["peak_bytes"] == max(64 * (1 << 20) + 512 * len(pc.point)
                                           for _, pc in jobs)


def test_precision_fp32_kahan_vs_fp64_accumulation():
    """The GPU's FP32 + Kahan accumulation (normals' covariance, ICP normal equations)
    against the oracle with FP64 accumulation (same search orders): sampled normals within a
    small angle, the same instance count, every instance pose within 0.1 deg and
    1e-3 * diameter."""
    from oracle import MODE_GRID, MatchParam as OMP, Oracle
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    cloud, surf, ctr = synth.model_cloud("gear", 8000, 60)
    sc = synth.scene_random(17, 80000, {"gear": surf}, {"gear": ctr}, 0.2, 0.2, 3,
                            box=((-120, -120, 0), (120, 120, 120)))
    det = Detector()
    det.trainModel(PointCloud(cloud.xyz, cloud.normal), SD)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), SD, KP, MS,
                                   MatchParam(numMatches=8, poseRefNumSteps=30))
    o = Oracle(mode=MODE_GRID, threads=8, fp64=True)
    m = o.train(cloud.xyz, cloud.normal, SD)
    r = o.match(m, sc.cloud.xyz, None, sc.viewpoint, SD, KP, MS,
                OMP(numMatches=8, poseRefNumSteps=30))
    ids = np.intersect1d(det.debug(0), r.sampled)
    a, b = det.debug(4)[ids].astype(np.float64), r.normals[ids].astype(np.float64)
    ang = np.degrees(np.arccos(np.clip(np.abs((a * b).sum(1)), 0, 1)))
    assert np.median(ang) < 1e-3 and np.percentile(ang, 99) < 0.1, (np.median(ang), ang.max())
    diam = float(np.linalg.norm(np.ptp(cloud.xyz, axis=0)))
    assert len(scores) == len(r.scores) and len(scores) > 0
    for P in poses:
        j = int(np.argmin([np.linalg.norm(P[:3, 3] - Q[:, 3]) for Q in r.poses]))
        Q = r.poses[j]
        R = P[:3, :3].astype(np.float64).T @ Q[:, :3].astype(np.float64)
        rot = np.degrees(np.arccos(np.clip((np.trace(R) - 1) / 2, -1, 1)))
        assert rot < 0.1 and np.linalg.norm(P[:3, 3] - Q[:, 3]) < 1e-3 * diam
