"""The opt-in kernel clock (sm_context_kernel_clock / sm_context_kernel_report): per-launch
event timing of the sampler phases, the scans and the refinement's correspondence search.
It counts launches and algorithmic bytes only while on, and does not change any result."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SD = 0.05


def test_kernel_clock_counts_and_leaves_results_unchanged():
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny(seed=3)
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    scene = PointCloud(sc.cloud.xyz, None, sc.viewpoint)
    p0, s0 = det.matchScene(scene, SD, 0.2, 0.2, MatchParam(numMatches=8))
    off = det.ctx.kernel_report()
    assert all(r["launches"] == 0 for r in off.values())
    det.ctx.kernel_clock(True)
    p1, s1 = det.matchScene(scene, SD, 0.2, 0.2, MatchParam(numMatches=8))
    rep = det.ctx.kernel_report()
    det.ctx.kernel_clock(False)
    np.testing.assert_array_equal(s0, s1)
    np.testing.assert_array_equal(p0.view(np.uint32), p1.view(np.uint32))
    st = det.last_stats
    # three samplings of 8 phases; 20 bytes per point of each sampling
    assert rep["k_sample_phase"]["launches"] == 24
    want = 20.0 * (st["n_valid"] + st["n_sampled"] + st["n_valid"])
    assert rep["k_sample_phase"]["bytes"] == pytest.approx(want)
    assert rep["k_scan_lookback"]["launches"] > 0
    assert len(s1) > 0 and rep["k_corr"]["launches"] > 0 and rep["k_corr"]["bytes"] > 0
    for r in rep.values():
        assert r["ms"] > 0
    # switched off: nothing more is counted (and on again starts from zero)
    det.matchScene(scene, SD, 0.2, 0.2, MatchParam(numMatches=8))
    assert det.ctx.kernel_report() == rep
    det.ctx.kernel_clock(True)
    assert all(r["launches"] == 0 for r in det.ctx.kernel_report().values())
    det.ctx.kernel_clock(False)
