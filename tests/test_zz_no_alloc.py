"""sm_vote_stage_noalloc: the voting stage for callers that may not allocate device memory
(a plugin whose host framework owns all device memory, a latency-critical loop that cannot
take cudaMalloc's implicit synchronisation). It takes caller-owned device buffers and keeps
its staging in a fixed array of the library's device image, so its results must equal
sm_vote_stage's (which stages through the context's allocated workspace) bit for bit, call
after call, while the shared array carries the previous call's contents.

Collected last on purpose (file name), so a run that stops at the first failure has run
every other test first; it builds all its inputs itself and runs alone as well.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev_ptr(t):
    return C.c_void_p(t.data_ptr())


def _workspace_bytes(det):
    from surface_match_gb300 import _lib
    b = C.c_int64(-1)
    assert _lib.load().sm_context_workspace_bytes(det.ctx.handle, C.byref(b)) == 0
    return b.value


def _inputs():
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    mc, _, _ = synth.gear_model(6000, seed=5)
    sc = synth.scene_tiny(seed=9, n_inst=2, pts=5000)
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), 0.05)
    det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), 0.05, 0.2, 0.2,
                   MatchParam(numMatches=4))
    pos, nrm = det.debug(3), det.debug(4)
    sampled, kp = det.debug(0), det.debug(1)
    diam = float(np.linalg.norm(np.ptp(mc.xyz, axis=0)))
    d = pos[kp][:, None, :] - pos[sampled][None, :, :]
    d2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    inside = d2 < np.float32(diam * diam)
    off = np.concatenate([[0], np.cumsum(inside.sum(1))]).astype(np.int32)
    ids = np.concatenate([sampled[row] for row in inside]).astype(np.int32)
    nrm = np.where(np.isfinite(nrm), nrm, 0).astype(np.float32)
    return det, pos.astype(np.float32), nrm, kp.astype(np.int32), off, ids


def _run_noalloc(det, L, pos, nrm, kp, off, ids, n_acc, dump):
    import torch
    K = len(kp)
    dpos = torch.from_numpy(pos).cuda()
    dnrm = torch.from_numpy(nrm).cuda()
    dkp = torch.from_numpy(kp).cuda()
    doff = torch.from_numpy(off).cuda()
    dids = torch.from_numpy(ids).cuda()
    stats = torch.full((K, 8), -7, dtype=torch.int64, device="cuda")
    cands = torch.full((K, 9), -7.0, dtype=torch.float32, device="cuda")
    poses = torch.full((K, 3, 18), -7.0, dtype=torch.float32, device="cuda")
    acc = torch.full((max(n_acc, 1),), -7, dtype=torch.int32, device="cuda")
    # the library works on its context's own stream: the inputs and the -7 fills, written on
    # torch's stream, must be complete before the call
    torch.cuda.synchronize()
    rc = L.sm_vote_stage_noalloc(det.model, _dev_ptr(dpos), _dev_ptr(dnrm), len(pos),
                                 _dev_ptr(dkp), K, _dev_ptr(doff), _dev_ptr(dids), 0.2,
                                 _dev_ptr(stats), _dev_ptr(cands), _dev_ptr(poses), dump,
                                 _dev_ptr(acc))
    return rc, stats.cpu().numpy(), cands.cpu().numpy(), poses.cpu().numpy(), \
        acc.cpu().numpy()[:n_acc]


def _check_equal(got, ref, what):
    stats, cands, poses, acc = got
    ref_stats, ref_cands, ref_poses, ref_acc = ref
    np.testing.assert_array_equal(stats, ref_stats, err_msg=what)
    np.testing.assert_array_equal(cands, ref_cands, err_msg=what)
    np.testing.assert_array_equal(poses.view(np.uint32), ref_poses.view(np.uint32), err_msg=what)
    np.testing.assert_array_equal(acc, ref_acc, err_msg=what)


def test_noalloc_vote_stage_matches_allocating_entry_twice():
    from surface_match_gb300 import _lib
    det, pos, nrm, kp, off, ids = _inputs()
    L = _lib.load()
    dump = 3
    ref = det.vote_stage(pos, nrm, kp, off, ids, 0.2, dump_k=dump)
    ws = _workspace_bytes(det)
    for call in range(2):
        rc, *got = _run_noalloc(det, L, pos, nrm, kp, off, ids, len(ref[3]), dump)
        assert rc == 0, _lib.last_error()
        _check_equal(got, ref, f"call {call}")
    # the entry's contract: nothing is allocated, the context's workspace did not grow
    assert _workspace_bytes(det) == ws
    assert (ref[0][:, 3] > 0).any(), "the case must cast votes"


def test_noalloc_vote_stage_matches_on_32bit_counters(monkeypatch):
    """The switch that forces 32-bit accumulator counters reaches both entries; their
    results still agree bit for bit."""
    from surface_match_gb300 import _lib
    det, pos, nrm, kp, off, ids = _inputs()
    L = _lib.load()
    monkeypatch.setenv("SM_VOTE_FORCE_WIDE", "1")
    ref = det.vote_stage(pos, nrm, kp, off, ids, 0.2, dump_k=2)
    rc, *got = _run_noalloc(det, L, pos, nrm, kp, off, ids, len(ref[3]), 2)
    assert rc == 0, _lib.last_error()
    _check_equal(got, ref, "32-bit counters")


def test_noalloc_vote_stage_rejects_bad_offsets_before_reading_lists():
    """Decreasing offsets whose last entry lies far beyond the ids buffer, and monotone
    offsets whose total runs past the ids allocation, are argument errors; the lists are
    never read with them."""
    from surface_match_gb300 import _lib
    det, pos, nrm, kp, off, ids = _inputs()
    L = _lib.load()
    bad = off.copy()
    bad[1] = bad[2] + 5  # decreasing at 1 -> 2
    bad[-1] = 1 << 30
    rc, *_ = _run_noalloc(det, L, pos, nrm, kp, bad, ids, 0, 0)
    assert rc == _lib.SM_ERR_ARG, _lib.last_error()
    # monotone lists of at most n entries each, whose total (2000 x n ids, tens of MB) runs
    # far past the small allocation that holds the ids
    kp2 = np.resize(kp, 2000).astype(np.int32)
    huge = (np.arange(2001, dtype=np.int64) * len(pos)).astype(np.int32)
    rc, *_ = _run_noalloc(det, L, pos, nrm, kp2, huge, ids, 0, 0)
    assert rc == _lib.SM_ERR_ARG, _lib.last_error()
    assert "nbr_ids" in _lib.last_error()
    # the context is still usable after the rejections
    ref = det.vote_stage(pos, nrm, kp, off, ids, 0.2)
    rc, *got = _run_noalloc(det, L, pos, nrm, kp, off, ids, 0, 0)
    assert rc == 0, _lib.last_error()
    _check_equal(got, (ref[0], ref[1], ref[2], np.zeros(0, np.int32)), "after rejections")


def test_noalloc_vote_stage_rejects_sizes_beyond_its_scratch():
    import torch
    from surface_match_gb300 import _lib
    det, pos, nrm, kp, off, ids = _inputs()
    L = _lib.load()
    big = 131072 + 1
    d = torch.zeros(16, dtype=torch.int64, device="cuda")
    p = _dev_ptr(d)
    rc = L.sm_vote_stage_noalloc(det.model, p, p, big, p, 1, p, p, 0.2, p, p, p, 0, None)
    assert rc == _lib.SM_ERR_CAPACITY
    assert "131072" in _lib.last_error()
    rc = L.sm_vote_stage_noalloc(det.model, p, p, 10, p, 65537, p, p, 0.2, p, p, p, 0, None)
    assert rc == _lib.SM_ERR_CAPACITY
