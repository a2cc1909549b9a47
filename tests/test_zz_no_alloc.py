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


def test_noalloc_vote_stage_matches_allocating_entry_twice():
    import torch
    from surface_match_gb300 import _lib
    det, pos, nrm, kp, off, ids = _inputs()
    L = _lib.load()
    dump = 3
    ref_stats, ref_cands, ref_poses, ref_acc = det.vote_stage(pos, nrm, kp, off, ids, 0.2,
                                                              dump_k=dump)
    K = len(kp)
    dpos = torch.from_numpy(pos).cuda()
    dnrm = torch.from_numpy(nrm).cuda()
    dkp = torch.from_numpy(kp).cuda()
    doff = torch.from_numpy(off).cuda()
    dids = torch.from_numpy(ids).cuda()
    for call in range(2):
        stats = torch.full((K, 8), -7, dtype=torch.int64, device="cuda")
        cands = torch.full((K, 9), -7.0, dtype=torch.float32, device="cuda")
        poses = torch.full((K, 3, 18), -7.0, dtype=torch.float32, device="cuda")
        acc = torch.full((len(ref_acc),), -7, dtype=torch.int32, device="cuda")
        rc = L.sm_vote_stage_noalloc(det.model, _dev_ptr(dpos), _dev_ptr(dnrm), len(pos),
                                     _dev_ptr(dkp), K, _dev_ptr(doff), _dev_ptr(dids), 0.2,
                                     _dev_ptr(stats), _dev_ptr(cands), _dev_ptr(poses), dump,
                                     _dev_ptr(acc))
        assert rc == 0, _lib.last_error()
        np.testing.assert_array_equal(stats.cpu().numpy(), ref_stats, err_msg=f"call {call}")
        np.testing.assert_array_equal(cands.cpu().numpy(), ref_cands, err_msg=f"call {call}")
        np.testing.assert_array_equal(poses.cpu().numpy().view(np.uint32),
                                      ref_poses.view(np.uint32), err_msg=f"call {call}")
        np.testing.assert_array_equal(acc.cpu().numpy(), ref_acc, err_msg=f"call {call}")
    assert (ref_stats[:, 3] > 0).any(), "the case must cast votes"


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
