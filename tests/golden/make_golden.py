"""Generate the golden fixtures of tests/golden/ (run in the build container, where the
reference source tree is present; the fixtures are committed and the GPU machine reads only
them).

* murmur_kat.json  - MurmurHash3_x86_32(4 words, len 16, seed 42) known answers from the
                     reference's own scalar murmurhash3 (util.cpp:643-688), compiled by
                     oracle/ref_probe/build_ref.py.
* kdtree_ref.npz   - build order (vAcc_) and unsorted radius-search order of the
                     reference's vendored nanoflann on a seeded cloud, plus 10-NN results.
* oracle_tiny.npz  - the oracle's stage outputs (sampled ids, keypoints, per-keypoint vote
                     statistics and candidates, final poses) on a seeded two-gear scene,
                     in both search-order modes: a regression pin of the restatement.
"""
import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_probe"))

f32p, i32p = C.POINTER(C.c_float), C.POINTER(C.c_int32)


def murmur_kat():
    import build_ref
    M = C.CDLL(build_ref.build_murmur())
    M.ref_murmur.restype = C.c_uint32
    M.ref_murmur.argtypes = [i32p, C.c_uint32, C.c_uint32]
    rng = np.random.default_rng(11)
    words = np.concatenate([rng.integers(0, 40, (48, 4)), rng.integers(0, 2 ** 31, (16, 4)),
                            np.array([[0, 0, 0, 0], [15, 15, 15, 25], [1, 2, 3, 4]])])
    out = []
    for w in words.astype(np.int32):
        out.append([[int(v) for v in w], int(M.ref_murmur(w.ctypes.data_as(i32p), 16, 42))])
    with open(os.path.join(HERE, "murmur_kat.json"), "w") as f:
        json.dump(out, f)


def kdtree_ref():
    import build_ref
    R = C.CDLL(build_ref.build_kd())
    R.ref_kd_probe.restype = C.c_int64
    R.ref_kd_probe.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_float, i32p, i32p, C.c_int64]
    R.ref_kd_knn.argtypes = [f32p, C.c_int64, f32p, f32p, C.c_int64, C.c_int, i32p, f32p]
    rng = np.random.default_rng(12)
    P = np.ascontiguousarray(np.concatenate([rng.uniform(-50, 50, (1500, 3)),
                                             np.round(rng.uniform(-5, 5, (500, 3)))])
                             .astype(np.float32))
    n = len(P)
    box = np.concatenate([P.min(0), P.max(0)]).astype(np.float32)
    qi = rng.integers(n, size=8)
    r2 = np.float32(30.0 ** 2)
    vacc = np.zeros(n, np.int32)
    found_off, found = [0], []
    for i in qi:
        q = np.ascontiguousarray(P[i])
        f = np.zeros(n, np.int32)
        k = R.ref_kd_probe(P.ctypes.data_as(f32p), n, box.ctypes.data_as(f32p),
                           q.ctypes.data_as(f32p), r2, vacc.ctypes.data_as(i32p),
                           f.ctypes.data_as(i32p), n)
        found.extend(f[:k].tolist())
        found_off.append(len(found))
    nq, k = 64, 10
    qs = np.ascontiguousarray(P[rng.integers(n, size=nq)] + rng.normal(0, 0.5, (nq, 3))
                              .astype(np.float32))
    ki, kd = np.zeros((nq, k), np.int32), np.zeros((nq, k), np.float32)
    R.ref_kd_knn(P.ctypes.data_as(f32p), n, box.ctypes.data_as(f32p), qs.ctypes.data_as(f32p),
                 nq, k, ki.ctypes.data_as(i32p), kd.ctypes.data_as(f32p))
    np.savez_compressed(os.path.join(HERE, "kdtree_ref.npz"), points=P, box=box, queries=qi,
                        r2=np.float32(r2), vacc=vacc, found=np.array(found, np.int32),
                        found_off=np.array(found_off, np.int32), knn_q=qs, knn_idx=ki,
                        knn_dist=kd)


def oracle_tiny():
    from oracle import MODE_GRID, MODE_REF, MatchParam, Oracle
    from surface_match_gb300 import synth
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny()
    out = {"model_xyz": mc.xyz, "model_nrm": mc.normal, "scene_xyz": sc.cloud.xyz,
           "viewpoint": sc.viewpoint}
    for mode, tag in ((MODE_REF, "ref"), (MODE_GRID, "grid")):
        o = Oracle(mode=mode, threads=1)
        m = o.train(mc.xyz, mc.normal, 0.05)
        r = o.match(m, sc.cloud.xyz, None, sc.viewpoint, 0.05, 0.2, 0.2,
                    MatchParam(numMatches=8))
        digest = hashlib.sha256(m.refs.tobytes() + m.alphas.tobytes()).hexdigest()
        out.update({f"{tag}_model_keys": m.keys, f"{tag}_model_offsets": m.offsets,
                    f"{tag}_model_entries_sha256": np.array(digest),
                    f"{tag}_sampled": r.sampled, f"{tag}_keypoints": r.keypoints,
                    f"{tag}_kp_stats": r.kp_stats, f"{tag}_kp_cands": r.kp_cands,
                    f"{tag}_results": r.results})
    np.savez_compressed(os.path.join(HERE, "oracle_tiny.npz"), **out)


if __name__ == "__main__":
    murmur_kat()
    kdtree_ref()
    oracle_tiny()
    print("golden fixtures written to", HERE)
