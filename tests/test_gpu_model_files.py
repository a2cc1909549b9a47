"""Model files: the reference's byte layout (ppf.cpp:512-547, serialize.cpp:5-186) written
and read by the GPU library.

* save -> load round trip: identical tables and bit-identical matchScene results;
* a file written here from the oracle's model, following serialize.cpp field by field with
  the buckets in a shuffled order (the reference writes them in its hash map's iteration
  order), loads into the oracle's tables and matches like the same arrays uploaded;
* bad magic, truncation and inconsistent counts raise the reference's std::runtime_error
  (SM_ERR_RUNTIME) without touching the loaded model.
"""
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SD = 0.05
MAGIC = 0x7F27F
VERSION = 100


@pytest.fixture(scope="module")
def data():
    from surface_match_gb300 import synth
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny(seed=3)
    return mc, sc


def _match(det, sc):
    from surface_match_gb300 import MatchParam, PointCloud
    return det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), SD, 0.2, 0.2,
                          MatchParam(numMatches=8))


def _tables_equal(a, b):
    for k in ("sampled", "sampled_normal", "resampled", "resampled_normal", "box", "keys",
              "offsets", "refs"):
        np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg=k)
    np.testing.assert_array_equal(np.asarray(a["alphas"]).view(np.uint32),
                                  np.asarray(b["alphas"]).view(np.uint32))


def _write_reference_file(path, m, sd, rng):
    """serialize.cpp's layout: int magic, int version, float samplingDistanceRel, TrainParam
    (float, int, float, int, bool), two PointClouds (u32 n + n xyz, u32 n + n normals,
    box min/max, viewPoint), then the hash map: u32 buckets, each u32 key, u32 n + n refInd,
    u32 n + n alphaAngle - buckets in `rng`'s shuffled order."""
    b = bytearray()
    b += struct.pack("<iif", MAGIC, VERSION, sd)
    b += struct.pack("<fifi?", 0.04, 30, 0.01, 10, True)

    def cloud(p, n):
        out = struct.pack("<I", len(p)) + np.asarray(p, "<f4").tobytes()
        out += struct.pack("<I", len(n)) + np.asarray(n, "<f4").tobytes()
        out += np.asarray(m.box, "<f4").tobytes()
        out += struct.pack("<fff", np.nan, np.nan, np.nan)
        return out

    b += cloud(m.sampled, m.sampled_normal)
    b += cloud(m.resampled, m.resampled_normal)
    nk = len(m.keys)
    b += struct.pack("<I", nk)
    for k in rng.permutation(nk):
        o0, o1 = int(m.offsets[k]), int(m.offsets[k + 1])
        b += struct.pack("<II", int(m.keys[k]), o1 - o0)
        b += np.asarray(m.refs[o0:o1], "<u4").tobytes()
        b += struct.pack("<I", o1 - o0)
        b += np.asarray(m.alphas[o0:o1], "<f4").tobytes()
    with open(path, "wb") as f:
        f.write(bytes(b))
    return bytes(b)


def test_save_load_round_trip(data, tmp_path):
    from surface_match_gb300 import Detector, PointCloud
    mc, sc = data
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    p0, s0 = _match(det, sc)
    path = str(tmp_path / "gear.model")
    det.save(path)
    raw = open(path, "rb").read()
    assert struct.unpack("<ii", raw[:8]) == (MAGIC, VERSION)
    det2 = Detector()
    det2.load(path)
    _tables_equal(det.download(), det2.download())
    p1, s1 = _match(det2, sc)
    assert len(s0) > 0
    np.testing.assert_array_equal(s0, s1)
    np.testing.assert_array_equal(p0.view(np.uint32), p1.view(np.uint32))
    # a second save of the loaded model writes the same bytes
    det2.save(str(tmp_path / "again.model"))
    assert open(str(tmp_path / "again.model"), "rb").read() == raw


def test_reference_layout_file_loads_into_the_same_tables(data, tmp_path):
    from oracle import MODE_REF, Oracle
    from surface_match_gb300 import Detector, TrainParam
    mc, sc = data
    om = Oracle(mode=MODE_REF, threads=4).train(mc.xyz, mc.normal, SD)
    path = str(tmp_path / "ref.model")
    _write_reference_file(path, om, SD, np.random.default_rng(3))
    det = Detector()
    det.load(path)
    want = {"sampled": om.sampled, "sampled_normal": om.sampled_normal,
            "resampled": om.resampled, "resampled_normal": om.resampled_normal,
            "box": om.box[:6], "keys": om.keys, "offsets": om.offsets, "refs": om.refs,
            "alphas": om.alphas}
    _tables_equal(det.download(), want)
    up = Detector()
    up.upload(om.sampled, om.sampled_normal, om.resampled, om.resampled_normal, om.box, om.keys,
              om.offsets, om.refs, om.alphas, SD, TrainParam())
    a, sa = _match(det, sc)
    b, sb = _match(up, sc)
    np.testing.assert_array_equal(sa, sb)
    np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("damage", ["magic", "truncated_header", "truncated_table",
                                    "count_mismatch", "normals_mismatch"])
def test_corrupt_files_raise_runtime_error(data, tmp_path, damage):
    from oracle import MODE_REF, Oracle
    from surface_match_gb300 import Detector, PointCloud
    mc, sc = data
    om = Oracle(mode=MODE_REF, threads=4).train(mc.xyz, mc.normal, SD)
    raw = bytearray(_write_reference_file(str(tmp_path / "ok.model"), om, SD,
                                          np.random.default_rng(1)))
    if damage == "magic":
        raw[0:4] = struct.pack("<i", 0x1234)
    elif damage == "truncated_header":
        raw = raw[:30]
    elif damage == "truncated_table":
        raw = raw[:len(raw) - 7]
    elif damage == "count_mismatch":
        # the first bucket's alpha count one larger than its reference count
        head = 4 + 4 + 4 + 17
        ns = len(om.sampled)
        nr = len(om.resampled)
        cl1 = 4 + ns * 12 + 4 + ns * 12 + 24 + 12
        cl2 = 4 + nr * 12 + 4 + nr * 12 + 24 + 12
        at = head + cl1 + cl2 + 4  # first bucket
        n1 = struct.unpack("<I", raw[at + 4:at + 8])[0]
        pos = at + 8 + 4 * n1
        raw[pos:pos + 4] = struct.pack("<I", n1 + 1)
    elif damage == "normals_mismatch":
        ns = len(om.sampled)
        pos = 4 + 4 + 4 + 17 + 4 + ns * 12
        raw[pos:pos + 4] = struct.pack("<I", ns - 1)
    path = str(tmp_path / "bad.model")
    with open(path, "wb") as f:
        f.write(bytes(raw))
    det = Detector()
    det.trainModel(PointCloud(mc.xyz, mc.normal), SD)
    before = det.download()
    with pytest.raises(RuntimeError) as e:
        det.load(path)
    if damage == "magic":
        assert "unsupported file format:" in str(e.value)
    # the failed load left the trained model as it was
    _tables_equal(before, det.download())
    p, s = _match(det, sc)
    assert len(s) > 0
