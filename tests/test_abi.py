"""The C ABI library builds, loads without a GPU, exports every entry point declared in
include/surface_match.h, and validates parameters like the reference's constructors."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "surface_match.h")).read()
    return sorted(set(re.findall(r"SM_API\s+[\w\s\*]+?\b(sm_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from surface_match_gb300 import _lib
    L = _lib.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(_lib.exported_names())
    assert b"sm_103a" in L.sm_version()


def test_param_defaults_and_validation_mirror_reference():
    from surface_match_gb300 import MatchParam, RangeError, TrainParam
    tp = TrainParam()
    assert (tp.featDistanceStepRel, tp.featAngleResolution, tp.poseRefRelSamplingDistance,
            tp.knnNormal, tp.smoothNormal) == (0.04, 30, 0.01, 10, True)
    mp = MatchParam()
    assert mp.numMatches == 1 and mp.poseRefNumSteps == 5 and mp.maxOverlapDistRel == 0.5
    with pytest.raises(RangeError, match="featDistanceStepRel"):
        TrainParam(featDistanceStepRel=0)
    with pytest.raises(RangeError, match="featAngleResolution"):
        TrainParam(featAngleResolution=0)
    with pytest.raises(RangeError, match="poseRefRelSamplingDistance"):
        TrainParam(poseRefRelSamplingDistance=1.5)
    with pytest.raises(RangeError, match="numMatches"):
        MatchParam(numMatches=0)
    with pytest.raises(RangeError, match="maxOverlapDist"):
        MatchParam(maxOverlapDistRel=-1, maxOverlapDistAbs=-1)
    with pytest.raises(RangeError, match="poseRefNumSteps"):
        MatchParam(densePoseRefinement=False, poseRefNumSteps=0)
    MatchParam(densePoseRefinement=True, poseRefNumSteps=0)  # only checked without dense


def test_context_without_gpu_reports_error():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from surface_match_gb300 import _lib
    L = _lib.load()
    h = C.c_void_p()
    rc = L.sm_context_create(0, None, C.byref(h))
    assert rc in (_lib.SM_ERR_CUDA, _lib.SM_ERR_ARG)
    assert L.sm_last_error()


def test_cpp_detector_header_compiles():
    """include/ppf.h (the C++ drop-in Detector) compiles against the C ABI."""
    import subprocess
    import tempfile
    src = r'''
#include <ppf.h>
int main() {
    ppf::PointCloud model;
    model.point.push_back(ppf::Vec3f(0, 0, 0));
    ppf::Detector d;
    std::vector<ppf::Mat4f> pose; std::vector<float> score;
    try { d.matchScene(model, pose, score, 0.04f, 0.2f, 0.2f, ppf::MatchParam(16)); }
    catch (const std::runtime_error &) { return 0; }
    return 1;
}
'''
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.cpp")
        open(p, "w").write(src)
        r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I",
                            os.path.join(ROOT, "include"), p], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
