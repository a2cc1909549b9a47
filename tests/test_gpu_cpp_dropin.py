"""The C++ drop-in run for real: a program written against include/ppf.h - the reference's
ppf::Detector API, used the way its example driver does (main.cpp:17-47: trainModel, save,
load, matchScene) - compiled with g++, linked against libsurface_match.so and run. Its poses
and scores must equal, bit for bit, the Python binding's on the same scene (both go through
the C ABI), in both search orders."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <cstdio>
#include <fstream>
#include <vector>
#include <ppf.h>

static std::vector<float> read_floats(const char *path) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    const std::streamsize n = f.tellg();
    std::vector<float> v(n / 4);
    f.seekg(0);
    f.read(reinterpret_cast<char *>(v.data()), n);
    return v;
}

static ppf::PointCloud cloud(const std::vector<float> &xyz, const std::vector<float> *nrm) {
    ppf::PointCloud pc;
    for (size_t i = 0; i + 2 < xyz.size(); i += 3) {
        pc.point.emplace_back(xyz[i], xyz[i + 1], xyz[i + 2]);
        if (nrm)
            pc.normal.emplace_back((*nrm)[i], (*nrm)[i + 1], (*nrm)[i + 2]);
    }
    return pc;
}

int main(int argc, char **argv) {
    // argv: model.xyz model.nrm scene.xyz vx vy vz order out.bin model.file
    const std::vector<float> mx = read_floats(argv[1]), mn = read_floats(argv[2]);
    const std::vector<float> sx = read_floats(argv[3]);
    const ppf::SearchOrder order = argv[7][0] == 'r' ? ppf::SearchOrder::Reference
                                                     : ppf::SearchOrder::Grid;
    ppf::PointCloud model = cloud(mx, &mn);
    ppf::PointCloud scene = cloud(sx, nullptr);
    scene.viewPoint = ppf::Vec3f((float)atof(argv[4]), (float)atof(argv[5]), (float)atof(argv[6]));
    try {
        ppf::Detector trained(order);
        trained.trainModel(model, 0.05f);
        trained.save(argv[9]);
        ppf::Detector detector(order);
        detector.load(argv[9]);
        std::vector<ppf::Mat4f> pose;
        std::vector<float>      score;
        ppf::MatchParam param;
        param.numMatches = 8;
        detector.matchScene(scene, pose, score, 0.05f, 0.2f, 0.2f, param);
        std::ofstream o(argv[8], std::ios::binary);
        const int n = (int)pose.size();
        o.write(reinterpret_cast<const char *>(&n), 4);
        for (int i = 0; i < n; i++) {
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++) {
                    const float v = pose[i](r, c);
                    o.write(reinterpret_cast<const char *>(&v), 4);
                }
            o.write(reinterpret_cast<const char *>(&score[i]), 4);
        }
        // the reference's exception types come through
        try {
            detector.matchScene(scene, pose, score, 1.5f, 0.2f, 0.2f, param);
            return 3;
        } catch (const std::range_error &) {
        }
    } catch (const std::exception &e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 2;
    }
    return 0;
}
"""


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("dropin")
    src = tmp / "app.cpp"
    src.write_text(PROGRAM)
    libdir = os.path.join(ROOT, "surface_match_gb300")
    exe = tmp / "app"
    subprocess.run(["g++", "-std=c++17", "-O1", "-DPPF_NO_EIGEN", "-I",
                    os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L", libdir,
                    "-lsurface_match", f"-Wl,-rpath,{libdir}"], check=True)
    return exe, tmp


@pytest.mark.parametrize("order", ["grid", "reference"])
def test_cpp_detector_matches_the_c_abi_path(program, order):
    from surface_match_gb300 import Detector, MatchParam, PointCloud, synth
    exe, tmp = program
    mc, _, _ = synth.gear_model(8000, seed=5)
    sc = synth.scene_tiny(seed=3)
    files = {"mx": tmp / "m.xyz", "mn": tmp / "m.nrm", "sx": tmp / "s.xyz"}
    np.ascontiguousarray(mc.xyz, np.float32).tofile(files["mx"])
    np.ascontiguousarray(mc.normal, np.float32).tofile(files["mn"])
    np.ascontiguousarray(sc.cloud.xyz, np.float32).tofile(files["sx"])
    out, mfile = tmp / f"out_{order}.bin", tmp / f"{order}.model"
    vp = [repr(float(v)) for v in sc.viewpoint]
    r = subprocess.run([str(exe), str(files["mx"]), str(files["mn"]), str(files["sx"]), *vp,
                        order, str(out), str(mfile)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, dtype=np.float32)
    n = int(raw[:1].view(np.int32)[0])
    rec = raw[1:].reshape(n, 17)
    det = Detector(search_order=order)
    det.trainModel(PointCloud(mc.xyz, mc.normal), 0.05)
    poses, scores = det.matchScene(PointCloud(sc.cloud.xyz, None, sc.viewpoint), 0.05, 0.2, 0.2,
                                   MatchParam(numMatches=8))
    assert n == len(scores) > 0
    np.testing.assert_array_equal(rec[:, 16], scores)
    np.testing.assert_array_equal(rec[:, :16].reshape(n, 4, 4).view(np.uint32),
                                  poses.astype(np.float32).view(np.uint32))
