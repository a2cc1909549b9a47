"""The reference's public helpers (util.h, helper.h, filePLY.h) as header-only C++ beside
ppf.h: a program shaped like the reference's example driver (main.cpp) compiles against
them, and the helpers give the reference's results on a cube mesh - mesh sampling (count,
points on the faces, face normals), transforms, boxes, NaN removal, extraction and normal
normalisation - checked against numpy. CPU only."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MAIN = r'''
#include <filePLY.h>
#include <helper.h>
#include <ppf.h>
#include <util.h>
int main(int argc, char *argv[]) {
    ppf::PointCloud model;
    ppf::readPLY(argv[1], model);
    ppf::PointCloud scene;
    ppf::readPLY(argv[2], scene);
    scene.viewPoint = {-200, -50, -500};
    auto tmp = model;
    {
        ppf::Timer    t("train model");
        ppf::Detector detector;
        detector.trainModel(model, 0.025f);
        detector.save("1.model");
    }
    std::vector<ppf::Mat4f> pose;
    std::vector<float>      score;
    ppf::MatchResult        result;
    ppf::Detector           detector;
    detector.load("1.model");
    {
        ppf::Timer t("match scene");
        detector.matchScene(scene, pose, score, 0.025f, 0.1f, 0.1f,
                            ppf::MatchParam{55, 10, true, false, 0.5, 0, true, true, 15, 0.3},
                            &result);
    }
    for (size_t i = 0; i < pose.size(); i++) {
        auto pc = ppf::transformPointCloud(tmp, pose[i]);
        ppf::writePLY(std::string("out") + std::to_string(i) + ".ply", pc);
    }
    ppf::writePLY("sampledScene.ply", result.sampledScene);
    ppf::writePLY("sampledKeypoint.ply", result.keyPoint);
    return 0;
}
'''

RUN = r'''
#include <util.h>
#include <cstdio>
int main() {
    // unit cube of side 2 centred at the origin: 8 corners, 12 outward triangles
    ppf::PointCloud cube;
    for (int i = 0; i < 8; i++)
        cube.point.emplace_back((i & 1) ? 1.f : -1.f, (i & 2) ? 1.f : -1.f, (i & 4) ? 1.f : -1.f);
    const int q[6][4] = {{0, 2, 3, 1}, {4, 5, 7, 6}, {0, 1, 5, 4}, {2, 6, 7, 3}, {0, 4, 6, 2}, {1, 3, 7, 5}};
    for (auto &f : q) {
        cube.face.emplace_back(f[0], f[1], f[2]);
        cube.face.emplace_back(f[0], f[2], f[3]);
    }
    auto s1 = ppf::sampleMesh(cube, 0.05f, 7u), s2 = ppf::sampleMesh(cube, 0.05f, 7u);
    std::printf("S %zu %zu %d\n", s1.point.size(), s1.normal.size(), s1.point.size() == s2.point.size() &&
                std::equal(s1.point.begin(), s1.point.end(), s2.point.begin(), [](const ppf::Vec3f &a, const ppf::Vec3f &b) {
                    return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }) ? 1 : 0);
    for (size_t i = 0; i < s1.point.size(); i++)
        std::printf("P %.9g %.9g %.9g %.9g %.9g %.9g\n", s1.point[i][0], s1.point[i][1], s1.point[i][2],
                    s1.normal[i][0], s1.normal[i][1], s1.normal[i][2]);
    ppf::Mat4f T;  // rotation by 90 degrees about z, then translation (1, 2, 3)
    T(0, 0) = 0; T(0, 1) = -1; T(1, 0) = 1; T(1, 1) = 0; T(0, 3) = 1; T(1, 3) = 2; T(2, 3) = 3;
    ppf::PointCloud pc;
    pc.point = {ppf::Vec3f(1, 0, 0), ppf::Vec3f(0, 2, 0), ppf::Vec3f(NAN, 0, 0), ppf::Vec3f(0, 0, 5)};
    pc.normal = {ppf::Vec3f(2, 0, 0), ppf::Vec3f(0, 0, 3), ppf::Vec3f(0, 1, 0), ppf::Vec3f(0, 0, 0)};
    auto t = ppf::transformPointCloud(pc, T);
    for (size_t i = 0; i < t.point.size(); i++)
        std::printf("T %.9g %.9g %.9g %.9g %.9g %.9g\n", t.point[i][0], t.point[i][1], t.point[i][2],
                    t.normal[i][0], t.normal[i][1], t.normal[i][2]);
    auto keep = ppf::removeNan(pc);
    std::printf("K");
    for (int k : keep) std::printf(" %d", k);
    std::printf("\n");
    auto b = ppf::computeBoundingBox(pc, keep);
    std::printf("B %g %g %g %g %g %g\n", b.min[0], b.min[1], b.min[2], b.max[0], b.max[1], b.max[2]);
    auto e = ppf::extraIndices(pc, {3, 1});
    std::printf("E %g %g %g %g %g %g %g\n", e.point[1][1], e.normal[0][2], e.normal[1][2],
                e.box.min[1], e.box.max[1], e.box.min[2], e.box.max[2]);
    ppf::normalizeNormal(pc, true);
    std::printf("N %g %g %g\n", pc.normal[0][0], pc.normal[1][2], pc.normal[3][2]);
    return 0;
}
'''


def compile_(src, out, tmp, syntax_only=False):
    p = tmp / (out + ".cpp")
    p.write_text(src)
    cmd = ["g++", "-std=c++17", "-DPPF_NO_EIGEN", "-I", os.path.join(ROOT, "include"), str(p)]
    cmd += ["-fsyntax-only"] if syntax_only else ["-O1", "-o", str(tmp / out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(tmp / out)


def test_reference_example_driver_compiles(tmp_path):
    compile_(MAIN, "main", tmp_path, syntax_only=True)


def test_helpers_on_a_cube(tmp_path):
    exe = compile_(RUN, "run", tmp_path)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    rows = {}
    for line in out:
        rows.setdefault(line.split()[0], []).append(line.split()[1:])
    n, nn, same = map(int, rows["S"][0])
    assert n == int(24.0 / 0.05 ** 2) == nn and same == 1  # area / radius^2; repeatable
    P = np.array(rows["P"], np.float64)
    pts, nrm = P[:, :3], P[:, 3:]
    # every point on the cube's surface, on the face its normal names
    assert np.all(np.abs(pts) <= 1 + 1e-6)
    axis = np.argmax(np.abs(nrm), 1)
    np.testing.assert_allclose(np.abs(nrm).max(1), 1.0, atol=1e-7)
    np.testing.assert_allclose(pts[np.arange(len(pts)), axis], np.sign(nrm[np.arange(len(pts)), axis]),
                               atol=1e-6)
    # area-proportional: each face holds about a sixth
    counts = np.bincount(axis * 2 + (nrm[np.arange(len(pts)), axis] > 0), minlength=6)
    assert np.all(np.abs(counts - n / 6) < 0.02 * n)
    T = np.array(rows["T"], np.float64)
    R = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float64)
    src = np.array([[1, 0, 0], [0, 2, 0], [np.nan, 0, 0], [0, 0, 5]])
    srcn = np.array([[2, 0, 0], [0, 0, 3], [0, 1, 0], [0, 0, 0]])
    np.testing.assert_allclose(T[:, :3], src @ R.T + [1, 2, 3])
    np.testing.assert_allclose(T[:, 3:], srcn @ R.T)
    assert rows["K"][0] == ["0", "1", "3"]
    assert list(map(float, rows["B"][0])) == [0, 0, 0, 1, 2, 5]
    # extraction keeps an empty box's recomputation and normalises normals
    assert list(map(float, rows["E"][0])) == [2, 0, 1, 0, 2, 0, 5]
    assert list(map(float, rows["N"][0])) == [-1, -1, 0]


def test_python_helpers_match_the_headers():
    """The Python mirror of the same helpers on the same cloud."""
    from surface_match_gb300 import PointCloud, util
    pc = PointCloud(np.array([[1, 0, 0], [0, 2, 0], [np.nan, 0, 0], [0, 0, 5]], np.float32),
                    np.array([[2, 0, 0], [0, 0, 3], [0, 1, 0], [0, 0, 0]], np.float32))
    T = np.eye(4, dtype=np.float32)
    T[:3, :3] = [[0, -1, 0], [1, 0, 0], [0, 0, 1]]
    T[:3, 3] = [1, 2, 3]
    t = util.transformPointCloud(pc, T)
    np.testing.assert_allclose(t.point, pc.point @ T[:3, :3].T + T[:3, 3])
    np.testing.assert_allclose(t.normal, pc.normal @ T[:3, :3].T)
    keep = util.removeNan(pc)
    assert keep.tolist() == [0, 1, 3]
    mn, mx = util.computeBoundingBox(pc, keep)
    assert mn.tolist() == [0, 0, 0] and mx.tolist() == [1, 2, 5]
    e = util.extraIndices(pc, [3, 1])
    assert e.normal[1].tolist() == [0, 0, 1] and e.normal[0].tolist() == [0, 0, 0]
    n = util.normalizeNormal(pc, invert=True)
    assert n.normal[0].tolist() == [-1, 0, 0] and n.normal[1].tolist() == [0, 0, -1]
    cube = PointCloud(np.array([[(i & 1) * 2 - 1, (i >> 1 & 1) * 2 - 1, (i >> 2 & 1) * 2 - 1]
                                for i in range(8)], np.float32), None, None,
                      np.array([[0, 2, 3], [0, 3, 1], [4, 5, 7], [4, 7, 6], [0, 1, 5], [0, 5, 4],
                                [2, 6, 7], [2, 7, 3], [0, 4, 6], [0, 6, 2], [1, 3, 7], [1, 7, 5]]))
    s = util.sampleMesh(cube, 0.05, seed=7)
    assert len(s.point) == int(24.0 / 0.05 ** 2)
    assert np.all(np.abs(s.point) <= 1 + 1e-6)
    assert len(util.sampleMesh(PointCloud(cube.point), 0.05).point) == 0  # no triangles
