"""PLY files (the reference's filePLY.h readPLY / writePLY): the C++ header include/filePLY.h and
the Python module read the same files to the same clouds - ASCII and binary of both byte
orders, foreign properties and elements skipped, polygons cut into triangles - and each
writer's files read back unchanged. CPU only."""
import os
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CPP = r'''
#include <ppf.h>
#include <filePLY.h>
#include <cstdio>
// usage: t read <in.ply> <out.txt> | t write <in.txt> <out.ply> <ascii 0/1>
int main(int argc, char **argv) {
    std::string mode = argv[1];
    if (mode == "read") {
        ppf::PointCloud pc;
        if (!ppf::readPLY(argv[2], pc)) return 2;
        FILE *f = std::fopen(argv[3], "w");
        std::fprintf(f, "%zu %zu %zu\n", pc.point.size(), pc.normal.size(), pc.face.size());
        for (auto &p : pc.point) std::fprintf(f, "%.9g %.9g %.9g\n", p[0], p[1], p[2]);
        for (auto &n : pc.normal) std::fprintf(f, "%.9g %.9g %.9g\n", n[0], n[1], n[2]);
        for (auto &t : pc.face) std::fprintf(f, "%d %d %d\n", t[0], t[1], t[2]);
        std::fclose(f);
        return 0;
    }
    FILE *f = std::fopen(argv[2], "r");
    size_t np, nn, nf;
    if (std::fscanf(f, "%zu %zu %zu", &np, &nn, &nf) != 3) return 3;
    ppf::PointCloud pc;
    for (size_t i = 0; i < np; i++) { float x, y, z; std::fscanf(f, "%f %f %f", &x, &y, &z); pc.point.emplace_back(x, y, z); }
    for (size_t i = 0; i < nn; i++) { float x, y, z; std::fscanf(f, "%f %f %f", &x, &y, &z); pc.normal.emplace_back(x, y, z); }
    for (size_t i = 0; i < nf; i++) { int a, b, c; std::fscanf(f, "%d %d %d", &a, &b, &c); pc.face.emplace_back(a, b, c); }
    std::fclose(f);
    return ppf::writePLY(argv[3], pc, argv[4][0] == '1') ? 0 : 4;
}
'''


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    d = tmp_path_factory.mktemp("ply")
    src, exe = d / "t.cpp", d / "t"
    src.write_text(CPP)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-DPPF_NO_EIGEN", "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def cpp_read(tool, path, tmp):
    out = str(tmp / "read.txt")
    r = subprocess.run([tool, "read", str(path), out], capture_output=True, text=True)
    if r.returncode:
        return None, r.stdout
    v = open(out).read().split()
    npt, nn, nf = int(v[0]), int(v[1]), int(v[2])
    x = np.array(v[3:], np.float64)
    P = x[:3 * npt].reshape(-1, 3).astype(np.float32)
    N = x[3 * npt:3 * (npt + nn)].reshape(-1, 3).astype(np.float32)
    F = x[3 * (npt + nn):].reshape(-1, 3).astype(np.int32)
    return (P, N if nn else None, F if nf else None), r.stdout


def cpp_write(tool, tmp, P, N, F, ascii_):
    txt = tmp / "in.txt"
    with open(txt, "w") as f:
        f.write(f"{len(P)} {0 if N is None else len(N)} {0 if F is None else len(F)}\n")
        for arr, fmt in ((P, "%.9g"), (N, "%.9g"), (F, "%d")):
            if arr is not None:
                for row in arr:
                    f.write(" ".join(fmt % v for v in row) + "\n")
    out = tmp / ("w_a.ply" if ascii_ else "w_b.ply")
    r = subprocess.run([tool, "write", str(txt), str(out), "1" if ascii_ else "0"])
    assert r.returncode == 0
    return out


def same(a, b):
    if a is None or b is None:
        assert a is None and b is None
    else:
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def cloud():
    rng = np.random.default_rng(3)
    P = rng.normal(size=(50, 3)).astype(np.float32) * 40
    N = rng.normal(size=(50, 3)).astype(np.float32)
    F = rng.integers(0, 50, (20, 3)).astype(np.int32)
    return P, N, F


@pytest.mark.parametrize("ascii_", [False, True])
@pytest.mark.parametrize("normals", [False, True])
def test_round_trips_between_the_writers_and_readers(tool, tmp_path, ascii_, normals):
    from surface_match_gb300 import PointCloud
    from surface_match_gb300.ply import read_ply, write_ply
    P, N, F = cloud()
    N = N if normals else None
    p_py = tmp_path / "py.ply"
    assert write_ply(p_py, PointCloud(P, N, None, F), write_ascii=ascii_)
    p_cpp = cpp_write(tool, tmp_path, P, N, F, ascii_)
    assert open(p_py, "rb").read() == open(p_cpp, "rb").read()  # the same bytes
    for path in (p_py, p_cpp):
        r = read_ply(path)
        same(r.point, P), same(r.normal, N), same(r.face, F)
        (Pc, Nc, Fc), _ = cpp_read(tool, path, tmp_path)
        same(Pc, P), same(Nc, N), same(Fc, F)


FOREIGN_P = np.array([[0, 0, 0], [2, 0, 0], [2, 2, 0], [0, 2, 0], [1, 1, 0],
                      [3, 0, 1], [5, 0, 1], [5, 3, 1], [4, 1, 1], [3, 3, 1]], np.float32)
FOREIGN_POLYS = [[0, 1, 2, 3], [1, 2, 4], [5, 6, 7, 8, 9]]


def write_foreign(tmp_path, fmt):
    """A hand-made file: extra vertex properties (colours, a double intensity, a list), an
    extra element before the vertices, quads and a concave pentagon."""
    P, polys = FOREIGN_P, FOREIGN_POLYS
    h = ["ply", f"format {fmt} 1.0", "comment made by hand", "element camera 1",
         "property float fx", "element vertex 10", "property uchar red", "property float x",
         "property float y", "property double intensity", "property float z",
         "property list uchar int tags", "property uchar green", "element face 3",
         "property list uchar uint vertex_indices", "end_header"]
    path = tmp_path / f"{fmt}.ply"
    with open(path, "wb") as f:
        f.write(("\n".join(h) + "\n").encode())
        if fmt == "ascii":
            f.write(b"500.5\n")
            for i, p in enumerate(P):
                f.write(f"7 {p[0]} {p[1]} 0.25 {p[2]} 2 {i} {i + 1} 9\n".encode())
            for poly in polys:
                f.write((f"{len(poly)} " + " ".join(map(str, poly)) + "\n").encode())
        else:
            e = "<" if fmt == "binary_little_endian" else ">"
            f.write(struct.pack(e + "f", 500.5))
            for i, p in enumerate(P):
                f.write(struct.pack(e + "Bffdf", 7, p[0], p[1], 0.25, p[2]))
                f.write(struct.pack(e + "Bii", 2, i, i + 1) + struct.pack(e + "B", 9))
            for poly in polys:
                f.write(struct.pack(e + "B" + "I" * len(poly), len(poly), *poly))
    return path


def test_foreign_layouts_polygons_and_byte_orders(tool, tmp_path):
    """Extra vertex properties (colours, a double intensity, a list), an extra element,
    quads and a concave pentagon cut into triangles; big-endian binary reads like ASCII."""
    from surface_match_gb300.ply import read_ply
    P = FOREIGN_P
    ref = None
    for fmt in ("ascii", "binary_little_endian", "binary_big_endian"):
        path = write_foreign(tmp_path, fmt)
        r = read_ply(path)
        same(r.point, P)
        assert r.normal is None
        (Pc, Nc, Fc), _ = cpp_read(tool, path, tmp_path)
        same(Pc, P), same(Nc, None), same(Fc, r.face)
        ref = r.face if ref is None else ref
        same(r.face, ref)
    tris = {tuple(t) for t in ref.tolist()}
    assert len(ref) == 2 + 1 + 3  # a quad, a triangle, a pentagon
    assert {(0, 1, 2), (0, 2, 3), (1, 2, 4)} <= tris
    # the pentagon is concave at corner 8: no triangle may cut across the notch
    assert (7, 8, 9) in tris or (6, 7, 8) in tris


def test_failures_like_the_reference(tool, tmp_path):
    from surface_match_gb300.ply import read_ply
    with pytest.raises(ValueError, match="unable to open file"):
        read_ply(tmp_path / "missing.ply")
    r, out = cpp_read(tool, tmp_path / "missing.ply", tmp_path)
    assert r is None and "unable to open file" in out
    bad = tmp_path / "empty.ply"
    bad.write_bytes(b"ply\nformat ascii 1.0\nelement vertex 0\nproperty float x\nend_header\n")
    with pytest.raises(ValueError, match="number of vertex <= 0"):
        read_ply(bad)
    r, out = cpp_read(tool, bad, tmp_path)
    assert r is None and "number of vertex <= 0" in out


def _ref_ply():
    """The reference's own PLY reader (its vendored rply, compiled in place by the oracle's
    recipe) or None where its source is absent."""
    import ctypes as C
    import sys
    from conftest import reference_dir
    if reference_dir() is None:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_probe"))
    try:
        import build_ref
        L = C.CDLL(build_ref.build_ply())
    finally:
        sys.path.pop(0)
    L.ref_ply_counts.argtypes = [C.c_char_p, C.POINTER(C.c_long)]
    L.ref_ply_read.argtypes = [C.c_char_p] + [C.c_void_p] * 4
    return L


def ref_read(L, path):
    import ctypes as C
    cnt = (C.c_long * 4)()
    assert L.ref_ply_counts(str(path).encode(), cnt) == 0
    nv, nn, nf, ni = (int(v) for v in cnt)
    P = np.zeros((nv, 3), np.float32)
    N = np.zeros((nn, 3), np.float32)
    ln = np.zeros(max(nf, 1), np.int32)
    ix = np.zeros(max(ni, 1), np.int32)
    assert L.ref_ply_read(str(path).encode(), P.ctypes.data, N.ctypes.data, ln.ctypes.data,
                          ix.ctypes.data) == 0
    polys, o = [], 0
    for k in ln[:nf]:
        polys.append(ix[o:o + k].tolist())
        o += k
    return P, (N if nn else None), polys


def test_readers_match_the_reference_rply(tool, tmp_path):
    """Both readers against the reference's own rply, read the way its readPLY reads
    (filePLY.cpp:199-257): identical vertices and normals (doubles stored to floats),
    triangles as written, and polygons cut into n - 2 triangles of their own corners."""
    L = _ref_ply()
    if L is None:
        pytest.skip("the reference's source tree is not present")
    from surface_match_gb300 import PointCloud
    from surface_match_gb300.ply import read_ply, write_ply
    P, N, F = cloud()
    files = []
    for ascii_ in (True, False):
        for normals in (True, False):
            path = tmp_path / f"w_{int(ascii_)}_{int(normals)}.ply"
            write_ply(path, PointCloud(P, N if normals else None, None, F), write_ascii=ascii_)
            files.append((path, None))
    for fmt in ("ascii", "binary_little_endian", "binary_big_endian"):
        files.append((write_foreign(tmp_path, fmt), FOREIGN_POLYS))
    for path, polys in files:
        rP, rN, rpolys = ref_read(L, path)
        r = read_ply(path)
        (Pc, Nc, Fc), _ = cpp_read(tool, path, tmp_path)
        for got_P, got_N, got_F in ((r.point, r.normal, r.face), (Pc, Nc, Fc)):
            same(got_P, rP), same(got_N, rN)
            if polys is None:
                same(got_F, np.array(rpolys, np.int32))
            else:
                assert rpolys == polys
                assert len(got_F) == sum(len(q) - 2 for q in rpolys)
                for t in got_F.tolist():
                    assert any(set(t) <= set(q) for q in rpolys), t
