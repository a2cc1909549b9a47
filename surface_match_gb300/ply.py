"""PLY point-cloud / mesh files (the reference's filePLY.h:6-9 readPLY / writePLY), the
Python counterpart of include/filePLY.h with the same rules: ASCII and binary files of either
byte order, any scalar type, list properties; the vertex element's x, y, z (and nx, ny, nz
when all three are present) and the face element's vertex_indices / vertex_index lists,
polygons with more than three corners cut into triangles by ear clipping (convex about
the polygon's normal, no other corner inside the triangle seen along z; filePLY.cpp:44-98).
Vertex data is read with numpy in one pass. read_ply raises ValueError where the reference
prints a message and returns false."""
from __future__ import annotations

import numpy as np

from .detector import PointCloud

_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "i2",
          "int16": "i2", "ushort": "u2", "uint16": "u2", "int": "i4", "int32": "i4",
          "uint": "u4", "uint32": "u4", "float": "f4", "float32": "f4", "double": "f8",
          "float64": "f8"}


def _header(f):
    if not f.readline().startswith(b"ply"):
        raise ValueError("Read PLY failed: unable to parse header.")
    fmt, elems = "ascii", []
    while True:
        line = f.readline()
        if not line:
            raise ValueError("Read PLY failed: unable to parse header.")
        w = line.decode("ascii", "replace").split()
        if not w:
            continue
        if w[0] == "format":
            fmt = w[1]
        elif w[0] == "element":
            elems.append((w[1], int(w[2]), []))
        elif w[0] == "property":
            if w[1] == "list":
                elems[-1][2].append((w[4], _TYPES[w[3]], _TYPES[w[2]]))
            else:
                elems[-1][2].append((w[2], _TYPES[w[1]], None))
        elif w[0] == "end_header":
            break
    if fmt not in ("ascii", "binary_little_endian", "binary_big_endian"):
        raise ValueError("Read PLY failed: unable to parse header.")
    return fmt, elems


def _inside_xy(a, b, c, x, y):
    inside = False
    for p, q in ((a, b), (b, c), (c, a)):
        if (p[1] <= y < q[1]) or (q[1] <= y < p[1]):
            cx = (q[0] - p[0]) * (y - p[1]) / (q[1] - p[1]) + p[0]
            if cx < x:
                inside = not inside
    return inside


def _triangulate(pts, idx, out):
    idx = list(idx)
    if any(i < 0 or i >= len(pts) for i in idx):
        return False
    n = len(idx)
    nrm = np.zeros(3, np.float32)
    if n > 3:
        for i in range(n):
            a, b, c = pts[idx[i]], pts[idx[(i + 1) % n]], pts[idx[(i + 2) % n]]
            nrm = nrm + np.cross(b - a, c - b)
        nrm = nrm / np.float32(np.sqrt(np.dot(nrm, nrm)))
    while n > 3:
        cut = False
        for i in range(1, n - 1):
            a, b, c = pts[idx[i - 1]], pts[idx[i]], pts[idx[i + 1]]
            if not float(np.dot(nrm, np.cross(b - a, c - b))) > 0.0:
                continue
            if any(_inside_xy(a, b, c, float(pts[idx[j]][0]), float(pts[idx[j]][1]))
                   for j in range(n) if not i - 1 <= j <= i + 1):
                continue
            out.append((idx[i - 1], idx[i], idx[i + 1]))
            del idx[i]
            n -= 1
            cut = True
            break
        if not cut:
            return False
    if n == 3:
        out.append(tuple(idx))
    return True


def read_ply(path, pinned: bool = False) -> PointCloud:
    """PointCloud with point (n, 3) float32, normal (n, 3) or None, face (m, 3) int32 or
    None. With `pinned`, point and normal sit in page-locked host memory (pinned_empty), so
    matchScene uploads them as an asynchronous DMA."""
    try:
        f = open(path, "rb")
    except OSError:
        raise ValueError(f"Read PLY failed: unable to open file: {path}") from None
    with f:
        fmt, elems = _header(f)
        body = f.read()
    nv = next((c for name, c, _ in elems if name == "vertex"), 0)
    if nv <= 0:
        raise ValueError("Read PLY failed: number of vertex <= 0.")
    order = {"binary_little_endian": "<", "binary_big_endian": ">"}.get(fmt)
    point, normal, faces = np.zeros((nv, 3), np.float32), None, []
    pos, tokens, tk = 0, (body.split() if order is None else None), 0
    for name, count, props in elems:
        scalars_only = all(p[2] is None for p in props)
        names = [p[0] for p in props]
        if scalars_only:
            if order is None:
                n = count * len(props)
                vals = np.array(tokens[tk:tk + n], dtype=np.float64).reshape(count, len(props))
                tk += n
                cols = {nm: vals[:, k] for k, nm in enumerate(names)}
            else:
                dt = np.dtype([(nm, order + t) for nm, t, _ in props])
                arr = np.frombuffer(body, dt, count, pos)
                pos += dt.itemsize * count
                cols = {nm: arr[nm] for nm in names}
            if name == "vertex":
                for a, nm in enumerate(("x", "y", "z")):
                    if nm in cols:
                        point[:, a] = cols[nm]
                if all(nm in cols for nm in ("nx", "ny", "nz")):
                    normal = np.stack([cols["nx"], cols["ny"], cols["nz"]], 1).astype(np.float32)
            continue
        face_k = next((k for k, p in enumerate(props)
                       if p[2] is not None and p[0] in ("vertex_indices", "vertex_index")), -1)
        has_n = name == "vertex" and all(nm in names for nm in ("nx", "ny", "nz"))
        if has_n:
            normal = np.zeros((nv, 3), np.float32)
        for r in range(count):
            poly, vals = None, {}
            for k, (nm, t, ct) in enumerate(props):
                if ct is None:
                    if order is None:
                        vals[nm] = float(tokens[tk])
                        tk += 1
                    else:
                        vals[nm] = float(np.frombuffer(body, order + t, 1, pos)[0])
                        pos += np.dtype(t).itemsize
                    continue
                if order is None:
                    cnt = int(float(tokens[tk]))
                    items = [int(float(x)) for x in tokens[tk + 1:tk + 1 + cnt]]
                    tk += 1 + cnt
                else:
                    cnt = int(np.frombuffer(body, order + ct, 1, pos)[0])
                    pos += np.dtype(ct).itemsize
                    items = np.frombuffer(body, order + t, cnt, pos).astype(np.int64).tolist()
                    pos += np.dtype(t).itemsize * cnt
                if k == face_k:
                    poly = items
            if name == "vertex":
                point[r] = [vals.get(a, 0.0) for a in ("x", "y", "z")]
                if has_n:
                    normal[r] = [vals[a] for a in ("nx", "ny", "nz")]
                continue
            if poly is not None and not _triangulate(point, poly, faces):
                raise ValueError("Read PLY failed: A polygon in the mesh could not be "
                                 "decomposed into triangles.")
    face = np.array(faces, np.int32).reshape(-1, 3) if faces else None
    if pinned:
        from .detector import pinned_empty
        p = pinned_empty(point.shape, np.float32)
        p[...] = point
        point = p
        if normal is not None:
            q = pinned_empty(normal.shape, np.float32)
            q[...] = normal
            normal = q
    return PointCloud(point, normal, None, face)


def write_ply(path, cloud: PointCloud, write_ascii: bool = False) -> bool:
    """float x, y, z (+ nx, ny, nz) and uchar/uint triangle lists; binary little-endian
    unless write_ascii (the reference's writePLY layout)."""
    pts = np.asarray(cloud.point, np.float32).reshape(-1, 3)
    if len(pts) == 0:
        print("Write PLY failed: mesh has 0 vertices.")
        return False
    nrm = None if cloud.normal is None else np.asarray(cloud.normal, np.float32).reshape(-1, 3)
    if nrm is not None and len(nrm) != len(pts):
        nrm = None
    faces = np.zeros((0, 3), np.uint32) if cloud.face is None else \
        np.asarray(cloud.face, np.int64).reshape(-1, 3).astype(np.uint32)
    head = ["ply", f"format {'ascii' if write_ascii else 'binary_little_endian'} 1.0",
            f"element vertex {len(pts)}", "property float x", "property float y",
            "property float z"]
    if nrm is not None:
        head += ["property float nx", "property float ny", "property float nz"]
    head += [f"element face {len(faces)}", "property list uchar uint vertex_indices",
             "end_header"]
    data = pts if nrm is None else np.concatenate([pts, nrm], 1)
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n").encode())
        if write_ascii:
            for row in data:
                f.write((" ".join("%.9g" % v for v in row) + "\n").encode())
            for tri in faces:
                f.write(f"3 {tri[0]} {tri[1]} {tri[2]}\n".encode())
        else:
            f.write(np.ascontiguousarray(data, "<f4").tobytes())
            if len(faces):
                rec = np.zeros(len(faces), np.dtype([("n", "u1"), ("i", "<u4", 3)]))
                rec["n"] = 3
                rec["i"] = faces
                f.write(rec.tobytes())
    return True
