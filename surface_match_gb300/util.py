"""The reference's public point-cloud helpers (util.h:8-21) for Python, as in
include/util.h: sampleMesh (util.cpp:20-84), removeNan (util.cpp:86-105), extraIndices
(util.cpp:141-161), normalizeNormal (util.cpp:163-176), computeBoundingBox
(util.cpp:178-207) and transformPointCloud (util.cpp:209-232), on numpy arrays.
computeBoundingBox returns (min, max)."""
from __future__ import annotations

import numpy as np

from .detector import PointCloud


def _unit(v):
    n = np.sqrt((v.astype(np.float32) ** 2).sum(1, keepdims=True))
    return np.where(n > 0, v / np.where(n > 0, n, 1), v).astype(np.float32)


def sampleMesh(pc: PointCloud, radius: float, seed: int | None = None) -> PointCloud:
    """About one point per radius^2 of surface, spread over the triangles in proportion to
    their areas (triangle i fills up to round(cumulative share x count)), at uniform
    barycentric coordinates, with the triangles' unit normals; no triangles, no points."""
    if pc.face is None or len(pc.face) == 0:
        return PointCloud(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.float32))
    P = np.asarray(pc.point, np.float32)
    F = np.asarray(pc.face, np.int64).reshape(-1, 3)
    p0, p1, p2 = P[F[:, 0]], P[F[:, 1]], P[F[:, 2]]
    k = np.cross(p1 - p0, p2 - p0)
    area = np.sqrt((k ** 2).sum(1)) / 2
    nrm = _unit(k)
    total = float(area.sum())
    cdf = np.cumsum(area / total)
    cdf[-1] = 1.0
    n = int(total / (radius * radius))
    ends = np.minimum(np.round(cdf * n).astype(np.int64), n)
    counts = np.diff(np.concatenate([[0], np.maximum.accumulate(ends)]))
    tri = np.repeat(np.arange(len(F)), counts)
    rng = np.random.default_rng(seed)
    r1, r2 = rng.random(n), rng.random(n)
    s = np.sqrt(r1)
    a, b, c = (1 - s)[:, None], (s * (1 - r2))[:, None], (s * r2)[:, None]
    pts = (a * p0[tri] + b * p1[tri] + c * p2[tri]).astype(np.float32)
    return PointCloud(pts, nrm[tri])


def removeNan(pc: PointCloud, checkNormal: bool = False) -> np.ndarray:
    """Ascending indices of the points with finite coordinates (and finite normals)."""
    ok = np.isfinite(np.asarray(pc.point, np.float32)).all(1)
    if checkNormal and pc.normal is not None and len(pc.normal) == len(pc.point):
        ok &= np.isfinite(np.asarray(pc.normal, np.float32)).all(1)
    return np.nonzero(ok)[0]


def computeBoundingBox(pc: PointCloud, validIndices=None):
    P = np.asarray(pc.point, np.float32)
    if validIndices is not None and len(validIndices):
        P = P[np.asarray(validIndices)]
    return P.min(0), P.max(0)


def extraIndices(pc: PointCloud, indices) -> PointCloud:
    """The named points; unit normals when the cloud has normals."""
    idx = np.asarray(indices, np.int64)
    pts = np.asarray(pc.point, np.float32)[idx]
    nrm = None
    if pc.normal is not None and len(pc.normal) == len(pc.point):
        nrm = _unit(np.asarray(pc.normal, np.float32)[idx])
    return PointCloud(pts, nrm, pc.viewPoint)


def normalizeNormal(pc: PointCloud, invert: bool = False) -> PointCloud:
    """Unit normals (reversed when invert); returns the cloud, whose normals are replaced."""
    n = _unit(np.asarray(pc.normal, np.float32))
    pc.normal = -n if invert else n
    return pc


def transformPointCloud(pc: PointCloud, pose, useNormal: bool = True) -> PointCloud:
    """R p + t for the points, R n for the normals, triangles kept."""
    T = np.asarray(pose, np.float32).reshape(4, 4)
    R, t = T[:3, :3], T[:3, 3]
    pts = (np.asarray(pc.point, np.float32) @ R.T + t).astype(np.float32)
    nrm = None
    if useNormal and pc.normal is not None and len(pc.normal) == len(pc.point):
        nrm = (np.asarray(pc.normal, np.float32) @ R.T).astype(np.float32)
    return PointCloud(pts, nrm, pc.viewPoint, pc.face)
