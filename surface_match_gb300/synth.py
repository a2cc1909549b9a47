"""Seeded procedural models and scenes for the matching workloads.

The reference ships no data (its README links an external Ensenso gear scan), so every
workload is generated here from a seed:

* ``gear``    - spur gear with trapezoidal teeth, a central bore and flat faces;
* ``bracket`` - L-bracket of two rectangular plates at 90 degrees with four round holes;
* ``torus``   - torus of major radius R and minor radius r.

Models are area-weighted surface samples with exact outward normals. Scenes place model
instances at uniform SO(3) rotations (normalised Gaussian quaternions) and uniform
translations without bounding-sphere overlap, add a ground plane and/or clutter (uniform
points, or surfaces of random boxes and spheres), isotropic Gaussian noise, and keep only
points whose true normal faces the viewpoint. Scenes are returned without normals, as a
range sensor delivers them. All randomness comes from one ``numpy.random.Generator``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class Cloud:
    xyz: np.ndarray  # (n, 3) float32
    normal: np.ndarray | None = None  # (n, 3) float32


@dataclass
class Instance:
    model: str
    R: np.ndarray  # (3, 3) float64
    t: np.ndarray  # (3,) float64


@dataclass
class Scene:
    cloud: Cloud
    instances: list
    viewpoint: np.ndarray


# --------------------------------------------------------------------------------------
# surface primitives: each returns (area, sampler(rng, m) -> (points, normals))
# --------------------------------------------------------------------------------------

def _polygon_area(poly):
    x, y = poly[:, 0], poly[:, 1]
    return 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))


def _point_in_polygon(px, py, poly):
    inside = np.zeros(px.shape, dtype=bool)
    n = len(poly)
    for i in range(n):
        x1, y1 = poly[i]
        x2, y2 = poly[(i + 1) % n]
        cond = (y1 > py) != (y2 > py)
        with np.errstate(divide="ignore", invalid="ignore"):
            xint = (x2 - x1) * (py - y1) / (y2 - y1) + x1
        inside ^= cond & (px < xint)
    return inside


def gear_profile(teeth=24, r_out=50.0, r_root=42.0):
    """CCW outline of a spur gear with trapezoidal teeth (4 vertices per tooth)."""
    pitch = 2 * math.pi / teeth
    pts = []
    for k in range(teeth):
        a0 = k * pitch
        pts.append((r_root * math.cos(a0), r_root * math.sin(a0)))
        a1 = a0 + 0.12 * pitch
        pts.append((r_out * math.cos(a1), r_out * math.sin(a1)))
        a2 = a0 + 0.38 * pitch
        pts.append((r_out * math.cos(a2), r_out * math.sin(a2)))
        a3 = a0 + 0.5 * pitch
        pts.append((r_root * math.cos(a3), r_root * math.sin(a3)))
    return np.array(pts, dtype=np.float64)


class _Surface:
    def __init__(self):
        self.parts = []  # (area, fn(rng, m) -> (p, n))

    def add(self, area, fn):
        if area > 0:
            self.parts.append((float(area), fn))

    def area(self):
        return sum(a for a, _ in self.parts)

    def sample(self, rng, m):
        areas = np.array([a for a, _ in self.parts])
        counts = rng.multinomial(m, areas / areas.sum())
        ps, ns = [], []
        for (a, fn), c in zip(self.parts, counts):
            if c:
                p, n = fn(rng, int(c))
                ps.append(p)
                ns.append(n)
        p = np.concatenate(ps)
        n = np.concatenate(ns)
        n = n / np.linalg.norm(n, axis=1, keepdims=True)
        return p, n


def _prism_with_holes(surface, poly, holes, z0, z1, frame=None):
    """Extrude a CCW polygon (with circular holes (cx, cy, r)) between z0 and z1.

    `frame` maps local (x, y, z) to world: a (3, 3) rotation and (3,) offset.
    """
    R = np.eye(3) if frame is None else frame[0]
    o = np.zeros(3) if frame is None else frame[1]
    area2d = _polygon_area(poly) - sum(math.pi * r * r for _, _, r in holes)
    lo, hi = poly.min(axis=0), poly.max(axis=0)

    def face(z, nz):
        def fn(rng, m):
            out = []
            while sum(len(a) for a in out) < m:
                k = max(64, 2 * m)
                x = rng.uniform(lo[0], hi[0], k)
                y = rng.uniform(lo[1], hi[1], k)
                ok = _point_in_polygon(x, y, poly)
                for cx, cy, r in holes:
                    ok &= (x - cx) ** 2 + (y - cy) ** 2 > r * r
                out.append(np.stack([x[ok], y[ok], np.full(ok.sum(), z)], 1))
            p = np.concatenate(out)[:m]
            n = np.tile([0.0, 0.0, nz], (m, 1))
            return p @ R.T + o, n @ R.T
        return fn

    surface.add(area2d, face(z1, 1.0))
    surface.add(area2d, face(z0, -1.0))
    npoly = len(poly)
    for i in range(npoly):
        a, b = poly[i], poly[(i + 1) % npoly]
        e = b - a
        L = float(np.hypot(*e))
        nrm = np.array([e[1], -e[0], 0.0]) / L

        def side(rng, m, a=a, e=e, nrm=nrm):
            u = rng.uniform(0, 1, m)
            z = rng.uniform(z0, z1, m)
            p = np.stack([a[0] + u * e[0], a[1] + u * e[1], z], 1)
            return p @ R.T + o, np.tile(nrm, (m, 1)) @ R.T
        surface.add(L * (z1 - z0), side)
    for cx, cy, r in holes:
        def wall(rng, m, cx=cx, cy=cy, r=r):
            th = rng.uniform(0, 2 * math.pi, m)
            z = rng.uniform(z0, z1, m)
            p = np.stack([cx + r * np.cos(th), cy + r * np.sin(th), z], 1)
            n = np.stack([-np.cos(th), -np.sin(th), np.zeros(m)], 1)  # into the hole axis
            return p @ R.T + o, n @ R.T
        surface.add(2 * math.pi * r * (z1 - z0), wall)


def gear_surface(teeth=24, r_out=50.0, r_root=42.0, bore=10.0, thickness=20.0):
    """Spur gear; `bore` is the bore diameter."""
    s = _Surface()
    _prism_with_holes(s, gear_profile(teeth, r_out, r_root), [(0.0, 0.0, bore / 2)],
                      -thickness / 2, thickness / 2)
    return s


def bracket_surface(width=60.0, depth=40.0, thick=8.0, hole=6.0):
    """L-bracket: two width x depth x thick plates joined at 90 degrees (an L-shaped
    profile extruded over `width`), each plate pierced by two round holes of diameter
    `hole`."""
    s = _Surface()
    # L profile in the (y, z) plane, extruded along x: local (x, y, z) -> world (y, z, x)
    prof = np.array([[0, 0], [depth, 0], [depth, thick], [thick, thick], [thick, depth],
                     [0, depth]], dtype=np.float64)
    Rf = np.array([[0.0, 0.0, 1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    inner = _Surface()
    _prism_with_holes(inner, prof, [], 0.0, width, (Rf, np.zeros(3)))
    r = hole / 2
    # (axis, centre in world coords, span along the axis)
    holes = [(2, (width * 0.25, depth * 0.6), (0.0, thick)),
             (2, (width * 0.75, depth * 0.6), (0.0, thick)),
             (1, (width * 0.25, depth * 0.6), (0.0, thick)),
             (1, (width * 0.75, depth * 0.6), (0.0, thick))]

    def outside_holes(p):
        ok = np.ones(len(p), dtype=bool)
        for axis, (a, b), (lo, hi) in holes:
            if axis == 2:  # vertical hole through the horizontal plate: centre (x, y)
                d2 = (p[:, 0] - a) ** 2 + (p[:, 1] - b) ** 2
                along = p[:, 2]
            else:  # hole along y through the vertical plate: centre (x, z)
                d2 = (p[:, 0] - a) ** 2 + (p[:, 2] - b) ** 2
                along = p[:, 1]
            ok &= ~((d2 < r * r) & (along >= lo - 1e-6) & (along <= hi + 1e-6))
        return ok

    def body(rng, m):
        out_p, out_n = [], []
        while sum(len(a) for a in out_p) < m:
            p, n = inner.sample(rng, int(m * 1.1) + 16)
            ok = outside_holes(p)
            out_p.append(p[ok])
            out_n.append(n[ok])
        return np.concatenate(out_p)[:m], np.concatenate(out_n)[:m]
    s.add(inner.area() - 8 * math.pi * r * r, body)
    for axis, (a, b), (lo, hi) in holes:
        def wall(rng, m, axis=axis, a=a, b=b, lo=lo, hi=hi):
            th = rng.uniform(0, 2 * math.pi, m)
            h = rng.uniform(lo, hi, m)
            c, sn = np.cos(th), np.sin(th)
            if axis == 2:
                p = np.stack([a + r * c, b + r * sn, h], 1)
                n = np.stack([-c, -sn, np.zeros(m)], 1)
            else:
                p = np.stack([a + r * c, h, b + r * sn], 1)
                n = np.stack([-c, np.zeros(m), -sn], 1)
            return p, n
        s.add(2 * math.pi * r * thick, wall)
    return s


def torus_surface(R=30.0, r=8.0):
    s = _Surface()

    def fn(rng, m):
        out_u, out_v = [], []
        while sum(len(a) for a in out_u) < m:
            k = 2 * m
            u = rng.uniform(0, 2 * math.pi, k)
            v = rng.uniform(0, 2 * math.pi, k)
            w = rng.uniform(0, 1, k)
            ok = w < (R + r * np.cos(v)) / (R + r)
            out_u.append(u[ok])
            out_v.append(v[ok])
        u = np.concatenate(out_u)[:m]
        v = np.concatenate(out_v)[:m]
        p = np.stack([(R + r * np.cos(v)) * np.cos(u), (R + r * np.cos(v)) * np.sin(u),
                      r * np.sin(v)], 1)
        n = np.stack([np.cos(v) * np.cos(u), np.cos(v) * np.sin(u), np.sin(v)], 1)
        return p, n
    s.add(4 * math.pi * math.pi * R * r, fn)
    return s


MODELS = {
    "gear": lambda: gear_surface(),
    "bracket": lambda: bracket_surface(),
    "torus": lambda: torus_surface(),
}


def model_cloud(name="gear", n=20000, seed=0, surface=None):
    """Model point cloud with exact normals, centred on its bounding-box centre."""
    rng = np.random.default_rng(seed)
    s = surface if surface is not None else MODELS[name]()
    p, nrm = s.sample(rng, n)
    c = 0.5 * (p.min(0) + p.max(0))
    return Cloud((p - c).astype(np.float32), nrm.astype(np.float32)), s, c


def random_rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def _box_surface(rng, center, size, R):
    s = _Surface()
    hx, hy, hz = size / 2

    def face(axis, sign):
        def fn(rng_, m):
            u = rng_.uniform(-1, 1, (m, 3)) * np.array([hx, hy, hz])
            u[:, axis] = sign * [hx, hy, hz][axis]
            n = np.zeros((m, 3))
            n[:, axis] = sign
            return u @ R.T + center, n @ R.T
        return fn
    dims = [hx, hy, hz]
    for axis in range(3):
        a, b = [d for k, d in enumerate(dims) if k != axis]
        for sign in (-1.0, 1.0):
            s.add(4 * a * b, face(axis, sign))
    return s


def _sphere_surface(center, radius):
    s = _Surface()

    def fn(rng, m):
        n = rng.standard_normal((m, 3))
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        return center + radius * n, n
    s.add(4 * math.pi * radius * radius, fn)
    return s


def make_scene(seed, models, n_instances, box, points_per_instance, plane=None,
               plane_points=0, clutter_frac=0.1, clutter="uniform", noise=0.2,
               viewpoint=(620.0, 100.0, 500.0), model_centers=None):
    """Generate a scene.

    models: dict name -> _Surface (model frame centred on its bbox centre: pass
    model_centers[name] to shift). box: ((xmin, ymin, zmin), (xmax, ymax, zmax)) for
    instance centres. plane: (size, z) of a square ground plane centred under the box.
    """
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(box[0], float), np.asarray(box[1], float)
    vp = np.asarray(viewpoint, dtype=np.float64)
    names = list(models)
    radii = {}
    for nm, s in models.items():
        p, _ = s.sample(np.random.default_rng(1), 4000)
        c = model_centers[nm] if model_centers else 0.5 * (p.min(0) + p.max(0))
        radii[nm] = float(np.linalg.norm(p - c, axis=1).max())
    placed, pts, nrms = [], [], []
    tries = 0
    while len(placed) < n_instances and tries < 20000:
        tries += 1
        nm = names[int(rng.integers(len(names)))]
        t = rng.uniform(lo, hi)
        r = radii[nm]
        if any(np.linalg.norm(t - q.t) < r + radii[q.model] for q in placed):
            continue
        R = random_rotation(rng)
        placed.append(Instance(nm, R, t))
    for inst in placed:
        s = models[inst.model]
        c = model_centers[inst.model] if model_centers else 0.0
        p, n = s.sample(rng, points_per_instance)
        p = (p - c) @ inst.R.T + inst.t
        n = n @ inst.R.T
        pts.append(p)
        nrms.append(n)
    if plane is not None and plane_points > 0:
        size, z = plane
        cx, cy = 0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1])
        p = np.stack([rng.uniform(cx - size / 2, cx + size / 2, plane_points),
                      rng.uniform(cy - size / 2, cy + size / 2, plane_points),
                      np.full(plane_points, z)], 1)
        pts.append(p)
        nrms.append(np.tile([0.0, 0.0, 1.0], (plane_points, 1)))
    P = np.concatenate(pts)
    Nn = np.concatenate(nrms)
    n_obj = len(P)
    n_clutter = int(round(clutter_frac / max(1e-9, 1 - clutter_frac) * n_obj))
    if n_clutter > 0:
        if clutter == "uniform":
            cp = rng.uniform(lo - 20, hi + 20, (n_clutter, 3))
            cn = rng.standard_normal((n_clutter, 3))
            cn /= np.linalg.norm(cn, axis=1, keepdims=True)
            # uniform clutter has no surface: orient toward the viewer so it survives culling
            flip = np.einsum("ij,ij->i", cn, vp - cp) < 0
            cn[flip] *= -1
        else:  # random boxes and spheres
            shapes = []
            n_shapes = int(rng.integers(6, 16))
            for _ in range(n_shapes):
                ctr = rng.uniform(lo, hi)
                if rng.random() < 0.5:
                    size = rng.uniform(15, 60, 3)
                    shapes.append(_box_surface(rng, ctr, size, random_rotation(rng)))
                else:
                    shapes.append(_sphere_surface(ctr, float(rng.uniform(8, 30))))
            areas = np.array([s.area() for s in shapes])
            counts = rng.multinomial(2 * n_clutter, areas / areas.sum())
            cps, cns = [], []
            for s, k in zip(shapes, counts):
                if k:
                    p, n = s.sample(rng, int(k))
                    cps.append(p)
                    cns.append(n)
            cp, cn = np.concatenate(cps), np.concatenate(cns)
        P = np.concatenate([P, cp])
        Nn = np.concatenate([Nn, cn])
    P = P + rng.normal(0, noise, P.shape)
    vis = np.einsum("ij,ij->i", Nn, vp - P) > 0
    P, Nn = P[vis], Nn[vis]
    perm = rng.permutation(len(P))
    P = P[perm].astype(np.float32)
    return Scene(Cloud(np.ascontiguousarray(P)), placed, vp.astype(np.float32))


# --------------------------------------------------------------------------------------
# The configured workloads
# --------------------------------------------------------------------------------------

def gear_model(n=20000, seed=7):
    cloud, s, c = model_cloud("gear", n, seed)
    return cloud, s, c


def scene_small(seed=1, model=None):
    """Three gears over a 400x400 ground plane, 10% uniform clutter, sigma 0.2 mm,
    about 100k points (plain method, small)."""
    _, s, c = model if model is not None else gear_model()
    return make_scene(seed, {"gear": s}, 3, ((-100, -100, 40), (100, 100, 140)),
                      points_per_instance=34000, plane=(400.0, 0.0), plane_points=42000,
                      clutter_frac=0.10, clutter="uniform", noise=0.2,
                      model_centers={"gear": c})


def scene_large(seed=2, model=None):
    """Ten gears in a 400x400x200 box, 30% clutter of random boxes and spheres, sigma
    0.3 mm, about 1M points (large single scene)."""
    _, s, c = model if model is not None else gear_model()
    return make_scene(seed, {"gear": s}, 10, ((-200, -200, 0), (200, 200, 200)),
                      points_per_instance=100000, clutter_frac=0.30, clutter="shapes",
                      noise=0.3, model_centers={"gear": c})


def scene_tiny(seed=3, model=None, n_inst=2, pts=6000, noise=0.2):
    """A small two-instance scene for quick parity tests."""
    _, s, c = model if model is not None else gear_model(8000, seed=5)
    return make_scene(seed, {"gear": s}, n_inst, ((-70, -70, 40), (70, 70, 100)),
                      points_per_instance=pts, plane=(220.0, 0.0), plane_points=pts,
                      clutter_frac=0.05, clutter="uniform", noise=noise,
                      model_centers={"gear": c})


def scene_random(seed, n_target, surfaces, centers, noise, clutter_frac, n_inst,
                 box=((-200, -200, 0), (200, 200, 200))):
    """A scene of about n_target points: n_inst instances of one model, clutter of random
    boxes and spheres, noise, viewpoint culling (batching / serving workloads)."""
    name = list(surfaces)[0]
    # about half of each instance's surface faces the viewer; clutter adds its fraction
    per = max(200, int(n_target * (1 - clutter_frac) * 2.0 / max(1, n_inst)))
    return make_scene(seed, {name: surfaces[name]}, n_inst, box, points_per_instance=per,
                      clutter_frac=clutter_frac, clutter="shapes", noise=noise,
                      model_centers={name: centers[name]})


def batch_models(seed=11):
    """The three procedural models of the batching workload, each sampled at 20k-40k
    points: name -> (Cloud, surface, centre)."""
    rng = np.random.default_rng(seed)
    out = {}
    for k, name in enumerate(["gear", "bracket", "torus"]):
        out[name] = model_cloud(name, int(rng.integers(20000, 40001)), seed + k)
    return out


def batch_scenes(n_scenes=64, seed=21, models=None, n_min=50_000, n_max=2_000_000):
    """The batching workload: scenes with log-uniform point counts in [n_min, n_max], 1-12
    instances of one of the models (drawn per scene), noise sigma U(0.2, 0.5) mm and
    clutter U(10%, 40%), all from the seed. Returns [(model name, Scene)]."""
    models = models or batch_models()
    rng = np.random.default_rng(seed)
    names = sorted(models)
    out = []
    for i in range(n_scenes):
        name = names[int(rng.integers(len(names)))]
        n = int(np.exp(rng.uniform(np.log(n_min), np.log(n_max))))
        sc = scene_random(int(rng.integers(1 << 30)), n, {name: models[name][1]},
                          {name: models[name][2]}, float(rng.uniform(0.2, 0.5)),
                          float(rng.uniform(0.10, 0.40)), int(rng.integers(1, 13)))
        out.append((name, sc))
    return out


def serving_models(seed=31):
    """Eight resident models: gear, L-bracket, torus, plus five gears and brackets with a
    random tooth count (12-40) or plate size (30-80 mm)."""
    rng = np.random.default_rng(seed)
    surfs = {"gear": gear_surface(), "bracket": bracket_surface(), "torus": torus_surface()}
    for k in range(5):
        if k % 2 == 0:
            teeth = int(rng.integers(12, 41))
            r_out = float(rng.uniform(30, 60))
            surfs[f"gear{teeth}"] = gear_surface(teeth=teeth, r_out=r_out, r_root=r_out * 0.84,
                                                 bore=r_out * 0.2, thickness=float(rng.uniform(10, 25)))
        else:
            w, d = (float(x) for x in rng.uniform(30, 80, 2))
            surfs[f"bracket{int(w)}x{int(d)}"] = bracket_surface(width=w, depth=d,
                                                                thick=float(rng.uniform(5, 10)))
    out = {}
    for k, (name, s) in enumerate(surfs.items()):
        out[name] = model_cloud(name, 20000, seed + k, surface=s)
    return out


def gear_symmetries(teeth=24):
    """Rotations mapping the procedural spur gear onto itself (model frame): turns about z
    by a tooth pitch, and half-turns about the in-plane axes through tooth and gap
    centres."""
    out = []
    pitch = 2 * np.pi / teeth
    for k in range(teeth):
        a = k * pitch
        out.append(np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]]))
    for k in range(teeth):
        phi = 0.25 * pitch + k * 0.5 * pitch
        u = np.array([np.cos(phi), np.sin(phi), 0.0])
        out.append(2 * np.outer(u, u) - np.eye(3))
    return out


def pose_error_sym(A, B, syms):
    """Rotation (deg) and translation error between 4x4 poses A and B of a symmetric model:
    B = A * S for the symmetry S closest to A^-1 B."""
    Ra, Rb = A[:3, :3].astype(np.float64), B[:3, :3].astype(np.float64)
    Rs = Ra.T @ Rb

    def angle(R):
        # atan2(sin, cos) of the rotation angle: the skew part gives the sine, so a float32
        # rotation compared with itself reads 0 (arccos of the trace alone reads its
        # non-orthonormality as a few hundredths of a degree)
        w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]]) / 2.0
        return np.degrees(np.arctan2(np.linalg.norm(w), (np.trace(R) - 1.0) / 2.0))

    ang = min(angle(S.T @ Rs) for S in syms)
    return ang, float(np.linalg.norm(A[:3, 3].astype(np.float64) - B[:3, 3]))


def match_poses(poses, ref_poses, syms):
    """Each pose paired with the unused reference pose nearest to it (rotation error modulo
    the symmetries, then translation); returns [(rotation deg, translation)]."""
    used, out = set(), []
    for P in poses:
        cands = [(i,) + pose_error_sym(P, Q, syms) for i, Q in enumerate(ref_poses) if i not in used]
        if not cands:
            break
        best = min(cands, key=lambda t: t[2])
        used.add(best[0])
        out.append(best[1:])
    return out

