"""Seeded synthetic scenes for the benchmark workloads (host-side, numpy).

Every scene is a list of axis-aligned rectangles subdivided into quad patches.
Quads are wound so that the reference's patch normal (v4-v1) x (v2-v1)
(source/Patch.cpp:272-276) points into the visible side, which is the side the
hemicube rasteriser treats as front-facing.

* ``cornell_box``   - the small plain workload: closed-on-5-sides 5.5 m box,
  tall and short block, 1.3 x 1.05 m ceiling light with emission (17,12,4),
  grey 0.73 / red-ish left / green-ish right walls, about ``target`` patches.
* ``room_with_boxes`` - the large plain workload: 20 x 20 x 5 m room, 40 random
  axis-aligned boxes with sides U[0.3, 3] m, 4 ceiling emitters with emission
  U[5, 20] per channel, reflectance U[0.1, 0.8] per channel per object,
  subdivided to about ``target`` patches (50,000 by default).

The returned dict holds vertices (N*12), color (N*3), reflectance (N*3),
radiosity (N*3, the emission = initial unshot energy), illumination (N*3, zeros)
as float32 arrays, plus ``n`` and ``object_id`` (N).
"""
from __future__ import annotations

import math

import numpy as np


def _rect(origin, u, v, normal_hint):
    """Corners of the rectangle origin + [0,1]u + [0,1]v, wound for normal_hint."""
    o = np.asarray(origin, np.float64)
    u = np.asarray(u, np.float64)
    v = np.asarray(v, np.float64)
    c = [o, o + u, o + u + v, o + v]
    n = np.cross(c[3] - c[0], c[1] - c[0])
    if np.dot(n, normal_hint) < 0:
        c = [c[0], c[3], c[2], c[1]]
    return c


def _subdivide(corners, edge):
    c0, c1, c2, c3 = corners
    lu = np.linalg.norm(c1 - c0)
    lv = np.linalg.norm(c3 - c0)
    ku = max(1, int(math.ceil(lu / edge - 1e-9)))
    kv = max(1, int(math.ceil(lv / edge - 1e-9)))
    du = (c1 - c0) / ku
    dv = (c3 - c0) / kv
    # grid points computed once, so neighbouring patches share bit-identical corners
    g = [[(c0 + du * i + dv * j).astype(np.float32) for i in range(ku + 1)] for j in range(kv + 1)]
    out = []
    for j in range(kv):
        for i in range(ku):
            out.append([g[j][i], g[j][i + 1], g[j + 1][i + 1], g[j + 1][i]])
    return out


def _box_faces(lo, hi, outward=True, with_bottom=False):
    """Rectangles of an axis-aligned box [lo, hi]; outward or inward normals."""
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    s = 1.0 if outward else -1.0
    faces = [
        ((x0, y1, z0), (x1 - x0, 0, 0), (0, 0, z1 - z0), (0, s, 0)),   # top
        ((x0, y0, z0), (x1 - x0, 0, 0), (0, y1 - y0, 0), (0, 0, -s)),  # z0 side
        ((x0, y0, z1), (x1 - x0, 0, 0), (0, y1 - y0, 0), (0, 0, s)),   # z1 side
        ((x0, y0, z0), (0, 0, z1 - z0), (0, y1 - y0, 0), (-s, 0, 0)),  # x0 side
        ((x1, y0, z0), (0, 0, z1 - z0), (0, y1 - y0, 0), (s, 0, 0)),   # x1 side
    ]
    if with_bottom:
        faces.append(((x0, y0, z0), (x1 - x0, 0, 0), (0, 0, z1 - z0), (0, -s, 0)))
    return [_rect(o, u, v, np.array(n, np.float64)) for o, u, v, n in faces]


def _assemble(parts, edge):
    """parts: list of (corners, rho(3), emission(3), object_id)."""
    verts, rho, emit, obj = [], [], [], []
    for corners, r, e, oid in parts:
        for q in _subdivide(corners, edge):
            verts.append(np.concatenate(q))
            rho.append(r)
            emit.append(e)
            obj.append(oid)
    n = len(verts)
    v = np.asarray(verts, np.float32).reshape(-1)
    rho_a = np.asarray(rho, np.float32).reshape(-1)
    e_a = np.asarray(emit, np.float32).reshape(-1)
    return dict(n=n, vertices=v, color=rho_a.copy(), reflectance=rho_a, radiosity=e_a,
                illumination=np.zeros(3 * n, np.float32), object_id=np.asarray(obj, np.int32))


def _fit_edge(parts, target):
    area = 0.0
    for corners, *_ in parts:
        c0, c1, _, c3 = corners
        area += np.linalg.norm(c1 - c0) * np.linalg.norm(c3 - c0)
    edge = math.sqrt(area / target)
    for _ in range(40):  # shrink/grow until the subdivided count is within 2% of target
        n = sum(len(_subdivide(p[0], edge)) for p in parts)
        if abs(n - target) <= 0.02 * target:
            break
        edge *= math.sqrt(n / target)
    return edge


def cornell_box(target: int = 5000, seed: int = 0) -> dict:
    S = 5.5
    grey = (0.73, 0.73, 0.73)
    zero = (0.0, 0.0, 0.0)
    parts = []
    parts.append((_rect((0, 0, 0), (S, 0, 0), (0, 0, S), np.array([0, 1.0, 0])), grey, zero, 0))      # floor
    parts.append((_rect((0, S, 0), (S, 0, 0), (0, 0, S), np.array([0, -1.0, 0])), grey, zero, 1))     # ceiling
    parts.append((_rect((0, 0, S), (S, 0, 0), (0, S, 0), np.array([0, 0, -1.0])), grey, zero, 2))     # back
    parts.append((_rect((0, 0, 0), (0, 0, S), (0, S, 0), np.array([1.0, 0, 0])),
                  (0.63, 0.065, 0.05), zero, 3))                                                    # left
    parts.append((_rect((S, 0, 0), (0, 0, S), (0, S, 0), np.array([-1.0, 0, 0])),
                  (0.14, 0.45, 0.09), zero, 4))                                                     # right
    for f in _box_faces((3.0, 0.0, 2.8), (4.65, 3.3, 4.45)):                                       # tall box
        parts.append((f, grey, zero, 5))
    for f in _box_faces((0.9, 0.0, 0.8), (2.55, 1.65, 2.45)):                                      # short box
        parts.append((f, grey, zero, 6))
    light = _rect((S / 2 - 0.65, S - 0.005, S / 2 - 0.525), (1.3, 0, 0), (0, 0, 1.05), np.array([0, -1.0, 0]))
    edge = _fit_edge(parts, target)
    scene = _assemble(parts, edge)
    lscene = _assemble([(light, (0.78, 0.78, 0.78), (17.0, 12.0, 4.0), 7)], edge)
    return _concat(scene, lscene)


def room_with_boxes(target: int = 50000, seed: int = 0, n_boxes: int = 40, n_emitters: int = 4) -> dict:
    rng = np.random.default_rng(seed)
    X, Y, Z = 20.0, 5.0, 20.0

    def rho():
        return tuple(rng.uniform(0.1, 0.8, 3))

    zero = (0.0, 0.0, 0.0)
    parts = []
    room = _box_faces((0, 0, 0), (X, Y, Z), outward=False, with_bottom=True)
    for k, f in enumerate(room):
        parts.append((f, rho(), zero, k))
    for b in range(n_boxes):
        sx, sy, sz = rng.uniform(0.3, 3.0, 3)
        x0 = rng.uniform(0.0, X - sx)
        z0 = rng.uniform(0.0, Z - sz)
        r = rho()
        for f in _box_faces((x0, 0.0, z0), (x0 + sx, sy, z0 + sz)):
            parts.append((f, r, zero, 100 + b))
    edge = _fit_edge(parts, target - 64)
    scene = _assemble(parts, edge)
    lights = []
    for e in range(n_emitters):
        w, d = rng.uniform(0.5, 2.0, 2)
        x0 = rng.uniform(0.5, X - w - 0.5)
        z0 = rng.uniform(0.5, Z - d - 0.5)
        em = tuple(rng.uniform(5.0, 20.0, 3))
        q = _rect((x0, Y - 0.01, z0), (w, 0, 0), (0, 0, d), np.array([0, -1.0, 0]))
        lights.append((q, (0.8, 0.8, 0.8), em, 1000 + e))
    return _concat(scene, _assemble(lights, edge))


def _concat(a: dict, b: dict) -> dict:
    out = {}
    for k in ("vertices", "color", "reflectance", "radiosity", "illumination", "object_id"):
        out[k] = np.concatenate([a[k], b[k]])
    out["n"] = a["n"] + b["n"]
    return out


def cornell_variant(target: int = 5000, seed: int = 0, n_lights: int = 1) -> dict:
    """A seeded variation of ``cornell_box`` for training data: box size, block sizes and
    positions, wall reflectances, and the lights' sizes, positions and emission vary."""
    rng = np.random.default_rng(seed)
    S = float(rng.uniform(4.0, 7.0))
    zero = (0.0, 0.0, 0.0)

    def rho():
        return tuple(rng.uniform(0.1, 0.8, 3))

    parts = []
    parts.append((_rect((0, 0, 0), (S, 0, 0), (0, 0, S), np.array([0, 1.0, 0])), rho(), zero, 0))
    parts.append((_rect((0, S, 0), (S, 0, 0), (0, 0, S), np.array([0, -1.0, 0])), rho(), zero, 1))
    parts.append((_rect((0, 0, S), (S, 0, 0), (0, S, 0), np.array([0, 0, -1.0])), rho(), zero, 2))
    parts.append((_rect((0, 0, 0), (0, 0, S), (0, S, 0), np.array([1.0, 0, 0])), rho(), zero, 3))
    parts.append((_rect((S, 0, 0), (0, 0, S), (0, S, 0), np.array([-1.0, 0, 0])), rho(), zero, 4))
    for b in range(2):
        w, h, d = rng.uniform(0.15, 0.35, 3) * S
        h *= 1.0 + b
        x0 = rng.uniform(0.05 * S, S - w - 0.05 * S)
        z0 = rng.uniform(0.05 * S, S - d - 0.05 * S)
        r = rho()
        for f in _box_faces((x0, 0.0, z0), (x0 + w, min(h, 0.8 * S), z0 + d)):
            parts.append((f, r, zero, 5 + b))
    lights = []
    for k in range(n_lights):
        lw, ld = rng.uniform(0.1, 0.3, 2) * S
        lx = rng.uniform(0.05 * S, S - lw - 0.05 * S)
        lz = rng.uniform(0.05 * S, S - ld - 0.05 * S)
        em = tuple(rng.uniform(5.0, 20.0, 3))
        light = _rect((lx, S - 0.005 - 0.001 * k, lz), (lw, 0, 0), (0, 0, ld), np.array([0, -1.0, 0]))
        lights.append((light, (0.8, 0.8, 0.8), em, 7 + k))
    edge = _fit_edge(parts, target)
    return _concat(_assemble(parts, edge), _assemble(lights, edge))
