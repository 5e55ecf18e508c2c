"""Generates tests/golden/sample_pixels.json: known-answer pixels of the
reference sample's scene and of the single-triangle workload, computed
analytically in float64 numpy, independently of both the CPU oracle and the
CUDA path.

Inputs are the sample's own constants (vulkan-raytraced-triangle/main.cpp):
  quad vertices and indices        :676-682
  geometry transforms (x = -2, +2) :684-695
  instance transforms (y = +2, -2) :835-846, custom index 100 :850,
  SBT offsets 0 / 2                :851, :857
  SBT record colours               :1310-1317
  camera {0, 0, 10, 60}            :1015
  raygen (pinhole, basis X, -Y, -Z):1033-1045, tmin 0, tmax 100 :1051
  miss colour (0, 0, 0.2)          :1065
  closest hit predicate            :1080-1091
  launch 1200 x 800                :13-14, :1355

Only pixels whose hit point lies at least MARGIN (in barycentric units) inside
a triangle, or whose ray misses every quad by at least MARGIN, are kept, so the
answer does not depend on how a renderer resolves shared edges.

    python tests/golden/make_golden.py      # rewrites the JSON
"""
from __future__ import annotations

import json
import math
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "sample_pixels.json"
MARGIN = 1e-3

QUAD = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float64)
QUAD_IDX = [(0, 1, 3), (1, 2, 3)]
GEOM_TX = [-2.0, 2.0]
INST_TY = [2.0, -2.0]
INST_SBT = [0, 2]
CUSTOM = 100
SBT = [(0.6, 0.1, 0.2), (0.1, 0.8, 0.4), (0.9, 0.7, 0.1), (0.3, 0.6, 0.9)]
MISS = (0.0, 0.0, 0.2)


def f32(x: float) -> float:
    return float(np.float32(x))


def ray_dir(x: int, y: int, w: int, h: int, fov: float):
    ay = math.tan(math.radians(fov) * 0.5)
    ax = ay * w / h
    ndx = (x + 0.5) / w * 2.0 - 1.0
    ndy = (y + 0.5) / h * 2.0 - 1.0
    return np.array([ndx * ax, -ndy * ay, -1.0])


def isect(o, d, v0, v1, v2):
    """Moller-Trumbore in float64: (t, u, v) or None."""
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d, e2)
    det = float(np.dot(e1, p))
    if abs(det) < 1e-300:
        return None
    s = o - v0
    u = float(np.dot(s, p)) / det
    q = np.cross(s, e1)
    v = float(np.dot(d, q)) / det
    t = float(np.dot(e2, q)) / det
    return t, u, v


def ref8_triangles():
    out = []  # (inst, geom, prim, v0, v1, v2)
    for inst, ty in enumerate(INST_TY):
        for g, tx in enumerate(GEOM_TX):
            for p, (a, b, c) in enumerate(QUAD_IDX):
                off = np.array([tx, ty, 0.0])
                out.append((inst, g, p, QUAD[a] + off, QUAD[b] + off, QUAD[c] + off))
    return out


def shade_ref8(x, y, w=1200, h=800):
    o = np.array([0.0, 0.0, 10.0])
    d = ray_dir(x, y, w, h, 60.0)
    best = None
    near_edge = False
    for inst, g, p, v0, v1, v2 in ref8_triangles():
        r = isect(o, d, v0, v1, v2)
        if r is None:
            continue
        t, u, v = r
        if not (0.0 <= t <= 100.0):
            continue
        wmin = min(u, v, 1.0 - u - v)
        if abs(wmin) < MARGIN:
            near_edge = True
        if wmin >= 0.0 and (best is None or t < best[0]):
            best = (t, u, v, inst, g, p)
    if near_edge:
        return None
    if best is None:
        return MISS
    t, u, v, inst, g, p = best
    if p == 1 and inst == 1 and CUSTOM == 100 and g == 1:
        return (1.0 - u - v, u, v)
    return SBT[INST_SBT[inst] + g]


def shade_tri(x, y, w=800, h=600):
    o = np.array([0.0, 0.0, 2.5])
    d = ray_dir(x, y, w, h, 60.0)
    v0, v1, v2 = np.array([-1.0, -1, 0]), np.array([1.0, -1, 0]), np.array([0.0, 1, 0])
    r = isect(o, d, v0, v1, v2)
    if r is not None:
        t, u, v = r
        wmin = min(u, v, 1.0 - u - v)
        if abs(wmin) < MARGIN:
            return None
        if wmin >= 0.0 and 0.0 <= t <= 100.0:
            return (1.0 - u - v, u, v)
    return MISS


def sample(shade, w, h, step_x, step_y):
    pix = []
    for y in range(3, h, step_y):
        for x in range(5, w, step_x):
            c = shade(x, y)
            if c is None or (c == MISS and (x // step_x + y // step_y) % 6 != 0):
                continue  # near an edge, or one of the many misses not kept
            pix.append([x, y, *[f32(v) if c in (MISS, *SBT) else v for v in c]])
    return pix


def main() -> None:
    data = {
        "note": "known-answer pixels of the reference sample (float64 analytic); see make_golden.py",
        "margin": MARGIN,
        "ref8": {"width": 1200, "height": 800, "camera": [[0.0, 0.0, 10.0], 60.0], "chit": "sample",
                 "pixels": sample(shade_ref8, 1200, 800, 23, 17)},
        "tri": {"width": 800, "height": 600, "camera": [[0.0, 0.0, 2.5], 60.0], "chit": "barycentric",
                "pixels": sample(shade_tri, 800, 600, 13, 11)},
    }
    OUT.write_text(json.dumps(data, indent=0))
    print(f"wrote {OUT}: ref8 {len(data['ref8']['pixels'])} px, tri {len(data['tri']['pixels'])} px")


if __name__ == "__main__":
    main()
