"""Seeded synthetic workloads as numpy arrays (host memory).

The generators themselves are host C++ in librtcore (include/rtcore_scene.h)
so that the C++ drop-in sample and the Python tests and benchmark produce the
same bits; this module only allocates the arrays and calls them.

Seeds follow one convention: 0x5EED0000 + workload number, where 1 is the
single-triangle sample, 2 the triangle soup, 3 the box scene, 4 the batched
form and 5 the learned form.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import RT_OK, RtError, load

SEED_BASE = 0x5EED0000

# rt_ray: org xyz, tmin, dir xyz, tmax (32 bytes)
RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
# rt_hit: t, prim, u, v (16 bytes)
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])
# rt_hit_ext (32 bytes)
HIT_EXT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance_id", "<u4"),
                          ("custom_index", "<u4"), ("geometry_index", "<u4"), ("primitive_id", "<u4"),
                          ("sbt_record", "<u4")])
MATERIAL_DTYPE = np.dtype([("albedo", "<f4", 3), ("emission", "<f4", 3)])


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def soup(seed: int, n_tris: int):
    """(vertices float32 [3n, 3], indices uint32 [n, 3]) of the triangle soup."""
    v = np.empty((3 * n_tris, 3), np.float32)
    i = np.empty((n_tris, 3), np.uint32)
    rc = load().rt_scene_soup(seed, n_tris, _ptr(v), _ptr(i))
    if rc != RT_OK:
        raise RtError(rc, "rt_scene_soup")
    return v, i


def box(seed: int, n_spheres: int, freq: int):
    """(vertices, indices, tri_material, materials) of the box scene."""
    lib = load()
    nv, nt, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
    rc = lib.rt_scene_box_counts(n_spheres, freq, C.byref(nv), C.byref(nt), C.byref(nm))
    if rc != RT_OK:
        raise RtError(rc, "rt_scene_box_counts")
    v = np.empty((nv.value, 3), np.float32)
    i = np.empty((nt.value, 3), np.uint32)
    tm = np.empty(nt.value, np.uint32)
    m = np.empty(nm.value, MATERIAL_DTYPE)
    rc = lib.rt_scene_box(seed, n_spheres, freq, _ptr(v), _ptr(i), _ptr(tm), _ptr(m))
    if rc != RT_OK:
        raise RtError(rc, "rt_scene_box")
    return v, i, tm, m


def load_obj(path):
    """(vertices float32 [n, 3], indices uint32 [m, 3], tri_material uint32 [m],
    number of materials) of a Wavefront OBJ file (rt_obj_load)."""
    import os
    lib = load()
    b = os.fsencode(str(path))
    nv, nt, nm = C.c_uint32(), C.c_uint32(), C.c_uint32()
    rc = lib.rt_obj_counts(b, C.byref(nv), C.byref(nt), C.byref(nm))
    if rc != RT_OK:
        raise RtError(rc, "rt_obj_counts")
    v = np.empty((nv.value, 3), np.float32)
    i = np.empty((nt.value, 3), np.uint32)
    tm = np.empty(nt.value, np.uint32)
    rc = lib.rt_obj_load(b, _ptr(v), _ptr(i), _ptr(tm))
    if rc != RT_OK:
        raise RtError(rc, "rt_obj_load")
    return v, i, tm, nm.value


def write_obj(path, v: np.ndarray, i: np.ndarray, tri_material: np.ndarray | None = None) -> None:
    """Writes vertices and triangles as OBJ text (floats with 9 significant
    digits, which read back to the same float32)."""
    lines = [f"v {a:.9g} {b:.9g} {c:.9g}" for a, b, c in np.asarray(v, np.float32).tolist()]
    cur = None
    for k, (a, b, c) in enumerate((np.asarray(i, np.int64) + 1).tolist()):
        if tri_material is not None and tri_material[k] != cur:
            cur = int(tri_material[k])
            lines.append(f"usemtl m{cur}")
        lines.append(f"f {a} {b} {c}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def incoherent_rays(seed: int, n: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), tmax: float = 1e30):
    rays = np.empty(n, RAY_DTYPE)
    lo_a = np.asarray(lo, np.float32)
    hi_a = np.asarray(hi, np.float32)
    rc = load().rt_scene_incoherent_rays(seed, n, _ptr(lo_a), _ptr(hi_a), tmax, _ptr(rays))
    if rc != RT_OK:
        raise RtError(rc, "rt_scene_incoherent_rays")
    return rays


# rt_instance: the bit layout of VkAccelerationStructureInstanceKHR (64 bytes)
INSTANCE_DTYPE = np.dtype([("transform", "<f4", (3, 4)), ("custom_index_and_mask", "<u4"),
                           ("sbt_offset_and_flags", "<u4"), ("accel_ref", "<u8")])

# The reference sample's scene (vulkan-raytraced-triangle/main.cpp).
REF8_VERTICES = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)       # :676-681
REF8_INDICES = np.array([[0, 1, 3], [1, 2, 3]], np.uint32)                                 # :682
REF8_GEOM_TRANSFORMS = np.array([[[1, 0, 0, -2], [0, 1, 0, 0], [0, 0, 1, 0]],               # :684-695
                                 [[1, 0, 0, 2], [0, 1, 0, 0], [0, 0, 1, 0]]], np.float32)
REF8_INSTANCE_TRANSFORMS = np.array([[[1, 0, 0, 0], [0, 1, 0, 2], [0, 0, 1, 0]],           # :835-846
                                     [[1, 0, 0, 0], [0, 1, 0, -2], [0, 0, 1, 0]]], np.float32)
REF8_CUSTOM_INDEX = 100                                                                    # :850
REF8_SBT_OFFSETS = (0, 2)                                                                  # :851, :857
REF8_SBT_COLORS = np.array([[0.6, 0.1, 0.2], [0.1, 0.8, 0.4], [0.9, 0.7, 0.1], [0.3, 0.6, 0.9]],
                           np.float32)                                                     # :1310-1317
REF8_CAMERA = ((0.0, 0.0, 10.0), 60.0)                                                     # :1015
REF8_SIZE = (1200, 800)                                                                    # :13-14

TRI1_VERTICES = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32)
TRI1_INDICES = np.array([[0, 1, 2]], np.uint32)
TRI1_CAMERA = ((0.0, 0.0, 2.5), 60.0)
TRI1_SIZE = (800, 600)

# rt_pt_light: three vertices and the emitted radiance (48 bytes)
LIGHT_DTYPE = np.dtype([("v0", "<f4", 3), ("v1", "<f4", 3), ("v2", "<f4", 3), ("emission", "<f4", 3)])

# The box workload's path-tracing setup: camera inside the box near the front
# wall, looking -z with the sample's raygen basis.
BOX_CAMERA = ((0.0, 0.0, 0.95), 60.0)


def emissive_lights(v: np.ndarray, i: np.ndarray, tri_material: np.ndarray, materials: np.ndarray) -> np.ndarray:
    """Every triangle whose material emits, as rt_pt_light records."""
    em = materials["emission"][tri_material]
    sel = np.nonzero((em > 0).any(axis=1))[0]
    out = np.zeros(len(sel), LIGHT_DTYPE)
    out["v0"] = v[i[sel, 0]]
    out["v1"] = v[i[sel, 1]]
    out["v2"] = v[i[sel, 2]]
    out["emission"] = em[sel]
    return out
