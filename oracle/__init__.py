"""CPU oracle of the ray-tracing core -- TEST INFRASTRUCTURE ONLY.

Builds oracle/oracle.cpp (a scalar C++ restatement of the reference sample's
shader math plus this project's BVH build and traversal) into
oracle/_build/liboracle.so and exposes it through ctypes.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
checker; the product never links or calls it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SRC = [HERE / "oracle.cpp"]
DEPS = SRC + [HERE / "oracle.h", Path(__file__)] + sorted((REPO / "include").glob("*.h"))

# -ffp-contract=off: one rounding per operation, as the GPU kernels
# (-fmad=false); no -march flags so x86-64 and aarch64 round alike.
CXXFLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in DEPS):
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", *CXXFLAGS, *map(str, SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stderr}")
    tmp.replace(LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    vp, u32, u64, i32, f = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
    protos = {
        "orc_blas_accel_bytes": (u64, [vp, u32]),
        "orc_tlas_accel_bytes": (u64, [u32]),
        "orc_build_blas": (i32, [vp, u32, u32, vp, u64, vp]),
        "orc_build_tlas": (i32, [vp, u32, u32, vp, u64]),
        "orc_refit_blas": (i32, [vp, u32, vp]),
        "orc_refit_tlas": (i32, [vp, u32, vp]),
        "orc_trace_closest": (None, [vp, vp, vp, vp, u32, u32, vp]),
        "orc_trace_any": (None, [vp, vp, vp, u32, u32, vp]),
        "orc_brute_closest": (None, [vp, u32, vp, vp, u32, i32, u32]),
        "orc_intersect_tri": (i32, [vp, vp, f, f, vp, vp, vp, vp, vp, vp]),
        "orc_raygen": (None, [vp, u32, u32, u32, u32, vp, vp]),
        "orc_trace_rays": (i32, [vp, vp, u32, u32, vp, vp, vp, u32, u32, u32]),
        "orc_sort_pairs": (None, [vp, vp, u32, u32]),
        "orc_hw_threads": (u32, []),
        "orc_path_trace": (i32, [vp, vp, vp, u32, vp, u32, vp, vp, u32]),
        "orc_sincos_q": (None, [f, vp, vp]),
        "orc_path_trace_pixels": (i32, [vp, vp, vp, u32, vp, u32, vp, u32, vp, u32, vp, u32]),
        "orc_scene_soup": (i32, [u64, u32, vp, vp]),
        "orc_scene_incoherent_rays": (i32, [u64, u32, vp, vp, f, vp]),
    }
    for name, (res, args) in protos.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class LbvhDebug(C.Structure):
    _fields_ = [("keys_unsorted", C.c_void_p), ("keys_sorted", C.c_void_p), ("ids_sorted", C.c_void_p),
                ("bin_nodes", C.c_void_p)]


class Geometry(C.Structure):
    """Host-memory rt_geometry_triangles (same 48-byte layout)."""
    _fields_ = [("vertices", C.c_void_p), ("vertex_stride", C.c_uint64), ("max_vertex", C.c_uint32),
                ("index_type", C.c_uint32), ("indices", C.c_void_p), ("tri_count", C.c_uint32),
                ("flags", C.c_uint32), ("transform", C.c_void_p)]


# numpy views of the plain-data records (rtcore.h)
import numpy as np  # noqa: E402

RAY_DTYPE = np.dtype([("org", "<f4", 3), ("tmin", "<f4"), ("dir", "<f4", 3), ("tmax", "<f4")])
HIT_DTYPE = np.dtype([("t", "<f4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4")])
HIT_EXT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance_id", "<u4"),
                          ("custom_index", "<u4"), ("geometry_index", "<u4"), ("primitive_id", "<u4"),
                          ("sbt_record", "<u4")])
INSTANCE_DTYPE = np.dtype([("transform", "<f4", (3, 4)), ("custom_index_and_mask", "<u4"),
                           ("sbt_offset_and_flags", "<u4"), ("accel_ref", "<u8")])


class HostGeoms:
    """Keeps numpy arrays alive behind an array of Geometry descriptors.

    items: list of (vertices float32 [V,3], indices uint32 [T,3] or None,
    transform float32 [3,4] or None)."""

    def __init__(self, items):
        self.keep = []
        self.arr = (Geometry * max(1, len(items)))()
        self.n = len(items)
        for k, (v, i, xf) in enumerate(items):
            v = np.ascontiguousarray(v, np.float32)
            self.keep.append(v)
            g = self.arr[k]
            g.vertices = v.ctypes.data
            g.vertex_stride = 12
            g.max_vertex = max(0, v.shape[0] - 1)
            if i is not None:
                i = np.ascontiguousarray(i, np.uint32)
                self.keep.append(i)
                g.index_type = 1
                g.indices = i.ctypes.data
                g.tri_count = i.shape[0]
            else:
                g.index_type = 0
                g.indices = None
                g.tri_count = v.shape[0] // 3
            g.flags = 1
            if xf is not None:
                xf = np.ascontiguousarray(xf, np.float32).reshape(3, 4)
                self.keep.append(xf)
                g.transform = xf.ctypes.data
            else:
                g.transform = None

    def counts(self):
        return [self.arr[k].tri_count for k in range(self.n)]


def build_blas(items, flags: int = 0, debug: bool = False):
    """Oracle BLAS build.  Returns the accel bytes (numpy uint8, 256-byte
    aligned storage) and, with debug, (keys_sorted, ids_sorted, bin_nodes)."""
    lib = load()
    hg = HostGeoms(items)
    counts = (C.c_uint32 * max(1, hg.n))(*hg.counts())
    nbytes = lib.orc_blas_accel_bytes(counts, hg.n)
    buf = _aligned_zeros(nbytes)
    n = sum(hg.counts())
    dbg = None
    arrays = None
    if debug:
        ks = np.zeros(n, np.uint64)
        ids = np.zeros(n, np.uint32)
        bn = np.zeros(max(0, n - 1) * 4, np.uint32)
        arrays = (ks, ids, bn.reshape(-1, 4))
        dbg = LbvhDebug(None, ks.ctypes.data, ids.ctypes.data, bn.ctypes.data if n > 1 else None)
    rc = lib.orc_build_blas(hg.arr, hg.n, flags, buf.ctypes.data, nbytes, C.byref(dbg) if dbg else None)
    return (buf, rc, arrays) if debug else (buf, rc)


def build_tlas(instances: np.ndarray, flags: int = 0):
    """instances: INSTANCE_DTYPE array whose accel_ref are host addresses of
    oracle BLAS buffers (buffer.ctypes.data)."""
    lib = load()
    instances = np.ascontiguousarray(instances, INSTANCE_DTYPE)
    nbytes = lib.orc_tlas_accel_bytes(len(instances))
    buf = _aligned_zeros(nbytes)
    rc = lib.orc_build_tlas(instances.ctypes.data, len(instances), flags, buf.ctypes.data, nbytes)
    return buf, rc


def refit_blas(accel: np.ndarray, items) -> int:
    """rt_refit_blas on the CPU, in place on an oracle BLAS buffer."""
    hg = HostGeoms(items)
    return load().orc_refit_blas(hg.arr, hg.n, accel.ctypes.data)


def refit_tlas(accel: np.ndarray, instances: np.ndarray) -> int:
    instances = np.ascontiguousarray(instances, INSTANCE_DTYPE)
    return load().orc_refit_tlas(instances.ctypes.data, len(instances), accel.ctypes.data)


def _aligned_zeros(nbytes: int) -> np.ndarray:
    raw = np.zeros(int(nbytes) + 256, np.uint8)
    off = (-raw.ctypes.data) % 256
    return raw[off:off + int(nbytes)]


def trace_closest(accel: np.ndarray, rays: np.ndarray, threads: int = 0, ext: bool = False):
    lib = load()
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits = np.zeros(len(rays), HIT_DTYPE)
    hx = np.zeros(len(rays), HIT_EXT_DTYPE) if ext else None
    stats = np.zeros(2, np.uint64)
    lib.orc_trace_closest(accel.ctypes.data, rays.ctypes.data, hits.ctypes.data,
                          hx.ctypes.data if ext else None, len(rays), threads, stats.ctypes.data)
    return (hits, stats, hx) if ext else (hits, stats)


def trace_any(accel: np.ndarray, rays: np.ndarray, threads: int = 0):
    lib = load()
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    occ = np.zeros(len(rays), np.uint8)
    stats = np.zeros(2, np.uint64)
    lib.orc_trace_any(accel.ctypes.data, rays.ctypes.data, occ.ctypes.data, len(rays), threads, stats.ctypes.data)
    return occ, stats


def brute_closest(items, rays: np.ndarray, precision: int = 32, threads: int = 0):
    lib = load()
    hg = HostGeoms(items)
    rays = np.ascontiguousarray(rays, RAY_DTYPE)
    hits = np.zeros(len(rays), HIT_DTYPE)
    lib.orc_brute_closest(hg.arr, hg.n, rays.ctypes.data, hits.ctypes.data, len(rays), precision, threads)
    return hits


class _Pipeline(C.Structure):
    _fields_ = [("chit", C.c_uint32), ("ray_flags", C.c_uint32), ("cull_mask", C.c_uint32),
                ("sbt_record_offset", C.c_uint32), ("sbt_record_stride", C.c_uint32),
                ("miss_index", C.c_uint32), ("tmin", C.c_float), ("tmax", C.c_float),
                ("miss_color", C.c_float * 3), ("max_recursion", C.c_uint32)]


class _Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("y_fov_degree", C.c_float)]


def trace_rays(accel: np.ndarray, camera, width: int, height: int, chit: int = 0, sbt_colors=None,
               ray_flags: int = 1, tmin: float = 0.0, tmax: float = 100.0, miss=(0.0, 0.0, 0.2),
               cull_mask: int = 0xFF, sbt_offset: int = 0, sbt_stride: int = 1, threads: int = 0):
    """The sample's vkCmdTraceRaysKHR on the CPU; returns (image float32
    [H, W, 4], status)."""
    lib = load()
    p = _Pipeline(chit, ray_flags, cull_mask, sbt_offset, sbt_stride, 0, tmin, tmax,
                  (C.c_float * 3)(*miss), 1)
    cam = _Camera((C.c_float * 3)(*camera[0]), camera[1])
    img = np.zeros((height, width, 4), np.float32)
    cols = np.ascontiguousarray(sbt_colors if sbt_colors is not None else np.zeros((0, 3)), np.float32)
    rc = lib.orc_trace_rays(C.byref(p), cols.ctypes.data if cols.size else None, cols.shape[0], 3,
                            accel.ctypes.data, C.byref(cam), img.ctypes.data, width, height, threads)
    return img, rc


def raygen(camera, width: int, height: int, x: int, y: int):
    lib = load()
    cam = _Camera((C.c_float * 3)(*camera[0]), camera[1])
    o = np.zeros(3, np.float32)
    d = np.zeros(3, np.float32)
    lib.orc_raygen(C.byref(cam), width, height, x, y, o.ctypes.data, d.ctypes.data)
    return o, d


def primary_rays(camera, width: int, height: int, tmin: float = 0.0, tmax: float = 100.0) -> np.ndarray:
    """All pinhole rays of a launch, row-major: orc_raygen vectorised in
    numpy float32 (one rounding per operation, the same sequence)."""
    import math
    f32 = np.float32
    half = f32(f32(f32(camera[1]) * f32(math.pi / 180.0)) * f32(0.5))
    ay = f32(math.tan(float(half)))
    ax = f32(f32(ay * f32(width)) / f32(height))
    xs = np.arange(width, dtype=np.float32) + f32(0.5)
    ys = np.arange(height, dtype=np.float32) + f32(0.5)
    ndx = (xs / f32(width)) * f32(2.0) - f32(1.0)
    ndy = (ys / f32(height)) * f32(2.0) - f32(1.0)
    p = (ndx * ax)[None, :].repeat(height, 0)
    q = (ndy * ay)[:, None].repeat(width, 1)
    rays = np.zeros(width * height, RAY_DTYPE)
    d = np.empty((height, width, 3), np.float32)
    d[..., 0] = (p * f32(1.0) + q * f32(0.0)) + f32(0.0)
    d[..., 1] = (p * f32(0.0) + q * f32(-1.0)) + f32(0.0)
    d[..., 2] = (p * f32(0.0) + q * f32(0.0)) + f32(-1.0)
    rays["dir"] = d.reshape(-1, 3)
    rays["org"] = np.asarray(camera[0], np.float32)
    rays["tmin"] = tmin
    rays["tmax"] = tmax
    return rays


def sort_pairs(keys: np.ndarray, vals: np.ndarray, bits: int):
    lib = load()
    k = np.ascontiguousarray(keys, np.uint64).copy()
    v = np.ascontiguousarray(vals, np.uint32).copy()
    lib.orc_sort_pairs(k.ctypes.data, v.ctypes.data, len(k), bits)
    return k, v


class _PtParams(C.Structure):
    _fields_ = [("camera", _Camera), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("sample_offset", C.c_uint32), ("max_depth", C.c_uint32), ("rr_depth", C.c_uint32),
                ("seed", C.c_uint64), ("ray_eps", C.c_float), ("flags", C.c_uint32)]


def path_trace(accel: np.ndarray, tri_material: np.ndarray, materials: np.ndarray, lights: np.ndarray, camera,
               width: int, height: int, spp: int, max_depth: int = 8, rr_depth: int = 3, seed: int = 0,
               eps: float = 1e-4, sample_offset: int = 0, accum: np.ndarray | None = None, threads: int = 0):
    """rt_path_trace on the CPU; returns the accumulation buffer
    (float32 [H, W, 4]: radiance sums, sample count)."""
    lib = load()
    if accum is None:
        accum = np.zeros((height, width, 4), np.float32)
    tm = np.ascontiguousarray(tri_material, np.uint32)
    mats = np.ascontiguousarray(materials)
    lts = np.ascontiguousarray(lights)
    p = _PtParams(_Camera((C.c_float * 3)(*camera[0]), camera[1]), width, height, spp, sample_offset, max_depth,
                  rr_depth, seed, eps, 0)
    rc = lib.orc_path_trace(accel.ctypes.data, tm.ctypes.data, mats.ctypes.data, len(mats),
                            lts.ctypes.data if len(lts) else None, len(lts), C.byref(p), accum.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"orc_path_trace returned {rc}")
    return accum


CACHE_INPUT_DTYPE = np.dtype([("pos", "<f4", 3), ("dir", "<f4", 3), ("normal", "<f4", 3), ("albedo", "<f4", 3)])
# orc_path_record (88 bytes)
PATH_RECORD_DTYPE = np.dtype([("kind", "<u4"), ("L", "<f4", 3), ("L_before", "<f4", 3), ("t1", "<f4", 3),
                              ("rec", CACHE_INPUT_DTYPE)])


def path_trace_pixels(accel: np.ndarray, tri_material: np.ndarray, materials: np.ndarray, lights: np.ndarray,
                      camera, width: int, height: int, pixels, spp: int = 1, max_depth: int = 8, rr_depth: int = 3,
                      seed: int = 0, eps: float = 1e-4, sample_offset: int = 0, train_stride: int = 0,
                      threads: int = 0) -> np.ndarray:
    """The paths of rt_path_trace (train_stride 0) or rt_path_trace_cached
    (its training stride) for the listed pixels only: PATH_RECORD_DTYPE
    [len(pixels), spp]."""
    lib = load()
    px = np.ascontiguousarray(pixels, np.uint32)
    out = np.zeros((len(px), spp), PATH_RECORD_DTYPE)
    tm = np.ascontiguousarray(tri_material, np.uint32)
    mats = np.ascontiguousarray(materials)
    lts = np.ascontiguousarray(lights)
    p = _PtParams(_Camera((C.c_float * 3)(*camera[0]), camera[1]), width, height, spp, sample_offset, max_depth,
                  rr_depth, seed, eps, 0)
    rc = lib.orc_path_trace_pixels(accel.ctypes.data, tm.ctypes.data, mats.ctypes.data, len(mats),
                                   lts.ctypes.data if len(lts) else None, len(lts), C.byref(p), train_stride,
                                   px.ctypes.data, len(px), out.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"orc_path_trace_pixels returned {rc}")
    return out


def scene_soup(seed: int, n_tris: int):
    """The triangle soup of rt_scene_soup, generated by the oracle:
    (vertices float32 [3n, 3], indices uint32 [n, 3])."""
    v = np.empty((3 * n_tris, 3), np.float32)
    i = np.empty((n_tris, 3), np.uint32)
    load().orc_scene_soup(seed, n_tris, v.ctypes.data, i.ctypes.data)
    return v, i


def incoherent_rays(seed: int, n: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), tmax: float = 1e30) -> np.ndarray:
    """The rays of rt_scene_incoherent_rays, generated by the oracle."""
    rays = np.empty(n, RAY_DTYPE)
    lo_a = np.asarray(lo, np.float32)
    hi_a = np.asarray(hi, np.float32)
    load().orc_scene_incoherent_rays(seed, n, lo_a.ctypes.data, hi_a.ctypes.data, tmax, rays.ctypes.data)
    return rays


def sincos_q(x: float):
    s, c = C.c_float(), C.c_float()
    load().orc_sincos_q(x, C.byref(s), C.byref(c))
    return s.value, c.value


def hw_threads() -> int:
    return int(load().orc_hw_threads())


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
