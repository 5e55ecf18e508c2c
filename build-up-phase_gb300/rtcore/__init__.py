"""Python binding of librtcore (the GB300 software ray-tracing core).

A thin ctypes mirror of include/rtcore.h: the same entry points, argument
meaning and status codes as the C ABI.  Device buffers are passed as raw
pointers; torch tensors are accepted for convenience (torch is only the
allocator and stream provider here).  There is no fallback: if the CUDA
library is missing or fails to load, every call raises.

The entry points mirror the Vulkan calls of the reference sample
(vulkan-raytraced-triangle/main.cpp): rt_get_*_build_sizes ->
vkGetAccelerationStructureBuildSizesKHR (:757, :893), rt_build_* ->
vkCmdBuildAccelerationStructuresKHR (:808, :932), rt_trace_rays ->
vkCmdTraceRaysKHR (:1349).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "lib" / "librtcore.so"

# ---------------------------------------------------------------------------
# status codes and flags (rtcore.h)
# ---------------------------------------------------------------------------
RT_OK = 0
RT_ERR_INVALID_ARG = -1
RT_ERR_OOM = -2
RT_ERR_CUDA = -3
RT_ERR_TIMEOUT = -4
RT_ERR_BOUNDS = -5
RT_ERR_UNSUPPORTED = -6
RT_ERR_NO_DEVICE = -7
RT_ERR_NOT_FOUND = -8
STATUS_NAMES = {0: "RT_OK", -1: "RT_ERR_INVALID_ARG", -2: "RT_ERR_OOM", -3: "RT_ERR_CUDA",
                -4: "RT_ERR_TIMEOUT", -5: "RT_ERR_BOUNDS", -6: "RT_ERR_UNSUPPORTED",
                -7: "RT_ERR_NO_DEVICE", -8: "RT_ERR_NOT_FOUND"}
RT_BUILD_WIDTH_MASK = 0xF << 16
RT_PT_OCTANT_BINNING = 1
RT_HOST_TRANSFER_AUTO = 0
RT_HOST_TRANSFER_STAGED = 1
RT_BATCH_GRAPH = 1
RT_BATCH_DISCARD = 2
RT_TUNE_FORCE = 1

RT_INDEX_NONE = 0
RT_INDEX_UINT32 = 1
RT_GEOMETRY_OPAQUE = 1
RT_BUILD_PREFER_FAST_TRACE = 1 << 0
RT_BUILD_MORTON30 = 1 << 8
RT_BUILD_MORTON63 = 1 << 9
RT_RAY_FLAG_OPAQUE = 1 << 0
RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT = 1 << 2
RT_RAY_FLAG_SKIP_CLOSEST_HIT = 1 << 3
RT_CHIT_SAMPLE = 0
RT_CHIT_BARYCENTRIC = 1
RT_CHIT_SBT_COLOR = 2
RT_NO_HIT = 0xFFFFFFFF
RT_STATIC_SCRATCH_MAX_TRIS = 131072
RT_GEOMETRY_INSTANCE_TRIANGLE_FACING_CULL_DISABLE = 1


class RtError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str = ""):
        self.code = code
        super().__init__(f"{where}: {STATUS_NAMES.get(code, code)}" + (f" ({msg})" if msg else ""))


# ---------------------------------------------------------------------------
# structs
# ---------------------------------------------------------------------------
class Transform3x4(C.Structure):
    _fields_ = [("m", (C.c_float * 4) * 3)]


class GeometryTriangles(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("vertex_stride", C.c_uint64), ("max_vertex", C.c_uint32),
                ("index_type", C.c_uint32), ("indices", C.c_void_p), ("tri_count", C.c_uint32),
                ("flags", C.c_uint32), ("transform", C.c_void_p)]


class Instance(C.Structure):
    _fields_ = [("transform", Transform3x4), ("custom_index_and_mask", C.c_uint32),
                ("sbt_offset_and_flags", C.c_uint32), ("accel_ref", C.c_uint64)]


class BuildSizes(C.Structure):
    _fields_ = [("accel_bytes", C.c_uint64), ("scratch_bytes", C.c_uint64)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("y_fov_degree", C.c_float)]


class Pipeline(C.Structure):
    _fields_ = [("chit", C.c_uint32), ("ray_flags", C.c_uint32), ("cull_mask", C.c_uint32),
                ("sbt_record_offset", C.c_uint32), ("sbt_record_stride", C.c_uint32),
                ("miss_index", C.c_uint32), ("tmin", C.c_float), ("tmax", C.c_float),
                ("miss_color", C.c_float * 3), ("max_recursion", C.c_uint32)]


class Sbt(C.Structure):
    _fields_ = [("hit_colors", C.c_void_p), ("hit_record_count", C.c_uint32),
                ("hit_record_stride", C.c_uint32)]


class TraceTuning(C.Structure):
    _fields_ = [("block_threads", C.c_uint32), ("blocks_per_sm", C.c_uint32),
                ("batch_rays", C.c_uint32), ("reserved", C.c_uint32)]


class PtLight(C.Structure):
    _fields_ = [("v0", C.c_float * 3), ("v1", C.c_float * 3), ("v2", C.c_float * 3), ("emission", C.c_float * 3)]


class PtScene(C.Structure):
    _fields_ = [("accel", C.c_uint64), ("tri_material", C.c_void_p), ("materials", C.c_void_p),
                ("n_materials", C.c_uint32), ("lights", C.c_void_p), ("n_lights", C.c_uint32)]


class PtParams(C.Structure):
    _fields_ = [("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32), ("spp", C.c_uint32),
                ("sample_offset", C.c_uint32), ("max_depth", C.c_uint32), ("rr_depth", C.c_uint32),
                ("seed", C.c_uint64), ("ray_eps", C.c_float), ("flags", C.c_uint32)]


class CacheConfig(C.Structure):
    _fields_ = [("scene_lo", C.c_float * 3), ("scene_hi", C.c_float * 3), ("lr", C.c_float), ("beta1", C.c_float),
                ("beta2", C.c_float), ("eps", C.c_float), ("seed", C.c_uint32), ("reserved", C.c_uint32)]


def cache_config(lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0), lr=1e-3, beta1=0.9, beta2=0.99, eps=1e-8,
                 seed=1) -> CacheConfig:
    return CacheConfig((C.c_float * 3)(*lo), (C.c_float * 3)(*hi), lr, beta1, beta2, eps, seed, 0)


class PtCacheParams(C.Structure):
    _fields_ = [("cache", C.c_void_p), ("train_paths", C.c_uint32), ("train_batch", C.c_uint32)]


class PtCacheLayout(C.Structure):
    """rt_debug_pt_cache_layout: byte offsets of the learned form's arrays."""
    _fields_ = [(f, C.c_uint64) for f in ("query_count", "query_in", "query_t1", "query_path", "query_out",
                                          "train_count", "train_in", "train_t1", "train_before", "train_path",
                                          "train_target")]


class BatchScene(C.Structure):
    _fields_ = [("scene", PtScene), ("camera", Camera), ("width", C.c_uint32), ("height", C.c_uint32),
                ("accum", C.c_void_p)]


class BatchParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("max_depth", C.c_uint32), ("rr_depth", C.c_uint32), ("flags", C.c_uint32),
                ("seed", C.c_uint64), ("ray_eps", C.c_float), ("reserved", C.c_uint32)]


class BatchTuning(C.Structure):
    _fields_ = [("trace_threads", C.c_uint32), ("trace_blocks_per_sm", C.c_uint32), ("stack_ring", C.c_uint32),
                ("refill", C.c_uint32), ("shade_threads", C.c_uint32), ("wave_paths", C.c_uint32),
                ("bvh_width", C.c_uint32), ("reserved", C.c_uint32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}


assert C.sizeof(BatchScene) == 80
assert C.sizeof(BatchParams) == 32
assert C.sizeof(BatchTuning) == 32
assert C.sizeof(PtLight) == 48
assert C.sizeof(GeometryTriangles) == 48
assert C.sizeof(Instance) == 64
assert C.sizeof(Camera) == 16

# Every symbol include/rtcore.h declares, with (restype, argtypes).
_vp, _u32, _u64, _i32, _f = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_float
PROTOTYPES = {
    "rt_context_create": (_i32, [_i32, C.POINTER(_vp)]),
    "rt_context_destroy": (_i32, [_vp]),
    "rt_last_error_string": (C.c_char_p, [_vp]),
    "rt_sync": (_i32, [_vp, _vp]),
    "rt_abi_version": (_u32, []),
    "rt_get_blas_build_sizes": (_i32, [_vp, C.POINTER(_u32), _u32, _u32, C.POINTER(BuildSizes)]),
    "rt_get_tlas_build_sizes": (_i32, [_vp, _u32, _u32, C.POINTER(BuildSizes)]),
    "rt_build_blas": (_i32, [_vp, _vp, C.POINTER(GeometryTriangles), _u32, _u32, _vp, _u64, _vp, _u64]),
    "rt_build_tlas": (_i32, [_vp, _vp, _vp, _u32, _u32, _vp, _u64, _vp, _u64]),
    "rt_build_blas_static_scratch": (_i32, [_vp, _vp, C.POINTER(GeometryTriangles), _u32, _u32, _vp, _u64]),
    "rt_get_refit_scratch_bytes": (_i32, [_u32, C.POINTER(_u64)]),
    "rt_refit_blas": (_i32, [_vp, _vp, C.POINTER(GeometryTriangles), _u32, _vp, _u64, _vp, _u64]),
    "rt_refit_tlas": (_i32, [_vp, _vp, _vp, _u32, _vp, _u64, _vp, _u64]),
    "rt_accel_address": (_u64, [_vp]),
    "rt_accel_info": (_i32, [_vp, _vp, _vp, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "rt_trace_rays": (_i32, [_vp, _vp, C.POINTER(Pipeline), C.POINTER(Sbt), _u64, C.POINTER(Camera), _vp,
                             _u32, _u32, _u32]),
    "rt_trace_closest": (_i32, [_vp, _vp, _u64, _vp, _vp, _vp, _u32]),
    "rt_trace_any": (_i32, [_vp, _vp, _u64, _vp, _vp, _u32]),
    "rt_generate_primary_rays": (_i32, [_vp, _vp, C.POINTER(Camera), _u32, _u32, _f, _f, _vp]),
    "rt_trace_host_scratch_bytes": (_i32, [_u32, _i32, C.POINTER(_u64)]),
    "rt_set_host_transfer": (_i32, [_vp, _u32]),
    "rt_trace_closest_host": (_i32, [_vp, _vp, _u64, _vp, _vp, _u32, _vp, _u64]),
    "rt_trace_any_host": (_i32, [_vp, _vp, _u64, _vp, _vp, _u32, _vp, _u64]),
    "rt_trace_stats": (_i32, [_vp, _vp, _u64, _vp, _u32, _i32, _vp]),
    "rt_set_trace_tuning": (_i32, [_vp, C.POINTER(TraceTuning)]),
    "rt_get_trace_tuning": (_i32, [_vp, C.POINTER(TraceTuning)]),
    "rt_write_ppm": (_i32, [_vp, _u32, _u32, C.c_char_p]),
    "rt_write_pfm": (_i32, [_vp, _u32, _u32, C.c_char_p]),
    # debug / utility entry points declared in include/rtcore_debug.h
    "rt_get_sort_scratch_bytes": (_i32, [_u32, _u32, C.POINTER(_u64)]),
    "rt_sort_pairs": (_i32, [_vp, _vp, _vp, _vp, _u32, _u32, _vp, _u64]),
    "rt_debug_blas_scratch_layout": (_i32, [_u32, _u32, C.POINTER(_u64), C.POINTER(_u64), C.POINTER(_u64)]),
    "rt_debug_set_sort_spin_limit": (_i32, [_vp, _u32]),
    "rt_debug_set_sort_withhold": (_i32, [_vp, _i32]),
    "rt_debug_host_in_place": (_i32, [_vp, _vp, _u64, C.POINTER(_i32)]),
    "rt_debug_read_sweep": (_i32, [_vp, _vp, _vp, _u64, _u32]),
    "rt_debug_pt_cache_layout": (_i32, [C.POINTER(PtParams), C.POINTER(PtCacheParams), _u32,
                                        C.POINTER(PtCacheLayout)]),
    # path tracer declared in include/rtcore_pt.h
    "rt_pt_scratch_bytes": (_i32, [C.POINTER(PtParams), C.POINTER(_u64)]),
    "rt_path_trace": (_i32, [_vp, _vp, C.POINTER(PtScene), C.POINTER(PtParams), _vp, _vp, _u64]),
    "rt_pt_ray_counts": (_i32, [_vp, _vp, C.POINTER(PtParams), _u32, _vp, C.POINTER(_u64), C.POINTER(_u64)]),
    "rt_pt_cached_scratch_bytes": (_i32, [C.POINTER(PtParams), C.POINTER(PtCacheParams), C.POINTER(_u64)]),
    "rt_path_trace_cached": (_i32, [_vp, _vp, C.POINTER(PtScene), C.POINTER(PtParams), C.POINTER(PtCacheParams), _vp,
                                    _vp, _u64]),
    # batched path tracing and its autotuner declared in include/rtcore_batch.h
    "rt_batch_default_tuning": (_i32, [C.POINTER(BatchTuning)]),
    "rt_batch_scratch_bytes": (_i32, [C.POINTER(BatchScene), _u32, C.POINTER(BatchParams), C.POINTER(BatchTuning),
                                      C.POINTER(_u64)]),
    "rt_batch_plan_create": (_i32, [_vp, C.POINTER(BatchScene), _u32, C.POINTER(BatchParams),
                                    C.POINTER(BatchTuning), _vp, _u64, _u32, C.POINTER(_vp)]),
    "rt_batch_launch": (_i32, [_vp, _vp, _u32]),
    "rt_batch_ray_counts": (_i32, [_vp, _vp, C.POINTER(_u64), C.POINTER(_u64)]),
    "rt_batch_plan_launches": (_i32, [_vp, C.POINTER(_u32)]),
    "rt_batch_plan_destroy": (_i32, [_vp]),
    "rt_batch_autotune": (_i32, [_vp, C.POINTER(BatchScene), _u32, C.POINTER(BatchParams), _vp, _u64, C.c_char_p,
                                 _u32, C.POINTER(BatchTuning), C.POINTER(_f)]),
    "rt_batch_tuning_key": (_i32, [_vp, C.POINTER(BatchScene), _u32, C.POINTER(BatchParams), C.c_char_p, _u32]),
    "rt_batch_tuning_cache_lookup": (_i32, [C.c_char_p, C.c_char_p, C.POINTER(BatchTuning), C.POINTER(_f)]),
    "rt_batch_tuning_cache_store": (_i32, [C.c_char_p, C.c_char_p, C.POINTER(BatchTuning), _f]),
    # MLP radiance cache declared in include/rtcore_cache.h
    "rt_cache_bytes": (_i32, [C.POINTER(_u64)]),
    "rt_cache_param_count": (_u32, []),
    "rt_cache_init": (_i32, [_vp, _vp, _vp, _vp]),
    "rt_cache_query": (_i32, [_vp, _vp, _vp, _vp, _vp, _u32]),
    "rt_cache_train": (_i32, [_vp, _vp, _vp, _vp, _vp, _u32, _u32, _vp]),
    "rt_cache_gradient": (_i32, [_vp, _vp, _vp, _vp, _vp, _u32, _vp]),
    "rt_cache_get_params": (_i32, [_vp, _vp, _vp, _vp]),
    "rt_cache_set_params": (_i32, [_vp, _vp, _vp, _vp]),
    "rt_cache_save": (_i32, [_vp, _vp, _vp, C.c_char_p]),
    "rt_cache_load": (_i32, [_vp, _vp, _vp, C.c_char_p]),
    # seeded scenes declared in include/rtcore_scene.h (host code)
    "rt_scene_soup": (_i32, [_u64, _u32, _vp, _vp]),
    "rt_scene_box_counts": (_i32, [_u32, _u32, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "rt_scene_box": (_i32, [_u64, _u32, _u32, _vp, _vp, _vp, _vp]),
    "rt_scene_incoherent_rays": (_i32, [_u64, _u32, _vp, _vp, _f, _vp]),
    "rt_obj_counts": (_i32, [C.c_char_p, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32)]),
    "rt_obj_load": (_i32, [C.c_char_p, _vp, _vp, _vp]),
}

_lib = None


def lib_path() -> Path:
    return LIB_PATH


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads librtcore.so (raises if it is missing: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RtError(RT_ERR_NO_DEVICE, "load", f"{p} is missing; build it with build-up-phase_gb300/build.py")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(x) -> int | None:
    """Device pointer of a torch tensor, an int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Context:
    """rt_context: owner of the device-side bookkeeping of the core."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.rt_context_create(device, C.byref(h))
        if rc != RT_OK:
            raise RtError(rc, "rt_context_create")
        self.h = h
        self.device = device

    def close(self) -> None:
        if self.h:
            self.lib.rt_context_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int, where: str) -> None:
        if rc != RT_OK:
            msg = self.lib.rt_last_error_string(self.h)
            raise RtError(rc, where, msg.decode() if msg else "")

    # ---- sizes / builds
    def blas_sizes(self, tri_counts, flags: int = 0) -> BuildSizes:
        arr = (C.c_uint32 * max(1, len(tri_counts)))(*tri_counts)
        out = BuildSizes()
        self.check(self.lib.rt_get_blas_build_sizes(self.h, arr, len(tri_counts), flags, C.byref(out)),
                   "rt_get_blas_build_sizes")
        return out

    def tlas_sizes(self, n: int, flags: int = 0) -> BuildSizes:
        out = BuildSizes()
        self.check(self.lib.rt_get_tlas_build_sizes(self.h, n, flags, C.byref(out)), "rt_get_tlas_build_sizes")
        return out

    def build_blas(self, geoms, flags, accel, accel_bytes, scratch, scratch_bytes, stream=None) -> None:
        arr = (GeometryTriangles * max(1, len(geoms)))(*geoms)
        self.check(self.lib.rt_build_blas(self.h, _stream_ptr(stream), arr, len(geoms), flags, _ptr(accel),
                                          accel_bytes, _ptr(scratch), scratch_bytes), "rt_build_blas")

    def build_blas_static_scratch(self, geoms, flags, accel, accel_bytes, stream=None) -> None:
        """rt_build_blas_static_scratch: the build without a caller scratch
        buffer (at most RT_STATIC_SCRATCH_MAX_TRIS triangles)."""
        arr = (GeometryTriangles * max(1, len(geoms)))(*geoms)
        self.check(self.lib.rt_build_blas_static_scratch(self.h, _stream_ptr(stream), arr, len(geoms), flags,
                                                         _ptr(accel), accel_bytes), "rt_build_blas_static_scratch")

    def build_tlas(self, instances, n, flags, accel, accel_bytes, scratch, scratch_bytes, stream=None) -> None:
        self.check(self.lib.rt_build_tlas(self.h, _stream_ptr(stream), _ptr(instances), n, flags, _ptr(accel),
                                          accel_bytes, _ptr(scratch), scratch_bytes), "rt_build_tlas")

    def set_host_transfer(self, mode: int) -> None:
        self.check(self.lib.rt_set_host_transfer(self.h, mode), "rt_set_host_transfer")

    def trace_host_scratch_bytes(self, n: int, any_hit: bool = False) -> int:
        out = C.c_uint64()
        self.check(self.lib.rt_trace_host_scratch_bytes(n, 1 if any_hit else 0, C.byref(out)),
                   "rt_trace_host_scratch_bytes")
        return out.value

    def trace_closest_host(self, accel_addr: int, rays, hits, n: int, scratch, scratch_bytes: int,
                           stream=None) -> None:
        """rays / hits: host buffers (torch CPU tensors or raw addresses);
        read and written in place by the traversal launch where the device
        reaches them (pinned memory; pageable memory on a Grace system), else
        staged through the scratch ring in chunks."""
        self.check(self.lib.rt_trace_closest_host(self.h, _stream_ptr(stream), accel_addr, _ptr(rays), _ptr(hits), n,
                                                  _ptr(scratch), scratch_bytes), "rt_trace_closest_host")

    def trace_any_host(self, accel_addr: int, rays, occluded, n: int, scratch, scratch_bytes: int,
                       stream=None) -> None:
        self.check(self.lib.rt_trace_any_host(self.h, _stream_ptr(stream), accel_addr, _ptr(rays), _ptr(occluded), n,
                                              _ptr(scratch), scratch_bytes), "rt_trace_any_host")

    def refit_blas(self, geoms, accel, accel_bytes, scratch, scratch_bytes, stream=None) -> None:
        arr = (GeometryTriangles * max(1, len(geoms)))(*geoms)
        self.check(self.lib.rt_refit_blas(self.h, _stream_ptr(stream), arr, len(geoms), _ptr(accel), accel_bytes,
                                          _ptr(scratch), scratch_bytes), "rt_refit_blas")

    def refit_tlas(self, instances, n, accel, accel_bytes, scratch, scratch_bytes, stream=None) -> None:
        self.check(self.lib.rt_refit_tlas(self.h, _stream_ptr(stream), _ptr(instances), n, _ptr(accel), accel_bytes,
                                          _ptr(scratch), scratch_bytes), "rt_refit_tlas")

    def accel_info(self, accel, stream=None):
        nc, pc, d = C.c_uint32(), C.c_uint32(), C.c_uint32()
        self.check(self.lib.rt_accel_info(self.h, _stream_ptr(stream), _ptr(accel), C.byref(nc), C.byref(pc),
                                          C.byref(d)), "rt_accel_info")
        return nc.value, pc.value, d.value

    def address(self, accel) -> int:
        return int(self.lib.rt_accel_address(_ptr(accel)))

    # ---- tracing
    def trace_closest(self, accel_addr: int, rays, hits, n: int, hits_ext=None, stream=None) -> None:
        self.check(self.lib.rt_trace_closest(self.h, _stream_ptr(stream), accel_addr, _ptr(rays), _ptr(hits),
                                             _ptr(hits_ext), n), "rt_trace_closest")

    def trace_any(self, accel_addr: int, rays, occluded, n: int, stream=None) -> None:
        self.check(self.lib.rt_trace_any(self.h, _stream_ptr(stream), accel_addr, _ptr(rays), _ptr(occluded), n),
                   "rt_trace_any")

    def trace_stats(self, accel_addr: int, rays, n: int, any_hit: bool, counters, stream=None) -> None:
        self.check(self.lib.rt_trace_stats(self.h, _stream_ptr(stream), accel_addr, _ptr(rays), n,
                                           1 if any_hit else 0, _ptr(counters)), "rt_trace_stats")

    def trace_rays(self, pipeline: Pipeline, sbt: Sbt | None, accel_addr: int, camera: Camera, out, width: int,
                   height: int, depth: int = 1, stream=None) -> None:
        self.check(self.lib.rt_trace_rays(self.h, _stream_ptr(stream), C.byref(pipeline),
                                          C.byref(sbt) if sbt is not None else None, accel_addr, C.byref(camera),
                                          _ptr(out), width, height, depth), "rt_trace_rays")

    def generate_primary_rays(self, camera: Camera, width: int, height: int, tmin: float, tmax: float, rays,
                              stream=None) -> None:
        self.check(self.lib.rt_generate_primary_rays(self.h, _stream_ptr(stream), C.byref(camera), width, height,
                                                     tmin, tmax, _ptr(rays)), "rt_generate_primary_rays")

    def sync(self, stream=None) -> None:
        self.check(self.lib.rt_sync(self.h, _stream_ptr(stream)), "rt_sync")

    def set_tuning(self, blocks_per_sm: int, batch_rays: int) -> None:
        t = TraceTuning(128, blocks_per_sm, batch_rays, 0)
        self.check(self.lib.rt_set_trace_tuning(self.h, C.byref(t)), "rt_set_trace_tuning")

    def get_tuning(self) -> TraceTuning:
        t = TraceTuning()
        self.check(self.lib.rt_get_trace_tuning(self.h, C.byref(t)), "rt_get_trace_tuning")
        return t

    # ---- path tracer
    def pt_scratch_bytes(self, params: PtParams) -> int:
        out = C.c_uint64()
        self.check(self.lib.rt_pt_scratch_bytes(C.byref(params), C.byref(out)), "rt_pt_scratch_bytes")
        return out.value

    def path_trace(self, scene: PtScene, params: PtParams, accum, scratch, scratch_bytes: int, stream=None) -> None:
        self.check(self.lib.rt_path_trace(self.h, _stream_ptr(stream), C.byref(scene), C.byref(params), _ptr(accum),
                                          _ptr(scratch), scratch_bytes), "rt_path_trace")

    def pt_cached_scratch_bytes(self, params: PtParams, cp: PtCacheParams) -> int:
        out = C.c_uint64()
        self.check(self.lib.rt_pt_cached_scratch_bytes(C.byref(params), C.byref(cp), C.byref(out)),
                   "rt_pt_cached_scratch_bytes")
        return out.value

    def path_trace_cached(self, scene: PtScene, params: PtParams, cp: PtCacheParams, accum, scratch,
                          scratch_bytes: int, stream=None) -> None:
        self.check(self.lib.rt_path_trace_cached(self.h, _stream_ptr(stream), C.byref(scene), C.byref(params),
                                                 C.byref(cp), _ptr(accum), _ptr(scratch), scratch_bytes),
                   "rt_path_trace_cached")

    def pt_ray_counts(self, params: PtParams, n_lights: int, scratch, stream=None):
        e, s = C.c_uint64(), C.c_uint64()
        self.check(self.lib.rt_pt_ray_counts(self.h, _stream_ptr(stream), C.byref(params), n_lights, _ptr(scratch),
                                             C.byref(e), C.byref(s)), "rt_pt_ray_counts")
        return e.value, s.value

    # ---- batched path tracing
    def batch_scratch_bytes(self, scenes, params: BatchParams, tuning: "BatchTuning | None" = None) -> int:
        arr = _scene_array(scenes)
        out = C.c_uint64()
        self.check(self.lib.rt_batch_scratch_bytes(arr, len(arr), C.byref(params),
                                                   C.byref(tuning) if tuning is not None else None, C.byref(out)),
                   "rt_batch_scratch_bytes")
        return out.value

    def batch_plan(self, scenes, params: BatchParams, scratch, scratch_bytes: int,
                   tuning: "BatchTuning | None" = None, graph: bool = True, discard: bool = False) -> "BatchPlan":
        arr = _scene_array(scenes)
        h = C.c_void_p()
        flags = (RT_BATCH_GRAPH if graph else 0) | (RT_BATCH_DISCARD if discard else 0)
        self.check(self.lib.rt_batch_plan_create(self.h, arr, len(arr), C.byref(params),
                                                 C.byref(tuning) if tuning is not None else None, _ptr(scratch),
                                                 scratch_bytes, flags, C.byref(h)), "rt_batch_plan_create")
        return BatchPlan(self, h)

    def batch_autotune(self, scenes, params: BatchParams, scratch, scratch_bytes: int, cache_path=None,
                       force: bool = False):
        """(BatchTuning, ms of one sample per pixel) chosen by the autotuner."""
        arr = _scene_array(scenes)
        t, ms = BatchTuning(), C.c_float()
        path = os.fsencode(str(cache_path)) if cache_path is not None else None
        self.check(self.lib.rt_batch_autotune(self.h, arr, len(arr), C.byref(params), _ptr(scratch), scratch_bytes,
                                              path, RT_TUNE_FORCE if force else 0, C.byref(t), C.byref(ms)),
                   "rt_batch_autotune")
        return t, ms.value

    def batch_tuning_key(self, scenes, params: BatchParams) -> str:
        arr = _scene_array(scenes)
        buf = C.create_string_buffer(160)
        self.check(self.lib.rt_batch_tuning_key(self.h, arr, len(arr), C.byref(params), buf, len(buf)),
                   "rt_batch_tuning_key")
        return buf.value.decode()

    # ---- MLP radiance cache
    def cache_bytes(self) -> int:
        out = C.c_uint64()
        self.check(self.lib.rt_cache_bytes(C.byref(out)), "rt_cache_bytes")
        return out.value

    def cache_init(self, cache, cfg: "CacheConfig", stream=None) -> None:
        self.check(self.lib.rt_cache_init(self.h, _stream_ptr(stream), _ptr(cache), C.byref(cfg)), "rt_cache_init")

    def cache_query(self, cache, inputs, out, n: int, stream=None) -> None:
        self.check(self.lib.rt_cache_query(self.h, _stream_ptr(stream), _ptr(cache), _ptr(inputs), _ptr(out), n),
                   "rt_cache_query")

    def cache_train(self, cache, inputs, targets, n: int, batch: int, loss_out=None, stream=None) -> None:
        self.check(self.lib.rt_cache_train(self.h, _stream_ptr(stream), _ptr(cache), _ptr(inputs), _ptr(targets), n,
                                           batch, _ptr(loss_out)), "rt_cache_train")

    def cache_gradient(self, cache, inputs, targets, n: int, grad_out, stream=None) -> None:
        self.check(self.lib.rt_cache_gradient(self.h, _stream_ptr(stream), _ptr(cache), _ptr(inputs), _ptr(targets),
                                              n, _ptr(grad_out)), "rt_cache_gradient")

    def cache_get_params(self, cache, params, stream=None) -> None:
        self.check(self.lib.rt_cache_get_params(self.h, _stream_ptr(stream), _ptr(cache), _ptr(params)),
                   "rt_cache_get_params")

    def cache_set_params(self, cache, params, stream=None) -> None:
        self.check(self.lib.rt_cache_set_params(self.h, _stream_ptr(stream), _ptr(cache), _ptr(params)),
                   "rt_cache_set_params")

    def cache_save(self, cache, path, stream=None) -> None:
        self.check(self.lib.rt_cache_save(self.h, _stream_ptr(stream), _ptr(cache), os.fsencode(str(path))),
                   "rt_cache_save")

    def cache_load(self, cache, path, stream=None) -> None:
        self.check(self.lib.rt_cache_load(self.h, _stream_ptr(stream), _ptr(cache), os.fsencode(str(path))),
                   "rt_cache_load")

    # ---- utilities
    def sort_pairs(self, keys, vals, n: int, key_bits: int, scratch, scratch_bytes: int, stream=None) -> None:
        self.check(self.lib.rt_sort_pairs(self.h, _stream_ptr(stream), _ptr(keys), _ptr(vals), n, key_bits,
                                          _ptr(scratch), scratch_bytes), "rt_sort_pairs")

    def read_sweep(self, buf, nbytes: int, passes: int, stream=None) -> None:
        """rt_debug_read_sweep: the bandwidth probe (reads buf `passes` times)."""
        self.check(self.lib.rt_debug_read_sweep(self.h, _stream_ptr(stream), _ptr(buf), nbytes, passes),
                   "rt_debug_read_sweep")

    def host_in_place(self, ptr: int, nbytes: int) -> bool:
        """rt_debug_host_in_place: would the host-memory ray API use
        [ptr, ptr + nbytes) in place?"""
        out = C.c_int()
        self.check(self.lib.rt_debug_host_in_place(self.h, ptr, nbytes, C.byref(out)), "rt_debug_host_in_place")
        return bool(out.value)

    def set_sort_spin_limit(self, spins: int) -> None:
        """rt_debug_set_sort_spin_limit (0 restores the default)."""
        self.check(self.lib.rt_debug_set_sort_spin_limit(self.h, spins), "rt_debug_set_sort_spin_limit")

    def set_sort_withhold(self, withhold: bool) -> None:
        """rt_debug_set_sort_withhold: the first tile of each pass publishes no status."""
        self.check(self.lib.rt_debug_set_sort_withhold(self.h, 1 if withhold else 0), "rt_debug_set_sort_withhold")

    @staticmethod
    def pt_cache_layout(params: PtParams, cp: PtCacheParams, n_lights: int) -> PtCacheLayout:
        """rt_debug_pt_cache_layout: where the last wave's learned-form arrays
        lie in the scratch of rt_path_trace_cached."""
        out = PtCacheLayout()
        rc = load().rt_debug_pt_cache_layout(C.byref(params), C.byref(cp), n_lights, C.byref(out))
        if rc != RT_OK:
            raise RtError(rc, "rt_debug_pt_cache_layout")
        return out


def _scene_array(scenes):
    if isinstance(scenes, C.Array):
        return scenes
    scenes = list(scenes)
    return (BatchScene * len(scenes))(*scenes)


class BatchPlan:
    """rt_batch_plan: one recorded launch of a batch of scenes."""

    def __init__(self, ctx: Context, h: C.c_void_p):
        self.ctx, self.h = ctx, h

    def launch(self, sample_offset: int, stream=None) -> None:
        self.ctx.check(self.ctx.lib.rt_batch_launch(self.h, _stream_ptr(stream), sample_offset), "rt_batch_launch")

    def ray_counts(self, stream=None):
        e, s = C.c_uint64(), C.c_uint64()
        self.ctx.check(self.ctx.lib.rt_batch_ray_counts(self.h, _stream_ptr(stream), C.byref(e), C.byref(s)),
                       "rt_batch_ray_counts")
        return e.value, s.value

    def launches(self) -> int:
        k = C.c_uint32()
        self.ctx.check(self.ctx.lib.rt_batch_plan_launches(self.h, C.byref(k)), "rt_batch_plan_launches")
        return k.value

    def close(self) -> None:
        if self.h:
            self.ctx.lib.rt_batch_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_batch_tuning() -> BatchTuning:
    t = BatchTuning()
    load().rt_batch_default_tuning(C.byref(t))
    return t


def tuning_cache_lookup(path, key: str):
    """(BatchTuning, ms) for key, or None when the file or key is absent."""
    t, ms = BatchTuning(), C.c_float()
    rc = load().rt_batch_tuning_cache_lookup(os.fsencode(str(path)), key.encode(), C.byref(t), C.byref(ms))
    if rc == RT_ERR_NOT_FOUND:
        return None
    if rc != RT_OK:
        raise RtError(rc, "rt_batch_tuning_cache_lookup")
    return t, ms.value


def tuning_cache_store(path, key: str, t: BatchTuning, ms: float) -> None:
    rc = load().rt_batch_tuning_cache_store(os.fsencode(str(path)), key.encode(), C.byref(t), ms)
    if rc != RT_OK:
        raise RtError(rc, "rt_batch_tuning_cache_store")


def build_width(w: int) -> int:
    """RT_BUILD_WIDTH(w): build flag for at most w children per wide node (4..8)."""
    return (w & 0xF) << 16


def refit_scratch_bytes(prim_count: int) -> int:
    out = C.c_uint64()
    rc = load().rt_get_refit_scratch_bytes(prim_count, C.byref(out))
    if rc != RT_OK:
        raise RtError(rc, "rt_get_refit_scratch_bytes")
    return out.value


def sort_scratch_bytes(n: int, key_bits: int) -> int:
    out = C.c_uint64()
    rc = load().rt_get_sort_scratch_bytes(n, key_bits, C.byref(out))
    if rc != RT_OK:
        raise RtError(rc, "rt_get_sort_scratch_bytes")
    return out.value


def blas_scratch_layout(n_tris: int, flags: int = 0):
    k, i, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
    load().rt_debug_blas_scratch_layout(n_tris, flags, C.byref(k), C.byref(i), C.byref(b))
    return k.value, i.value, b.value


def pack_custom_mask(custom_index: int, mask: int) -> int:
    return (custom_index & 0xFFFFFF) | ((mask & 0xFF) << 24)


def pack_sbt_flags(sbt_offset: int, flags: int) -> int:
    return (sbt_offset & 0xFFFFFF) | ((flags & 0xFF) << 24)


def sample_pipeline(chit: int = RT_CHIT_SAMPLE) -> Pipeline:
    """The constant arguments of the sample's raygen traceRayEXT call
    (main.cpp:1047-1052) and its miss colour (main.cpp:1065)."""
    p = Pipeline()
    p.chit = chit
    p.ray_flags = RT_RAY_FLAG_OPAQUE
    p.cull_mask = 0xFF
    p.sbt_record_offset = 0
    p.sbt_record_stride = 1
    p.miss_index = 0
    p.tmin = 0.0
    p.tmax = 100.0
    p.miss_color[:] = [0.0, 0.0, 0.2]
    p.max_recursion = 1
    return p
