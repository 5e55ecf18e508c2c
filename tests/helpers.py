"""Helpers shared by the tests: numpy <-> device buffers and the two builds
(CUDA path through the C ABI, CPU oracle) of the same inputs."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"

HEADER_DTYPE = np.dtype([
    ("magic", "<u4"), ("version", "<u4"), ("kind", "<u4"), ("prim_count", "<u4"), ("node_count", "<u4"),
    ("geom_count", "<u4"), ("build_flags", "<u4"), ("status", "<u4"), ("depth", "<u4"), ("morton_bits", "<u4"),
    ("node_capacity", "<u4"), ("reserved0", "<u4"), ("bounds_lo", "<f4", 4), ("bounds_hi", "<f4", 4),
    ("node_offset", "<u8"), ("prim_offset", "<u8"), ("geom_offset", "<u8"), ("total_bytes", "<u8"),
    ("reserved", "u1", 144)])
assert HEADER_DTYPE.itemsize == 256

NODE_DTYPE = np.dtype([("origin", "<f4", 3), ("exp", "i1", 3), ("imask", "u1"), ("child_base", "<u4"),
                       ("prim_base", "<u4"), ("meta", "u1", 8), ("qlo", "u1", (3, 8)), ("qhi", "u1", (3, 8))])
assert NODE_DTYPE.itemsize == 80


def golden() -> dict:
    return json.loads((GOLDEN / "sample_pixels.json").read_text())


def header(buf: np.ndarray) -> np.void:
    return buf[:256].view(HEADER_DTYPE)[0]


def nodes(buf: np.ndarray) -> np.ndarray:
    h = header(buf)
    off = int(h["node_offset"])
    return buf[off:off + 80 * int(h["node_count"])].view(NODE_DTYPE)


def prims(buf: np.ndarray, rec_bytes: int) -> np.ndarray:
    h = header(buf)
    off = int(h["prim_offset"])
    return buf[off:off + rec_bytes * int(h["prim_count"])]


def compare_accels(gpu: np.ndarray, orc: np.ndarray, rec_bytes: int, ignore_ref: bool = False) -> None:
    """Asserts that two built structures are byte-identical in every field the
    build defines (the unused node capacity tail excepted)."""
    hg, ho = header(gpu), header(orc)
    for f in ("magic", "version", "kind", "prim_count", "node_count", "geom_count", "build_flags", "status",
              "depth", "morton_bits", "node_capacity", "node_offset", "prim_offset", "geom_offset", "total_bytes"):
        assert hg[f] == ho[f], f"header field {f}: gpu {hg[f]} oracle {ho[f]}"
    assert hg["bounds_lo"].tobytes() == ho["bounds_lo"].tobytes(), "bounds_lo"
    assert hg["bounds_hi"].tobytes() == ho["bounds_hi"].tobytes(), "bounds_hi"
    ng, no = nodes(gpu), nodes(orc)
    if ng.tobytes() != no.tobytes():
        bad = np.nonzero(ng.view(np.uint8).reshape(-1, 80) != no.view(np.uint8).reshape(-1, 80))
        k = int(bad[0][0])
        raise AssertionError(f"node {k} differs (first of {len(set(bad[0].tolist()))}):\n gpu {ng[k]}\n orc {no[k]}")
    pg, po = prims(gpu, rec_bytes), prims(orc, rec_bytes)
    if ignore_ref:  # instance records: bytes 48..55 hold device vs host BLAS addresses
        pg = pg.reshape(-1, rec_bytes).copy()
        po = po.reshape(-1, rec_bytes).copy()
        pg[:, 48:56] = 0
        po[:, 48:56] = 0
    if pg.tobytes() != po.tobytes():
        a, b = pg.reshape(-1, rec_bytes), po.reshape(-1, rec_bytes)
        k = int(np.nonzero((a != b).any(1))[0][0])
        raise AssertionError(f"leaf record {k} differs:\n gpu {a[k].view(np.float32)}\n orc {b[k].view(np.float32)}")
    if int(hg["kind"]) == 1:
        off = int(hg["geom_offset"])
        n = int(hg["geom_count"]) + 1
        assert gpu[off:off + 4 * n].tobytes() == orc[off:off + 4 * n].tobytes(), "geometry table"


# ---------------------------------------------------------------------------
# GPU side (torch only as allocator)
# ---------------------------------------------------------------------------

def dev(a: np.ndarray):
    import torch
    t = torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).reshape(-1).copy())
    return t.cuda()


def host(t, dtype=np.uint8) -> np.ndarray:
    return t.cpu().numpy().view(dtype)


class GpuBlas:
    """A BLAS built through rt_get_blas_build_sizes + rt_build_blas."""

    def __init__(self, ctx, items, flags: int = 0, stream=None):
        import torch
        self.keep = []
        geoms = self._geoms(items, self.keep)
        self.sizes = ctx.blas_sizes([g.tri_count for g in geoms], flags)
        self.accel = torch.empty(self.sizes.accel_bytes, dtype=torch.uint8, device="cuda")
        self.scratch = torch.empty(self.sizes.scratch_bytes, dtype=torch.uint8, device="cuda")
        ctx.build_blas(geoms, flags, self.accel, self.sizes.accel_bytes, self.scratch, self.sizes.scratch_bytes,
                       stream)
        ctx.sync(stream)
        self.addr = ctx.address(self.accel)

    def refit(self, ctx, items, stream=None) -> None:
        """rt_refit_blas with new (vertices, indices, transform) items."""
        import rtcore
        import torch
        keep = []
        geoms = self._geoms(items, keep)
        n = sum(g.tri_count for g in geoms)
        nb = rtcore.refit_scratch_bytes(n)
        scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
        ctx.refit_blas(geoms, self.accel, self.sizes.accel_bytes, scratch, nb, stream)
        ctx.sync(stream)

    @staticmethod
    def _geoms(items, keep):
        import rtcore
        geoms = []
        for v, i, xf in items:
            g = rtcore.GeometryTriangles()
            dv = dev(np.ascontiguousarray(v, np.float32))
            keep.append(dv)
            g.vertices = dv.data_ptr()
            g.vertex_stride = 12
            g.max_vertex = max(0, len(v) - 1)
            if i is not None:
                di = dev(np.ascontiguousarray(i, np.uint32))
                keep.append(di)
                g.index_type = rtcore.RT_INDEX_UINT32
                g.indices = di.data_ptr()
                g.tri_count = len(i)
            else:
                g.index_type = rtcore.RT_INDEX_NONE
                g.tri_count = len(v) // 3
            g.flags = rtcore.RT_GEOMETRY_OPAQUE
            if xf is not None:
                dx = dev(np.ascontiguousarray(xf, np.float32))
                keep.append(dx)
                g.transform = dx.data_ptr()
            geoms.append(g)
        return geoms

    def bytes(self) -> np.ndarray:
        return host(self.accel)


class GpuTlas:
    def __init__(self, ctx, instances: np.ndarray, flags: int = 0):
        import torch
        self.inst = dev(instances)
        self.sizes = ctx.tlas_sizes(len(instances), flags)
        self.accel = torch.empty(self.sizes.accel_bytes, dtype=torch.uint8, device="cuda")
        self.scratch = torch.empty(self.sizes.scratch_bytes, dtype=torch.uint8, device="cuda")
        ctx.build_tlas(self.inst, len(instances), flags, self.accel, self.sizes.accel_bytes, self.scratch,
                       self.sizes.scratch_bytes)
        ctx.sync()
        self.addr = ctx.address(self.accel)

    def refit(self, ctx, instances: np.ndarray) -> None:
        import rtcore
        import torch
        di = dev(instances)
        nb = rtcore.refit_scratch_bytes(len(instances))
        scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
        ctx.refit_tlas(di, len(instances), self.accel, self.sizes.accel_bytes, scratch, nb)
        ctx.sync()

    def bytes(self) -> np.ndarray:
        return host(self.accel)


def gpu_trace_closest(ctx, addr: int, rays: np.ndarray, ext: bool = False):
    import torch
    from oracle import HIT_DTYPE, HIT_EXT_DTYPE
    n = len(rays)
    dr = dev(rays)
    hits = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    hx = torch.empty(max(1, n) * 32, dtype=torch.uint8, device="cuda") if ext else None
    ctx.trace_closest(addr, dr, hits, n, hits_ext=hx)
    ctx.sync()
    h = host(hits).view(HIT_DTYPE)
    return (h, host(hx)[:n * 32].view(HIT_EXT_DTYPE)) if ext else h


def gpu_trace_any(ctx, addr: int, rays: np.ndarray):
    import torch
    n = len(rays)
    dr = dev(rays)
    occ = torch.empty(max(1, n), dtype=torch.uint8, device="cuda")
    ctx.trace_any(addr, dr, occ, n)
    ctx.sync()
    return host(occ)[:n]


def gpu_trace_stats(ctx, addr: int, rays: np.ndarray, any_hit: bool = False):
    import torch
    dr = dev(rays)
    c = torch.zeros(2, dtype=torch.int64, device="cuda")
    ctx.trace_stats(addr, dr, len(rays), any_hit, c)
    ctx.sync()
    return c.cpu().numpy().astype(np.uint64)


def ref8_items():
    import rtcore.scenes as S
    return [(S.REF8_VERTICES, S.REF8_INDICES, S.REF8_GEOM_TRANSFORMS[g]) for g in range(2)]


def ref8_instances(blas_refs) -> np.ndarray:
    """blas_refs: one address per instance (device or host)."""
    import rtcore.scenes as S
    from oracle import INSTANCE_DTYPE
    inst = np.zeros(2, INSTANCE_DTYPE)
    for k in range(2):
        inst[k]["transform"] = S.REF8_INSTANCE_TRANSFORMS[k]
        inst[k]["custom_index_and_mask"] = S.REF8_CUSTOM_INDEX | (0xFF << 24)
        inst[k]["sbt_offset_and_flags"] = S.REF8_SBT_OFFSETS[k] | (1 << 24)
        inst[k]["accel_ref"] = blas_refs[k]
    return inst


def single_instance(blas_ref: int) -> np.ndarray:
    from oracle import INSTANCE_DTYPE
    inst = np.zeros(1, INSTANCE_DTYPE)
    inst[0]["transform"] = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], np.float32)
    inst[0]["custom_index_and_mask"] = 0xFF << 24
    inst[0]["sbt_offset_and_flags"] = 1 << 24
    inst[0]["accel_ref"] = blas_ref
    return inst


def ptr_of(a: np.ndarray) -> int:
    return a.ctypes.data_as(C.c_void_p).value


def radix_tree_canonical(bn):
    """The radix tree of a (left, right, first, last) node array without its
    numbering: per internal node its key range and each child's range (leaf
    flag, first, last), sorted by range."""
    bn = bn.astype(np.int64)
    first, last = bn[:, 2], bn[:, 3]

    def child(x):
        leaf = (x & 0x80000000) != 0
        idx = x & 0x7FFFFFFF
        inner = np.where(leaf, 0, idx)
        return np.stack([leaf.astype(np.int64), np.where(leaf, idx, first[inner]), np.where(leaf, idx, last[inner])], 1)

    rows = np.concatenate([bn[:, 2:4], child(bn[:, 0]), child(bn[:, 1])], 1)
    return rows[np.lexsort((rows[:, 1], rows[:, 0]))]
