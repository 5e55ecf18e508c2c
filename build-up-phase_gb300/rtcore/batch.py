"""The batched form: many seeded scenes of uneven triangle count and
resolution, traced by one CUDA-graph launch of rt_batch_launch against one
rt_path_trace launch per scene.

    python -m rtcore.batch [--scenes 64] [--min-tris 10000] [--max-tris 5000000]
                           [--spp 16] [--depth 8] [--tune-cache FILE] [--retune]
                           [--widths 4,6,8] [--repeat 2] [--out result.json]

Scenes (seed 0x5EED0004): each is a lit triangle soup or a box scene with
probability 1/2, triangle count exp(U(ln min, ln max)), square resolution
drawn from {512, 1024, 1536, 2048}, its own jittered camera.  Both forms trace
the same samples (the batch adds to each scene's image exactly what
rt_path_trace adds), so their times compare equal work; the batch's launch
shapes come from the autotuner (rt_batch_autotune) and its JSON cache.  With
--retune and more than one --widths value, the BVH width is tuned too: every
scene is rebuilt with RT_BUILD_WIDTH(w) for each w and one-sample graph
launches of the tuned shape are timed; the fastest width is stored with the
launch shapes.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import math
import os
import time
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from . import (BatchParams, BatchScene, Camera, Context, GeometryTriangles, PtParams, PtScene, build_width,
               default_batch_tuning, load, tuning_cache_lookup, tuning_cache_store)
from . import scenes as S

BATCH_SEED = S.SEED_BASE + 4
RESOLUTIONS = (512, 1024, 1536, 2048)
DEFAULT_CACHE = Path(__file__).resolve().parent / "tuning" / "batch_gb300.json"

# Lit soup: the soup of [0,1]^3 above a floor, under a ceiling light.
SOUP_FLOOR = (-0.05, (-1.0, 2.0))          # y, x/z extent
SOUP_LIGHT = (1.25, (0.25, 0.75), 10.0)    # y, x/z extent, radiance
SOUP_ALBEDO = (0.7, 0.7, 0.7)
SOUP_FLOOR_ALBEDO = (0.5, 0.5, 0.5)


def lit_soup(seed: int, n_tris: int):
    """(vertices, indices, tri_material, materials) of the soup plus a floor
    quad and a downward-facing light quad (2 triangles each)."""
    v, i = S.soup(seed, n_tris)
    fy, (f0, f1) = SOUP_FLOOR
    ly, (l0, l1), le = SOUP_LIGHT
    # floor faces +y: (v1 - v0) x (v2 - v0) = (0, +, 0) with v1 along +z, v2 along +x
    quad_v = np.array([[f0, fy, f0], [f0, fy, f1], [f1, fy, f0], [f1, fy, f1],
                       # light faces -y: v1 along +x, v2 along +z
                       [l0, ly, l0], [l1, ly, l0], [l0, ly, l1], [l1, ly, l1]], np.float32)
    base = len(v)
    quad_i = np.array([[0, 1, 2], [2, 1, 3], [4, 5, 6], [6, 5, 7]], np.uint32) + np.uint32(base)
    v = np.concatenate([v, quad_v])
    i = np.concatenate([i, quad_i])
    tm = np.zeros(len(i), np.uint32)
    tm[-4:-2] = 1
    tm[-2:] = 2
    m = np.zeros(3, S.MATERIAL_DTYPE)
    m["albedo"][0] = SOUP_ALBEDO
    m["albedo"][1] = SOUP_FLOOR_ALBEDO
    m["emission"][2] = (le, le, le)
    return v, i, tm, m


def box_shape(n_tris: int):
    """(spheres, frequency) of a box scene with about n_tris triangles."""
    spheres = int(min(max(n_tris // 25000, 1), 200))
    freq = max(1, int(round(math.sqrt(max(n_tris - 14, 20) / (20.0 * spheres)))))
    return spheres, freq


@dataclass
class SceneSpec:
    kind: str          # "soup" or "box"
    tris: int          # requested triangle count
    width: int
    height: int
    camera: tuple      # ((x, y, z), y_fov_degree)
    seed: int


def batch_specs(n: int = 64, min_tris: int = 10_000, max_tris: int = 5_000_000, seed: int = BATCH_SEED,
                resolutions=RESOLUTIONS) -> list[SceneSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for s in range(n):
        kind = "box" if rng.random() < 0.5 else "soup"
        tris = int(round(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))))
        res = int(resolutions[int(rng.integers(len(resolutions)))])
        j = rng.uniform(-1.0, 1.0, 3)
        fov = float(rng.uniform(50.0, 70.0))
        if kind == "box":
            cam = ((float(0.2 * j[0]), float(0.2 * j[1]), 0.95), fov)
        else:
            cam = ((float(0.5 + 0.1 * j[0]), float(0.5 + 0.1 * j[1]), float(2.2 + 0.3 * j[2])), fov - 15.0)
        out.append(SceneSpec(kind, tris, res, res, cam, seed * 1000 + s))
    return out


def host_scene(spec: SceneSpec):
    if spec.kind == "soup":
        return lit_soup(spec.seed, spec.tris)
    return S.box(spec.seed, *box_shape(spec.tris))


class GpuScene:
    """One scene on the device: bottom-level structure, materials, lights and
    its accumulation image."""

    def __init__(self, ctx: Context, spec: SceneSpec, host, scratch=None, width: int = 8):
        import torch
        v, i, tm, m = host
        self.spec = spec
        self.n_tris = len(i)
        lights = S.emissive_lights(v, i, tm, m)
        self.n_lights = len(lights)
        # the geometry stays on the device for rebuilds with another width
        self.dv = torch.from_numpy(np.ascontiguousarray(v).reshape(-1)).cuda()
        self.di = torch.from_numpy(np.ascontiguousarray(i).reshape(-1).view(np.int32)).cuda()
        self.n_vertices = len(v)
        self.keep = [torch.from_numpy(tm.view(np.int32)).cuda(), torch.from_numpy(m.view(np.uint8)).cuda(),
                     torch.from_numpy(lights.view(np.uint8)).cuda()]
        sz = ctx.blas_sizes([len(i)])
        self.accel = torch.empty(sz.accel_bytes, dtype=torch.uint8, device="cuda")
        self.scratch = self.build(ctx, width, scratch)  # reusable by the next build
        self.accum = torch.zeros(spec.width * spec.height * 4, dtype=torch.float32, device="cuda")
        self.pt = PtScene(ctx.address(self.accel), self.keep[0].data_ptr(), self.keep[1].data_ptr(), len(m),
                          self.keep[2].data_ptr(), len(lights))

    def build(self, ctx: Context, width: int = 8, scratch=None):
        """(Re)builds the structure with at most `width` children per node;
        returns the scratch buffer used (for reuse)."""
        import torch
        g = GeometryTriangles()
        g.vertices, g.vertex_stride, g.max_vertex = self.dv.data_ptr(), 12, self.n_vertices - 1
        g.index_type, g.indices, g.tri_count, g.flags = 1, self.di.data_ptr(), self.n_tris, 1
        sz = ctx.blas_sizes([self.n_tris])
        if scratch is None or scratch.numel() < sz.scratch_bytes:
            scratch = torch.empty(sz.scratch_bytes, dtype=torch.uint8, device="cuda")
        ctx.build_blas([g], build_width(width) if width != 8 else 0, self.accel, sz.accel_bytes, scratch,
                       sz.scratch_bytes)
        ctx.sync()
        self.bvh_width = width
        return scratch

    def camera(self) -> Camera:
        return Camera(self.spec.camera[0], self.spec.camera[1])

    def batch_scene(self) -> BatchScene:
        return BatchScene(self.pt, self.camera(), self.spec.width, self.spec.height, self.accum.data_ptr())

    def pt_params(self, spp: int, offset: int, depth: int, seed: int, rr: int = 3, eps: float = 1e-4) -> PtParams:
        return PtParams(self.camera(), self.spec.width, self.spec.height, spp, offset, depth, rr, seed, eps, 0)


def build_scenes(ctx: Context, specs: list[SceneSpec], threads: int | None = None, width: int = 8) -> list[GpuScene]:
    """Generates the scenes on host threads (the generators release the GIL)
    and builds their structures on the device, in order."""
    threads = threads or min(16, os.cpu_count() or 4)
    out, scratch = [], None
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        for spec, host in zip(specs, ex.map(host_scene, specs)):
            sc = GpuScene(ctx, spec, host, scratch, width)
            scratch = sc.scratch
            sc.scratch = None
            out.append(sc)
    return out


def rebuild_scenes(ctx: Context, scenes: list[GpuScene], width: int) -> None:
    scratch = None
    for sc in scenes:
        if sc.bvh_width != width:
            scratch = sc.build(ctx, width, scratch)


def sweep_widths(ctx: Context, scenes: list[GpuScene], p: BatchParams, tuning, scratch, nb: int, widths,
                 stream) -> dict:
    """{width: ms of one sample per pixel} with the given launch shape, best of
    three graph launches after a warm-up (results discarded); the scenes are
    left built with the fastest width."""
    import torch
    one = BatchParams(1, p.max_depth, p.rr_depth, 0, p.seed, p.ray_eps, 0)
    times = {}
    for w in widths:
        rebuild_scenes(ctx, scenes, w)
        t = type(tuning).from_buffer_copy(tuning)
        t.bvh_width = w
        plan = ctx.batch_plan([sc.batch_scene() for sc in scenes], one, scratch, nb, t, graph=True, discard=True)
        plan.launch(0, stream)
        times[w] = min(time_ms(lambda: plan.launch(0, stream), stream) for _ in range(3))
        plan.close()
        torch.cuda.synchronize()
    rebuild_scenes(ctx, scenes, min(times, key=times.get))
    return times


def batch_params(spp: int, depth: int = 8, seed: int = BATCH_SEED, rr: int = 3, eps: float = 1e-4) -> BatchParams:
    return BatchParams(spp, depth, rr, 0, seed, eps, 0)


class Sequential:
    """One rt_path_trace per scene (the unbatched form)."""

    def __init__(self, ctx: Context, scenes: list[GpuScene], spp: int, depth: int, seed: int = BATCH_SEED):
        import torch
        self.ctx, self.scenes, self.spp, self.depth, self.seed = ctx, scenes, spp, depth, seed
        self.nb = max(ctx.pt_scratch_bytes(sc.pt_params(spp, 0, depth, seed)) for sc in scenes)
        self.scratch = torch.empty(self.nb, dtype=torch.uint8, device="cuda")

    def launch(self, offset: int, stream=None) -> None:
        for sc in self.scenes:
            self.ctx.path_trace(sc.pt, sc.pt_params(self.spp, offset, self.depth, self.seed), sc.accum, self.scratch,
                                self.nb, stream)


def _record_width_trials(path, key: str, width_ms: dict) -> None:
    """Adds the width sweep's times to the key's entry of the tuning cache."""
    p = Path(path)
    doc = json.loads(p.read_text())
    doc["entries"][key]["width_trials"] = [[f"bvh width {w}", round(ms, 3)] for w, ms in sorted(width_ms.items())]
    tmp = p.with_name(p.name + f".tmp.{os.getpid()}")
    tmp.write_text(json.dumps(doc, indent=2) + "\n")
    os.replace(tmp, p)


def time_ms(fn, stream) -> float:
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--min-tris", type=int, default=10_000)
    ap.add_argument("--max-tris", type=int, default=5_000_000)
    ap.add_argument("--spp", type=int, default=16)
    ap.add_argument("--depth", type=int, default=8)
    ap.add_argument("--tune-cache", default=str(DEFAULT_CACHE))
    ap.add_argument("--retune", action="store_true")
    ap.add_argument("--widths", default="8", help="BVH widths to tune over with --retune, e.g. 4,6,8")
    ap.add_argument("--repeat", type=int, default=2, help="timed launches of each form (after one warm-up)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    import torch
    load()
    ctx = Context(0)
    t0 = time.time()
    specs = batch_specs(a.scenes, a.min_tris, a.max_tris)
    scenes = build_scenes(ctx, specs)
    t_build = time.time() - t0
    st = torch.cuda.current_stream()
    p = batch_params(a.spp, a.depth)
    table = [sc.batch_scene() for sc in scenes]
    nb = ctx.batch_scratch_bytes(table, p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    t1 = time.time()
    tuning, tune_ms = ctx.batch_autotune(table, p, scratch, nb, a.tune_cache, force=a.retune)
    widths = sorted({int(w) for w in a.widths.split(",")})
    width_ms = None
    key = ctx.batch_tuning_key(table, p)
    if a.retune and len(widths) > 1:
        width_ms = sweep_widths(ctx, scenes, p, tuning, scratch, nb, widths, st)
        best = min(width_ms, key=width_ms.get)
        tuning.bvh_width = best
        tuning_cache_store(a.tune_cache, key, tuning, width_ms[best])
        _record_width_trials(a.tune_cache, key, width_ms)
    elif tuning.bvh_width != 8:
        rebuild_scenes(ctx, scenes, tuning.bvh_width)
    table = [sc.batch_scene() for sc in scenes]
    t_tune = time.time() - t1
    plan = ctx.batch_plan(table, p, scratch, nb, tuning, graph=True)
    seq = Sequential(ctx, scenes, a.spp, a.depth)
    off = 0
    plan.launch(off, st)  # warm-up of both forms
    seq.launch(off, st)
    torch.cuda.synchronize()
    batch_ms, seq_ms = [], []
    for r in range(a.repeat):
        off += a.spp
        batch_ms.append(time_ms(lambda: plan.launch(off, st), st))
        seq_ms.append(time_ms(lambda: seq.launch(off, st), st))
    ext, shadow = plan.ray_counts(st)
    ctx.sync()
    pixels = sum(s.width * s.height for s in specs)
    res = {
        "scenes": len(specs), "tris": int(sum(sc.n_tris for sc in scenes)), "pixels": pixels, "spp": a.spp,
        "depth": a.depth, "build_wall_s": round(t_build, 1), "tune_wall_s": round(t_tune, 1),
        "tuning": tuning.as_dict(), "tuning_key": key, "tuning_1spp_ms": round(tune_ms, 3),
        "width_1spp_ms": {str(k): round(v, 3) for k, v in width_ms.items()} if width_ms else None,
        "graph_kernels": plan.launches(),
        "batch_ms": [round(x, 3) for x in batch_ms], "sequential_ms": [round(x, 3) for x in seq_ms],
        "rays_per_launch": {"extension": ext, "shadow": shadow},
        "batch_mrays_s": round((ext + shadow) / (min(batch_ms) * 1e3), 1),
        "sequential_mrays_s": round((ext + shadow) / (min(seq_ms) * 1e3), 1),
        "speedup": round(min(seq_ms) / min(batch_ms), 3),
    }
    js = json.dumps(res)
    print(js)
    if a.out:
        Path(a.out).write_text(js + "\n")
    plan.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
