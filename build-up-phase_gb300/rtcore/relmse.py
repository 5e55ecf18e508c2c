"""Equal-time relMSE of the learned form (MLP radiance cache) against the plain
path tracer, both measured against a converged plain reference.

    python -m rtcore.relmse [--spheres 160 --freq 50] [--width 1920 --height 1080]
                            [--ref-spp 16384] [--budget-ms 4000] [--out result.json]

relMSE = mean over pixels and channels of (I - R)^2 / (R^2 + 0.01).  Both
forms run four samples per call (one wave of four samples of every pixel; the
learned form queries the cache once per wave and trains after it on the
wave's training paths).  Each call is timed twice: its CUDA-event duration
(training included for the learned form) and its wall time (a host clock
from just before the call to the end of a synchronisation after it); image
read-backs for the relMSE are outside both.
The curve is sampled at sample counts growing by 1.25x and at the end of the
budget; the time to a target relMSE is interpolated log-log between the two
samples around the crossing.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import Camera, Context, GeometryTriangles, PtCacheParams, PtParams, PtScene, cache_config, load
from . import scenes as S


# Adam batch of the learned form's online training.  Smaller batches mean more
# optimiser steps per frame for the same 65,536 samples, and on the GB300 the
# steps are cheap next to the path tracing: on the 8M-triangle box at
# 1920x1080 (four samples per call) the learned form reached the relMSE the
# plain form has after 3 s of GPU time in 611 ms with batches of 4,096,
# 759 ms with 8,192, 1,189 ms with 16,384, and it reached relMSE 1e-3 (against
# 16,384 spp) in 2,579 / 4,095 / 6,623 ms with 16,384 / 32,768 / 65,536.
TRAIN_BATCH = 4096


def relmse(img: np.ndarray, ref: np.ndarray) -> float:
    return float(np.mean((img - ref) ** 2 / (ref * ref + 0.01)))


class GpuBox:
    """The box workload on the device: BLAS, materials, lights."""

    def __init__(self, ctx: Context, n_spheres: int, freq: int, seed: int = S.SEED_BASE + 3):
        import torch
        self.ctx = ctx
        v, i, tm, m = S.box(seed, n_spheres, freq)
        self.n_tris = len(i)
        lights = S.emissive_lights(v, i, tm, m)
        self.keep = [torch.from_numpy(v.reshape(-1)).cuda(), torch.from_numpy(i.reshape(-1).view(np.int32)).cuda(),
                     torch.from_numpy(tm.view(np.int32)).cuda(), torch.from_numpy(m.view(np.uint8)).cuda(),
                     torch.from_numpy(lights.view(np.uint8)).cuda()]
        g = GeometryTriangles()
        g.vertices, g.vertex_stride, g.max_vertex = self.keep[0].data_ptr(), 12, len(v) - 1
        g.index_type, g.indices, g.tri_count, g.flags = 1, self.keep[1].data_ptr(), len(i), 1
        sz = ctx.blas_sizes([len(i)])
        self.accel = torch.empty(sz.accel_bytes, dtype=torch.uint8, device="cuda")
        scratch = torch.empty(sz.scratch_bytes, dtype=torch.uint8, device="cuda")
        ctx.build_blas([g], 0, self.accel, sz.accel_bytes, scratch, sz.scratch_bytes)
        ctx.sync()
        del scratch
        self.n_lights = len(lights)
        self.scene = PtScene(ctx.address(self.accel), self.keep[2].data_ptr(), self.keep[3].data_ptr(), len(m),
                             self.keep[4].data_ptr(), len(lights))


def params(w: int, h: int, spp: int, offset: int, seed: int) -> PtParams:
    return PtParams(Camera(S.BOX_CAMERA[0], S.BOX_CAMERA[1]), w, h, spp, offset, 8, 3, seed, 1e-4, 0)


def _image(accum) -> np.ndarray:
    a = accum.cpu().numpy().view(np.float32).reshape(-1, 4)
    return a[:, :3] / np.maximum(a[:, 3:4], 1.0)


def reference(ctx: Context, box: GpuBox, w: int, h: int, spp: int, chunk: int = 256, seed: int = 12345) -> np.ndarray:
    import torch
    p = params(w, h, min(chunk, spp), 0, seed)
    nb = ctx.pt_scratch_bytes(p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    accum = torch.zeros(w * h * 16, dtype=torch.uint8, device="cuda")
    done = 0
    while done < spp:
        p = params(w, h, min(chunk, spp - done), done, seed)
        ctx.path_trace(box.scene, p, accum, scratch, nb)
        done += p.spp
    ctx.sync()
    return _image(accum)


def _checkpoints(n: int):
    k = 1
    while k <= n:
        yield k
        k = max(k + 1, int(math.ceil(k * 1.25)))


def run(ctx: Context, box: GpuBox, w: int, h: int, ref: np.ndarray, budget_ms: float, cached: bool,
        train_paths: int = 65536, train_batch: int = TRAIN_BATCH, seed: int = 777, lr: float = 1e-3,
        spp_per_call: int = 1):
    """[(gpu_ms, wall_ms, samples, relmse)] until the GPU time reaches the
    budget: cumulative CUDA-event and wall-clock times of the calls."""
    import torch
    st = torch.cuda.current_stream()
    accum = torch.zeros(w * h * 16, dtype=torch.uint8, device="cuda")
    spc = max(1, spp_per_call)
    p = params(w, h, spc, 0, seed)
    cache = None
    if cached:
        cache = torch.zeros(ctx.cache_bytes(), dtype=torch.uint8, device="cuda")
        ctx.cache_init(cache, cache_config(lr=lr, seed=3))
        cp = PtCacheParams(cache.data_ptr(), train_paths, train_batch)
        nb = ctx.pt_cached_scratch_bytes(p, cp)
    else:
        nb = ctx.pt_scratch_bytes(p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    curve, elapsed, wall, s = [], 0.0, 0.0, 0
    marks = set(_checkpoints(1 << 20))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    while elapsed < budget_ms:
        p = params(w, h, spc, s, seed)
        t0 = time.perf_counter()
        e0.record(st)
        if cached:
            ctx.path_trace_cached(box.scene, p, cp, accum, scratch, nb)
        else:
            ctx.path_trace(box.scene, p, accum, scratch, nb)
        e1.record(st)
        e1.synchronize()
        wall += (time.perf_counter() - t0) * 1e3
        elapsed += e0.elapsed_time(e1)
        s += spc
        if any(k in marks for k in range(s - spc + 1, s + 1)) or elapsed >= budget_ms:
            curve.append((round(elapsed, 3), round(wall, 3), s, relmse(_image(accum), ref)))
    ctx.sync()
    return curve


def time_to(curve, target: float, clock: str = "gpu"):
    """Elapsed time (clock "gpu": CUDA events, "wall": host clock) at which
    relMSE first reaches target, interpolated log-log between the samples
    around the crossing (None if never)."""
    col = 0 if clock == "gpu" else 1
    prev = None
    for row in curve:
        ms, r = row[col], row[3]
        if r <= target:
            if prev is None or prev[1] <= r or prev[0] <= 0.0:
                return ms
            lt0, lt1 = math.log(prev[0]), math.log(ms)
            lr0, lr1 = math.log(prev[1]), math.log(r)
            f = (math.log(target) - lr0) / (lr1 - lr0)
            return round(math.exp(lt0 + f * (lt1 - lt0)), 3)
        prev = (ms, r)
    return None


def equal_time(ctx: Context, box: GpuBox, w: int, h: int, ref: np.ndarray, budget_ms: float, target: float = 1e-3,
               train_paths: int = 65536, train_batch: int = TRAIN_BATCH, lr: float = 1e-3, spp_per_call: int = 4) -> dict:
    """Both forms against the reference within the budget: their curves,
    relMSE at the end of the budget, the time each takes to reach `target`
    on both clocks and the learned form's share of the plain form's time."""
    plain = run(ctx, box, w, h, ref, budget_ms, False, spp_per_call=spp_per_call)
    cached = run(ctx, box, w, h, ref, budget_ms, True, train_paths=train_paths, train_batch=train_batch, lr=lr,
                 spp_per_call=spp_per_call)
    out = {"curve_columns": ["gpu_ms", "wall_ms", "spp", "relmse"], "plain": plain, "cached": cached,
           "relmse_at_budget": {"plain": plain[-1][3], "cached": cached[-1][3],
                                "plain_spp": plain[-1][2], "cached_spp": cached[-1][2]},
           "target": target}
    for clock in ("gpu", "wall"):
        tp, tc = time_to(plain, target, clock), time_to(cached, target, clock)
        out[f"time_to_target_{clock}_ms"] = {"plain": tp, "cached": tc,
                                             "ratio_cached_over_plain": round(tc / tp, 3) if tp and tc else None}
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--spheres", type=int, default=160)
    ap.add_argument("--freq", type=int, default=50)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--budget-ms", type=float, default=4000.0)
    ap.add_argument("--target", type=float, default=1e-3)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--train-paths", type=int, default=65536, help="training paths per frame")
    ap.add_argument("--train-batch", type=int, default=TRAIN_BATCH)
    ap.add_argument("--plain-spp-per-call", type=int, default=4,
                    help="samples per call of the plain form (4: one wave of four samples)")
    ap.add_argument("--cached-spp-per-call", type=int, default=4,
                    help="samples per call of the learned form (the cache trains after each call's wave)")
    ap.add_argument("--out", default=None)
    a = ap.parse_args(argv)
    load()
    ctx = Context(0)
    t0 = time.time()
    box = GpuBox(ctx, a.spheres, a.freq)
    ref = reference(ctx, box, a.width, a.height, a.ref_spp)
    t_ref = time.time() - t0
    plain = run(ctx, box, a.width, a.height, ref, a.budget_ms, False, spp_per_call=a.plain_spp_per_call)
    cached = run(ctx, box, a.width, a.height, ref, a.budget_ms, True, train_paths=a.train_paths,
                 train_batch=a.train_batch, lr=a.lr, spp_per_call=a.cached_spp_per_call)
    res = {"tris": box.n_tris, "width": a.width, "height": a.height, "ref_spp": a.ref_spp,
           "train_paths": a.train_paths, "train_batch": a.train_batch, "lr": a.lr,
           "plain_spp_per_call": a.plain_spp_per_call, "cached_spp_per_call": a.cached_spp_per_call,
           "reference_wall_s": round(t_ref, 1), "budget_ms": a.budget_ms,
           "curve_columns": ["gpu_ms", "wall_ms", "spp", "relmse"], "plain": plain, "cached": cached,
           "relmse_at_budget": {"plain": plain[-1][3], "cached": cached[-1][3]}}
    for clock in ("gpu", "wall"):
        tp, tc = time_to(plain, a.target, clock), time_to(cached, a.target, clock)
        res[f"time_to_target_{clock}_ms"] = {"target": a.target, "plain": tp, "cached": tc,
                                             "ratio_cached_over_plain": round(tc / tp, 3) if tp and tc else None}
    js = json.dumps(res)
    print(js)
    if a.out:
        with open(a.out, "w") as f:
            f.write(js + "\n")
    ctx.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
