"""Benchmark of the GB300 software ray-tracing core.

Workload (one "step"): closest-hit traversal of 1920x1080 coherent primary
rays plus 1920x1080 incoherent rays (origins uniform in the unit cube,
directions uniform on the sphere) against a seeded soup of 1,000,000 FP32
triangles in the unit cube (LBVH -> BVH8 built once, outside the timed
region), submitted as one rt_trace_closest call over the step's 4.15M rays
(primary, then incoherent).  Metric: Mrays/s over both ray sets, inputs
resident in HBM.  The breakdown times each ray set in a launch of its own.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  Besides the headline value it reports:
  e2e           the same metric through the C ABI with rays in pinned host
                memory and hits returned there: the traversal launch reads
                the rays and writes the hits over NVLink-C2C inside the
                timed region (132.7 MB in, 66.4 MB out per step)
  roofline      achieved algorithmic GB/s of the traversal kernel (rays x
                (48 B ray I/O + 80 B x nodes visited + 36 B x triangles
                tested), counts from the instrumented kernel) over measured
                HBM bandwidth; beside it the step's L2 traffic over the L2
                read bandwidth measured in the same run, and the issue-slot
                bound (warp instructions per ray at the sampled SM clock)
  cpu_baseline  the CPU oracle (same BVH8, same traversal, all host threads)
                timed by the reference arm's function on all of the step's
                rays
  shadow/build  any-hit shadow-ray Mrays/s and BVH build ms (not in value)
  secondary     the 2M-triangle box scene, the path tracer, the MLP cache,
                the 64-scene batch and (relmse) the equal-time relMSE of the
                learned form against the plain path tracer on the 8M-triangle
                box against a 16,384-spp reference (--no-relmse skips it)
  clocks        nvidia-smi samples taken during the timed region
--impl reference times the CPU implementation (the oracle port: the
reference's own ray tracing runs in a Vulkan driver, which does not exist on
this machine) on the same workload and config, all 4,147,200 rays per step,
with inputs from the oracle's own generators (the product library is not
loaded), and prints the same line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
PKG = REPO / "build-up-phase_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

N_TRIS = 1_000_000
W, H = 1920, 1080
CAMERA = ((0.5, 0.5, 2.5), 60.0)
LIGHT = (0.5, 2.0, 0.5)
SEED_BASE = 0x5EED0000   # seeded workloads: 0x5EED0000 + workload number (2: the soup)
METRIC = "Mrays/s primary+incoherent (closest hit), 1M-triangle soup, 1920x1080 each"
WORKLOAD = "triangle soup 1M tris (unit cube, edges U(0.001,0.02)); 1920x1080 primary + 1920x1080 incoherent rays"
BYTES_RAY_IO = 48   # 32 B ray in + 16 B hit out
BYTES_NODE = 80     # compressed BVH8 node
BYTES_TRI = 36      # FP32 vertex triplet
# LBVH build, algorithmic bytes per triangle: 48 read for bounds and
# centroids (12 B indices + 36 B vertices), 12 written as Morton key + id,
# 24 per sort pass (8 passes of 63-bit keys), 2 x 24 for the radix tree and
# its refit, 80 / 8 for the BVH8 node share of one leaf-equivalent
BYTES_BUILD_PER_TRI = 48 + 12 + 24 * 8 + 2 * 24 + 80 // 8
# DRAM bytes (read + write) of one step's traversal launch measured by ncu
# (cold caches): 436.9 MB read + 68.0 MB written
TRAFFIC_BYTES_PER_STEP = 504_800_000
# From the same ncu capture of the step's launch: L2 sectors (32 B) moved,
# warp instructions issued and the SIMT efficiency (active threads per warp
# instruction / 32)
L2_SECTORS_PER_STEP = 235_000_000
WARP_INST_PER_STEP = 1_861_000_000
SIMT_EFFICIENCY = 16.5 / 32
TRAFFIC_SOURCE = "constant from one ncu capture of the step's launch (cold caches), not measured in this run"
SMS, SMSP_PER_SM = 152, 4   # GB300: 152 SMs, four schedulers (one warp instruction per cycle each)
L2_NOTE = ("GPU arm: L2 flushed between steps (256 MB write, outside the step events); "
           "CPU arm: no cache flush, every step traces all 4.15M rays (133 MB of rays, 71 MB of BVH)")


def config(world: int) -> dict:
    """The workload's config, the same in both arms."""
    return {"workload": WORKLOAD, "tris": N_TRIS, "rays_per_step": 2 * W * H,
            "parallelism": f"replicas{world}" if world > 1 else "single", "l2": L2_NOTE}


def _env_int(name: str, default: int) -> int:
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def _peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock/throttle samples while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path("/tmp") / f"rt_bench_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def primary_rays_np():
    """The sample's pinhole raygen for the 1920x1080 launch, in numpy float32
    (the same op sequence as rt_generate_primary_rays)."""
    import math
    f32 = np.float32
    from rtcore.scenes import RAY_DTYPE
    half = f32(f32(f32(CAMERA[1]) * f32(math.pi / 180.0)) * f32(0.5))
    ay = f32(math.tan(float(half)))
    ax = f32(f32(ay * f32(W)) / f32(H))
    ndx = ((np.arange(W, dtype=np.float32) + f32(0.5)) / f32(W)) * f32(2) - f32(1)
    ndy = ((np.arange(H, dtype=np.float32) + f32(0.5)) / f32(H)) * f32(2) - f32(1)
    rays = np.zeros(W * H, RAY_DTYPE)
    d = np.empty((H, W, 3), np.float32)
    p = (ndx * ax)[None, :]
    q = (ndy * ay)[:, None]
    d[..., 0] = (p * f32(1) + q * f32(0)) + f32(0)
    d[..., 1] = (p * f32(0) + q * f32(-1)) + f32(0)
    d[..., 2] = (p * f32(0) + q * f32(0)) + f32(-1)
    rays["dir"] = d.reshape(-1, 3)
    rays["org"] = np.asarray(CAMERA[0], np.float32)
    rays["tmax"] = 100.0
    return rays


def workload():
    """The GPU arm's inputs, from the library's seeded generators."""
    import rtcore.scenes as S
    seed = SEED_BASE + 2
    v, i = S.soup(seed, N_TRIS)
    prim = primary_rays_np()
    inc = S.incoherent_rays(seed, W * H, (0, 0, 0), (1, 1, 1), 1e30)
    return v, i, prim, inc


def workload_cpu():
    """The same inputs (byte for byte: tests/test_pt_oracle.py) from the
    oracle's restatement of the generators, so that the CPU arm loads nothing
    of the product library."""
    import oracle
    seed = SEED_BASE + 2
    v, i = oracle.scene_soup(seed, N_TRIS)
    prim = oracle.primary_rays(CAMERA, W, H, 0.0, 100.0)
    inc = oracle.incoherent_rays(seed, W * H, (0, 0, 0), (1, 1, 1), 1e30)
    return v, i, prim, inc


# ---------------------------------------------------------------------------
# CPU side (oracle port): the reference arm and the cpu_baseline leg
# ---------------------------------------------------------------------------

def cpu_trace_rate(v, i, rays, warmup: int, steps: int, threads: int = 0):
    """Mrays/s of the oracle's BVH8 closest-hit traversal on all host threads:
    `warmup` untimed calls over all of `rays`, then `steps` timed calls.  Both
    CPU figures (the reference arm and the GPU arm's cpu_baseline) come from
    this function on the step's full 4,147,200 rays.  Returns (Mrays/s,
    seconds per step, threads, the oracle structure)."""
    import oracle
    accel, rc = oracle.build_blas([(v, i, None)])
    if rc != 0:
        raise RuntimeError(f"oracle build failed: {rc}")
    threads = threads or oracle.hw_threads()
    for _ in range(warmup):
        oracle.trace_closest(accel, rays, threads)
    t0 = time.perf_counter()
    for _ in range(steps):
        oracle.trace_closest(accel, rays, threads)
    dt = (time.perf_counter() - t0) / max(1, steps)
    return len(rays) / dt / 1e6, dt, threads, accel


def whole_job(ms_step: float, units_per_rank: int, world: int, device=None):
    """(step time, whole-job M units/s): the slowest rank's step time (max over
    ranks through torch.distributed when `device` is given -- the replicas
    each trace the full workload, no data-path collective) and the units all
    ranks processed per second at that time."""
    if device is not None and world > 1:
        import torch
        import torch.distributed as tdist
        t = torch.tensor([ms_step], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms_step = float(t.item())
    return ms_step, units_per_rank * world / (ms_step * 1e-3) / 1e6


def run_reference(args) -> int:
    """The reference arm: the CPU restatement of the path (the reference's own
    ray tracing runs inside a Vulkan driver on RT cores, and no Vulkan stack
    exists on this machine) on the same workload, every step all 4,147,200
    rays, with inputs made by the oracle's own generators."""
    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    if rank != 0:
        return 0
    v, i, prim, inc = workload_cpu()
    rays = np.concatenate([prim, inc])
    value, dt, threads, accel = cpu_trace_rate(v, i, rays, args.warmup, args.steps)
    hdr = accel[:256]
    sample = f"all {len(rays)} rays of the workload per step (2073600 primary + 2073600 incoherent)"
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded PCG32 scene and rays)",
            "config": config(world),
            "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "bvh": {"nodes": int(hdr[16:20].view(np.uint32)[0]), "depth": int(hdr[32:36].view(np.uint32)[0])},
            "note": "the reference's ray tracing runs inside a Vulkan driver on RT cores; no Vulkan stack exists "
                    "on this machine, so the CPU port of the same algorithm (oracle/: same BVH8, same traversal "
                    "order) is timed on all host threads"}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

def run_ours(args) -> int:
    import torch
    import rtcore
    from rtcore.scenes import RAY_DTYPE
    sys.path.insert(0, str(PKG))
    import build as rt_build
    rt_build.build()

    rank, world = _env_int("RANK", 0), _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    ctx = rtcore.Context(local)
    stream = torch.cuda.current_stream()

    v, i, prim, inc = workload()
    n_p, n_i = len(prim), len(inc)
    n_all = n_p + n_i

    # ---- scene upload + build (timed separately: build ms)
    dv = torch.from_numpy(v.reshape(-1)).to(dev)
    di = torch.from_numpy(i.reshape(-1).view(np.int32)).to(dev)
    g = rtcore.GeometryTriangles()
    g.vertices, g.vertex_stride, g.max_vertex = dv.data_ptr(), 12, len(v) - 1
    g.index_type, g.indices, g.tri_count, g.flags = rtcore.RT_INDEX_UINT32, di.data_ptr(), N_TRIS, 1
    sz = ctx.blas_sizes([N_TRIS])
    accel = torch.empty(sz.accel_bytes, dtype=torch.uint8, device=dev)
    scratch = torch.empty(sz.scratch_bytes, dtype=torch.uint8, device=dev)
    # twelve builds back to back (the GPU stays busy, so its clocks are up);
    # the median of the last eight
    ev = []
    for k in range(12):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.build_blas([g], 0, accel, sz.accel_bytes, scratch, sz.scratch_bytes, stream)
        e1.record(stream)
        ev.append((e0, e1))
    ctx.sync(stream)
    build_ms = [e0.elapsed_time(e1) for e0, e1 in ev[4:]]
    n_nodes, _, depth = ctx.accel_info(accel, stream)
    addr = ctx.address(accel)

    # ---- rays resident in HBM
    rays_p = torch.from_numpy(prim.view(np.uint8)).to(dev)
    rays_i = torch.from_numpy(inc.view(np.uint8)).to(dev)
    hits_p = torch.empty(n_p * 16, dtype=torch.uint8, device=dev)
    hits_i = torch.empty(n_i * 16, dtype=torch.uint8, device=dev)

    # ---- traversal statistics (instrumented kernel, untimed)
    cnt = torch.zeros(2, dtype=torch.int64, device=dev)
    ctx.trace_stats(addr, rays_p, n_p, False, cnt, stream)
    ctx.sync(stream)
    st_p = cnt.cpu().numpy().astype(float) / n_p
    ctx.trace_stats(addr, rays_i, n_i, False, cnt, stream)
    ctx.sync(stream)
    st_i = cnt.cpu().numpy().astype(float) / n_i
    bytes_p = BYTES_RAY_IO + BYTES_NODE * st_p[0] + BYTES_TRI * st_p[1]
    bytes_i = BYTES_RAY_IO + BYTES_NODE * st_i[0] + BYTES_TRI * st_i[1]

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2

    # the step's rays in one array: one call traces the whole batch
    rays_all = torch.cat([rays_p, rays_i])
    hits_all = torch.empty(n_all * 16, dtype=torch.uint8, device=dev)

    def step(ev=None):
        if ev:
            ev[0].record(stream)
        ctx.trace_closest(addr, rays_all, hits_all, n_all, stream=stream)
        if ev:
            ev[1].record(stream)

    def step_split(ev):
        ev[0].record(stream)
        ctx.trace_closest(addr, rays_p, hits_p, n_p, stream=stream)
        ev[1].record(stream)
        ctx.trace_closest(addr, rays_i, hits_i, n_i, stream=stream)
        ev[2].record(stream)

    for _ in range(max(3, args.warmup)):
        step()
        flush.fill_(1)
    ctx.sync(stream)

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        t_wall0 = time.perf_counter()
        for k in range(args.steps):
            step(evs[k])
            flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall0
    if dist:
        tdist.barrier()
    ctx.sync(stream)
    ms_step = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    ms_step, value = whole_job(ms_step, n_all, world, dev if dist else None)

    # ---- breakdown: each ray set in a launch of its own (L2 flushed between steps)
    k_split = min(args.steps, 50)
    evs_s = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(k_split)]
    for k in range(k_split):
        step_split(evs_s[k])
        flush.fill_(k & 0xFF)
    ctx.sync(stream)
    t_p = [e[0].elapsed_time(e[1]) for e in evs_s]
    t_i = [e[1].elapsed_time(e[2]) for e in evs_s]

    # ---- roofline of the traversal kernel (the step's launch)
    peaks = _peaks()
    alg_bytes = n_p * bytes_p + n_i * bytes_i
    achieved = alg_bytes / (ms_step * 1e-3) / 1e9
    l2_gbs = l2_read_bandwidth(ctx, stream, dev)
    l2_traffic = L2_SECTORS_PER_STEP * 32
    warp_inst_per_ray = WARP_INST_PER_STEP / n_all
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": round(achieved / peaks["hbm_gbs"], 4),
                "traffic": TRAFFIC_BYTES_PER_STEP,
                "traffic_source": TRAFFIC_SOURCE,
                "algorithmic_bytes_per_step": round(alg_bytes),
                "peak_source": peaks["source"],
                "kernel": "k_trace_blas (closest hit)",
                "bytes_per_ray": {"primary": round(bytes_p, 1), "incoherent": round(bytes_i, 1)},
                "nodes_per_ray": {"primary": round(st_p[0], 3), "incoherent": round(st_i[0], 3)},
                "tris_per_ray": {"primary": round(st_p[1], 3), "incoherent": round(st_i[1], 3)},
                # the pure ray I/O lower bound: 32 B ray in + 16 B hit out
                "io_only": {"bytes_per_ray": BYTES_RAY_IO,
                            "achieved": round(n_all * BYTES_RAY_IO / (ms_step * 1e-3) / 1e9, 1),
                            "frac": round(n_all * BYTES_RAY_IO / (ms_step * 1e-3) / 1e9 / peaks["hbm_gbs"], 4)},
                # the BVH stays in L2: the step's L2 traffic over the L2 read
                # bandwidth measured in this run (a 64 MB buffer read repeatedly)
                "l2": {"achieved": round(l2_traffic / (ms_step * 1e-3) / 1e9, 1), "peak": round(l2_gbs, 1),
                       "unit": "GB/s", "frac": round(l2_traffic / (ms_step * 1e-3) / 1e9 / l2_gbs, 4),
                       "traffic_per_step": l2_traffic, "traffic_source": TRAFFIC_SOURCE,
                       "peak_source": "measured in this run: 64 MB buffer resident in L2, 16-byte L1-bypassing "
                                      "loads, CUDA events"},
                # issue slots: the kernel's warp instructions per ray against
                # one warp instruction per scheduler per cycle at the sampled clock
                "issue": None}

    # ---- shadow rays (any hit) toward a point light from primary hits
    hp = hits_p.cpu().numpy().view(np.float32).reshape(-1, 4)
    hitmask = hp[:, 1].view(np.uint32) != 0xFFFFFFFF
    pts = prim["org"][hitmask] + hp[hitmask, 0:1] * prim["dir"][hitmask]
    sh = np.zeros(int(hitmask.sum()), RAY_DTYPE)
    sh["org"] = pts + np.float32(1e-4) * np.float32([0, 0, 1])
    sh["dir"] = np.float32(LIGHT) - sh["org"]
    sh["tmax"] = 1.0
    rays_s = torch.from_numpy(sh.view(np.uint8)).to(dev)
    occ = torch.empty(max(1, len(sh)), dtype=torch.uint8, device=dev)
    for _ in range(3):
        ctx.trace_any(addr, rays_s, occ, len(sh), stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(5):
        ctx.trace_any(addr, rays_s, occ, len(sh), stream)
    e1.record(stream)
    ctx.sync(stream)
    shadow_mrays = len(sh) * 5 / (e0.elapsed_time(e1) * 1e-3) / 1e6

    # ---- the step's rays through a TLAS of one identity instance over the
    # same BLAS (the sample's two-level layout): the persistent two-level walk
    from rtcore.scenes import INSTANCE_DTYPE
    inst = np.zeros(1, INSTANCE_DTYPE)
    inst[0]["transform"] = np.eye(3, 4, dtype=np.float32)
    inst[0]["custom_index_and_mask"] = 0xFF << 24
    inst[0]["accel_ref"] = addr
    d_inst = torch.from_numpy(inst.view(np.uint8)).to(dev)
    tsz = ctx.tlas_sizes(1)
    tl_accel = torch.empty(tsz.accel_bytes, dtype=torch.uint8, device=dev)
    tl_scratch = torch.empty(tsz.scratch_bytes, dtype=torch.uint8, device=dev)
    ctx.build_tlas(d_inst, 1, 0, tl_accel, tsz.accel_bytes, tl_scratch, tsz.scratch_bytes, stream)
    tl_addr = ctx.address(tl_accel)
    t_tl = []
    for k in range(7):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.trace_closest(tl_addr, rays_all, hits_all, n_all, stream=stream)
        e1.record(stream)
        flush.fill_(k & 0xFF)
        ctx.sync(stream)
        if k >= 2:
            t_tl.append(e0.elapsed_time(e1))
    tlas_mrays = n_all / (statistics.median(t_tl) * 1e-3) / 1e6

    # ---- e2e: rays from pinned host memory, hits back to host
    hp_rays = torch.from_numpy(prim.view(np.uint8)).pin_memory()
    hi_rays = torch.from_numpy(inc.view(np.uint8)).pin_memory()

    # rt_trace_closest_host: the step's rays (primary, then incoherent) read
    # from and its hits written to pinned host memory -- in place by the
    # traversal launch, over NVLink-C2C (the copy path with chunked, overlapped
    # copies serves pageable buffers)
    h_rays = torch.cat([hp_rays, hi_rays]).pin_memory()
    h_hits = torch.empty(n_all * 16, dtype=torch.uint8).pin_memory()
    hnb = ctx.trace_host_scratch_bytes(n_all)
    hscratch = torch.empty(hnb, dtype=torch.uint8, device=dev)

    def e2e_step():
        ctx.trace_closest_host(addr, h_rays, h_hits, n_all, hscratch, hnb, stream)

    def e2e_time(k_steps):
        """ms per call, each call between its own events, L2 flushed between
        calls outside them (as for the device-resident steps)."""
        for _ in range(2):
            e2e_step()
            flush.fill_(1)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k_steps)]
        for k in range(k_steps):
            ev[k][0].record(stream)
            e2e_step()
            ev[k][1].record(stream)
            flush.fill_(k & 0xFF)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / k_steps

    k_e2e = max(3, args.steps)
    e2e_ms = e2e_time(k_e2e)
    # the same calls with the rays and hits staged through the scratch ring
    # (chunked copies on two copy streams, traced on three trace streams)
    ctx.set_host_transfer(rtcore.RT_HOST_TRANSFER_STAGED)
    e2e_staged_ms = e2e_time(min(k_e2e, 50))
    ctx.set_host_transfer(rtcore.RT_HOST_TRANSFER_AUTO)
    e2e_value = n_all * world / (e2e_ms * 1e-3) / 1e6

    extra = secondary_workloads(ctx, stream, dev) if (rank == 0 and not args.no_secondary) else {}
    if rank == 0 and not args.no_relmse:
        extra["relmse"] = relmse_workload(ctx, args.relmse_ref_spp, args.relmse_budget_ms)

    out = None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            cv, _, cores, _ = cpu_trace_rate(v, i, np.concatenate([prim, inc]), 1, 3)
            cpu = {"value": round(cv, 3), "unit": "Mrays/s", "cores": cores, "kind": "port",
                   "sample": f"all {n_all} rays of the workload per step, 1 warm-up + 3 timed steps, oracle BVH8 "
                             f"traversal on {cores} host threads (the reference arm's function)"}
        clk = clocks.summary()
        mhz = clk.get("sm_mhz") or 2070.0
        issue_rate = SMS * SMSP_PER_SM * mhz * 1e6 / warp_inst_per_ray / 1e6  # M rays/s at full issue
        roofline["issue"] = {"achieved": round(value / world, 1), "peak": round(issue_rate, 1), "unit": "Mrays/s",
                             "frac": round(value / world / issue_rate, 4),
                             "warp_instructions_per_ray": round(warp_inst_per_ray, 1),
                             "simt_efficiency": round(SIMT_EFFICIENCY, 3),
                             "peak_all_lanes_active": round(issue_rate / SIMT_EFFICIENCY, 1),
                             "sm_mhz": mhz, "source": "warp instructions and SIMT efficiency: " + TRAFFIC_SOURCE}
        out = {"metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
               "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": round(ms_step, 4),
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic (seeded PCG32 scene and rays)",
               "config": config(world),
               "bvh": {"nodes": n_nodes, "depth": depth},
               "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s",
                       "h2d_bytes_per_step": n_all * 32, "d2h_bytes_per_step": n_all * 16,
                       "transfer": "rt_trace_closest_host on pinned host buffers: the traversal launch reads "
                                   "the rays and writes the hits in place over NVLink-C2C",
                       "staged_value": round(n_all * world / (e2e_staged_ms * 1e-3) / 1e6, 3),
                       "staged_transfer": "RT_HOST_TRANSFER_STAGED: chunked copies through the scratch ring, "
                                          "overlapped with the traversal",
                       "l2": "flushed between calls (256 MB write, outside the call events)"},
               "gpu_launches": 2 * args.steps,
               "roofline": roofline,
               "cpu_baseline": cpu,
               "breakdown": {"primary_mrays": round(n_p * k_split / (sum(t_p) * 1e-3) / 1e6, 2),
                             "incoherent_mrays": round(n_i * k_split / (sum(t_i) * 1e-3) / 1e6, 2),
                             "separate_launches_mrays": round(n_all * k_split / ((sum(t_p) + sum(t_i)) * 1e-3) / 1e6, 2),
                             "shadow_anyhit_mrays": round(shadow_mrays, 2),
                             "tlas_1instance_mrays": round(tlas_mrays, 2),
                             "build_ms": round(statistics.median(build_ms), 3),
                             "build_roofline": {
                                 "bytes_per_tri": BYTES_BUILD_PER_TRI,
                                 "achieved_gbs": round(N_TRIS * BYTES_BUILD_PER_TRI / (statistics.median(build_ms) * 1e-3) / 1e9, 1),
                                 "frac_of_hbm": round(N_TRIS * BYTES_BUILD_PER_TRI / (statistics.median(build_ms) * 1e-3) / 1e9
                                                      / peaks["hbm_gbs"], 4),
                                 "note": "latency-bound: 15 dependent launches (eight sort passes), the collapse a cooperative grid of level barriers"},
                             "wall_s_timed_region": round(t_wall, 3)},
               "secondary": extra,
               "clocks": clk}
        print(json.dumps(out), flush=True)
    ctx.close()
    if dist:
        tdist.destroy_process_group()
    return 0


def l2_read_bandwidth(ctx, stream, dev, mbytes: int = 64, passes: int = 40) -> float:
    """GB/s of reading an L2-resident buffer (64 MB, below the 129 MB L2):
    rt_debug_read_sweep reads it `passes` times per launch with 16-byte
    loads that bypass L1; best of five launches after a warm-up, CUDA events
    on the launching stream."""
    import torch
    buf = torch.ones(mbytes << 20, dtype=torch.uint8, device=dev)
    ctx.read_sweep(buf, buf.numel(), passes, stream)
    best = None
    for _ in range(5):
        ms = _events(torch, stream, lambda: ctx.read_sweep(buf, buf.numel(), passes, stream), 1)
        best = ms if best is None else min(best, ms)
    ctx.sync(stream)
    return buf.numel() * passes / (best * 1e-3) / 1e9


def _events(torch, stream, fn, reps: int) -> float:
    """Mean milliseconds of fn() over reps calls, CUDA events on `stream`."""
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def secondary_workloads(ctx, stream, dev) -> dict:
    """Untimed-by-the-headline figures of the other targets: the 2M-triangle
    box scene (build, primary and incoherent rays), the path tracer on it at
    1920x1080, and the MLP cache's query and training throughput."""
    import torch
    import rtcore
    import rtcore.scenes as S
    out = {}
    v, i, tm, m = S.box(S.SEED_BASE + 3, 40, 50)
    lights = S.emissive_lights(v, i, tm, m)
    keep = [torch.from_numpy(v.reshape(-1)).to(dev), torch.from_numpy(i.reshape(-1).view(np.int32)).to(dev),
            torch.from_numpy(tm.view(np.int32)).to(dev), torch.from_numpy(m.view(np.uint8)).to(dev),
            torch.from_numpy(lights.view(np.uint8)).to(dev)]
    g = rtcore.GeometryTriangles()
    g.vertices, g.vertex_stride, g.max_vertex = keep[0].data_ptr(), 12, len(v) - 1
    g.index_type, g.indices, g.tri_count, g.flags = rtcore.RT_INDEX_UINT32, keep[1].data_ptr(), len(i), 1
    sz = ctx.blas_sizes([len(i)])
    accel = torch.empty(sz.accel_bytes, dtype=torch.uint8, device=dev)
    scratch = torch.empty(sz.scratch_bytes, dtype=torch.uint8, device=dev)
    build = lambda: ctx.build_blas([g], 0, accel, sz.accel_bytes, scratch, sz.scratch_bytes, stream)
    build()
    ms_build = _events(torch, stream, build, 5)
    ctx.sync(stream)
    del scratch
    rnb = rtcore.refit_scratch_bytes(len(i))
    rscratch = torch.empty(rnb, dtype=torch.uint8, device=dev)
    refit = lambda: ctx.refit_blas([g], accel, sz.accel_bytes, rscratch, rnb, stream)
    refit()
    ms_refit = _events(torch, stream, refit, 5)
    ctx.sync(stream)
    del rscratch
    addr = ctx.address(accel)
    n = W * H
    rays = torch.empty(n * 32, dtype=torch.uint8, device=dev)
    ctx.generate_primary_rays(rtcore.Camera(S.BOX_CAMERA[0], S.BOX_CAMERA[1]), W, H, 0.0, 1e30, rays, stream)
    inc = torch.from_numpy(S.incoherent_rays(S.SEED_BASE + 3, n, (-0.99,) * 3, (0.99,) * 3, 1e30).view(np.uint8)).to(dev)
    hits = torch.empty(n * 16, dtype=torch.uint8, device=dev)
    for r in (rays, inc):
        ctx.trace_closest(addr, r, hits, n, stream=stream)
    ms_p = _events(torch, stream, lambda: ctx.trace_closest(addr, rays, hits, n, stream=stream), 20)
    ms_i = _events(torch, stream, lambda: ctx.trace_closest(addr, inc, hits, n, stream=stream), 20)
    out["box_2M"] = {"tris": len(i), "build_ms": round(ms_build, 3), "refit_ms": round(ms_refit, 3),
                     "primary_mrays": round(n / ms_p / 1e3, 1),
                     "incoherent_mrays": round(n / ms_i / 1e3, 1),
                     "targets": ">= 2000 primary, >= 500 incoherent Mrays/s on the 2M-triangle scene"}
    # path tracer, 1920x1080, 4 samples per call, depth 8, RR from 3
    sc = rtcore.PtScene(addr, keep[2].data_ptr(), keep[3].data_ptr(), len(m), keep[4].data_ptr(), len(lights))
    p = rtcore.PtParams(rtcore.Camera(S.BOX_CAMERA[0], S.BOX_CAMERA[1]), W, H, 4, 0, 8, 3, S.SEED_BASE + 3, 1e-4, 0)
    nb = ctx.pt_scratch_bytes(p)
    pscr = torch.empty(nb, dtype=torch.uint8, device=dev)
    acc = torch.zeros(n * 16, dtype=torch.uint8, device=dev)
    ctx.path_trace(sc, p, acc, pscr, nb, stream)
    ms_pt = _events(torch, stream, lambda: ctx.path_trace(sc, p, acc, pscr, nb, stream), 3)
    ext, shadow = ctx.pt_ray_counts(p, len(lights), pscr, stream)
    # the same samples with the bounce rays grouped by direction octant
    pu = rtcore.PtParams(p.camera, W, H, 4, 0, 8, 3, S.SEED_BASE + 3, 1e-4, rtcore.RT_PT_OCTANT_BINNING)
    ctx.path_trace(sc, pu, acc, pscr, nb, stream)
    ms_pu = _events(torch, stream, lambda: ctx.path_trace(sc, pu, acc, pscr, nb, stream), 3)
    out["path_tracer"] = {"resolution": [W, H], "spp_per_call": 4, "ms_per_spp": round(ms_pt / 4, 3),
                          "mrays_per_s": round((ext + shadow) / ms_pt / 1e3, 1),
                          "rays_per_spp": round((ext + shadow) / 4 / n, 3),
                          "ms_per_spp_octant_binning": round(ms_pu / 4, 3)}
    del pscr, acc
    # MLP cache: 2M queries (43,520 FLOP each, algorithmic) and 65,536 training
    # samples per pass (120,192 FLOP each)
    cache = torch.zeros(ctx.cache_bytes(), dtype=torch.uint8, device=dev)
    ctx.cache_init(cache, rtcore.cache_config(seed=1), stream)
    rng = np.random.default_rng(0)
    qn = n
    qin = np.zeros((qn, 12), np.float32)
    qin[:, 0:3] = rng.uniform(-1, 1, (qn, 3))
    for c0 in (3, 6):
        d = rng.normal(size=(qn, 3))
        qin[:, c0:c0 + 3] = d / np.linalg.norm(d, axis=1, keepdims=True)
    qin[:, 9:12] = rng.uniform(0, 1, (qn, 3))
    dq = torch.from_numpy(qin.reshape(-1)).to(dev)
    qo = torch.empty(qn * 16, dtype=torch.uint8, device=dev)
    ctx.cache_query(cache, dq, qo, qn, stream)
    ms_q = _events(torch, stream, lambda: ctx.cache_query(cache, dq, qo, qn, stream), 10)
    tn = 65536
    tg = torch.from_numpy(rng.uniform(0, 1, (tn, 4)).astype(np.float32).reshape(-1)).to(dev)
    from rtcore.relmse import TRAIN_BATCH
    train_ms = {}
    for tb in (16384, TRAIN_BATCH):
        ctx.cache_train(cache, dq, tg, tn, tb, None, stream)
        train_ms[tb] = _events(torch, stream, lambda: ctx.cache_train(cache, dq, tg, tn, tb, None, stream), 5)
    ms_t = train_ms[16384]
    peaks = json.loads((REPO / "MEASURED_PEAKS.json").read_text()) if (REPO / "MEASURED_PEAKS.json").exists() else {}
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    q_tflops = qn * 43520 / (ms_q * 1e-3) / 1e12
    out["mlp_cache"] = {"query_ms_2M": round(ms_q, 3), "query_tflops": round(q_tflops, 2),
                        "query_frac_of_bf16_peak": round(q_tflops / bf16_peak, 4),
                        "train_ms_65536": round(ms_t, 3),
                        "train_tflops": round(tn * 120192 / (ms_t * 1e-3) / 1e12, 2),
                        "train_frac_of_bf16_peak": round(tn * 120192 / (ms_t * 1e-3) / 1e12 / bf16_peak, 4),
                        "train_batch": 16384,
                        # the learned form's own batch (more, cheaper Adam steps)
                        "train_ms_65536_learned_batch": round(train_ms[TRAIN_BATCH], 3),
                        "learned_batch": TRAIN_BATCH}
    ctx.sync(stream)
    del cache, dq, qo, tg, keep, accel, rays, inc, hits
    out["batch_64"] = batch_workload(ctx, stream, dev)
    return out


def relmse_workload(ctx, ref_spp: int, budget_ms: float) -> dict:
    """The second half of the metric: equal-time relMSE of the learned form
    (MLP radiance cache ending paths at their second vertex) against the
    plain path tracer, on the learned workload -- the box with 160 icospheres
    (8,000,014 triangles), 1920x1080, depth 8, Russian roulette from 3,
    65,536 training paths per sample in Adam batches of 4,096 (lr 1e-3),
    four samples per call for both forms -- measured against a plain
    reference of ref_spp samples per pixel.  Reports each form's curve, the
    relMSE both reach in the same time, and the time each needs to reach
    relMSE 1e-3 on the CUDA-event clock and the wall clock; the target is a
    learned/plain time ratio of at most 0.5."""
    from rtcore.relmse import TRAIN_BATCH, GpuBox, equal_time, reference
    t0 = time.perf_counter()
    box = GpuBox(ctx, 160, 50)
    t1 = time.perf_counter()
    ref = reference(ctx, box, W, H, ref_spp)
    t2 = time.perf_counter()
    res = equal_time(ctx, box, W, H, ref, budget_ms, target=1e-3, train_paths=65536, train_batch=TRAIN_BATCH, lr=1e-3,
                     spp_per_call=4)
    ratio = res["time_to_target_wall_ms"]["ratio_cached_over_plain"]
    out = {"workload": "box scene, 160 icospheres (8,000,014 triangles), 1920x1080, depth 8, RR from 3",
           "tris": box.n_tris, "reference_spp": ref_spp, "reference_wall_s": round(t2 - t1, 1),
           "setup_wall_s": round(t1 - t0, 1), "budget_gpu_ms": budget_ms, "train_paths": 65536,
           "train_batch": TRAIN_BATCH, "lr": 1e-3, "spp_per_call": 4, "target_relmse": 1e-3,
           "target_time_ratio": 0.5,
           "meets_target": bool(ratio is not None and ratio <= 0.5)}
    out.update(res)
    return out


def batch_workload(ctx, stream, dev) -> dict:
    """The batched form: 64 seeded scenes (lit soups and box scenes of
    10k-5M triangles, 512^2-2048^2 pixels, own cameras), 16 spp, depth 8:
    one CUDA-graph launch of rt_batch_launch against 64 rt_path_trace
    launches over the same samples (the images are equal bit for bit).  The
    launch shape comes from the committed autotuner cache when it holds the
    batch's key, else from a live autotuner run."""
    import torch
    import rtcore
    from rtcore import batch as B
    t0 = time.time()
    specs = B.batch_specs()
    scenes = B.build_scenes(ctx, specs)
    t_build = time.time() - t0
    p = B.batch_params(16, 8)
    table = [sc.batch_scene() for sc in scenes]
    key = ctx.batch_tuning_key(table, p)
    hit = rtcore.tuning_cache_lookup(B.DEFAULT_CACHE, key) if B.DEFAULT_CACHE.exists() else None
    tuning = hit[0] if hit else None
    if tuning is not None and tuning.bvh_width != 8:
        B.rebuild_scenes(ctx, scenes, tuning.bvh_width)
        table = [sc.batch_scene() for sc in scenes]
    nb = ctx.batch_scratch_bytes(table, p, tuning)
    scratch = torch.empty(nb, dtype=torch.uint8, device=dev)
    if tuning is None:
        tuning, _ = ctx.batch_autotune(table, p, scratch, nb, None)
    plan = ctx.batch_plan(table, p, scratch, nb, tuning, graph=True)
    seq = B.Sequential(ctx, scenes, 16, 8)
    plan.launch(0, stream)
    seq.launch(0, stream)
    ms_b = B.time_ms(lambda: plan.launch(16, stream), stream)
    ms_s = B.time_ms(lambda: seq.launch(16, stream), stream)
    ext, shadow = plan.ray_counts(stream)
    ctx.sync(stream)
    res = {"scenes": len(specs), "tris": int(sum(sc.n_tris for sc in scenes)),
           "pixels": int(sum(s.width * s.height for s in specs)), "spp": 16, "depth": 8,
           "setup_wall_s": round(t_build, 1), "tuning": tuning.as_dict(), "tuning_key": key,
           "tuning_source": "cache" if hit else "live", "graph_kernels": plan.launches(),
           "batch_ms": round(ms_b, 2), "sequential_ms": round(ms_s, 2),
           "rays": ext + shadow, "batch_mrays_s": round((ext + shadow) / (ms_b * 1e3), 1),
           "sequential_mrays_s": round((ext + shadow) / (ms_s * 1e3), 1), "speedup": round(ms_s / ms_b, 3)}
    plan.close()
    return res


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    # ~2.5 ms per step: 1000 steps keep the timed region near 3 s, long
    # enough for a dozen clock samples
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU oracle leg")
    ap.add_argument("--no-secondary", action="store_true", help="skip the box-scene / path-tracer / MLP figures")
    ap.add_argument("--no-relmse", action="store_true", help="skip the learned form's equal-time relMSE block")
    ap.add_argument("--relmse-ref-spp", type=int, default=16384,
                    help="samples per pixel of the plain reference image of the relMSE block")
    ap.add_argument("--relmse-budget-ms", type=float, default=12000.0,
                    help="GPU time given to each form in the relMSE block")
    args = ap.parse_args(argv)
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
