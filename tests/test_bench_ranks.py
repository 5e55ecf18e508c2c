"""The multi-rank path of bench.py on the CPU: two gloo ranks, each with its
own step time, agree on the slowest and report the whole-job rate; the
reference arm's non-zero ranks exit at once without work."""
from __future__ import annotations

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    import torch
    import torch.distributed as tdist
    sys.path.insert(0, str(REPO))
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.whole_job(2.0 + rank, 4_147_200, world, torch.device("cpu"))
    q.put((rank, ms, value))
    tdist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_step():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == 3.0  # the slower rank's step
        assert abs(value - 2 * 4_147_200 / 3e-3 / 1e6) < 1e-6


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(REPO))
    import bench
    ms, value = bench.whole_job(2.0, 1000, 1)
    assert ms == 2.0 and abs(value - 0.5) < 1e-12


def test_reference_arm_other_ranks_exit_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "3",
                        "--warmup", "3"], capture_output=True, text=True, timeout=120, env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_loads_only_the_oracle():
    """The reference arm makes its inputs with the oracle's generators and
    times the oracle: the product library is never mapped into its process
    (a small soup and frame here; the arm itself runs the full workload)."""
    code = (
        "import sys, json, types; sys.path.insert(0, %r); import bench\n"
        "bench.N_TRIS, bench.W, bench.H = 20000, 64, 32\n"
        "bench.run_reference(types.SimpleNamespace(gpus=1, steps=1, warmup=1))\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'librtcore': 'librtcore' in maps, 'liboracle': 'liboracle' in maps,"
        " 'rtcore_imported': 'rtcore' in sys.modules}))\n" % str(REPO))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    import json
    lines = r.stdout.strip().splitlines()
    line, probe = json.loads(lines[0]), json.loads(lines[-1])
    assert line["impl"] == "reference" and line["config"]["rays_per_step"] == 2 * 64 * 32
    assert probe == {"librtcore": False, "liboracle": True, "rtcore_imported": False}, probe


def test_primary_rays_of_both_arms_are_equal():
    """The GPU arm's numpy raygen and the oracle's give the same rays."""
    sys.path.insert(0, str(REPO))
    import bench
    import oracle
    a = bench.primary_rays_np()
    b = oracle.primary_rays(bench.CAMERA, bench.W, bench.H, 0.0, 100.0)
    assert a.tobytes() == b.tobytes()
