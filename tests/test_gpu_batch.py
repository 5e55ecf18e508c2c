"""GPU checks of the batched path tracer (rtcore_batch.h): every scene of a
batch receives exactly the image rt_path_trace -- and the CPU oracle -- give
for it, whatever the launch shape, wave size, graph or direct launch; and the
autotuner chooses among shapes and caches its choice."""
from __future__ import annotations

import json

import numpy as np
import pytest

from helpers import host

pytestmark = pytest.mark.gpu

SEED = 0x5EED0004


def _scenes(ctx, specs):
    from rtcore.batch import GpuScene, host_scene
    return [GpuScene(ctx, sp, host_scene(sp)) for sp in specs]


def _spec(kind, tris, w, h, cam=None, seed=1):
    from rtcore.batch import SceneSpec
    import rtcore.scenes as S
    if cam is None:
        cam = S.BOX_CAMERA if kind == "box" else ((0.5, 0.5, 2.2), 45.0)
    return SceneSpec(kind, tris, w, h, cam, seed)


def _plan_run(ctx, scenes, spp, depth=8, tuning=None, graph=True, offsets=(0,)):
    import torch
    from rtcore.batch import batch_params
    p = batch_params(spp, depth, SEED)
    for sc in scenes:
        sc.accum.zero_()
    table = [sc.batch_scene() for sc in scenes]
    nb = ctx.batch_scratch_bytes(table, p, tuning)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    plan = ctx.batch_plan(table, p, scratch, nb, tuning, graph=graph)
    for off in offsets:
        plan.launch(off)
    ctx.sync()
    out = [host(sc.accum).copy() for sc in scenes]
    counts = plan.ray_counts()
    plan.close()
    return out, counts


def _sequential(ctx, scenes, spp, offsets=(0,), depth=8):
    from rtcore.batch import Sequential
    for sc in scenes:
        sc.accum.zero_()
    seq = Sequential(ctx, scenes, spp, depth, SEED)
    for off in offsets:
        seq.launch(off)
    ctx.sync()
    return [host(sc.accum).copy() for sc in scenes]


SMALL = [("soup", 3000, 48, 32), ("box", 2000, 40, 30), ("soup", 500, 0, 0), ("box", 9000, 33, 17),
         ("soup", 20000, 1, 1), ("box", 14, 25, 20)]


def test_batch_matches_oracle_across_waves(ctx, orc):
    """Six scenes (one without pixels, one 1x1, one empty box), waves of 997
    paths that split scenes: each image equals the oracle's bit for bit."""
    import rtcore
    from rtcore.batch import host_scene
    specs = [_spec(k, t, w, h, seed=100 + j) for j, (k, t, w, h) in enumerate(SMALL)]
    scenes = _scenes(ctx, specs)
    tun = rtcore.default_batch_tuning()
    tun.wave_paths = 997
    for graph in (True, False):
        got, (ext, shadow) = _plan_run(ctx, scenes, 2, tuning=tun, graph=graph)
        assert ext >= 2 * sum(s.width * s.height for s in specs) and shadow > 0
        for sp, sc, g in zip(specs, scenes, got):
            if sp.width * sp.height == 0:
                continue
            v, i, tm, m = host_scene(sp)
            ob, _ = orc.build_blas([(v, i, None)])
            import rtcore.scenes as S
            lights = S.emissive_lights(v, i, tm, m)
            o = orc.path_trace(ob, tm, m, lights, sp.camera, sp.width, sp.height, 2, 8, 3, SEED, 1e-4)
            gg = g.view(np.float32).reshape(sp.height, sp.width, 4)
            assert gg.tobytes() == o.tobytes(), (sp, graph, np.abs(gg - o).max())


@pytest.fixture(scope="module")
def mid_scenes(ctx):
    specs = [_spec("box", 60000, 128, 128, seed=7), _spec("soup", 250000, 96, 96, seed=8),
             _spec("soup", 12000, 200, 150, ((0.45, 0.55, 2.4), 40.0), seed=9), _spec("box", 300000, 64, 64, seed=10),
             _spec("box", 20000, 160, 90, ((0.1, -0.1, 0.9), 65.0), seed=11), _spec("soup", 90000, 77, 111, seed=12)]
    return _scenes(ctx, specs)


def test_batch_equals_sequential_progressive(ctx, mid_scenes):
    """Two graph launches (samples 0-2 and 3-5) equal one rt_path_trace per
    scene over the same samples, bit for bit."""
    got, _ = _plan_run(ctx, mid_scenes, 3, offsets=(0, 3))
    ref = _sequential(ctx, mid_scenes, 3, offsets=(0, 3))
    for g, r in zip(got, ref):
        assert g.tobytes() == r.tobytes()
    img = got[0].view(np.float32).reshape(-1, 4)
    assert (img[:, 3] == 6).all() and img[:, :3].max() > 0


@pytest.mark.parametrize("threads,bps,ring,refill,shade,wave", [
    (128, 8, 8, 1, 128, 0), (128, 6, 32, 32, 512, 0), (256, 4, 16, 4, 256, 4096), (256, 2, 8, 16, 512, 50000),
    (256, 4, 32, 2, 128, 0), (128, 4, 16, 8, 256, 1 << 20)])
def test_every_launch_shape_gives_the_same_images(ctx, mid_scenes, threads, bps, ring, refill, shade, wave):
    import rtcore
    base, _ = _plan_run(ctx, mid_scenes, 2)
    t = rtcore.BatchTuning(threads, bps, ring, refill, shade, wave, 8, 0)
    got, _ = _plan_run(ctx, mid_scenes, 2, tuning=t)
    for g, b in zip(got, base):
        assert g.tobytes() == b.tobytes()


def test_autotune_and_cache(ctx, mid_scenes, tmp_path):
    import torch
    import rtcore
    from rtcore.batch import batch_params
    p = batch_params(4, 8, SEED)
    table = [sc.batch_scene() for sc in mid_scenes]
    nb = ctx.batch_scratch_bytes(table, p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    cache = tmp_path / "tune.json"
    for sc in mid_scenes:
        sc.accum.zero_()
    t, ms = ctx.batch_autotune(table, p, scratch, nb, cache)
    ctx.sync()
    assert ms > 0
    # timing launches discard their samples
    assert all(float(sc.accum.abs().max()) == 0.0 for sc in mid_scenes)
    doc = json.loads(cache.read_text())
    key = ctx.batch_tuning_key(table, p)
    assert key.startswith("sm103-") and "/n2^2/" in key and key.endswith("/d8")
    entry = doc["entries"][key]
    assert len(entry["trials"]) >= 10
    assert {k: entry[k] for k in t.as_dict()} == t.as_dict()
    # the second call reads the cache (same tuning, the stored time)
    t2, ms2 = ctx.batch_autotune(table, p, scratch, nb, cache)
    assert t2.as_dict() == t.as_dict() and abs(ms2 - entry["ms"]) < 1e-3
    # the chosen tuning gives the default tuning's images
    got, _ = _plan_run(ctx, mid_scenes, 2, tuning=t)
    base, _ = _plan_run(ctx, mid_scenes, 2)
    assert all(g.tobytes() == b.tobytes() for g, b in zip(got, base))
    assert rtcore.tuning_cache_lookup(cache, "no-such-key") is None


def test_batch_argument_errors(ctx, mid_scenes):
    import torch
    import rtcore
    from rtcore.batch import batch_params
    p = batch_params(1, 8, SEED)
    table = [sc.batch_scene() for sc in mid_scenes[:2]]
    nb = ctx.batch_scratch_bytes(table, p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    bad = rtcore.default_batch_tuning()
    bad.stack_ring = 12
    with pytest.raises(rtcore.RtError) as e:
        ctx.batch_plan(table, p, scratch, nb, bad)
    assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    with pytest.raises(rtcore.RtError) as e:
        ctx.batch_plan(table, p, scratch, nb - 256)
    assert e.value.code == rtcore.RT_ERR_OOM
    t2 = [sc.batch_scene() for sc in mid_scenes[:2]]
    t2[1].scene.accel = 0
    with pytest.raises(rtcore.RtError) as e:
        ctx.batch_scratch_bytes(t2, p)
    assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    with pytest.raises(rtcore.RtError):
        ctx.batch_plan(table, batch_params(1, 0, SEED), scratch, nb)


def test_batch_with_octant_binning_gives_the_same_images(ctx, mid_scenes):
    import rtcore
    import torch
    from rtcore.batch import batch_params
    base, _ = _plan_run(ctx, mid_scenes, 2)
    p = batch_params(2, 8, SEED)
    p.flags = rtcore.RT_PT_OCTANT_BINNING
    for sc in mid_scenes:
        sc.accum.zero_()
    table = [sc.batch_scene() for sc in mid_scenes]
    nb = ctx.batch_scratch_bytes(table, p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    plan = ctx.batch_plan(table, p, scratch, nb)
    plan.launch(0)
    ctx.sync()
    plan.close()
    for sc, b in zip(mid_scenes, base):
        assert host(sc.accum).tobytes() == b.tobytes()
