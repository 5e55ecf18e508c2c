"""GPU parity of traversal and of the sample pipeline (through the C ABI).

The GPU and the oracle traverse the same (bit-exact) BVH8 in the same order
with the same FP32 operations, so hits, occlusion and traversal statistics
are compared bit for bit; the oracle itself is checked against brute force
and float64 in test_oracle.py."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import (GpuBlas, GpuTlas, dev, golden, gpu_trace_any, gpu_trace_closest, gpu_trace_stats, host,
                     ref8_instances, ref8_items, ptr_of, single_instance)

pytestmark = pytest.mark.gpu
REPO = Path(__file__).resolve().parent.parent


def soup(n, seed=31):
    import rtcore.scenes as S
    v, i = S.soup(seed, n)
    return [(v, i, None)]


def ray_mix(orc, n_inc, w, h, seed=13, cam=((0.5, 0.5, 2.5), 60.0)):
    import rtcore.scenes as S
    inc = S.incoherent_rays(seed, n_inc, (0, 0, 0), (1, 1, 1), 1e30)
    prim = orc.primary_rays(cam, w, h, 0.0, 100.0)
    return np.concatenate([inc, prim])


@pytest.fixture(scope="module")
def soup_scene(ctx, orc):
    items = soup(200000)
    g = GpuBlas(ctx, items)
    o, _ = orc.build_blas(items)
    return items, g, o


def test_closest_and_any_bit_exact(ctx, orc, soup_scene):
    items, g, o = soup_scene
    rays = ray_mix(orc, 60000, 256, 192)
    hg, xg = gpu_trace_closest(ctx, g.addr, rays, ext=True)
    ho, so, xo = orc.trace_closest(o, rays, ext=True)
    assert hg.tobytes() == ho.tobytes()
    assert xg.tobytes() == xo.tobytes()
    assert (hg["prim"] != 0xFFFFFFFF).sum() > 20000
    og = gpu_trace_any(ctx, g.addr, rays)
    oo, _ = orc.trace_any(o, rays)
    np.testing.assert_array_equal(og, oo)
    np.testing.assert_array_equal(gpu_trace_stats(ctx, g.addr, rays), so)


def test_shadow_rays_and_ranges(ctx, orc, soup_scene):
    """Any-hit rays toward a point light from primary hit points, plus rays
    with tmin > 0 and tiny tmax."""
    items, g, o = soup_scene
    prim = orc.primary_rays(((0.5, 0.5, 2.5), 60.0), 200, 150)
    hp, _ = orc.trace_closest(o, prim)
    hit = hp["prim"] != 0xFFFFFFFF
    p = prim["org"][hit] + hp["t"][hit, None] * prim["dir"][hit]
    sh = np.zeros(hit.sum(), prim.dtype)
    sh["org"] = p + np.float32(1e-4) * np.float32([0, 0, 1])
    sh["dir"] = np.float32([0.5, 2.0, 0.5]) - sh["org"]
    sh["tmin"] = 0.0
    sh["tmax"] = 1.0
    np.testing.assert_array_equal(gpu_trace_any(ctx, g.addr, sh), orc.trace_any(o, sh)[0])
    rr = ray_mix(orc, 20000, 64, 48)
    rr["tmin"] = 0.05
    rr["tmax"] = np.where(np.arange(len(rr)) % 2 == 0, 0.3, 1e30).astype(np.float32)
    assert gpu_trace_closest(ctx, g.addr, rr).tobytes() == orc.trace_closest(o, rr)[0].tobytes()


def test_box_scene_closest(ctx, orc):
    import rtcore.scenes as S
    v, i, tm, m = S.box(S.SEED_BASE + 3, 8, 16)
    items = [(v, i, None)]
    g = GpuBlas(ctx, items)
    o, _ = orc.build_blas(items)
    rays = orc.primary_rays(((0.0, 0.0, 0.95), 60.0), 320, 240)
    inc = S.incoherent_rays(4, 30000, (-0.9, -0.9, -0.9), (0.9, 0.9, 0.9), 1e30)
    rays = np.concatenate([rays, inc])
    hg = gpu_trace_closest(ctx, g.addr, rays)
    assert hg.tobytes() == orc.trace_closest(o, rays)[0].tobytes()
    assert np.all(hg["prim"] != 0xFFFFFFFF)  # closed box: every ray hits


def test_tlas_trace_ids(ctx, orc):
    import rtcore.scenes as S
    g = GpuBlas(ctx, ref8_items())
    ob, _ = orc.build_blas(ref8_items())
    gt = GpuTlas(ctx, ref8_instances([g.addr, g.addr]))
    ot, _ = orc.build_tlas(ref8_instances([ptr_of(ob), ptr_of(ob)]))
    rays = orc.primary_rays(S.REF8_CAMERA, 300, 200)
    hg, xg = gpu_trace_closest(ctx, gt.addr, rays, ext=True)
    ho, so, xo = orc.trace_closest(ot, rays, ext=True)
    assert hg.tobytes() == ho.tobytes() and xg.tobytes() == xo.tobytes()
    assert set(np.unique(xg["instance_id"])) >= {0, 1}
    np.testing.assert_array_equal(gpu_trace_any(ctx, gt.addr, rays), orc.trace_any(ot, rays)[0])
    np.testing.assert_array_equal(gpu_trace_stats(ctx, gt.addr, rays), so)


def _instance_field(n, seed):
    """n rotated, scaled and translated instances (ids 0..n-1): every 7th
    masked out, pairs (10k, 10k+1) identical so their hits tie on t."""
    from oracle import INSTANCE_DTYPE
    rng = np.random.default_rng(seed)
    inst = np.zeros(n, INSTANCE_DTYPE)
    for k in range(n):
        if k % 10 == 1:
            inst[k] = inst[k - 1]
        else:
            ang = rng.uniform(0, 6.28)
            s = rng.uniform(0.5, 2)
            inst[k]["transform"] = np.array([[np.cos(ang) * s, -np.sin(ang) * s, 0, rng.uniform(-3, 3)],
                                             [np.sin(ang) * s, np.cos(ang) * s, 0, rng.uniform(-3, 3)],
                                             [0, 0, s, rng.uniform(-3, 3)]], np.float32)
        mask = 0 if k % 7 == 3 else 0xFF
        inst[k]["custom_index_and_mask"] = (k * 3) | (mask << 24)
        inst[k]["sbt_offset_and_flags"] = (k % 4) | (1 << 24)
    return inst


@pytest.mark.parametrize("n_inst", [1, 37, 300])
def test_tlas_instance_field_trace(ctx, orc, n_inst):
    """The persistent two-level walk against the oracle: overlapping
    instances of three BLASes (a soup, the sample's quads, an empty one),
    masked and duplicated instances; hits, extended ids, occlusion and
    traversal statistics bit for bit."""
    import rtcore.scenes as S
    items = [soup(3000, seed=5), ref8_items(), [(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), None)]]
    gb = [GpuBlas(ctx, it) for it in items]
    ob = [orc.build_blas(it)[0] for it in items]
    inst_g = _instance_field(n_inst, seed=n_inst)
    inst_o = inst_g.copy()
    which = [k % 3 if k % 11 else 2 for k in range(n_inst)]
    for k in range(n_inst):
        if k % 10 == 1:
            which[k] = which[k - 1]  # the duplicate of instance k - 1, same BLAS
    if n_inst == 1:
        which = [1]
    inst_g["accel_ref"] = [gb[w].addr for w in which]
    inst_o["accel_ref"] = [ptr_of(ob[w]) for w in which]
    gt = GpuTlas(ctx, inst_g)
    ot, rc = orc.build_tlas(inst_o)
    assert rc == 0
    inc = S.incoherent_rays(77 + n_inst, 40000, (-4, -4, -4), (4, 4, 4), 1e30)
    prim = orc.primary_rays(((0.0, 0.0, 12.0), 60.0), 160, 120, 0.0, 100.0)
    rays = np.concatenate([inc, prim])
    hg, xg = gpu_trace_closest(ctx, gt.addr, rays, ext=True)
    ho, so, xo = orc.trace_closest(ot, rays, ext=True)
    assert hg.tobytes() == ho.tobytes()
    assert xg.tobytes() == xo.tobytes()
    assert np.count_nonzero(hg["prim"] != 0xFFFFFFFF) > 500
    np.testing.assert_array_equal(gpu_trace_any(ctx, gt.addr, rays), orc.trace_any(ot, rays)[0])
    np.testing.assert_array_equal(gpu_trace_stats(ctx, gt.addr, rays), so)
    np.testing.assert_array_equal(gpu_trace_stats(ctx, gt.addr, rays, any_hit=True), orc.trace_any(ot, rays)[1])


def _pipeline_image(ctx, accel_addr, camera, w, h, chit, sbt_colors=None):
    import rtcore
    import torch
    p = rtcore.sample_pipeline(chit)
    sbt = None
    keep = None
    if sbt_colors is not None:
        keep = dev(np.asarray(sbt_colors, np.float32))
        sbt = rtcore.Sbt(keep.data_ptr(), len(sbt_colors), 3)
    cam = rtcore.Camera((camera[0][0], camera[0][1], camera[0][2]), camera[1])
    out = torch.empty(w * h * 16, dtype=torch.uint8, device="cuda")
    ctx.trace_rays(p, sbt, accel_addr, cam, out, w, h, 1)
    ctx.sync()
    return host(out).view(np.float32).reshape(h, w, 4)


def _golden_check(img, gd, tol=1e-5):
    px = np.array(gd["pixels"], np.float64)
    xs, ys = px[:, 0].astype(int), px[:, 1].astype(int)
    err = np.abs(img[ys, xs, :3] - px[:, 2:5]).max(1)
    assert err.max() <= tol, err.max()
    assert np.all(img[ys, xs, 3] == 0.0)


def test_trace_rays_reference_scene(ctx, orc):
    """vkCmdTraceRaysKHR of the sample: bit-exact with the oracle and within
    1e-5 of the float64 known answers."""
    import rtcore.scenes as S
    g = GpuBlas(ctx, ref8_items())
    gt = GpuTlas(ctx, ref8_instances([g.addr, g.addr]))
    img = _pipeline_image(ctx, gt.addr, S.REF8_CAMERA, *S.REF8_SIZE, 0, S.REF8_SBT_COLORS)
    ob, _ = orc.build_blas(ref8_items())
    ot, _ = orc.build_tlas(ref8_instances([ptr_of(ob), ptr_of(ob)]))
    oimg, rc = orc.trace_rays(ot, S.REF8_CAMERA, *S.REF8_SIZE, chit=0, sbt_colors=S.REF8_SBT_COLORS)
    assert img.tobytes() == oimg.tobytes()
    _golden_check(img, golden()["ref8"])


def test_trace_rays_single_triangle(ctx, orc):
    import rtcore.scenes as S
    items = [(S.TRI1_VERTICES, S.TRI1_INDICES, None)]
    g = GpuBlas(ctx, items)
    # traced through a BLAS directly and through a one-instance TLAS
    gt = GpuTlas(ctx, single_instance(g.addr))
    for addr in (g.addr, gt.addr):
        img = _pipeline_image(ctx, addr, S.TRI1_CAMERA, *S.TRI1_SIZE, 1)
        _golden_check(img, golden()["tri"])
    o, _ = orc.build_blas(items)
    oimg, _ = orc.trace_rays(o, S.TRI1_CAMERA, *S.TRI1_SIZE, chit=1)
    assert img.tobytes() == oimg.tobytes()


def test_primary_ray_generation(ctx, orc):
    import rtcore
    import torch
    cam = ((0.5, 0.5, 2.5), 60.0)
    w, h = 333, 217
    out = torch.empty(w * h * 32, dtype=torch.uint8, device="cuda")
    ctx.generate_primary_rays(rtcore.Camera(cam[0], cam[1]), w, h, 0.0, 100.0, out)
    ctx.sync()
    assert host(out).tobytes() == orc.primary_rays(cam, w, h, 0.0, 100.0).tobytes()


def test_empty_structure_misses(ctx, orc):
    g = GpuBlas(ctx, [(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), None)])
    rays = ray_mix(orc, 1000, 16, 16)
    hg = gpu_trace_closest(ctx, g.addr, rays)
    assert np.all(hg["prim"] == 0xFFFFFFFF) and np.all(np.isinf(hg["t"]))
    assert not gpu_trace_any(ctx, g.addr, rays).any()


def test_tuning_does_not_change_results(ctx, orc, soup_scene):
    items, g, o = soup_scene
    rays = ray_mix(orc, 30000, 128, 96, seed=3)
    ref = orc.trace_closest(o, rays)[0].tobytes()
    t0 = ctx.get_tuning()
    try:
        for bps, batch in ((1, 32), (4, 1), (8, 16), (16, 8)):
            ctx.set_tuning(bps, batch)
            assert gpu_trace_closest(ctx, g.addr, rays).tobytes() == ref
    finally:
        ctx.set_tuning(t0.blocks_per_sm, t0.batch_rays)


def test_trace_rays_argument_errors(ctx):
    import rtcore
    import torch
    g = GpuBlas(ctx, ref8_items())
    out = torch.empty(16 * 16, dtype=torch.uint8, device="cuda")
    cam = rtcore.Camera((0, 0, 10), 60.0)
    with pytest.raises(rtcore.RtError) as e:
        ctx.trace_rays(rtcore.sample_pipeline(), None, g.addr, cam, out, 4, 4, 2)
    assert e.value.code == rtcore.RT_ERR_UNSUPPORTED
    p = rtcore.sample_pipeline()
    p.chit = 7
    with pytest.raises(rtcore.RtError) as e:
        ctx.trace_rays(p, None, g.addr, cam, out, 4, 4, 1)
    assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    # a hit whose SBT record is out of range: black pixel + RT_ERR_BOUNDS,
    # reported by rt_sync, no out-of-range read
    p = rtcore.sample_pipeline(rtcore.RT_CHIT_SBT_COLOR)
    out8 = torch.empty(8 * 8 * 16, dtype=torch.uint8, device="cuda")
    with pytest.raises(rtcore.RtError) as e:
        ctx.trace_rays(p, None, g.addr, rtcore.Camera((0, 0, 10), 60.0), out8, 8, 8, 1)
        ctx.sync()
    assert e.value.code == rtcore.RT_ERR_BOUNDS
    img = host(out8).view(np.float32).reshape(8, 8, 4)
    assert (img[..., :3] == 0).all(axis=2).any()  # the hit pixels are black


def test_rt_sample_executable(rtlib, orc, tmp_path):
    """The headless drop-in of the sample's main(): its raw RGBA32F frame is
    the oracle's image, and its PPM is the 8-bit quantisation of it."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rtcore.scenes as S
    exe = REPO / "build-up-phase_gb300" / "_build" / "rt_sample"
    raw = tmp_path / "f.bin"
    ppm = tmp_path / "f.ppm"
    r = subprocess.run([str(exe), "--scene", "ref8", "--raw", str(raw), "--out", str(ppm)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    img = np.fromfile(raw, np.float32).reshape(800, 1200, 4)
    ob, _ = orc.build_blas(ref8_items())
    ot, _ = orc.build_tlas(ref8_instances([ptr_of(ob), ptr_of(ob)]))
    oimg, _ = orc.trace_rays(ot, S.REF8_CAMERA, *S.REF8_SIZE, chit=0, sbt_colors=S.REF8_SBT_COLORS)
    assert img.tobytes() == oimg.tobytes()
    body = ppm.read_bytes()
    hdr = b"P6\n1200 800\n255\n"
    px = np.frombuffer(body[len(hdr):], np.uint8).reshape(800, 1200, 3)
    want = np.clip(np.rint(np.clip(oimg[..., :3], 0, 1) * np.float32(255)), 0, 255).astype(np.uint8)
    assert np.abs(px.astype(int) - want.astype(int)).max() <= 1


def test_rt_sample_obj_mesh(rtlib, orc, tmp_path):
    """rt_sample --obj: an OBJ file (the box scene written as text) loaded by
    rt_obj_load, built and traced by the drop-in sample, equals the oracle's
    image of the same arrays under one identity instance."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import rtcore.scenes as S
    from helpers import single_instance
    v, i, tm, m = S.box(S.SEED_BASE + 3, 6, 6)
    obj = tmp_path / "box.obj"
    S.write_obj(obj, v, i, tm)
    exe = REPO / "build-up-phase_gb300" / "_build" / "rt_sample"
    raw = tmp_path / "o.bin"
    cam = ((0.1, -0.2, 0.9), 70.0)
    r = subprocess.run([str(exe), "--obj", str(obj), "--camera", *map(str, cam[0]), str(cam[1]), "--width", "320",
                        "--height", "240", "--raw", str(raw), "--out", str(tmp_path / "o.ppm")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    img = np.fromfile(raw, np.float32).reshape(240, 320, 4)
    ob, _ = orc.build_blas([(v, i, None)])
    ot, _ = orc.build_tlas(single_instance(ptr_of(ob)))
    oimg, _ = orc.trace_rays(ot, cam, 320, 240, chit=1)
    assert img.tobytes() == oimg.tobytes()
    assert (img[..., 2] != np.float32(0.2)).mean() > 0.5  # the box fills the view


@pytest.mark.parametrize("n", [0, 1, 1000, (1 << 20) + 12345, 3 * (1 << 20) + 1])
def test_host_memory_rays(ctx, orc, n):
    """rt_trace_closest_host / rt_trace_any_host (rays and results in host
    memory: read and written in place where the device reaches them -- pinned,
    and pageable on a Grace system -- else chunked copies overlapping the
    traversal) give the device API's results, over repeated calls; pinned
    buffers forced to the staged path and a pinned buffer at an odd offset
    (staged) as well."""
    import torch
    import rtcore.scenes as S
    items = soup(50_000, seed=3)
    g = GpuBlas(ctx, items)
    rays = S.incoherent_rays(77, max(n, 1), (0, 0, 0), (1, 1, 1), 1e30)[:n]
    want = gpu_trace_closest(ctx, g.addr, rays) if n else np.zeros(0, np.uint8)
    want_occ = gpu_trace_any(ctx, g.addr, rays) if n else np.zeros(0, np.uint8)
    nb = max(ctx.trace_host_scratch_bytes(n), ctx.trace_host_scratch_bytes(n, True))
    scratch = torch.empty(max(nb, 256), dtype=torch.uint8, device="cuda")
    for pinned in (True, False):
        hr = torch.from_numpy(rays.view(np.uint8).copy() if n else np.zeros(32, np.uint8))
        hh = torch.full((max(n, 1) * 16,), 0xAB, dtype=torch.uint8)
        ho = torch.full((max(n, 1),), 7, dtype=torch.uint8)
        if pinned:
            hr, hh, ho = hr.pin_memory(), hh.pin_memory(), ho.pin_memory()
        for _ in range(2):
            ctx.trace_closest_host(g.addr, hr, hh, n, scratch, nb)
            ctx.trace_any_host(g.addr, hr, ho, n, scratch, nb)
        ctx.sync()
        if n:
            assert hh.numpy()[:n * 16].tobytes() == want.tobytes()
            assert ho.numpy()[:n].tobytes() == want_occ.tobytes()
    if n:
        # pinned buffers forced through the staged (copy) path
        import rtcore
        ctx.set_host_transfer(rtcore.RT_HOST_TRANSFER_STAGED)
        try:
            hr = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
            hh = torch.full((n * 16,), 0xAB, dtype=torch.uint8).pin_memory()
            ctx.trace_closest_host(g.addr, hr, hh, n, scratch, nb)
            ctx.sync()
            assert hh.numpy().tobytes() == want.tobytes()
            with pytest.raises(rtcore.RtError) as e:
                ctx.set_host_transfer(7)
            assert e.value.code == rtcore.RT_ERR_INVALID_ARG
        finally:
            ctx.set_host_transfer(rtcore.RT_HOST_TRANSFER_AUTO)
        # pinned but not 16-byte aligned: rays and hits one byte into their buffers
        hr1 = torch.zeros(n * 32 + 16, dtype=torch.uint8).pin_memory()
        hr1[1:1 + n * 32] = torch.from_numpy(rays.view(np.uint8).copy())
        hh1 = torch.full((n * 16 + 16,), 0xAB, dtype=torch.uint8).pin_memory()
        ctx.trace_closest_host(g.addr, hr1.data_ptr() + 1, hh1.data_ptr() + 1, n, scratch, nb)
        ctx.sync()
        assert hh1.numpy()[1:1 + n * 16].tobytes() == want.tobytes()


def test_host_memory_rays_small_scratch(ctx, orc):
    """The staged path (RT_HOST_TRANSFER_STAGED) from pageable buffers with a
    scratch sized for 5,000-ray chunks: 200,003 rays go round the four-slot
    ring in 41 chunks on three trace streams, closest and any-hit calls
    alternating on one scratch; results equal the device API's."""
    import torch
    import rtcore.scenes as S
    n = 200_003
    items = soup(50_000, seed=5)
    g = GpuBlas(ctx, items)
    rays = S.incoherent_rays(91, n, (0, 0, 0), (1, 1, 1), 1e30)
    want = gpu_trace_closest(ctx, g.addr, rays)
    want_occ = gpu_trace_any(ctx, g.addr, rays)
    nb = ctx.trace_host_scratch_bytes(5000)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    hr = torch.from_numpy(rays.view(np.uint8).copy())
    hh = torch.full((n * 16,), 0xAB, dtype=torch.uint8)
    ho = torch.full((n,), 7, dtype=torch.uint8)
    import rtcore
    ctx.set_host_transfer(rtcore.RT_HOST_TRANSFER_STAGED)
    try:
        for _ in range(3):
            ctx.trace_closest_host(g.addr, hr, hh, n, scratch, nb)
            ctx.trace_any_host(g.addr, hr, ho, n, scratch, nb)
        ctx.sync()
    finally:
        ctx.set_host_transfer(rtcore.RT_HOST_TRANSFER_AUTO)
    assert hh.numpy().tobytes() == want.tobytes()
    assert ho.numpy().tobytes() == want_occ.tobytes()


def test_full_size_soup_sampled(ctx, orc):
    """The 1M-triangle soup at full size: build bit-exact, and 2x2.07M rays
    traced on the GPU of which a seeded 40k sample is re-traced by the oracle
    bit for bit; every hit is in range."""
    import rtcore.scenes as S
    items = soup(1_000_000, seed=S.SEED_BASE + 2)
    g = GpuBlas(ctx, items)
    o, _ = orc.build_blas(items)
    gb = g.bytes()
    assert gb[:256].tobytes()[:48] == o[:256].tobytes()[:48]
    from helpers import compare_accels
    compare_accels(gb, o, 48)
    rays = np.concatenate([orc.primary_rays(((0.5, 0.5, 2.5), 60.0), 1920, 1080),
                           S.incoherent_rays(S.SEED_BASE + 2, 1920 * 1080, (0, 0, 0), (1, 1, 1), 1e30)])
    hg = gpu_trace_closest(ctx, g.addr, rays)
    hit = hg["prim"] != 0xFFFFFFFF
    assert np.all(hg["prim"][hit] < 1_000_000)
    assert np.all((hg["t"][hit] >= rays["tmin"][hit]) & (hg["t"][hit] <= rays["tmax"][hit]))
    idx = np.random.default_rng(0).choice(len(rays), 40000, replace=False)
    assert hg[idx].tobytes() == orc.trace_closest(o, rays[idx])[0].tobytes()
