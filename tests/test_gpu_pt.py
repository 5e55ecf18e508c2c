"""GPU parity of the wavefront path tracer: the image accumulated by
rt_path_trace equals the CPU oracle's bit for bit (same BVH8, same traversal,
same per-pixel random streams, same float operation order)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuBlas, dev, host

pytestmark = pytest.mark.gpu


def _scene(ctx, n_spheres, freq, seed=0x5EED0003):
    import rtcore
    import rtcore.scenes as S
    v, i, tm, m = S.box(seed, n_spheres, freq)
    lights = S.emissive_lights(v, i, tm, m)
    blas = GpuBlas(ctx, [(v, i, None)])
    keep = [dev(tm), dev(m), dev(lights)]
    sc = rtcore.PtScene(blas.addr, keep[0].data_ptr(), keep[1].data_ptr(), len(m), keep[2].data_ptr(), len(lights))
    return (v, i, tm, m, lights), blas, sc, keep


def _params(w, h, spp, offset=0, depth=8, rr=3, seed=0x5EED0003):
    import rtcore
    import rtcore.scenes as S
    cam = rtcore.Camera(S.BOX_CAMERA[0], S.BOX_CAMERA[1])
    return rtcore.PtParams(cam, w, h, spp, offset, depth, rr, seed, 1e-4, 0)


def _run(ctx, sc, p, accum=None):
    import torch
    nb = ctx.pt_scratch_bytes(p)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    if accum is None:
        accum = torch.zeros(p.width * p.height * 16, dtype=torch.uint8, device="cuda")
    ctx.path_trace(sc, p, accum, scratch, nb)
    ctx.sync()
    return accum, scratch


@pytest.mark.parametrize("n_spheres,freq,w,h,spp", [(0, 1, 32, 24, 8), (6, 8, 64, 48, 4), (12, 16, 96, 64, 2)])
def test_path_trace_bit_exact(ctx, orc, n_spheres, freq, w, h, spp):
    import rtcore.scenes as S
    (v, i, tm, m, lights), blas, sc, keep = _scene(ctx, n_spheres, freq)
    p = _params(w, h, spp)
    acc, scratch = _run(ctx, sc, p)
    g = host(acc).view(np.float32).reshape(h, w, 4)
    ob, _ = orc.build_blas([(v, i, None)])
    o = orc.path_trace(ob, tm, m, lights, S.BOX_CAMERA, w, h, spp, 8, 3, 0x5EED0003, 1e-4)
    if g.tobytes() != o.tobytes():
        diff = np.abs(g - o).max(axis=2)
        k = np.argwhere(diff > 0)
        raise AssertionError(f"{len(k)} pixels differ, max {diff.max()}, first at {k[0]}: gpu {g[tuple(k[0])]} "
                             f"oracle {o[tuple(k[0])]}")
    ext, shadow = ctx.pt_ray_counts(p, len(lights), scratch)
    assert ext >= w * h * spp and shadow > 0


def test_progressive_and_depth_limits(ctx, orc):
    import rtcore.scenes as S
    (v, i, tm, m, lights), blas, sc, keep = _scene(ctx, 4, 6)
    w, h = 40, 30
    one, _ = _run(ctx, sc, _params(w, h, 5))
    acc, _ = _run(ctx, sc, _params(w, h, 2))
    _run(ctx, sc, _params(w, h, 3, offset=2), accum=acc)
    assert host(one).tobytes() == host(acc).tobytes()
    ob, _ = orc.build_blas([(v, i, None)])
    for depth, rr in ((1, 99), (2, 0), (16, 1)):
        g, _ = _run(ctx, sc, _params(w, h, 2, depth=depth, rr=rr))
        o = orc.path_trace(ob, tm, m, lights, S.BOX_CAMERA, w, h, 2, depth, rr, 0x5EED0003, 1e-4)
        assert host(g).view(np.float32).tobytes() == o.tobytes(), (depth, rr)


def test_octant_binning_does_not_change_images(ctx, orc):
    """Bounce rays traced in shading order (the default) or grouped by
    direction octant (RT_PT_OCTANT_BINNING): the same image bit for bit, and
    the oracle's."""
    import rtcore
    import rtcore.scenes as S
    (v, i, tm, m, lights), blas, sc, keep = _scene(ctx, 10, 12)
    w, h = 96, 72
    binned, _ = _run(ctx, sc, _params(w, h, 3))
    p = _params(w, h, 3)
    p.flags = rtcore.RT_PT_OCTANT_BINNING
    plain, _ = _run(ctx, sc, p)
    assert host(binned).tobytes() == host(plain).tobytes()
    ob, _ = orc.build_blas([(v, i, None)])
    o = orc.path_trace(ob, tm, m, lights, S.BOX_CAMERA, w, h, 3, 8, 3, 0x5EED0003, 1e-4)
    assert host(binned).view(np.float32).tobytes() == o.tobytes()
