"""GPU refit (rt_refit_blas / rt_refit_tlas) against the oracle's refit:
byte-identical structures after moving vertices, transforms and instances,
identity on unchanged inputs, rejection of inputs that do not match."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuBlas, GpuTlas, compare_accels, gpu_trace_closest, ptr_of, single_instance

pytestmark = pytest.mark.gpu


def _soup(n, seed=7):
    import rtcore.scenes as S
    return S.soup(seed, n)


def _moved(v, seed=3, amount=0.01):
    rng = np.random.default_rng(seed)
    return (v + rng.uniform(-amount, amount, v.shape)).astype(np.float32)


def _rays(orc, n, seed=11):
    import rtcore.scenes as S
    inc = S.incoherent_rays(seed, n, (0, 0, 0), (1, 1, 1), 1e30)
    prim = orc.primary_rays(((0.5, 0.5, 2.5), 60.0), 64, 48, 0.0, 100.0)
    return np.concatenate([inc, prim])


@pytest.mark.parametrize("n", [1, 2, 9, 1000, 100_000])
def test_blas_refit_matches_oracle(ctx, orc, n):
    v, i = _soup(n)
    xf = np.array([[1, 0, 0, 0.25], [0, 0.5, 0, 0], [0, 0, 1, -1]], np.float32)
    half = n // 2 + 1
    items = [(v, i, None), (v[:3 * half], i[:half], xf)]
    g = GpuBlas(ctx, items)
    built = g.bytes().copy()
    g.refit(ctx, items)  # unchanged inputs: the build itself
    assert g.bytes().tobytes() == built.tobytes()
    xf2 = xf.copy()
    xf2[:, 3] += (0.1, -0.2, 0.05)
    moved = [(_moved(v), i, None), (_moved(v[:3 * half], 5), i[:half], xf2)]
    g.refit(ctx, moved)
    o, _ = orc.build_blas(items)
    assert orc.refit_blas(o, moved) == 0
    compare_accels(g.bytes(), o, 48)
    rays = _rays(orc, 2000)
    assert gpu_trace_closest(ctx, g.addr, rays).tobytes() == orc.brute_closest(moved, rays, 32).tobytes()


def test_tlas_refit_matches_oracle(ctx, orc):
    v, i = _soup(3000)
    gb = GpuBlas(ctx, [(v, i, None)])
    ob, _ = orc.build_blas([(v, i, None)])

    def instances(ref, shift):
        inst = np.concatenate([single_instance(ref) for _ in range(40)])
        for k in range(40):
            inst[k]["transform"][:, 3] = ((k % 8) * 1.2, (k // 8) * 1.2 + shift * np.sin(k), shift * k * 0.01)
            inst[k]["custom_index_and_mask"] = k | (0xFF << 24)
        return inst

    gt = GpuTlas(ctx, instances(gb.addr, 0.0))
    ot, _ = orc.build_tlas(instances(ptr_of(ob), 0.0))
    built = gt.bytes().copy()
    gt.refit(ctx, instances(gb.addr, 0.0))
    assert gt.bytes().tobytes() == built.tobytes()
    gt.refit(ctx, instances(gb.addr, 0.3))
    assert orc.refit_tlas(ot, instances(ptr_of(ob), 0.3)) == 0
    compare_accels(gt.bytes(), ot, 80, ignore_ref=True)


def test_refit_rejects_other_inputs(ctx, orc):
    import rtcore
    v, i = _soup(200)
    g = GpuBlas(ctx, [(v, i, None)])
    before = g.bytes().copy()
    with pytest.raises(rtcore.RtError) as e:
        g.refit(ctx, [(v[:597], i[:199], None)])  # one triangle fewer
    assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    assert g.bytes().tobytes() == before.tobytes()
    with pytest.raises(rtcore.RtError) as e:  # the same 200 triangles as two geometries
        g.refit(ctx, [(v[:300], i[:100], None), (v[300:], i[100:] - 300, None)])
    assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    assert g.bytes().tobytes() == before.tobytes()
    with pytest.raises(rtcore.RtError) as e:  # more triangles than the structure holds: refused on the host
        g.refit(ctx, [(v, i, None), (v, i, None)])
    assert e.value.code == rtcore.RT_ERR_OOM
    assert g.bytes().tobytes() == before.tobytes()


def test_deforming_mesh_frames(ctx, orc):
    """A box scene whose spheres breathe over 6 frames: refit each frame and
    trace; every frame's hits equal the oracle's refit of the same frame."""
    import rtcore.scenes as S
    v, i, tm, m = S.box(S.SEED_BASE + 3, 8, 10)
    centre = v.mean(axis=0)
    g = GpuBlas(ctx, [(v, i, None)])
    o, _ = orc.build_blas([(v, i, None)])
    rays = np.concatenate([orc.primary_rays((S.BOX_CAMERA[0], S.BOX_CAMERA[1]), 96, 64, 0.0, 1e30),
                           S.incoherent_rays(5, 4000, (-0.9,) * 3, (0.9,) * 3, 1e30)])
    for f in range(1, 7):
        vf = (centre + (v - centre) * np.float32(1.0 + 0.03 * np.sin(f))).astype(np.float32)
        g.refit(ctx, [(vf, i, None)])
        assert orc.refit_blas(o, [(vf, i, None)]) == 0
        assert gpu_trace_closest(ctx, g.addr, rays).tobytes() == orc.trace_closest(o, rays)[0].tobytes()
