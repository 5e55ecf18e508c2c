"""CPU checks of the oracle's path tracer (the checker of the GPU one): its
sin/cos polynomials, a closed-form direct-lighting answer, determinism and
progressive accumulation."""
from __future__ import annotations

import math

import numpy as np


def test_polynomial_sincos_accuracy(orc):
    xs = np.linspace(-math.pi / 4, math.pi / 4, 2001, dtype=np.float32)
    err = 0.0
    for x in xs:
        s, c = orc.sincos_q(float(x))
        err = max(err, abs(s - math.sin(float(x))), abs(c - math.cos(float(x))))
    assert err < 3e-7  # truncation < 3e-8 plus float rounding


def _box(rtlib, n_spheres=3, freq=4, seed=0x5EED0003):
    import rtcore.scenes as S
    v, i, tm, m = S.box(seed, n_spheres, freq)
    lights = S.emissive_lights(v, i, tm, m)
    return v, i, tm, m, lights


def test_box_image_sane(orc, rtlib):
    """The box image is finite, non-negative, lit, and counts its samples;
    the red and green walls tint the left and right edges."""
    import rtcore.scenes as S
    v, i, tm, m, lights = _box(rtlib, 0, 1)
    accel, _ = orc.build_blas([(v, i, None)])
    acc = orc.path_trace(accel, tm, m, lights, S.BOX_CAMERA, 32, 24, 64, seed=1)
    img = acc[..., :3] / acc[..., 3:4]
    assert np.isfinite(acc).all() and (acc[..., :3] >= 0).all()
    assert np.all(acc[..., 3] == 64)
    assert img.mean() > 0.01
    left, right = img[:, :3].mean((0, 1)), img[:, -3:].mean((0, 1))
    assert left[0] > left[1] and right[1] > right[0]


def test_direct_lighting_closed_form(orc, rtlib):
    """A white floor (albedo 1) under a small square light of radiance Le at
    height h: with max_depth 1 the path tracer computes direct lighting only,
    so the floor radiance directly below the light converges to
    Le / pi * (solid-angle integral of cos_s cos_l / d^2) = Le * F where F is
    the analytic form factor of a square seen from a point on its axis."""
    a, h, Le = 0.05, 1.0, 10.0
    # the sample's camera basis always looks down -z, so the "floor" is the
    # wall z = 0 and the light a square at z = h facing -z (winding chosen so
    # that (v1 - v0) x (v2 - v0) points to -z); the camera sits between them
    wall = np.array([[-10, -10, 0], [10, -10, 0], [10, 10, 0], [-10, 10, 0]], np.float32)
    light = np.array([[-a, -a, h], [a, -a, h], [a, a, h], [-a, a, h]], np.float32)
    v = np.concatenate([wall, light])
    i = np.array([[0, 1, 2], [0, 2, 3], [4, 6, 5], [4, 7, 6]], np.uint32)
    from rtcore.scenes import MATERIAL_DTYPE, emissive_lights
    m = np.zeros(2, MATERIAL_DTYPE)
    m[0]["albedo"] = (1, 1, 1)
    m[1]["emission"] = (Le, Le, Le)
    tm = np.array([0, 0, 1, 1], np.uint32)
    lights = emissive_lights(v, i, tm, m)
    accel, _ = orc.build_blas([(v, i, None)])
    # the centre pixel of a 9x9 image looks exactly down the light's axis
    cam = ((0.0, 0.0, 0.5), 10.0)
    acc = orc.path_trace(accel, tm, m, lights, cam, 9, 9, 4096, max_depth=1, rr_depth=99, seed=7)
    assert np.all(light[:, 2] == h) and lights["v0"][:, 2].max() == h
    img = acc[..., :3] / acc[..., 3:4]
    # form factor from a differential area to a parallel square of side 2a
    # at distance h (on its axis): F = 4 * (1/(2 pi)) * [x/sqrt(1+x^2) atan(y/sqrt(1+x^2)) + y/sqrt(1+y^2)
    # atan(x/sqrt(1+y^2))] with x = y = a/h
    x = a / h
    f = (2.0 / math.pi) * (x / math.sqrt(1 + x * x) * math.atan(x / math.sqrt(1 + x * x)) +
                           x / math.sqrt(1 + x * x) * math.atan(x / math.sqrt(1 + x * x)))
    want = Le * f
    # the centre pixels look at floor points within a few cm of the axis
    centre = img[4, 4, 0]
    assert abs(centre - want) / want < 0.05, (centre, want)


def test_progressive_accumulation_equals_one_call(orc, rtlib):
    import rtcore.scenes as S
    v, i, tm, m, lights = _box(rtlib)
    accel, _ = orc.build_blas([(v, i, None)])
    one = orc.path_trace(accel, tm, m, lights, S.BOX_CAMERA, 24, 16, 6, seed=3)
    two = orc.path_trace(accel, tm, m, lights, S.BOX_CAMERA, 24, 16, 2, seed=3)
    orc.path_trace(accel, tm, m, lights, S.BOX_CAMERA, 24, 16, 4, seed=3, sample_offset=2, accum=two)
    assert one.tobytes() == two.tobytes()
    again = orc.path_trace(accel, tm, m, lights, S.BOX_CAMERA, 24, 16, 6, seed=3, threads=1)
    assert again.tobytes() == one.tobytes()


def test_pixel_subset_paths_equal_the_full_image(orc, rtlib):
    """orc_path_trace_pixels (the per-pixel paths the full-size GPU tests
    compare against) sums to orc_path_trace's image bit for bit; in the
    learned form, exactly the training pixels of each sample -- the residue
    class (pixel + offset) % stride == 0 -- that reach a second reflective
    vertex train, the other such pixels end in a query with the radiance they
    had before it, and a training path's radiance is the plain path's."""
    import rtcore.scenes as S
    v, i, tm, m = S.box(S.SEED_BASE + 3, 3, 6)
    lights = S.emissive_lights(v, i, tm, m)
    ob, rc = orc.build_blas([(v, i, None)])
    assert rc == 0
    w, h, spp, seed = 64, 48, 3, 99
    img = orc.path_trace(ob, tm, m, lights, S.BOX_CAMERA, w, h, spp, 8, 3, seed, 1e-4, sample_offset=5)
    px = np.arange(w * h, dtype=np.uint32)
    rec = orc.path_trace_pixels(ob, tm, m, lights, S.BOX_CAMERA, w, h, px, spp=spp, seed=seed, sample_offset=5)
    acc = np.zeros((w * h, 3), np.float32)
    for s in range(spp):
        acc = acc + rec["L"][:, s]
    assert acc.tobytes() == img.reshape(-1, 4)[:, :3].tobytes()
    assert (rec["kind"] == 0).all()
    stride = 7
    lrn = orc.path_trace_pixels(ob, tm, m, lights, S.BOX_CAMERA, w, h, px, spp=spp, seed=seed, sample_offset=5,
                                train_stride=stride)
    assert (lrn["kind"] == 1).any() and (lrn["kind"] == 2).any()
    for s in range(spp):
        k = lrn["kind"][:, s]
        reached = k > 0
        # the offset is drawn per sample: that sample's training pixels form one residue class
        classes = {int(p % stride) for p in np.nonzero(k == 2)[0]}
        assert len(classes) == 1, classes
        c = classes.pop()
        assert ((px % stride == c) == (k == 2))[reached].all()
        train = k == 2
        assert lrn["L"][train, s].tobytes() == rec["L"][train, s].tobytes()
        query = k == 1
        assert lrn["L_before"][query, s].tobytes() == lrn["L"][query, s].tobytes()


def test_oracle_generators_equal_the_library(orc, rtlib):
    """The oracle's restatement of the seeded soup and incoherent-ray
    generators writes the library's bytes at the benchmark's full sizes (1M
    triangles, 1920x1080 rays), so a CPU-only run can make the benchmark's
    inputs without loading the product library."""
    import rtcore.scenes as S
    seed = S.SEED_BASE + 2
    v, i = S.soup(seed, 1_000_000)
    vo, io = orc.scene_soup(seed, 1_000_000)
    assert v.tobytes() == vo.tobytes() and i.tobytes() == io.tobytes()
    for lo, hi, tmax in (((0, 0, 0), (1, 1, 1), 1e30), ((-0.99,) * 3, (0.99,) * 3, 1e30), ((0, 0, 0), (1, 2, 3), 5.0)):
        r = S.incoherent_rays(seed, 1920 * 1080, lo, hi, tmax)
        ro = orc.incoherent_rays(seed, 1920 * 1080, lo, hi, tmax)
        assert r.tobytes() == ro.tobytes()
