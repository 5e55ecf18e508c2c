"""GPU parity of the acceleration-structure build (through the C ABI):
Morton keys, sort order, radix tree and the final BVH8 bytes are bit-exact
against the CPU oracle."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import (GpuBlas, GpuTlas, compare_accels, dev, header, host, ptr_of, radix_tree_canonical, ref8_instances,
                     ref8_items)

pytestmark = pytest.mark.gpu

M30 = 1 << 8


def soup(n, seed=21):
    import rtcore.scenes as S
    v, i = S.soup(seed, n)
    return [(v, i, None)]


@pytest.mark.parametrize("n,flags", [(0, 0), (1, 0), (2, 0), (3, 0), (4, 0), (9, 0), (100, 0), (4097, 0),
                                     (20000, 0), (250000, 0), (20000, M30), (250000, M30)])
def test_blas_bit_exact(ctx, orc, n, flags):
    items = soup(n)
    g = GpuBlas(ctx, items, flags)
    o, rc = orc.build_blas(items, flags)
    assert rc == 0
    compare_accels(g.bytes(), o, 48)


@pytest.mark.parametrize("n", [9, 20000, 250000])
@pytest.mark.parametrize("width", [4, 6])
def test_narrow_blas_bit_exact(ctx, orc, n, width):
    """RT_BUILD_WIDTH(4..7): trees of at most `width` children per node,
    byte-identical to the oracle's."""
    import rtcore
    items = soup(n, seed=8)
    flags = rtcore.build_width(width)
    g = GpuBlas(ctx, items, flags)
    o, rc = orc.build_blas(items, flags)
    assert rc == 0
    compare_accels(g.bytes(), o, 48)


def test_invalid_width_rejected(ctx):
    import rtcore
    for w in (2, 3, 9):
        with pytest.raises(rtcore.RtError) as e:
            GpuBlas(ctx, soup(50), rtcore.build_width(w))
        assert e.value.code == rtcore.RT_ERR_INVALID_ARG


def test_blas_stages_bit_exact(ctx, orc):
    """Sorted keys and primitive ids byte for byte; the binary radix tree
    node for node (the oracle numbers its nodes top-down, the GPU's
    bottom-up build numbers internal node i by its split between keys i and
    i + 1: the trees are compared by key ranges)."""
    import rtcore
    n = 50000
    items = soup(n, seed=5)
    g = GpuBlas(ctx, items)
    o, rc, (ks, ids, bn) = orc.build_blas(items, 0, debug=True)
    koff, ioff, boff = rtcore.blas_scratch_layout(n)
    s = host(g.scratch)
    np.testing.assert_array_equal(s[koff:koff + 8 * n].view(np.uint64), ks)
    np.testing.assert_array_equal(s[ioff:ioff + 4 * n].view(np.uint32), ids)
    gb = s[boff:boff + 16 * (n - 1)].view(np.uint32).reshape(-1, 4)
    np.testing.assert_array_equal(radix_tree_canonical(gb), radix_tree_canonical(bn))
    # internal node i splits between keys i and i + 1
    left = gb[:, 0].astype(np.int64)
    leaf = (left & 0x80000000) != 0
    left_last = np.where(leaf, left & 0x7FFFFFFF, gb[np.where(leaf, 0, left), 3])
    assert np.array_equal(left_last, np.arange(n - 1))


def test_blas_duplicates_degenerates_and_bad_indices(ctx, orc):
    # 300 identical triangles (equal Morton keys), 50 zero-area, 1 NaN vertex
    base = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    v = np.concatenate([np.tile(base, (300, 1)), np.tile(np.array([[0.5, 0.5, 0.5]] * 3, np.float32), (50, 1)),
                        np.array([[np.nan, 0, 0], [1, 1, 1], [0, 1, 1]], np.float32)])
    items = [(v, None, None)]
    g = GpuBlas(ctx, items)
    o, rc = orc.build_blas(items)
    compare_accels(g.bytes(), o, 48)
    # an index beyond max_vertex: the triangle is inactive, the build and
    # rt_sync report RT_ERR_BOUNDS, nothing is read out of range
    import rtcore
    bad = [(base, np.array([[0, 1, 2], [0, 1, 9]], np.uint32), None)]
    with pytest.raises(rtcore.RtError) as e:
        GpuBlas(ctx, bad)
    assert e.value.code == rtcore.RT_ERR_BOUNDS
    o2, rc2 = orc.build_blas(bad)
    assert rc2 == rtcore.RT_ERR_BOUNDS


@pytest.mark.parametrize("seed,frac", [(1, 1.0), (3, 1.0), (7, 0.5), (11, 0.5)])
def test_blas_extreme_coordinates_bit_exact(ctx, orc, seed, frac):
    """Vertices at +-1e30..3e38 mixed with unit-cube ones: box centres
    overflow, so some octant-slot costs are inf - inf = NaN.  These seeds
    make the slot assignment meet a NaN both as the first (child, slot) pair
    of a round -- which the sequential scan then keeps -- and after it (where
    it never wins); the eight-lane assignment must make the same choices."""
    rng = np.random.default_rng(seed)
    big = np.array([-3.0e38, -1.7e38, -1e30, 1e30, 1.7e38, 3.0e38], np.float32)
    nb = int(600 * frac)
    v = np.concatenate([rng.choice(big, size=(nb * 3, 3)).astype(np.float32),
                        rng.uniform(0, 1, size=((600 - nb) * 3, 3)).astype(np.float32)])
    idx = rng.permutation(len(v)).astype(np.uint32).reshape(-1, 3)
    items = [(v, idx, None)]
    g = GpuBlas(ctx, items)
    o, rc = orc.build_blas(items)
    assert rc == 0
    compare_accels(g.bytes(), o, 48)


@pytest.mark.parametrize("kind,flags", [("box", M30), ("all_large", 0), ("half_large", 0), ("half_large", M30)])
def test_blas_large_primitives_bit_exact(ctx, orc, kind, flags):
    """Primitives longer than RT_LARGE_PRIM_FRACTION of the centroid bounds
    take the key bit above the Morton code (bit 63, or bit 31 with 30-bit
    keys): a room's walls among small objects, a scene of large triangles
    only, and an even mix -- bit-exact with the oracle."""
    import rtcore.scenes as S
    rng = np.random.default_rng(17)
    if kind == "box":
        v, i, _, _ = S.box(S.SEED_BASE + 3, 3, 6)
    else:
        n_big = 400 if kind == "all_large" else 200
        c = rng.uniform(0, 1, size=(n_big, 1, 3)).astype(np.float32)
        big = (c + rng.uniform(-0.6, 0.6, size=(n_big, 3, 3))).astype(np.float32).reshape(-1, 3)
        parts = [big]
        if kind == "half_large":
            c2 = rng.uniform(0, 1, size=(200, 1, 3)).astype(np.float32)
            parts.append((c2 + rng.uniform(-0.01, 0.01, size=(200, 3, 3))).astype(np.float32).reshape(-1, 3))
        v = np.concatenate(parts)
        i = np.arange(len(v), dtype=np.uint32).reshape(-1, 3)
    items = [(v, i, None)]
    g = GpuBlas(ctx, items, flags)
    o, rc = orc.build_blas(items, flags)
    assert rc == 0
    compare_accels(g.bytes(), o, 48)


def test_blas_box_scene_bit_exact(ctx, orc):
    import rtcore.scenes as S
    v, i, tm, m = S.box(S.SEED_BASE + 3, 6, 12)
    items = [(v, i, None)]
    g = GpuBlas(ctx, items)
    o, _ = orc.build_blas(items)
    compare_accels(g.bytes(), o, 48)


def test_blas_geometries_with_transforms(ctx, orc):
    items = ref8_items() + soup(500, seed=2) + [(soup(64, seed=4)[0][0], None,
                                                 np.array([[0.5, 0.1, 0, 3], [0, 2, 0, -1], [0.2, 0, 1, 0.25]],
                                                          np.float32))]
    g = GpuBlas(ctx, items)
    o, _ = orc.build_blas(items)
    compare_accels(g.bytes(), o, 48)


def test_tlas_bit_exact(ctx, orc):
    g = GpuBlas(ctx, ref8_items())
    ob, _ = orc.build_blas(ref8_items())
    compare_accels(g.bytes(), ob, 48)
    gt = GpuTlas(ctx, ref8_instances([g.addr, g.addr]))
    ot, rc = orc.build_tlas(ref8_instances([ptr_of(ob), ptr_of(ob)]))
    assert rc == 0
    compare_accels(gt.bytes(), ot, 80, ignore_ref=True)


def test_tlas_many_instances(ctx, orc):
    """300 instances with rotations/scales over two BLASes."""
    from oracle import INSTANCE_DTYPE
    a_items, b_items = soup(200, seed=8), ref8_items()
    ga, gb = GpuBlas(ctx, a_items), GpuBlas(ctx, b_items)
    oa, _ = orc.build_blas(a_items)
    ob, _ = orc.build_blas(b_items)
    rng = np.random.default_rng(3)
    n = 300
    inst_g = np.zeros(n, INSTANCE_DTYPE)
    for k in range(n):
        ang = rng.uniform(0, 6.28)
        s = rng.uniform(0.5, 2)
        m = np.array([[np.cos(ang) * s, -np.sin(ang) * s, 0, rng.uniform(-5, 5)],
                      [np.sin(ang) * s, np.cos(ang) * s, 0, rng.uniform(-5, 5)],
                      [0, 0, s, rng.uniform(-5, 5)]], np.float32)
        inst_g[k]["transform"] = m
        inst_g[k]["custom_index_and_mask"] = k | (0xFF << 24)
        inst_g[k]["sbt_offset_and_flags"] = (k % 4) | (1 << 24)
    inst_o = inst_g.copy()
    inst_g["accel_ref"] = [ga.addr if k % 3 else gb.addr for k in range(n)]
    inst_o["accel_ref"] = [ptr_of(oa) if k % 3 else ptr_of(ob) for k in range(n)]
    gt = GpuTlas(ctx, inst_g)
    ot, _ = orc.build_tlas(inst_o)
    compare_accels(gt.bytes(), ot, 80, ignore_ref=True)


@pytest.mark.parametrize("n", [1, 4095, 4096, 4097, 100003, 1 << 20])
@pytest.mark.parametrize("dist", ["random", "equal", "few", "descending"])
def test_sort_pairs_matches_stable_sort(ctx, orc, n, dist):
    import rtcore
    import torch
    rng = np.random.default_rng(n)
    if dist == "random":
        keys = rng.integers(0, 1 << 63, n, dtype=np.uint64)
    elif dist == "equal":
        keys = np.full(n, 0x123456789, np.uint64)
    elif dist == "few":
        keys = rng.integers(0, 4, n, dtype=np.uint64) << np.uint64(40)
    else:
        keys = np.arange(n, 0, -1, dtype=np.uint64)
    vals = np.arange(n, dtype=np.uint32)
    for bits in (64, 30, 20):
        mask = np.uint64((1 << bits) - 1) if bits < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
        kd, vd = dev(keys), dev(vals)
        nb = rtcore.sort_scratch_bytes(n, bits)
        scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
        ctx.sort_pairs(kd, vd, n, bits, scratch, nb)
        ctx.sync()
        order = np.argsort(keys & mask, kind="stable")
        np.testing.assert_array_equal(host(vd).view(np.uint32), vals[order])
        np.testing.assert_array_equal(host(kd).view(np.uint64), keys[order])


def test_build_argument_errors(ctx):
    import rtcore
    import torch
    items = soup(1000)
    g = GpuBlas(ctx, items)
    geo = rtcore.GeometryTriangles()
    vd = dev(items[0][0])
    idd = dev(items[0][1])
    geo.vertices, geo.vertex_stride, geo.max_vertex = vd.data_ptr(), 12, 2999
    geo.index_type, geo.indices, geo.tri_count, geo.flags = 1, idd.data_ptr(), 1000, 1
    sz = ctx.blas_sizes([1000])
    acc = torch.empty(sz.accel_bytes, dtype=torch.uint8, device="cuda")
    scr = torch.empty(sz.scratch_bytes, dtype=torch.uint8, device="cuda")
    cases = [
        (dict(accel_bytes=sz.accel_bytes - 256), rtcore.RT_ERR_OOM),
        (dict(scratch_bytes=sz.scratch_bytes - 1), rtcore.RT_ERR_OOM),
        (dict(flags=M30 | (1 << 9)), rtcore.RT_ERR_INVALID_ARG),
        (dict(accel=acc.data_ptr() + 16), rtcore.RT_ERR_INVALID_ARG),
    ]
    for over, code in cases:
        kw = dict(accel=acc, accel_bytes=sz.accel_bytes, scratch=scr, scratch_bytes=sz.scratch_bytes, flags=0)
        kw.update(over)
        with pytest.raises(rtcore.RtError) as e:
            ctx.build_blas([geo], kw["flags"], kw["accel"], kw["accel_bytes"], kw["scratch"], kw["scratch_bytes"])
        assert e.value.code == code
    ctx.sync()
    # the earlier good build is intact
    assert header(g.bytes())["status"] == 0
    nodes, prims, depth = ctx.accel_info(g.accel)
    assert prims == 1000 and 1 <= nodes <= 999 and depth >= 2
