"""CPU tests of the oracle: pinned to the reference sample's known answers,
then used as the checker of the CUDA path.  No GPU needed."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import golden, header, nodes, prims, ref8_instances, ref8_items, ptr_of

BARY_TOL = 1e-5  # barycentric tolerance against float64


def _golden_check(img: np.ndarray, g: dict, bary_tol: float = BARY_TOL) -> None:
    px = np.array(g["pixels"], np.float64)
    xs, ys = px[:, 0].astype(int), px[:, 1].astype(int)
    got = img[ys, xs, :3].astype(np.float64)
    want = px[:, 2:5]
    assert np.all(img[ys, xs, 3] == 0.0), "alpha must be 0 (imageStore of vec4(hitValue, 0.0))"
    err = np.abs(got - want).max(axis=1)
    bad = np.nonzero(err > bary_tol)[0]
    assert len(bad) == 0, f"{len(bad)} golden pixels differ, first {px[bad[0]]} got {got[bad[0]]}"


def _ref8_oracle(orc):
    import rtcore.scenes as S
    blas, rc = orc.build_blas(ref8_items())
    assert rc == 0
    tlas, rc = orc.build_tlas(ref8_instances([ptr_of(blas), ptr_of(blas)]))
    assert rc == 0
    return blas, tlas


def test_golden_reference_scene(orc):
    """The sample's scene, camera, SBT and closest-hit predicate
    (main.cpp:676-695, 835-858, 1015, 1033-1091, 1310-1317)."""
    import rtcore.scenes as S
    blas, tlas = _ref8_oracle(orc)
    img, rc = orc.trace_rays(tlas, S.REF8_CAMERA, *S.REF8_SIZE, chit=0, sbt_colors=S.REF8_SBT_COLORS)
    assert rc == 0
    _golden_check(img, golden()["ref8"])
    # the four SBT colours and the barycentric branch all appear
    cols = {tuple(np.round(c, 4)) for c in img.reshape(-1, 4)[:, :3]}
    for c in S.REF8_SBT_COLORS:
        assert tuple(np.round(c, 4)) in cols


def test_golden_single_triangle(orc):
    import rtcore.scenes as S
    blas, rc = orc.build_blas([(S.TRI1_VERTICES, S.TRI1_INDICES, None)])
    assert rc == 0
    img, rc = orc.trace_rays(blas, S.TRI1_CAMERA, *S.TRI1_SIZE, chit=1)
    assert rc == 0
    _golden_check(img, golden()["tri"])


def test_raygen_vectorised_matches_scalar(orc):
    cam = ((0.5, 0.5, 2.5), 60.0)
    rays = orc.primary_rays(cam, 64, 48)
    for (x, y) in [(0, 0), (63, 47), (17, 5), (32, 24)]:
        o, d = orc.raygen(cam, 64, 48, x, y)
        r = rays[y * 64 + x]
        assert r["dir"].tobytes() == d.tobytes() and r["org"].tobytes() == o.tobytes()


def _soup_items(n, seed=7):
    import rtcore.scenes as S
    v, i = S.soup(seed, n)
    return [(v, i, None)]


def _rays(orc, n, seed=11):
    import rtcore.scenes as S
    inc = S.incoherent_rays(seed, n, (0, 0, 0), (1, 1, 1), 1e30)
    prim = orc.primary_rays(((0.5, 0.5, 2.5), 60.0), 80, 60, 0.0, 100.0)
    return np.concatenate([inc, prim])


@pytest.mark.parametrize("n", [1, 2, 3, 5, 64, 3000])
def test_bvh_traversal_equals_brute_force(orc, n):
    """The BVH8 traversal finds exactly the brute-force FP32 closest hit
    (same watertight test, same tie rule) and the same occlusion."""
    items = _soup_items(n)
    accel, rc = orc.build_blas(items)
    assert rc == 0
    rays = _rays(orc, 4000)
    hits, stats = orc.trace_closest(accel, rays)
    brute = orc.brute_closest(items, rays, 32)
    assert hits.tobytes() == brute.tobytes()
    occ, _ = orc.trace_any(accel, rays)
    np.testing.assert_array_equal(occ, (brute["prim"] != 0xFFFFFFFF).astype(np.uint8))
    assert stats[0] >= len(rays)


def test_fp32_hits_agree_with_fp64(orc):
    """>= 99.99% triangle-id agreement with the float64 oracle off grazing
    edges, barycentrics within 1e-5 where the ids agree."""
    items = _soup_items(20000, seed=3)
    accel, _ = orc.build_blas(items)
    rays = _rays(orc, 20000, seed=5)
    h32, _ = orc.trace_closest(accel, rays)
    h64 = orc.brute_closest(items, rays, 64)
    same = h32["prim"] == h64["prim"]

    def edge_dist(h):
        w = np.minimum(np.minimum(h["u"], h["v"]), 1 - h["u"] - h["v"])
        return np.where(h["prim"] != 0xFFFFFFFF, np.abs(w), np.inf)

    # grazing: either precision's hit lies within 1e-5 (barycentric) of an edge
    grazing = (edge_dist(h64) < 1e-5) | (edge_dist(h32) < 1e-5)
    off = ~grazing
    assert (h64["prim"] != 0xFFFFFFFF).sum() > 1000  # the rays do hit the soup
    agree = (same & off).sum() / max(1, off.sum())
    assert agree >= 0.9999, agree
    # Barycentrics of millimetre triangles seen from metres away cannot hold
    # 1e-5 in FP32 (error ~ ulp(|v - o|) / edge).  The bound checked here is
    # the hit point: |P32 - P64| <= 1e-6 * (1 + |o| + t|d|), i.e. a few FP32
    # ulps of the scene scale.  The 1e-5 barycentric bound is checked on the
    # reference scene (golden pixels).
    hit = same & (h64["prim"] != 0xFFFFFFFF)
    v = items[0][0].reshape(-1, 3, 3).astype(np.float64)[h32["prim"][hit]]

    def point(h):
        u, w = h["u"][hit].astype(np.float64), h["v"][hit].astype(np.float64)
        return (1 - u - w)[:, None] * v[:, 0] + u[:, None] * v[:, 1] + w[:, None] * v[:, 2]

    err = np.linalg.norm(point(h32) - point(h64), axis=1)
    scale = 1 + np.linalg.norm(rays["org"][hit], axis=1) + h64["t"][hit] * np.linalg.norm(rays["dir"][hit], axis=1)
    assert (err / scale).max() < 1e-6


def test_bvh8_structure(orc):
    """Every primitive sits in exactly one leaf; every decoded child box
    contains its leaf boxes in exact arithmetic; node links are in range."""
    items = _soup_items(5000, seed=9)
    accel, _ = orc.build_blas(items)
    h = header(accel)
    nd = nodes(accel)
    tri = prims(accel, 48).view(np.float32).reshape(-1, 12)
    assert h["node_count"] <= h["node_capacity"]
    seen = np.zeros(h["prim_count"], np.int32)
    for k, node in enumerate(nd):
        scale = np.ldexp(1.0, node["exp"].astype(np.int64))
        for s in range(8):
            lo = node["origin"].astype(np.float64) + node["qlo"][:, s] * scale
            hi = node["origin"].astype(np.float64) + node["qhi"][:, s] * scale
            if node["imask"] & (1 << s):
                c = node["child_base"] + bin(int(node["imask"]) & ((1 << s) - 1)).count("1")
                assert k < c < h["node_count"]
                cn = nd[c]
                cs = np.ldexp(1.0, cn["exp"].astype(np.int64))
                # the child's own grid origin lies inside this slot's box
                assert np.all(cn["origin"] >= lo) and np.all(cn["origin"] <= hi)
            elif node["meta"][s]:
                m = int(node["meta"][s])
                cnt = bin(m >> 5).count("1")
                for j in range(cnt):
                    r = node["prim_base"] + (m & 31) + j
                    seen[r] += 1
                    t = tri[r].reshape(3, 4)[:, :3].astype(np.float64)
                    assert np.all(t.min(0) >= lo) and np.all(t.max(0) <= hi), (k, s)
    assert np.all(seen == 1)
    ids = np.sort(tri[:, 3].view(np.uint32))
    np.testing.assert_array_equal(ids, np.arange(h["prim_count"], dtype=np.uint32))


def test_sort_oracle_is_stable_sort(orc):
    rng = np.random.default_rng(1)
    keys = rng.integers(0, 1 << 20, 5000, dtype=np.uint64) * np.uint64(1 << 40)
    vals = np.arange(5000, dtype=np.uint32)
    k, v = orc.sort_pairs(keys, vals, 64)
    order = np.argsort(keys, kind="stable")
    np.testing.assert_array_equal(k, keys[order])
    np.testing.assert_array_equal(v, vals[order])


def test_empty_and_degenerate_builds(orc):
    empty, rc = orc.build_blas([(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32), None)])
    assert rc == 0 and header(empty)["node_count"] == 1
    rays = _rays(orc, 100)
    hits, _ = orc.trace_closest(empty, rays)
    assert np.all(hits["prim"] == 0xFFFFFFFF)
    # duplicated triangles: identical Morton keys, index tie-break
    v = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (50, 1))
    dup, rc = orc.build_blas([(v, None, None)])
    assert rc == 0
    r = np.zeros(1, orc.RAY_DTYPE)
    r["org"] = (0.2, 0.2, 1.0)
    r["dir"] = (0, 0, -1)
    r["tmax"] = 10
    h, _ = orc.trace_closest(dup, r)
    assert h["prim"][0] == 0  # equal t: smallest triangle index wins
    # an index beyond max_vertex makes the triangle inactive and is reported
    bad_i = np.array([[0, 1, 7]], np.uint32)
    buf, rc = orc.build_blas([(v[:3], bad_i, None)])
    assert rc == -5


def test_scene_generators_deterministic(rtlib):
    import rtcore.scenes as S
    v1, i1 = S.soup(S.SEED_BASE + 2, 1000)
    v2, i2 = S.soup(S.SEED_BASE + 2, 1000)
    assert v1.tobytes() == v2.tobytes() and i1.tobytes() == i2.tobytes()
    t = v1.reshape(-1, 3, 3)
    c = t.mean(1)
    assert c.min() > -0.05 and c.max() < 1.05
    e = np.linalg.norm(t[:, 1] - t[:, 0], axis=1)
    assert e.min() >= 0.0009 and e.max() <= 0.0201
    v, i, tm, m = S.box(S.SEED_BASE + 3, 2, 4)
    assert len(i) == 14 + 2 * 20 * 16 and i.max() < len(v)
    assert m["emission"][3][0] == 15.0 and (tm == 3).sum() == 2
    r = S.incoherent_rays(1, 1000)
    n = np.linalg.norm(r["dir"], axis=1)
    assert np.abs(n - 1).max() < 1e-6


def test_tlas_walk_matches_flattened_geometry(orc):
    """The oracle's two-level walk against one world-space BLAS of the same
    instances: each unmasked instance's triangles transformed to world space
    as one geometry.  Object-space and world-space arithmetic round
    differently, so the check is the hit's identity -- which instance and
    which triangle, hit or miss -- on all but grazing rays, and t to 1e-4 of
    max(t, 1)."""
    import rtcore.scenes as S
    from oracle import INSTANCE_DTYPE
    v, i, _, _ = S.box(17, 3, 4)  # closed box walls and three small spheres
    blas, rc = orc.build_blas([(v, i, None)])
    assert rc == 0
    rng = np.random.default_rng(5)
    n_inst = 24
    inst = np.zeros(n_inst, INSTANCE_DTYPE)
    world_items, geom_of = [], {}
    for k in range(n_inst):
        ang = rng.uniform(0, 6.28)
        s = rng.uniform(0.5, 2.0)
        m = np.array([[np.cos(ang) * s, -np.sin(ang) * s, 0, rng.uniform(-2, 2)],
                      [np.sin(ang) * s, np.cos(ang) * s, 0, rng.uniform(-2, 2)],
                      [0, 0, s, rng.uniform(-2, 2)]], np.float32)
        mask = 0 if k % 5 == 2 else 0xFF
        inst[k]["transform"] = m
        inst[k]["custom_index_and_mask"] = k | (mask << 24)
        inst[k]["accel_ref"] = ptr_of(blas)
        if mask:
            wv = (v.astype(np.float64) @ m[:, :3].T.astype(np.float64) + m[:, 3]).astype(np.float32)
            geom_of[len(world_items)] = k
            world_items.append((wv, i, None))
    tlas, rc = orc.build_tlas(inst)
    assert rc == 0
    flat, rc = orc.build_blas(world_items)
    assert rc == 0
    rays = np.concatenate([S.incoherent_rays(23, 20000, (-3, -3, -3), (3, 3, 3), 1e30),
                           orc.primary_rays(((0.0, 0.0, 8.0), 60.0), 120, 90, 0.0, 100.0)])
    ht, _, xt = orc.trace_closest(tlas, rays, ext=True)
    hf, _, xf = orc.trace_closest(flat, rays, ext=True)
    hit_t, hit_f = ht["prim"] != 0xFFFFFFFF, hf["prim"] != 0xFFFFFFFF
    assert hit_t.sum() > 2000
    assert np.mean(hit_t == hit_f) >= 0.999
    both = np.nonzero(hit_t & hit_f)[0]
    inst_f = np.array([geom_of[g] for g in xf["geometry_index"][both]])
    same = (xt["instance_id"][both] == inst_f) & (xt["primitive_id"][both] == xf["primitive_id"][both])
    assert np.mean(same) >= 0.999
    assert not np.isin(xt["instance_id"][hit_t], [k for k in range(n_inst) if k % 5 == 2]).any()
    agree = both[same]
    # t error relative to max(t, 1): rays that start on a wall have t ~ 0
    rel = np.abs(ht["t"][agree] - hf["t"][agree]) / np.maximum(np.abs(hf["t"][agree]), 1.0)
    assert np.quantile(rel, 0.999) <= 1e-4
