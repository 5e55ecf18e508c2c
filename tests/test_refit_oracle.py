"""The refit restatement in the oracle (rt_refit_blas / rt_refit_tlas on
the CPU): unchanged inputs give back the build byte for byte; moved inputs
give a structure whose traversal finds exactly the brute-force hits of the
moved geometry; mismatched inputs are rejected."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import header, ptr_of, single_instance


def _soup(n, seed=7):
    import rtcore.scenes as S
    v, i = S.soup(seed, n)
    return v, i


def _moved(v, seed=3, amount=0.01):
    rng = np.random.default_rng(seed)
    return (v + rng.uniform(-amount, amount, v.shape)).astype(np.float32)


def _rays(orc, n, seed=11):
    import rtcore.scenes as S
    inc = S.incoherent_rays(seed, n, (0, 0, 0), (1, 1, 1), 1e30)
    prim = orc.primary_rays(((0.5, 0.5, 2.5), 60.0), 80, 60, 0.0, 100.0)
    return np.concatenate([inc, prim])


@pytest.mark.parametrize("n", [1, 2, 9, 3000])
def test_refit_with_same_inputs_is_the_build(orc, n):
    v, i = _soup(n)
    xf = np.array([[1, 0, 0, 0.25], [0, 0.5, 0, 0], [0, 0, 1, -1]], np.float32)
    items = [(v, i, None), (v[: 3 * (n // 2 + 1)], i[: n // 2 + 1] if n > 1 else i, xf)]
    a, rc = orc.build_blas(items)
    b = a.copy()
    assert orc.refit_blas(b, items) == 0
    assert a.tobytes() == b.tobytes()


def test_refit_after_moving_vertices_traces_the_new_geometry(orc):
    v, i = _soup(4000)
    a, _ = orc.build_blas([(v, i, None)])
    nodes_before = a[:256].copy()
    v2 = _moved(v)
    assert orc.refit_blas(a, [(v2, i, None)]) == 0
    h = header(a)
    assert h["node_count"] == header(nodes_before)["node_count"]
    rays = _rays(orc, 3000)
    hits, _ = orc.trace_closest(a, rays)
    brute = orc.brute_closest([(v2, i, None)], rays, 32)
    assert hits.tobytes() == brute.tobytes()
    # bounds of the refitted structure are the new geometry's
    assert np.allclose(h["bounds_lo"][:3], v2.min(axis=0)) and np.allclose(h["bounds_hi"][:3], v2.max(axis=0))


def test_tlas_refit(orc):
    v, i = _soup(500)
    b, _ = orc.build_blas([(v, i, None)])
    inst = np.concatenate([single_instance(ptr_of(b)) for _ in range(5)])
    for k in range(5):
        inst[k]["transform"][:, 3] = (k * 1.5, 0.0, 0.0)
    t, _ = orc.build_tlas(inst)
    same = t.copy()
    assert orc.refit_tlas(same, inst) == 0 and same.tobytes() == t.tobytes()
    moved = inst.copy()
    for k in range(5):
        moved[k]["transform"][:, 3] = (k * 1.5, 0.1 * k, -0.2 * k)
    assert orc.refit_tlas(t, moved) == 0
    fresh, _ = orc.build_tlas(moved)
    rays = _rays(orc, 2000)
    rays["org"][:, 0] *= 7.5
    hr, _ = orc.trace_closest(t, rays, ext=False)
    hf, _ = orc.trace_closest(fresh, rays, ext=False)
    assert hr.tobytes() == hf.tobytes()


def test_mismatched_inputs_are_rejected(orc):
    import rtcore
    v, i = _soup(100)
    a, _ = orc.build_blas([(v, i, None)])
    before = a.tobytes()
    assert orc.refit_blas(a, [(v[:297], i[:99], None)]) == rtcore.RT_ERR_INVALID_ARG  # one triangle fewer
    assert orc.refit_blas(a, [(v, i, None), (v, i, None)]) == rtcore.RT_ERR_INVALID_ARG  # two geometries
    assert a.tobytes() == before


@pytest.mark.parametrize("width", [4, 5, 6, 8])
def test_narrow_trees(orc, width):
    """RT_BUILD_WIDTH(w): at most w children per node, the same hits."""
    import rtcore
    from helpers import nodes
    v, i = _soup(3000)
    a, rc = orc.build_blas([(v, i, None)], rtcore.build_width(width))
    assert rc == 0
    nd = nodes(a)
    children = np.array([bin(int(im)).count("1") for im in nd["imask"]]) + \
        np.array([sum(1 for s in range(8) if m[s] and not (im >> s) & 1) for m, im in zip(nd["meta"], nd["imask"])])
    assert children.max() <= width and children.max() >= min(width, 4)
    rays = _rays(orc, 2000)
    assert orc.trace_closest(a, rays)[0].tobytes() == orc.brute_closest([(v, i, None)], rays, 32).tobytes()
    if width < 8:
        a8, _ = orc.build_blas([(v, i, None)])
        assert len(nodes(a8)) < len(nd)


def test_invalid_width_rejected(orc):
    import rtcore
    v, i = _soup(10)
    for w in (1, 2, 3, 9, 15):
        _, rc = orc.build_blas([(v, i, None)], rtcore.build_width(w))
        assert rc == rtcore.RT_ERR_INVALID_ARG, w
