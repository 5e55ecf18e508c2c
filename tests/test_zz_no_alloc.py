"""rt_build_blas_static_scratch: the bottom-level build for callers that
cannot allocate device memory (its scratch is a fixed array inside the
library).  Its output must equal the regular rt_build_blas on the same
inputs, on two calls in a row -- the second smaller than the first, so that
anything the first call left in the shared array would show -- and it must
refuse inputs beyond its stated maximum before touching the GPU.

This file is named to be collected last: if it fails, a run stopped at the
first failure has already run every other test."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import GpuBlas, compare_accels, dev, gpu_trace_closest, host

pytestmark = pytest.mark.gpu


def _geometry(v: np.ndarray, i: np.ndarray, keep: list):
    import rtcore
    g = rtcore.GeometryTriangles()
    dv, di = dev(v), dev(i)
    keep += [dv, di]
    g.vertices, g.vertex_stride, g.max_vertex = dv.data_ptr(), 12, len(v) - 1
    g.index_type, g.indices, g.tri_count, g.flags = rtcore.RT_INDEX_UINT32, di.data_ptr(), len(i), 1
    return g


def test_static_scratch_build_equals_regular_build(ctx):
    import torch
    import rtcore.scenes as S
    import rtcore
    for seed, n in ((101, rtcore.RT_STATIC_SCRATCH_MAX_TRIS), (202, 37_000)):
        v, i = S.soup(seed, n)
        regular = GpuBlas(ctx, [(v, i, None)])
        keep: list = []
        g = _geometry(v, i, keep)
        sz = ctx.blas_sizes([n])
        accel = torch.zeros(sz.accel_bytes, dtype=torch.uint8, device="cuda")
        ctx.build_blas_static_scratch([g], 0, accel, sz.accel_bytes)
        ctx.sync()
        compare_accels(host(accel), regular.bytes(), 48)
        rays = S.incoherent_rays(seed, 20000, (0, 0, 0), (1, 1, 1), 1e30)
        a = gpu_trace_closest(ctx, ctx.address(accel), rays)
        b = gpu_trace_closest(ctx, regular.addr, rays)
        assert a.tobytes() == b.tobytes()


def test_static_scratch_rejects_oversize(ctx):
    import torch
    import rtcore
    import rtcore.scenes as S
    n = rtcore.RT_STATIC_SCRATCH_MAX_TRIS + 1
    v, i = S.soup(5, n)
    keep: list = []
    g = _geometry(v, i, keep)
    sz = ctx.blas_sizes([n])
    accel = torch.zeros(sz.accel_bytes, dtype=torch.uint8, device="cuda")
    with pytest.raises(rtcore.RtError) as e:
        ctx.build_blas_static_scratch([g], 0, accel, sz.accel_bytes)
    assert e.value.code == rtcore.RT_ERR_UNSUPPORTED
    assert "131072" in str(e.value)
    ctx.sync()
    assert not host(accel).any()  # nothing was written
