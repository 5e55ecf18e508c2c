"""The learned form (MLP radiance cache at the second path vertex) against
the plain path tracer: what the trained network gains.

1. The same learned form with and without training: after some frames the
   trained cache's image is much closer to the converged reference.
2. Equal time against the plain path tracer at 1920x1080 on the 2M-triangle
   box scene: the learned form reaches a lower relMSE.  (At low resolution
   the fixed training cost per frame dominates and the plain form wins; the
   cache pays off at the resolution it is designed for.)
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def box(ctx):
    from rtcore.relmse import GpuBox
    return GpuBox(ctx, 40, 50)


def _frames(ctx, box, w, h, frames, train_batch, train_paths, seed=11, spc=1):
    """frames training samples then 32 measured ones, spc samples per call
    (one wave of spc samples: the cache trains after each call)."""
    import torch
    import rtcore
    from rtcore.relmse import _image, params
    cache = torch.zeros(ctx.cache_bytes(), dtype=torch.uint8, device="cuda")
    ctx.cache_init(cache, rtcore.cache_config(seed=5))
    cp = rtcore.PtCacheParams(cache.data_ptr(), train_paths, train_batch)
    p = params(w, h, spc, 0, seed)
    nb = ctx.pt_cached_scratch_bytes(p, cp)
    scratch = torch.empty(nb, dtype=torch.uint8, device="cuda")
    warm = torch.zeros(w * h * 16, dtype=torch.uint8, device="cuda")
    for s in range(0, frames, spc):  # training frames (their image is discarded)
        ctx.path_trace_cached(box.scene, params(w, h, spc, s, seed), cp, warm, scratch, nb)
    accum = torch.zeros(w * h * 16, dtype=torch.uint8, device="cuda")
    for s in range(frames, frames + 32, spc):
        ctx.path_trace_cached(box.scene, params(w, h, spc, s, seed), cp, accum, scratch, nb)
    ctx.sync()
    img = _image(accum)
    assert np.isfinite(img).all() and (img >= 0).all()
    return img


@pytest.mark.parametrize("spc", [1, 4])
def test_training_gains_over_untrained_cache(ctx, box, spc):
    """One sample per call (training after every sample) and four (one wave
    of four samples per call, training after the wave)."""
    from rtcore.relmse import reference, relmse
    w, h = 480, 270
    ref = reference(ctx, box, w, h, 1024)
    trained = _frames(ctx, box, w, h, 64, 4096, 4096, spc=spc)
    untrained = _frames(ctx, box, w, h, 64, 0, 4096, spc=spc)
    r_t, r_u = relmse(trained, ref), relmse(untrained, ref)
    assert r_t < 0.5 * r_u, (r_t, r_u)


def test_equal_time_beats_plain(ctx, box):
    """1920x1080, 65,536 training paths per frame in batches of 16,384 (the
    learned form's configuration), 1.5 s of GPU time each."""
    from rtcore.relmse import reference, run
    w, h = 1920, 1080
    ref = reference(ctx, box, w, h, 512)
    plain = run(ctx, box, w, h, ref, 1500.0, False)
    cached = run(ctx, box, w, h, ref, 1500.0, True, train_paths=65536, train_batch=16384)
    # same wall time (within one frame), lower error
    assert abs(plain[-1][0] - cached[-1][0]) < 50.0
    assert cached[-1][2] < 0.9 * plain[-1][2], (plain[-1], cached[-1])
    assert cached[-1][1] > plain[-1][1]  # cheaper samples
