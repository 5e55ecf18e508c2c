"""The learned form (MLP radiance cache at the second path vertex) against
the plain path tracer: what the trained network gains.

1. The same learned form with and without training: after some frames the
   trained cache's image is much closer to the converged reference.
2. The learned workload's criterion at 1920x1080 on the 8M-triangle box
   scene (160 icospheres): the learned form reaches the relMSE the plain form
   has after its whole time budget in at most half of that time.  (At low
   resolution the fixed training cost per frame dominates and the plain form
   wins; the cache pays off at the resolution it is designed for.)
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


def test_learned_form_needs_at_most_half_the_time(ctx):
    """1920x1080 on the learned workload's 8,000,014-triangle box, 65,536
    training paths per sample in Adam batches of 4,096, four samples per
    call for both forms, 3 s of GPU time each, against a 2,048-spp plain
    reference.  The target is the relMSE the plain form reaches at the end
    of its budget; the learned form must reach it in at most half the plain
    form's time, on the CUDA-event clock and on the wall clock.  (Against a
    2,048-spp reference both curves carry the same reference noise, which
    cancels in this comparison.)"""
    from rtcore.relmse import GpuBox, equal_time, reference, time_to
    box8 = GpuBox(ctx, 160, 50)
    w, h = 1920, 1080
    ref = reference(ctx, box8, w, h, 2048)
    res = equal_time(ctx, box8, w, h, ref, 3000.0, target=1.0, spp_per_call=4)
    plain, cached = res["plain"], res["cached"]
    target = plain[-1][3]
    for clock in ("gpu", "wall"):
        tp, tc = time_to(plain, target, clock), time_to(cached, target, clock)
        print(f"{clock}: plain reaches relMSE {target:.3e} at {tp} ms, learned at {tc} ms "
              f"(ratio {tc / tp if tc and tp else None})")
        assert tc is not None and tc <= 0.5 * tp, (clock, tp, tc, plain[-1], cached[-1])
    assert cached[-1][2] > plain[-1][2]  # cheaper samples
