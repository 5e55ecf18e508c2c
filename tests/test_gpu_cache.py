"""GPU checks of the MLP radiance cache against the float64 oracle
(oracle/mlp.py): forward outputs, gradients, one Adam step, and that online
training on a known target actually reduces the loss."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import dev, host

pytestmark = pytest.mark.gpu

# Tolerances against the float64 oracle (which rounds where the kernels
# round to BF16): about twice the errors observed on a GB300 (printed).
FWD_TOL = 1e-2    # max |y - y_oracle| / max |y_oracle|
GRAD_TOL = 3e-2   # per layer: max |g - g_oracle| / max |g_oracle|

INPUT_DTYPE = np.dtype([("pos", "<f4", 3), ("dir", "<f4", 3), ("normal", "<f4", 3), ("albedo", "<f4", 3)])


def random_inputs(n, seed=0):
    rng = np.random.default_rng(seed)
    x = np.zeros(n, INPUT_DTYPE)
    x["pos"] = rng.uniform(-1, 1, (n, 3))
    d = rng.normal(size=(n, 3))
    x["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    nn = rng.normal(size=(n, 3))
    x["normal"] = nn / np.linalg.norm(nn, axis=1, keepdims=True)
    x["albedo"] = rng.uniform(0, 1, (n, 3))
    return x


def smooth_target(x):
    p, nrm, alb = x["pos"], x["normal"], x["albedo"]
    base = 0.5 + 0.4 * np.sin(2.0 * p[:, 0:1]) * np.cos(1.5 * p[:, 1:2]) + 0.2 * nrm[:, 2:3]
    t = np.zeros((len(x), 4), np.float32)
    t[:, :3] = np.maximum(base * (0.3 + alb), 0.0)
    return t


@pytest.fixture()
def cache(ctx):
    import rtcore
    import torch
    buf = torch.zeros(ctx.cache_bytes(), dtype=torch.uint8, device="cuda")
    ctx.cache_init(buf, rtcore.cache_config(seed=7))
    return buf


def get_params(ctx, cache):
    import rtcore
    import torch
    n = rtcore.load().rt_cache_param_count()
    p = torch.empty(n * 4, dtype=torch.uint8, device="cuda")
    ctx.cache_get_params(cache, p)
    ctx.sync()
    return host(p).view(np.float32).copy()


def test_forward_matches_oracle(ctx, cache):
    from oracle import mlp
    import torch
    x = random_inputs(1000, 1)
    out = torch.empty(len(x) * 16, dtype=torch.uint8, device="cuda")
    ctx.cache_query(cache, dev(x), out, len(x))
    ctx.sync()
    y = host(out).view(np.float32).reshape(-1, 4)
    p = get_params(ctx, cache)
    yo = mlp.forward(p, x, (-1, -1, -1), (1, 1, 1))[:, :3]
    scale = np.abs(yo).max()
    err = np.abs(y[:, :3] - yo).max() / scale
    print(f"forward, 1,000 rows: max error / max output {err:.3e} (tolerance {FWD_TOL:g})")
    assert err < FWD_TOL
    assert np.all(y[:, 3] == 0)


def test_forward_many_tiles_matches_oracle(ctx, cache):
    """100,003 rows: several 128-row tiles per CTA and a ragged last tile."""
    from oracle import mlp
    import torch
    x = random_inputs(100003, 11)
    out = torch.full((len(x) * 4,), -7.0, dtype=torch.float32, device="cuda")
    ctx.cache_query(cache, dev(x), out, len(x))
    ctx.sync()
    y = out.cpu().numpy().reshape(-1, 4)
    assert np.isfinite(y).all() and not (y[:, 0] == -7.0).any()
    idx = np.r_[np.random.default_rng(0).choice(len(x) - 64, 2000, replace=False), np.arange(len(x) - 64, len(x))]
    p = get_params(ctx, cache)
    yo = mlp.forward(p, x[idx], (-1, -1, -1), (1, 1, 1))[:, :3]
    err = np.abs(y[idx, :3] - yo).max() / np.abs(yo).max()
    print(f"forward, 100,003 rows: max error / max output {err:.3e} (tolerance {FWD_TOL:g})")
    assert err < FWD_TOL


def test_gradient_matches_oracle(ctx, cache):
    from oracle import mlp
    import torch
    x = random_inputs(1000, 2)
    t = smooth_target(x)
    n = len(x)
    g = torch.empty(mlp.N_PARAMS * 4, dtype=torch.uint8, device="cuda")
    ctx.cache_gradient(cache, dev(x), dev(t), n, g)
    ctx.sync()
    gg = host(g).view(np.float32).astype(np.float64)
    p = get_params(ctx, cache)
    go, loss = mlp.gradient(p, x, t, (-1, -1, -1), (1, 1, 1))
    seen = []
    for L in range(6):
        wo, bo = mlp.W_OFF[L]
        a, b = gg[wo:bo], go[wo:bo]
        rel = np.abs(a - b).max() / max(np.abs(b).max(), 1e-30)
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
        ab, bb = gg[bo:bo + mlp.OUT[L]], go[bo:bo + mlp.OUT[L]]
        relb = np.abs(ab - bb).max() / max(np.abs(bb).max(), 1e-30)
        seen.append((L, float(rel), cos, float(relb)))
    print("gradient per layer (layer, weight error / max, cosine, bias error / max): "
          + ", ".join(f"({L}, {r:.2e}, {c:.6f}, {rb:.2e})" for L, r, c, rb in seen) + f"; tolerance {GRAD_TOL:g}")
    for L, rel, cos, relb in seen:
        assert rel < GRAD_TOL and cos > 0.999 and relb <= GRAD_TOL, (L, rel, cos, relb)
    # padded inputs / outputs never receive gradient
    assert np.all(gg[mlp.W_OFF[0][0]:mlp.W_OFF[0][1]].reshape(64, 96)[:, 81:] == 0)
    assert np.all(gg[mlp.W_OFF[5][0]:mlp.W_OFF[5][1]].reshape(8, 64)[3:] == 0)


def test_adam_step_matches_oracle(ctx, cache):
    from oracle import mlp
    import torch
    x = random_inputs(512, 3)
    t = smooth_target(x)
    p0 = get_params(ctx, cache)
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    ctx.cache_train(cache, dev(x), dev(t), len(x), 512, loss)
    ctx.sync()
    p1 = get_params(ctx, cache)
    go, lo = mlp.gradient(p0, x, t, (-1, -1, -1), (1, 1, 1))
    po, _, _ = mlp.adam(p0.astype(np.float64), go, np.zeros_like(go), np.zeros_like(go), 1)
    # one Adam step moves each parameter by about lr * sign(g): compare moves
    moved = np.abs(p1 - p0)
    assert moved.max() <= 1.01e-3
    agree = np.sign(p1 - p0) == np.sign(po - p0)
    big = np.abs(go) > 1e-3 * np.abs(go).max()
    assert agree[big].mean() > 0.99
    assert abs(float(loss.item()) - lo) / lo < 2e-2


def _held_out_relmse(ctx, cache, xv, tv):
    import torch
    out = torch.empty(len(xv) * 16, dtype=torch.uint8, device="cuda")
    ctx.cache_query(cache, dev(xv), out, len(xv))
    ctx.sync()
    y = host(out).view(np.float32).reshape(-1, 4)[:, :3]
    return float(np.mean((y - tv) ** 2 / (tv ** 2 + 0.01)))


def test_training_reduces_loss(ctx, cache):
    """120 Adam steps (lr 1e-3, batches of 16384): the training loss falls
    by more than 5x and the held-out relative error by more than 2x.  The
    float64 oracle with the same optimiser shows the same curve (a fast
    drop, a plateau near 0.5, then a slow descent), so the bound is set by
    the optimisation, not by the kernels."""
    import torch
    x = random_inputs(65536, 4)
    t = smooth_target(x)
    xv = random_inputs(4096, 5)
    tv = smooth_target(xv)[:, :3]
    before = _held_out_relmse(ctx, cache, xv, tv)
    dx, dt = dev(x), dev(t)
    losses = []
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    for epoch in range(30):
        ctx.cache_train(cache, dx, dt, len(x), 16384, loss)
        ctx.sync()
        losses.append(float(loss.item()))
    assert losses[-1] < 0.2 * losses[0], losses
    after = _held_out_relmse(ctx, cache, xv, tv)
    assert after < 0.5 * before, (before, after)


def test_params_roundtrip(ctx, cache):
    import torch
    p = get_params(ctx, cache)
    q = (p * 0.5).astype(np.float32)
    ctx.cache_set_params(cache, dev(q))
    ctx.sync()
    assert get_params(ctx, cache).tobytes() == q.tobytes()


def test_checkpoint_restores_training_state(ctx, cache, tmp_path):
    """Save after some Adam steps: a fresh cache loaded from the file holds the
    saved state byte for byte (weights, Adam moments, step count), and the
    next step from it matches the original's next step (to the rounding of
    the gradients' atomic accumulation).  Damaged files are rejected without
    touching the cache."""
    import rtcore
    import torch
    from oracle import mlp
    x = random_inputs(8192, 21)
    t = smooth_target(x)
    dx, dt = dev(x), dev(t)
    for _ in range(3):
        ctx.cache_train(cache, dx, dt, len(x), 8192)
    path = tmp_path / "cache.rtmc"
    ctx.cache_save(cache, path)
    ctx.sync()
    saved = host(cache).copy()
    other = torch.zeros(ctx.cache_bytes(), dtype=torch.uint8, device="cuda")
    ctx.cache_init(other, rtcore.cache_config(seed=99))
    ctx.cache_load(other, path)
    ctx.sync()
    n_state = path.stat().st_size - 64
    assert host(other)[:n_state].tobytes() == saved[:n_state].tobytes()
    ctx.cache_train(cache, dx, dt, len(x), 8192)
    ctx.cache_train(other, dx, dt, len(x), 8192)
    ctx.sync()
    a = host(cache)[:4 * mlp.N_PARAMS].view(np.float32)
    b = host(other)[:4 * mlp.N_PARAMS].view(np.float32)
    assert np.abs(a - b).max() <= 1e-5 * np.abs(a).max()
    step_off = 4 * 4 * mlp.N_PARAMS + 2 * mlp.N_PARAMS
    assert host(cache)[step_off:step_off + 4].view(np.uint32)[0] == 4
    assert host(other)[step_off:step_off + 4].view(np.uint32)[0] == 4
    data = path.read_bytes()
    before = host(other).copy()
    for bad in (data[:-1], data + b"x", data[:100] + bytes([data[100] ^ 1]) + data[101:], b"RTMX" + data[4:]):
        p2 = tmp_path / "bad.rtmc"
        p2.write_bytes(bad)
        with pytest.raises(rtcore.RtError) as e:
            ctx.cache_load(other, p2)
        assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    assert host(other).tobytes() == before.tobytes()


def test_misaligned_cache_is_rejected(ctx, cache):
    """A cache buffer that is not 256-byte aligned is refused on the host with
    RT_ERR_INVALID_ARG by every entry point that launches a kernel on it;
    nothing is launched and the aligned cache is untouched."""
    import rtcore
    import torch
    p0 = get_params(ctx, cache)
    x = random_inputs(64, 8)
    t = smooth_target(x)
    off = torch.zeros(ctx.cache_bytes() + 256, dtype=torch.uint8, device="cuda")[16:]
    out = torch.empty(64 * 16, dtype=torch.uint8, device="cuda")
    g = torch.empty(rtcore.load().rt_cache_param_count() * 4, dtype=torch.uint8, device="cuda")
    calls = [
        lambda: ctx.cache_init(off, rtcore.cache_config(seed=7)),
        lambda: ctx.cache_query(off, dev(x), out, 64),
        lambda: ctx.cache_train(off, dev(x), dev(t), 64, 64),
        lambda: ctx.cache_gradient(off, dev(x), dev(t), 64, g),
        lambda: ctx.cache_set_params(off, dev(p0)),
    ]
    for call in calls:
        with pytest.raises(rtcore.RtError) as e:
            call()
        assert e.value.code == rtcore.RT_ERR_INVALID_ARG
    ctx.sync()
    assert get_params(ctx, cache).tobytes() == p0.tobytes()
