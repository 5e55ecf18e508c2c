"""CPU check of the MLP oracle's backpropagation against torch autograd
(float64, no BF16 rounding), so the oracle that checks the GPU gradients is
itself pinned to an independent differentiation."""
from __future__ import annotations

import numpy as np


def test_oracle_gradient_equals_autograd():
    import torch
    from oracle import mlp
    rng = np.random.default_rng(0)
    dt = np.dtype([("pos", "<f4", 3), ("dir", "<f4", 3), ("normal", "<f4", 3), ("albedo", "<f4", 3)])
    x = np.zeros(64, dt)
    for f in dt.names:
        x[f] = rng.uniform(-1, 1, (64, 3))
    t = rng.uniform(0, 1, (64, 4)).astype(np.float32)
    p = (rng.normal(size=mlp.N_PARAMS) * 0.2).astype(np.float32)
    g, loss = mlp.gradient(p, x, t, (-1, -1, -1), (1, 1, 1), exact=True)

    enc = torch.tensor(mlp.encode(x, (-1, -1, -1), (1, 1, 1), exact=True))
    pt = torch.tensor(p.astype(np.float64), requires_grad=True)
    a = enc
    for L in range(6):
        wo, bo = mlp.W_OFF[L]
        w = pt[wo:bo].reshape(mlp.OUT[L], mlp.IN[L])
        b = pt[bo:bo + mlp.OUT[L]]
        a = a @ w.T + b
        if L < 5:
            a = torch.relu(a)
    y = a[:, :3]
    tt = torch.tensor(t[:, :3].astype(np.float64))
    den = (y.detach() ** 2 + 0.01)
    lt = ((y - tt) ** 2 / den).mean()
    lt.backward()
    np.testing.assert_allclose(g, pt.grad.numpy(), rtol=1e-9, atol=1e-12)
    assert abs(loss - float(lt.detach())) < 1e-12
