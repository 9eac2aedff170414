"""The CPU oracle of the learned preconditioner's network: its autograd gradients against
central finite differences (FP64, no BF16 emulation), and the emulation's closeness to the
exact network."""
import numpy as np

import unet_oracle as U


def _params(seed):
    rng = np.random.default_rng(seed)
    parts = []
    for ci, co, k, _ in U.LAYERS:
        parts.append(rng.normal(0, np.sqrt(2.0 / (ci * k * k)), co * k * k * ci))
        parts.append(rng.normal(0, 0.05, co))
    return np.concatenate(parts)


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    p = _params(1)
    x = rng.normal(size=(1, 16, 16))
    f = rng.normal(size=(1, 16, 16))
    t = rng.normal(size=(1, 16, 16))
    loss, g = U.loss_and_grads(p, x, f, t, emulate_bf16=False)
    assert g.shape == p.shape and np.isfinite(loss)
    # a spread of parameters: first/last weights and biases of several layers
    idx = [0, 5, 100, 2000, 30000, 150000, p.size - 40, p.size - 1]
    h = 1e-6
    for i in idx:
        e = np.zeros_like(p)
        e[i] = h
        lp, _ = U.loss_and_grads(p + e, x, f, t, emulate_bf16=False)
        lm, _ = U.loss_and_grads(p - e, x, f, t, emulate_bf16=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_oracle_bf16_emulation_is_close_to_exact():
    rng = np.random.default_rng(4)
    p = _params(2)
    x = rng.normal(size=(2, 16, 16))
    f = rng.normal(size=(2, 16, 16))
    a = U.forward(p, x, f, emulate_bf16=False)
    b = U.forward(p, x, f, emulate_bf16=True)
    rel = np.linalg.norm(a - b) / np.linalg.norm(a)
    assert 1e-5 < rel < 3e-2
