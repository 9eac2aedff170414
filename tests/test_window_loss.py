"""The windowed energy-norm training loss (train_preconditioner.window_energy_loss) against its
definition: the A-norm error left after flexible CG's step along z made A-orthogonal to the
window, on a dense SPD matrix standing in for the normal operator (CPU, no GPU)."""
import numpy as np
import pytest
import torch

from lentils_gb300 import train_preconditioner as T


def _setup(seed, B=3, H=4, W=5, m=3, used=(3, 1, 0)):
    n = H * W
    rng = np.random.default_rng(seed)
    G = rng.normal(size=(B, n, n))
    A = np.einsum("bij,bkj->bik", G, G) + n * np.eye(n)[None]
    Q = np.zeros((B, m, n))
    for b in range(B):  # A-orthogonal directions p_j, stored as q_j = A p_j / sqrt(p_j.A p_j)
        P = []
        for _ in range(used[b]):
            p = rng.normal(size=n)
            for pj in P:
                p -= (p @ A[b] @ pj) / (pj @ A[b] @ pj) * pj
            P.append(p)
        for j, p in enumerate(P):
            Q[b, j] = A[b] @ p / np.sqrt(p @ A[b] @ p)
    e = rng.normal(size=(B, n))
    r = np.einsum("bij,bj->bi", A, e)
    data = {"r": torch.tensor(r, dtype=torch.float32), "e": torch.tensor(e, dtype=torch.float32),
            "Q": torch.tensor(Q, dtype=torch.float32),
            "er": torch.tensor((e * r).sum(1)), "A": torch.tensor(A, dtype=torch.float32)}
    z = torch.tensor(rng.normal(size=(B, H, W)), dtype=torch.float32)
    return data, z, A, Q, e, r


def _fake_apply(data, ids, z):
    return torch.einsum("bij,bj->bi", data["A"][ids], z.reshape(z.shape[0], -1)).view_as(z)


def _projected_frac(A, Q, e, r, z):
    """1 - (p.r)|p.r| / ((p.Ap)(e.r)), p = z - sum_j (z.A p_j / p_j.A p_j) p_j, computed with
    the directions p_j = A^-1 q_j recovered explicitly."""
    out = []
    for b in range(A.shape[0]):
        p = z[b].copy()
        for q in Q[b]:
            if not q.any():
                continue
            pj = np.linalg.solve(A[b], q)
            p -= (p @ A[b] @ pj) / (pj @ A[b] @ pj) * pj
        pr = p @ r[b]
        out.append(1.0 - pr * abs(pr) / ((p @ A[b] @ p) * (e[b] @ r[b])))
    return np.array(out)


def test_window_loss_matches_projected_direction(monkeypatch):
    monkeypatch.setattr(T, "_apply_batch", _fake_apply)
    data, z, A, Q, e, r = _setup(3)
    ids = torch.arange(z.shape[0])
    frac, _ = T.window_energy_loss(data, ids, z)
    ref = _projected_frac(A, Q, e, r, z.reshape(z.shape[0], -1).double().numpy())
    np.testing.assert_allclose(frac.numpy(), ref, rtol=2e-4, atol=2e-5)
    assert (frac.numpy() >= -1e-5).all() and (frac.numpy() <= 2 + 1e-5).all()
    # the reversed direction scores 2 - frac: same line, but rejected by the solver
    fneg, _ = T.window_energy_loss(data, ids, -z)
    np.testing.assert_allclose(fneg.numpy(), 2.0 - frac.numpy(), rtol=1e-5, atol=1e-6)
    # an empty window reduces to the plain energy loss
    data0 = dict(data, Q=torch.zeros_like(data["Q"]))
    f0, g0 = T.window_energy_loss(data0, ids, z)
    f1, g1 = T.energy_loss(data0, ids, z)
    np.testing.assert_allclose(f0.numpy(), f1.numpy(), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(g0.numpy(), g1.numpy(), rtol=1e-4, atol=1e-7)


@pytest.mark.parametrize("sign", [1.0, -1.0])
def test_window_loss_gradient_matches_finite_differences(monkeypatch, sign):
    monkeypatch.setattr(T, "_apply_batch", _fake_apply)
    data, z, A, Q, e, r = _setup(5)
    z = sign * z
    B = z.shape[0]
    ids = torch.arange(B)
    _, grad = T.window_energy_loss(data, ids, z)
    zz = z.reshape(B, -1).double().numpy()
    rng = np.random.default_rng(0)
    h = 1e-4
    for b in range(B):
        for i in rng.choice(zz.shape[1], 5, replace=False):
            zp, zm = zz.copy(), zz.copy()
            zp[b, i] += h
            zm[b, i] -= h
            fd = (_projected_frac(A, Q, e, r, zp)[b] - _projected_frac(A, Q, e, r, zm)[b]) / (2 * h)
            # the loss is the batch mean: its gradient carries 1 / B
            assert grad.reshape(B, -1)[b, i].item() == pytest.approx(fd / B, rel=2e-2, abs=1e-6)
