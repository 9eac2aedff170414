"""Host-side pieces of the preconditioner training (CPU, no GPU): merging two training sets
and the deployment policy read from a weight file's metadata."""
import numpy as np
import torch

from lentils_gb300 import train_preconditioner as T


def _set(ndraws, npairs, n=12, m=3, seed=0):
    g = torch.Generator().manual_seed(seed)
    r = torch.randn(npairs, n, generator=g)
    e = torch.randn(npairs, n, generator=g)
    return {"r": r, "e": e, "er": (e.double() * r.double()).sum(1),
            "dinv": torch.rand(ndraws, n, generator=g), "feat": torch.randn(ndraws, n, generator=g),
            "draw": torch.randint(0, ndraws, (npairs,), generator=g),
            "Q": torch.randn(npairs, m, n, generator=g), "window": m,
            "inversions": [f"op{seed}-{k}" for k in range(ndraws)],
            "cg_iterations": [10 * (k + 1) for k in range(ndraws)], "seconds": 1.5}


def test_merge_sets_keeps_each_pair_with_its_draw():
    a, b = _set(3, 7, seed=1), _set(2, 5, seed=2)
    m = T.merge_sets(a, b)
    assert m["r"].shape[0] == 12 and m["Q"].shape == (12, 3, 12)
    assert m["dinv"].shape[0] == 5 and len(m["inversions"]) == 5
    # every pair still points at its own draw's diagonal and operator
    for k in range(12):
        src, kk = (a, k) if k < 7 else (b, k - 7)
        d = int(m["draw"][k])
        assert torch.equal(m["dinv"][d], src["dinv"][int(src["draw"][kk])])
        assert m["inversions"][d] == src["inversions"][int(src["draw"][kk])]
        assert torch.equal(m["r"][k], src["r"][kk]) and torch.equal(m["Q"][k], src["Q"][kk])
    assert m["window"] == 3 and m["seconds"] == 3.0
    assert m["cg_iterations"] == a["cg_iterations"] + b["cg_iterations"]


def test_deploy_policy_defaults_and_overrides():
    assert T.deploy_policy({}) == T.DEFAULT_POLICY
    pol = T.deploy_policy({"deploy": {"jacobi_weight": 0.0, "net_every": 4}})
    assert pol == {"jacobi_weight": 0.0, "window": T.DEFAULT_POLICY["window"], "net_every": 4}
    # the committed weights carry the policy their evaluation measured
    _, meta = T.load(T.DEFAULT_WEIGHTS)
    pol = T.deploy_policy(meta)
    assert pol["window"] == 8 and pol["net_every"] >= 1 and np.isfinite(pol["jacobi_weight"])
