"""Train the learned CG preconditioner on the GPU and compare it with plain Jacobi-CG.

    python -m lentils_gb300.train_preconditioner --draws 100 --pairs 100 --steps 4000 \
        --out lentils_gb300/weights/unet_source128.npz

1. Training set: for each of `draws` random lens models (PEMD + shear from the sweep priors,
   learned.lens_draw) and random sources, the inversion workload's normal equations are solved
   by plain Jacobi-CG from zero; `pairs` iterates x_k along the trajectory give pairs
   (r_k = b - A x_k, e_k = x* - x_k) with x* the FP64-refined solution (learned.trajectory_pairs).
   All draws share the workload's visibility set and NUFFT operator.
   With --loss window the pairs come from truncated flexible-CG trajectories instead
   (learned.window_pairs) and carry the solver's window of A-orthogonalised directions.
2. Training: Adam on the energy-norm loss -- the fraction of the A-norm error left after a
   line search along the network's direction, 1 - (z.r)|z.r| / ((z.Az)(e.r)), each sample
   with its own normal operator; with --loss window the direction is first made A-orthogonal
   to the pair's window, as flexible CG does (window_energy_loss); --refine-draws adds a
   second stage on pairs from flexible-CG trajectories with the trained network in the loop
   -- or (--loss mse) on the mean squared error against the
   correction's direction e / rms(e) with minibatches of random pairs under random flips and transposes of the grid
   (applied to residual, correction and diagonal together), cosine learning-rate decay; every
   step is the network's own forward and backward kernels.
3. Evaluation: the workload inversion solved to a true FP64 relative residual of 1e-6 by plain
   Jacobi-CG (lentils_cg_solve) and by flexible CG with the network (lentils_fcg_solve) for
   each Jacobi share, window and network period; the fastest combination is stored with the
   weights as their deployment policy (deploy_policy).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import time

import numpy as np
import torch

from . import learned, workloads

DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights",
                               "unet_source128.npz")


def build_training_set(nufft, geom, draws, pairs, seed, log=print, keep_operators=True,
                       lam=workloads.LAMBDA, z_src=workloads.Z_SRC, max_iter=8000, window=0,
                       net=None):
    """Pairs from `draws` random lens models and sources on geom = (visibility space, image
    space, source space, uvw), all sharing `nufft`: along plain Jacobi-CG trajectories
    (window = 0, learned.trajectory_pairs) or along flexible-CG trajectories with a
    `window`-direction A-orthogonalisation -- Jacobi, or with `net` as the preconditioner --
    together with each pair's window (learned.window_pairs)."""
    from .inversion import SourceInversion
    vs, ims, srcs, _ = geom
    rng = np.random.default_rng(seed)
    R, E, D, Fe, idx, iters, invs, Qs = [], [], [], [], [], [], [], []
    t0 = time.perf_counter()
    for k in range(draws):
        glm = learned.lens_draw(rng, centre=(0.25 * ims.dx, 0.25 * ims.dy))
        s = learned.random_source(rng, srcs)
        d = workloads.simulate(nufft, ims, srcs, glm, s, rng, z_src=z_src)
        inv = SourceInversion(vs, d, 1.0, ims, srcs, glm, z_src, lam, nufft=nufft)
        if window:
            r, e, Q, K = learned.window_pairs(inv, pairs, rng, window=window, net=net)
            Qs.append(Q)
        else:
            r, e, K, _ = learned.trajectory_pairs(inv, pairs, rng, max_iter=max_iter)
        R.append(r)
        E.append(e)
        D.append(inv.inv_diag32.clone())
        Fe.append(learned.features(inv.inv_diag32))
        idx.append(torch.full((r.shape[0],), k, dtype=torch.long, device="cuda"))
        iters.append(K)
        if keep_operators:
            invs.append(inv)
        del inv
        if (k + 1) % 10 == 0 or k + 1 == draws:
            log(f"draw {k + 1}/{draws}: {sum(x.shape[0] for x in R)} pairs, "
                f"{'flexible' if window else 'plain'} CG iterations {K}, "
                f"{time.perf_counter() - t0:.1f} s")
    r, e = torch.cat(R), torch.cat(E)
    return {"r": r, "e": e, "er": (e.double() * r.double()).sum(dim=1),
            "dinv": torch.stack(D), "feat": torch.stack(Fe), "draw": torch.cat(idx),
            "Q": torch.cat(Qs) if window else None, "window": window,
            "inversions": invs, "cg_iterations": iters, "seconds": time.perf_counter() - t0}


def merge_sets(a, b):
    """One training set from two built on the same grid (the second's draw indices shifted)."""
    nd = a["dinv"].shape[0]
    out = {k: torch.cat([a[k], b[k]]) for k in ("r", "e", "er", "dinv", "feat")}
    out["draw"] = torch.cat([a["draw"], b["draw"] + nd])
    out["Q"] = torch.cat([a["Q"], b["Q"]]) if a.get("Q") is not None else None
    out["window"] = a.get("window", 0)
    out["inversions"] = a["inversions"] + b["inversions"]
    out["cg_iterations"] = a["cg_iterations"] + b["cg_iterations"]
    out["seconds"] = a["seconds"] + b["seconds"]
    return out


def _dihedral(t, k):
    """One of the 8 flips/transposes of the last two axes."""
    if k & 4:
        t = t.transpose(-2, -1)
    if k & 1:
        t = t.flip(-2)
    if k & 2:
        t = t.flip(-1)
    return t


def batch(data, ids, H, W, aug):
    r = data["r"][ids].view(-1, H, W)
    e = data["e"][ids].view(-1, H, W)
    di = data["draw"][ids]
    dinv = data["dinv"][di].view(-1, H, W)
    feat = data["feat"][di].view(-1, H, W)
    if aug is not None:  # square grids: the 8 symmetries keep the shape
        aug = torch.as_tensor(aug, device=r.device)
        ts = [r.clone(), e.clone(), dinv.clone(), feat.clone()]
        for k in range(1, 8):
            m = aug == k
            if bool(m.any()):
                for dst, src in zip(ts, (r, e, dinv, feat)):
                    dst[m] = _dihedral(src[m], k)
        r, e, dinv, feat = ts
    return learned.scaled_inputs(r, dinv, feat, e)


def train(net, data, steps, batch_size, lr, seed, val_frac=0.05, log=print, log_every=250):
    H, W = net.H, net.W
    n = data["r"].shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=g)
    nval = max(batch_size, int(val_frac * n))
    val, tr = perm[:nval].cuda(), perm[nval:].cuda()
    losses = torch.zeros(steps, device="cuda")
    t0 = time.perf_counter()

    def val_loss():
        tot = 0.0
        for i in range(0, nval - batch_size + 1, batch_size):
            x, f, t = batch(data, val[i:i + batch_size], H, W, None)
            tot += net.gradients(x, f, t)[1]
        return tot / max(1, nval // batch_size)

    history = [{"step": 0, "val": val_loss()}]
    for it in range(steps):
        ids = tr[torch.randint(0, tr.numel(), (batch_size,), generator=g).cuda()]
        aug = torch.randint(0, 8, (batch_size,), generator=g).tolist()
        x, f, t = batch(data, ids, H, W, aug)
        lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * it / steps))
        net.train_step(x, f, t, lr_t, losses[it:it + 1])
        if (it + 1) % log_every == 0 or it + 1 == steps:
            tl = float(losses[max(0, it + 1 - log_every):it + 1].mean())
            vl = val_loss()
            history.append({"step": it + 1, "train": tl, "val": vl})
            log(f"step {it + 1}/{steps}: train {tl:.4g} val {vl:.4g} "
                f"({time.perf_counter() - t0:.1f} s)")
    torch.cuda.synchronize()
    if net.error_flag():
        raise RuntimeError("a tensor-core wait gave up during training")
    return history, time.perf_counter() - t0


def _apply_batch(data, ids, z):
    """A_j z_j with each sample's own normal operator (FP32)."""
    import ctypes
    from . import _native as N
    from .gridding import _ptr
    L = N.lib()
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    az = torch.empty_like(z)
    zf = z.reshape(z.shape[0], -1)
    af = az.reshape(z.shape[0], -1)
    for j, d in enumerate(data["draw"][ids].tolist()):
        N.check(L.lentils_normal_op_apply(data["inversions"][d].handle, _ptr(zf[j]),
                                          _ptr(af[j]), sp))
    return az


def energy_loss(data, ids, z):
    """Per-sample fraction of the A-norm error left after a line search along z,
    1 - (z.r)|z.r| / ((z.A z)(e.r)), and its gradient with respect to z. The signed numerator
    equals (z.r)^2 for a descent direction and puts directions with z.r < 0, which the solver
    rejects, above 1 (the plain fraction is blind to the sign of z)."""
    B = z.shape[0]
    r = data["r"][ids].view_as(z)
    az = _apply_batch(data, ids, z)
    zr = (z.double() * r.double()).sum(dim=(1, 2))
    zaz = (z.double() * az.double()).sum(dim=(1, 2))
    er = data["er"][ids]
    zaz = torch.where(zaz > 0, zaz, torch.ones_like(zaz))
    frac = 1.0 - zr * zr.abs() / (zaz * er)
    coef = (-2.0 * zr.abs() / (zaz * er) / B).float()[:, None, None]
    step = (zr / zaz).float()[:, None, None]
    grad = coef * (r - step * az)
    return frac, grad


def window_energy_loss(data, ids, z):
    """energy_loss for the direction flexible CG takes from z: p = z made A-orthogonal to the
    pair's window of directions p_j, stored as q_j = A p_j / sqrt(p_j.A p_j) (data["Q"], zero
    rows unused). With r = A e, p_j.r / sqrt(p_j.A p_j) = q_j.e, so
        p.r = z.r~,  r~ = r - sum_j (q_j.e) q_j,      p.Ap = D = z.Az - sum_j (z.q_j)^2,
    the error left is 1 - (z.r~)^2 / (D (e.r)). As in energy_loss the numerator is signed,
    (z.r~)|z.r~|, so that directions the solver rejects (z.r <= 0) score above 1; the gradient
    is -2 |z.r~| / (D (e.r)) * (r~ - (z.r~ / D) (Az - sum_j (z.q_j) q_j))."""
    B = z.shape[0]
    r = data["r"][ids].view_as(z)
    e = data["e"][ids].reshape(B, -1)
    az = _apply_batch(data, ids, z)
    Q = data["Q"][ids]                                   # (B, m, n)
    Qd = Q.double()
    zf = z.reshape(B, -1).double()
    zq = torch.bmm(Qd, zf.unsqueeze(2)).squeeze(2)      # (B, m): z.q_j
    eq = torch.bmm(Qd, e.double().unsqueeze(2)).squeeze(2)  # (B, m): e.q_j
    rt = r.reshape(B, -1).double() - torch.bmm(eq.unsqueeze(1), Qd).squeeze(1)
    zr = (zf * rt).sum(dim=1)
    zaz = (zf * az.reshape(B, -1).double()).sum(dim=1)
    D = zaz - (zq * zq).sum(dim=1)
    er = data["er"][ids]
    D = torch.where(D > 0, D, torch.ones_like(D))
    frac = 1.0 - zr * zr.abs() / (D * er)
    coef = (-2.0 * zr.abs() / (D * er) / B)[:, None]
    step = (zr / D)[:, None]
    proj = torch.bmm(zq.unsqueeze(1), Qd).squeeze(1)    # sum_j (z.q_j) q_j
    grad = coef * (rt - step * (az.reshape(B, -1).double() - proj))
    return frac, grad.float().view_as(z)


def train_energy(net, data, steps, batch_size, lr, seed, val_frac=0.05, log=print,
                 log_every=250, gamma=0.0):
    """Adam on the mean energy-norm loss of the direction z = gamma u/rms(u) + net(u/rms(u), f)
    (the preconditioner's output over rms(u), u = dinv r): energy_loss on plain-CG pairs,
    window_energy_loss on pairs that carry a flexible-CG window."""
    loss = window_energy_loss if data.get("Q") is not None else energy_loss
    H, W = net.H, net.W
    n = data["r"].shape[0]
    g = torch.Generator(device="cpu").manual_seed(seed)
    perm = torch.randperm(n, generator=g)
    nval = max(batch_size, int(val_frac * n))
    val, tr = perm[:nval].cuda(), perm[nval:].cuda()
    t0 = time.perf_counter()

    def inputs(ids):
        r = data["r"][ids].view(-1, H, W)
        di = data["draw"][ids]
        return learned.scaled_inputs(r, data["dinv"][di].view(-1, H, W),
                                     data["feat"][di].view(-1, H, W))

    def val_loss():
        tot, totj, cnt = 0.0, 0.0, 0
        for i in range(0, nval - batch_size + 1, batch_size):
            ids = val[i:i + batch_size]
            x, f = inputs(ids)
            tot += float(loss(data, ids, gamma * x + net.forward(x, f))[0].sum())
            totj += float(loss(data, ids, x)[0].sum())  # Jacobi direction
            cnt += ids.numel()
        return tot / cnt, totj / cnt

    v, vj = val_loss()
    history = [{"step": 0, "val": v, "val_jacobi": vj}]
    log(f"energy loss at start: val {v:.4f} (Jacobi direction {vj:.4f})")
    run = []
    for it in range(steps):
        ids = tr[torch.randint(0, tr.numel(), (batch_size,), generator=g).cuda()]
        x, f = inputs(ids)
        out = net.forward(x, f)
        frac, grad = loss(data, ids, gamma * x + out)
        run.append(frac.mean())
        lr_t = lr * 0.5 * (1.0 + math.cos(math.pi * it / steps))
        net.backward(grad, lr=lr_t)
        if (it + 1) % log_every == 0 or it + 1 == steps:
            tl = float(torch.stack(run).mean())
            run = []
            v, vj = val_loss()
            history.append({"step": it + 1, "train": tl, "val": v, "val_jacobi": vj})
            log(f"step {it + 1}/{steps}: train {tl:.4f} val {v:.4f} (Jacobi {vj:.4f}) "
                f"({time.perf_counter() - t0:.1f} s)")
    torch.cuda.synchronize()
    if net.error_flag():
        raise RuntimeError("a tensor-core wait gave up during training")
    return history, time.perf_counter() - t0


DEFAULT_POLICY = {"jacobi_weight": 0.3, "window": 8, "net_every": 1}


def deploy_policy(meta):
    """How the solver uses a trained network: Jacobi share gamma of the preconditioner, the
    flexible-CG window, and the network proposing every net_every-th direction (the descent
    check takes the Jacobi direction where it does not descend). Weight files record the
    policy their evaluation measured best under "deploy"; older files get DEFAULT_POLICY."""
    pol = dict(DEFAULT_POLICY)
    pol.update(meta.get("deploy", {}))
    return pol


def evaluate(net, inv, tol=1e-6, inner_tol=1e-3, repeats=2, gammas=(0.0,), windows=(1,),
             every=(1,)):
    """Plain Jacobi-CG against flexible CG with the network on one inversion (best of
    `repeats` after a warm-up solve of each), for each Jacobi share gamma, direction window
    and network period net_every."""
    def best_of(fn):
        best = None
        for _ in range(repeats):
            _, info = fn()
            if best is None or info["seconds"] < best["seconds"]:
                best = info
        return best

    inv.solve(tol=1e-2)
    inv.solve_flexible(net, tol=1e-2)
    out = {"plain": best_of(lambda: inv.solve(tol=tol, inner_tol=inner_tol)), "learned": {}}
    out["jacobi_fcg"] = {}
    for w in windows:
        out["jacobi_fcg"][str(w)] = best_of(lambda: inv.solve_flexible(
            None, tol=tol, inner_tol=inner_tol, window=w))
        for g in gammas:
            net.set_jacobi_weight(g)
            for ev in every:
                out["learned"][f"{g}/{w}/{ev}"] = best_of(lambda: inv.solve_flexible(
                    net, tol=tol, inner_tol=inner_tol, window=w, net_every=ev))
    key = min(out["learned"], key=lambda k: out["learned"][k]["seconds"])
    lb = out["learned"][key]
    g, w, ev = key.split("/")
    out["best"] = {"jacobi_weight": float(g), "window": int(w), "net_every": int(ev)}
    out["iteration_ratio"] = out["plain"]["inner_total"] / max(1, lb["inner_total"])
    out["time_ratio"] = out["plain"]["seconds"] / max(1e-12, lb["seconds"])
    net.set_jacobi_weight(float(g))
    return out


def save(path, params, meta):
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.savez_compressed(path, params=params, meta=json.dumps(meta))


def load(path):
    z = np.load(path)
    return z["params"], json.loads(str(z["meta"]))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--draws", type=int, default=100)
    ap.add_argument("--pairs", type=int, default=100)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--no-eval", action="store_true")
    ap.add_argument("--loss", choices=["energy", "window", "mse"], default="energy",
                    help="energy: plain-CG pairs; window: flexible-CG pairs with the "
                         "A-orthogonalisation window; mse: correction direction")
    ap.add_argument("--window", type=int, default=8, help="directions kept (--loss window)")
    ap.add_argument("--gamma", type=float, default=0.0,
                    help="Jacobi share of the trained direction (energy and window losses)")
    ap.add_argument("--refine-draws", type=int, default=0,
                    help="--loss window: draws of a second stage whose pairs come from "
                         "flexible-CG trajectories with the trained network in the loop")
    ap.add_argument("--refine-steps", type=int, default=3000)
    ap.add_argument("--refine-lr", type=float, default=3e-4)
    ap.add_argument("--reevaluate", action="store_true",
                    help="no training: measure the deployment policy of the weights in --out "
                         "again (network period 1, 2, 4, 8 with gamma 0 on the workload "
                         "inversion) and store it, keeping the previous evaluation")
    a = ap.parse_args(argv)

    def log(msg):
        print(msg, flush=True)

    if a.reevaluate:
        params, meta = load(a.out)
        inv, _, _ = workloads.inversion()
        pnet = learned.UNet(workloads.SRC, workloads.SRC, max_batch=1, params=params)
        ev = evaluate(pnet, inv, repeats=3, gammas=(0.0,), windows=(8,), every=(1, 2, 4, 8))
        if "evaluation" in meta:
            meta.setdefault("evaluation_history", []).append(
                {"evaluation": meta["evaluation"], "deploy": meta.get("deploy", {})})
        meta["evaluation"] = ev
        meta["deploy"] = ev["best"]
        log(json.dumps({k: ev[k] for k in ("best", "iteration_ratio", "time_ratio")}))
        log(json.dumps({k: (v["inner_total"], round(v["seconds"], 5)) for k, v in ev["learned"].items()}))
        log(json.dumps({k: (v["inner_total"], round(v["seconds"], 5)) for k, v in ev["jacobi_fcg"].items()}))
        save(a.out, params, meta)
        log(f"saved {a.out}")
        return 0

    from .operators import NUFFTOperator
    vs, ims, srcs, uvw, _ = workloads.geometry()
    F = NUFFTOperator(vs, ims)
    energy = a.loss in ("energy", "window")
    window = a.window if a.loss == "window" else 0
    data = build_training_set(F, (vs, ims, srcs, uvw), a.draws, a.pairs, a.seed, log,
                              keep_operators=energy, window=window)
    net = learned.UNet(workloads.SRC, workloads.SRC, max_batch=a.batch, seed=a.seed)
    if energy:
        history, train_s = train_energy(net, data, a.steps, a.batch, a.lr, a.seed, log=log,
                                        gamma=a.gamma)
    else:
        history, train_s = train(net, data, a.steps, a.batch, a.lr, a.seed, log=log)
    refine = {}
    if window and a.refine_draws > 0:
        pnet = learned.UNet(workloads.SRC, workloads.SRC, max_batch=1, params=net.params)
        pnet.set_jacobi_weight(a.gamma)
        extra = build_training_set(F, (vs, ims, srcs, uvw), a.refine_draws, a.pairs,
                                   a.seed + 1, log, window=window, net=pnet)
        del pnet
        refine = {"draws": a.refine_draws, "pairs": int(extra["r"].shape[0]),
                  "steps": a.refine_steps, "lr": a.refine_lr,
                  "trajectory_iterations_mean": float(np.mean(extra["cg_iterations"]))}
        data = merge_sets(data, extra)
        del extra
        h2, t2 = train_energy(net, data, a.refine_steps, a.batch, a.refine_lr, a.seed + 1,
                              log=log, gamma=a.gamma)
        refine["history"], refine["train_seconds"] = h2, t2
    meta = {"loss": a.loss, "draws": a.draws, "pairs": int(data["r"].shape[0]), "steps": a.steps,
            "batch": a.batch, "lr": a.lr, "seed": a.seed, "window": window, "gamma": a.gamma,
            "data_seconds": data["seconds"], "train_seconds": train_s, "history": history,
            "trajectory_iterations_mean": float(np.mean(data["cg_iterations"]))}
    if refine:
        meta["refine"] = refine
    del data
    if not a.no_eval:
        inv, _, _ = workloads.inversion(nufft=F)
        pnet = learned.UNet(workloads.SRC, workloads.SRC, max_batch=1, params=net.params)
        gammas = tuple(sorted({0.0, 0.3, a.gamma}))
        meta["evaluation"] = evaluate(pnet, inv, gammas=gammas, windows=(8,), every=(1, 2, 4, 8))
        meta["deploy"] = meta["evaluation"]["best"]
        log(json.dumps(meta["evaluation"]))
    save(a.out, net.params, meta)
    log(f"saved {a.out}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
