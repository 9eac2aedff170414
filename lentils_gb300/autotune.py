"""Autotuner for the gridding plans: Kaiser-Bessel width from an accuracy target, tile size and
work-item size (bin occupancy) from timing, cached in JSON.

KB width. With beta = 2.34 W and 2x oversampling the KB NUFFT differs from the direct Fourier
sum (dft_matrix_csr, lentils/backend/nufft.c:128-161) by a relative L2 error of about 1e-5 at
W = 6 and 9e-8 at W = 8 (measured against the oracle; KB_ERROR holds bounds of those
figures); width_for(tol) returns the narrowest width whose error bound meets tol.

Tile and chunk. For a workload class -- grid size, KB width, visibility-count bucket
(powers of two) and GPU architecture -- every (tile, chunk) candidate is timed on a seeded
synthetic visibility set of the class (density ~ 1/|uv| out to 0.45 of Nyquist) as one
degrid + grid pass with CUDA events (best of a few runs after a warm-up); the fastest wins.
Results are stored per class in a JSON file (default lentils_gb300/tuning/<arch>.json, or the
LENTILS_TUNING_CACHE path) and reused.

Batched mode (mode="batched", for the persistent lens sweep) times every candidate inside the
sweep kernel itself, on a small batch of synthetic samples of the class, because there the
parallelism comes from the many samples: fewer, larger work items win where a single plan
needs many small ones to fill the GPU. Its cache is <arch>_batched.json.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np
import torch

KB_ERROR = {6: 1.2e-5, 8: 1.2e-7}
TILES = (8, 16, 32)
CHUNKS = (256, 512, 1024, 2048)
DEFAULT_CACHE_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning")


def width_for(tol):
    """Narrowest KB width (6 or 8) whose NUFFT error bound meets the relative L2 target tol."""
    for w2 in sorted(KB_ERROR):
        if KB_ERROR[w2] <= tol:
            return w2
    return max(KB_ERROR)


def kb_beta(w2):
    return 2.34 * w2


def arch_name():
    if not torch.cuda.is_available():
        return "cpu"
    major, minor = torch.cuda.get_device_capability()
    return f"sm_{major}{minor}"


def nvis_bucket(nvis):
    return int(round(math.log2(max(1, nvis))))


BATCH_TILES = (8, 16)
BATCH_CHUNKS = (1024, 2048, 4096)


class Autotuner:
    def __init__(self, path=None, tiles=None, chunks=None, reps=3, mode="single"):
        if mode not in ("single", "batched"):
            raise ValueError("mode: 'single' or 'batched'")
        self.mode = mode
        suffix = "" if mode == "single" else "_batched"
        self.path = path or os.environ.get("LENTILS_TUNING_CACHE") or os.path.join(
            DEFAULT_CACHE_DIR, f"{arch_name()}{suffix}.json")
        if tiles is None:
            tiles = TILES if mode == "single" else BATCH_TILES
        if chunks is None:
            chunks = CHUNKS if mode == "single" else BATCH_CHUNKS
        self.tiles, self.chunks, self.reps = tuple(tiles), tuple(chunks), int(reps)
        self.cache = {}
        if os.path.exists(self.path):
            with open(self.path) as f:
                self.cache = json.load(f)
        self.tuned = 0

    @staticmethod
    def key(nu, nv, w2, nvis):
        return f"{nu}x{nv}/W{w2}/n2^{nvis_bucket(nvis)}"

    def params(self, nu, nv, du, dv, w2, nvis):
        """(tile, chunk) for the class of this plan, tuning it on first use."""
        k = self.key(nu, nv, w2, nvis)
        if k not in self.cache:
            fn = self.tune if self.mode == "single" else self.tune_batched
            self.cache[k] = fn(nu, nv, du, dv, w2, 2 ** nvis_bucket(nvis))
            self.tuned += 1
        c = self.cache[k]
        return int(c["tile"]), int(c["chunk"])

    def tune(self, nu, nv, du, dv, w2, nvis, seed=0):
        from .gridding import GriddingPlan
        from .synthetic import synth_uv

        class _Four:
            pass
        four = _Four()
        four.nu, four.nv, four.du, four.dv = nu, nv, du, dv
        rng = np.random.default_rng(seed)
        uvw = synth_uv(rng, int(nvis), four, 0.45, w2 // 2)
        dev = torch.device("cuda")
        grid = torch.randn((nu, nv // 2 + 1), dtype=torch.complex64, device=dev)
        vis = torch.randn(int(nvis), dtype=torch.complex64, device=dev)
        out_g = torch.empty_like(grid)
        out_v = torch.empty_like(vis)
        results = []
        for T in self.tiles:
            if T > nu // 2 or T > nv // 2:
                continue
            for chunk in self.chunks:
                plan = GriddingPlan(uvw, [1.0], nu, nv, du, dv, 0.0, 0.0, w2 // 2, kb_beta(w2),
                                    tile=T, chunk=chunk)
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                best = float("inf")
                for r in range(self.reps + 1):
                    torch.cuda.synchronize()
                    ev[0].record()
                    plan.degrid(grid, out_v)
                    plan.grid(vis, out_g)
                    ev[1].record()
                    torch.cuda.synchronize()
                    if r > 0:
                        best = min(best, ev[0].elapsed_time(ev[1]))
                results.append({"tile": T, "chunk": chunk, "ms": best})
                plan.close()
        best = min(results, key=lambda r: r["ms"])
        return {"tile": best["tile"], "chunk": best["chunk"], "ms": best["ms"],
                "candidates": results}

    def tune_batched(self, nu, nv, du, dv, w2, nvis, nsamples=8, seed=0):
        """Best (tile, chunk) for samples of this class inside the persistent sweep."""
        from .sweep import BatchedSweep, draw_samples
        rng = np.random.default_rng(seed)
        n = nu // 2
        samples = draw_samples(rng, nsamples, sizes=(n,), nvis_range=(nvis, nvis))
        pix = 0.02
        for smp in samples:
            smp.tol = KB_ERROR[w2]
            smp.pix = pix

        class _Fixed:
            def __init__(self, t, c):
                self.t, self.tuned = (t, c), 0

            def params(self, *a):
                return self.t

        results = []
        for T in self.tiles:
            if T > nu // 2 or T > nv // 2:
                continue
            for chunk in self.chunks:
                sw = BatchedSweep(samples, tuner=_Fixed(T, chunk))
                s = sw.stream
                ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
                sw.run()
                best = float("inf")
                for _ in range(self.reps):
                    s.synchronize()
                    ev[0].record(s)
                    sw.run()
                    ev[1].record(s)
                    s.synchronize()
                    best = min(best, ev[0].elapsed_time(ev[1]))
                results.append({"tile": T, "chunk": chunk, "ms": best})
                sw.close()
        best = min(results, key=lambda r: r["ms"])
        return {"tile": best["tile"], "chunk": best["chunk"], "ms": best["ms"],
                "candidates": results}

    def save(self):
        os.makedirs(os.path.dirname(os.path.abspath(self.path)), exist_ok=True)
        with open(self.path, "w") as f:
            json.dump(self.cache, f, indent=1, sort_keys=True)
