"""Batched lens-parameter sweep on one GPU (lentils_sweep_*; no counterpart in the reference,
whose operators run one lens model at a time).

Each sample is a lens model (PEMD + external shear drawn from priors), an n x n image plane
(pixel centres deflected to the source plane), and its own visibility set on the 2n x 2n
r2c grid of that image; its KB width follows from its accuracy target (autotune.width_for)
and its tile and work-item size from the autotuner (batched mode: timed inside the sweep
kernel). One run degrids every sample's grid,
grids every sample's visibilities and deflects every sample's pixel grid in one persistent
kernel launch, replayed as a CUDA graph.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _native as N
from .autotune import Autotuner, kb_beta, width_for
from .gridding import GriddingPlan, _ptr
from .lens_models import ExternalPotential, GlobalLensModel, PowerLawEllipsoid


@dataclass
class SweepSample:
    n: int                    # image edge (pixels)
    nvis: int                 # visibilities
    lenses: list              # mass models (PowerLawEllipsoid, ExternalPotential, ...)
    tol: float = 1e-5         # relative L2 accuracy target of the gridding (sets the KB width)
    pix: float = 0.02         # pixel size (arcsec)
    seed: int = 0             # uv draw
    info: dict = field(default_factory=dict)


def draw_samples(rng, nsamples=256, sizes=(128, 256, 384, 512), nvis_range=(1e5, 2e6),
                 eps=0.01):
    """The sweep workload: lens parameters from uniform priors (b in [0.8, 1.6], q in
    [0.5, 0.95], gamma in [1.8, 2.3], shear strength up to 0.1, angles uniform), image sizes
    from `sizes`, visibility counts log-uniform in nvis_range, and a per-sample accuracy target
    eps / sqrt(nvis) (the model error kept below the noise level of the sample's data, which
    falls as 1/sqrt(N) at fixed per-visibility signal-to-noise)."""
    out = []
    for k in range(nsamples):
        n = int(rng.choice(sizes))
        nvis = int(round(np.exp(rng.uniform(np.log(nvis_range[0]), np.log(nvis_range[1])))))
        b = rng.uniform(0.8, 1.6)
        q = rng.uniform(0.5, 0.95)
        gamma = rng.uniform(1.8, 2.3)
        th = rng.uniform(0.0, 180.0)
        ss = rng.uniform(0.0, 0.1)
        sa = rng.uniform(0.0, 180.0)
        x0, y0 = rng.uniform(-0.05, 0.05, 2)
        lenses = [PowerLawEllipsoid(z=0.5, b=b, th=th, f=q, x=x0, y=y0, rc=0.0,
                                    qh=0.5 * (gamma - 1.0)),
                  ExternalPotential(z=0.5, x=x0, y=y0, ss=ss, sa=sa)]
        out.append(SweepSample(n=n, nvis=nvis, lenses=lenses, tol=eps / np.sqrt(nvis),
                               seed=int(rng.integers(0, 2 ** 31))))
    return out


def _lens_array(lenses, z_s=2.0):
    return GlobalLensModel(lenses).setup_raytracing(z_s)


class BatchedSweep:
    """Plans, synthetic inputs (seeded), outputs and the native sweep of a list of samples.

    Per sample s: grid_in[s] (2n x (n+1) complex64 half plane), vis_in[s] (plan-order
    complex64), and after run(): vis_out[s] = degrid(grid_in[s]), grid_out[s] =
    grid(vis_in[s]), beta_out[s] (n*n, 2) float32 source-plane positions of the pixel centres
    (x-major). form selects the sweep kernel's item functions (lentils_sweep_create flags)."""

    def __init__(self, samples, tuner=None, seed=1, form=0):
        from .spaces import ImageSpace
        from .synthetic import padded_fourier_space, synth_uv
        self.samples = list(samples)
        self.uvw = []
        self.tuner = tuner if tuner is not None else Autotuner(mode="batched")
        self.stream = torch.cuda.Stream()
        gen = torch.Generator(device="cuda").manual_seed(seed)
        self.plans, self.grid_in, self.vis_in = [], [], []
        self.grid_out, self.vis_out, self.beta_out, self._lens = [], [], [], []
        cs = (N.SweepSampleC * max(1, len(self.samples)))()
        with torch.cuda.stream(self.stream):
            for k, s in enumerate(self.samples):
                half = 0.5 * s.n * s.pix
                four = padded_fourier_space(ImageSpace((s.n, s.n), [(-half, half),
                                                                    (-half, half)]), 2)
                nu, nv, du, dv = four.nu, four.nv, four.du, four.dv
                w2 = width_for(s.tol)
                tile, chunk = self.tuner.params(nu, nv, du, dv, w2, s.nvis)
                uvw = synth_uv(np.random.default_rng(s.seed), s.nvis, four, 0.45, w2 // 2)
                self.uvw.append(uvw)
                plan = GriddingPlan(uvw, [1.0], nu, nv, du, dv, 0.0, 0.0, w2 // 2, kb_beta(w2),
                                    tile=tile, chunk=chunk, stream=self.stream)
                s.info = {"w2": w2, "tile": tile, "chunk": chunk}
                gi = torch.randn((nu, nv // 2 + 1), dtype=torch.complex64, device="cuda",
                                 generator=gen)
                vi = torch.randn(s.nvis, dtype=torch.complex64, device="cuda", generator=gen)
                go = torch.empty_like(gi)
                vo = torch.empty_like(vi)
                bo = torch.empty((s.n * s.n, 2), dtype=torch.float32, device="cuda")
                la = _lens_array(s.lenses)
                self.plans.append(plan)
                self.grid_in.append(gi)
                self.vis_in.append(vi)
                self.grid_out.append(go)
                self.vis_out.append(vo)
                self.beta_out.append(bo)
                self._lens.append(la)
                c = cs[k]
                c.plan = plan.handle
                c.grid_in, c.vis_out = _ptr(gi), _ptr(vo)
                c.vis_in, c.grid_out = _ptr(vi), _ptr(go)
                c.lenses = ctypes.c_void_p(la.ctypes.data)
                c.nlenses = len(la)
                c.nx = c.ny = s.n
                dx = s.pix
                c.x0 = c.y0 = -half + 0.5 * dx
                c.dx = c.dy = dx
                c.beta_out = _ptr(bo)
            self._h = ctypes.c_void_p()
            N.check(N.lib().lentils_sweep_create(ctypes.byref(self._h), cs, len(self.samples),
                                                 int(form),
                                                 ctypes.c_void_p(self.stream.cuda_stream)))
        self.stream.synchronize()

    def pixel_points(self, k):
        """Pixel centres of sample k, (n*n, 2) float64, x-major (the deflected points)."""
        s = self.samples[k]
        half = 0.5 * s.n * s.pix
        c = -half + 0.5 * s.pix + s.pix * np.arange(s.n)
        xs, ys = np.meshgrid(c, c, indexing="ij")
        return np.stack([xs.reshape(-1), ys.reshape(-1)], axis=1)

    @property
    def handle(self):
        return self._h

    def run(self, use_graph=True, stream=None):
        st = self.stream if stream is None else stream
        N.check(N.lib().lentils_sweep_run(self._h, 1 if use_graph else 0,
                                          ctypes.c_void_p(st.cuda_stream)))

    def stats(self):
        s = N.SweepStatsC()
        N.check(N.lib().lentils_sweep_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            N.lib().lentils_sweep_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
