"""Benchmark: Kaiser-Bessel degrid + grid throughput (Mvis/s) on one GB300.

Workload (the full-size single-operator configuration): 1024^2 image at 0.02" pixels,
2x-padded 2048 x 2048 uv grid (r2c half plane 2048 x 1025, complex64), KB width W = 8
(w = 4, beta = 2.34*W), 1e7 visibilities: 90% with areal density ~ 1/|uv| out to 0.48 of the
grid's Nyquist extent, 10% in 50 Gaussian blobs of width 0.005 Nyquist. Synthetic, seeded.

One step = one degrid (grid -> visibilities) + one grid (visibilities -> zeroed grid) over
all 1e7 visibilities, plan-ordered and resident in HBM (`value`). Per step the kernels stream
coordinates, visibilities and outputs (~240 MB) -- more than the 129 MB L2 -- so no L2
flush is inserted between steps. `e2e` runs the same pair through the C ABI's host-buffer
entry points (lentils_degrid_host / lentils_grid_host) on pinned complex128 host buffers in
the reference's row order, host<->device copies and conversions inside the timed region.

`--impl reference` times the reference's CPU gridder (the compiled reference C from
oracle/_ref when present, else the oracle's C port of it) with all host threads on a bounded
sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "degrid+grid Mvis/s"
UNIT = "Mvis/s"
NVIS = 10_000_000
IMG = 1024
PIX = 0.02
WSUP = 4
BETA = 2.34 * 2 * WSUP
SEED = 1234


def workload_config():
    return {"workload": "KB degrid+grid, 1024^2 image -> 2048x2048 grid (half plane "
                        "2048x1025 c64), W=8, 1e7 vis (10% in 50 blobs)",
            "nvis": NVIS, "grid": [2 * IMG, 2 * IMG], "kernel_width": 2 * WSUP,
            "kb_beta": BETA, "pixel_arcsec": PIX, "seed": SEED,
            "l2": "per-step inputs (~240 MB) exceed the 129 MB L2; no flush",
            "parallelism": "replicas"}


def make_uv():
    import numpy as np
    from lentils_gb300.spaces import ImageSpace
    from lentils_gb300.synthetic import padded_fourier_space, synth_uv_blobs
    rng = np.random.default_rng(SEED)
    half = 0.5 * IMG * PIX
    four = padded_fourier_space(ImageSpace((IMG, IMG), [(-half, half), (-half, half)]), 2)
    uvw = synth_uv_blobs(rng, NVIS, four, 0.48, WSUP)
    return four, uvw


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
        self.dev = device_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                stderr=subprocess.DEVNULL)
            time.sleep(0.6)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [ln.strip().split(",") for ln in self.f.read().splitlines() if ln.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax = max(smax, float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "samples": len(sm),
                "reasons": sorted(reasons)}


def load_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# The default kernels of the two directions at W = 8, and their DRAM bytes (read + write) per
# launch on this workload from one ncu capture of the same plan (dram__bytes_read.sum +
# dram__bytes_write.sum, tile 16, chunk 4096).
DEGRID_KERNEL, GRID_KERNEL = "degrid_chunk_kernel", "grid_pairs_kernel"
TRAFFIC = {DEGRID_KERNEL: 130845440, GRID_KERNEL: 167329792}
# FP32 lanes: 152 SMs x 128 FMA per clock x 2 FLOP at the 2.07 GHz maximum SM clock (nominal).
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def cpu_reference_lib():
    """The compiled reference gridder when present (oracle/_ref), else the oracle C port."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    if O.ref_available():
        try:
            O.ref_lib("nufft")
            return O, True
        except OSError:
            pass
    O.build_port()
    O.port_lib()
    return O, False


def _oracle_fourier(O, four):
    """The oracle's geometry record for a package FourierSpace."""
    import numpy as np
    f = O.FourierGeom.__new__(O.FourierGeom)
    f.nu, f.nv, f.half_nv = int(four.nu), int(four.nv), int(four.half_nv)
    f.du, f.dv, f.gcx, f.gcy = float(four.du), float(four.dv), float(four.gcx), float(four.gcy)
    f._chan = np.zeros(1)
    return f


def time_cpu_gridder(O, use_ref, four, uvw, nsample, reps=1):
    import numpy as np
    four = _oracle_fourier(O, four)
    rng = np.random.default_rng(SEED + 1)
    idx = rng.choice(uvw.shape[0], nsample, replace=False)
    vis = O.VisGeom(uvw[idx], [1.0])
    g = (rng.normal(size=four.shape) + 1j * rng.normal(size=four.shape))
    y = O.complex_normal(rng, vis.nvis)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        O.degrid(vis, four, g, WSUP, BETA, use_ref=use_ref)
        O.grid(vis, four, y, WSUP, BETA, use_ref=use_ref)
        times.append(time.perf_counter() - t0)
    return times


class Ranks:
    """Process-group plumbing of an N-GPU run: one process per GPU, launched by torchrun
    (RANK / LOCAL_RANK / WORLD_SIZE / MASTER_* in the environment). Every rank runs its own
    replica of the workload; the only collectives are the barriers around the timed region and
    the maximum of the ranks' times."""

    def __init__(self, backend="nccl"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = backend
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend, init_method="env://")

    def _device(self):
        import torch
        return torch.device("cuda", self.local) if self.backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()

    def max(self, x):
        """The maximum of x over the ranks (x itself on one rank)."""
        if self.world == 1:
            return float(x)
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64, device=self._device())
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


def whole_job_rate(world, units_per_rank, seconds):
    """Whole-job throughput in millions of units per second: every rank processes
    units_per_rank in `seconds` (the slowest rank's time)."""
    return world * units_per_rank / seconds / 1e6


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    O, use_ref = cpu_reference_lib()
    four, uvw = make_uv()
    # calibrate, then size each step's sample so the whole run stays within ~2-3 minutes
    cal = 20000
    t = time_cpu_gridder(O, use_ref, four, uvw, cal)[0]
    rate = cal / t
    per_step = min(10.0, 150.0 / max(1, args.steps + args.warmup))
    nsample = int(max(5000, min(2_000_000, rate * per_step)))
    time_cpu_gridder(O, use_ref, four, uvw, nsample, reps=args.warmup)
    ts = time_cpu_gridder(O, use_ref, four, uvw, nsample, reps=args.steps)
    total = sum(ts)
    value = nsample * args.steps / total / 1e6
    kind = "reference" if use_ref else "port"
    sample = (f"{nsample} of the 1e7 visibilities (random subset incl. blobs), full 2048x1025 "
              f"grid, degrid+grid per step, OMP_NUM_THREADS={os.environ['OMP_NUM_THREADS']}")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import numpy as np
    import torch

    ranks = Ranks("nccl")
    world, rank, local = ranks.world, ranks.rank, ranks.local
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from lentils_gb300 import _native as N
    from lentils_gb300.gridding import GriddingPlan

    four, uvw = make_uv()
    plan_t0 = time.perf_counter()
    plan = GriddingPlan(uvw, [1.0], four.nu, four.nv, four.du, four.dv, four.gcx, four.gcy,
                        WSUP, BETA)
    torch.cuda.synchronize()
    plan_s = time.perf_counter() - plan_t0
    st = plan.stats
    nvis = plan.nvis

    gen = torch.Generator(device=dev).manual_seed(SEED)
    grid_in = torch.complex(torch.randn((four.nu, four.half_nv), generator=gen, device=dev),
                            torch.randn((four.nu, four.half_nv), generator=gen, device=dev))
    vis_in = torch.complex(torch.randn(nvis, generator=gen, device=dev),
                           torch.randn(nvis, generator=gen, device=dev))
    vis_out = torch.empty(nvis, dtype=torch.complex64, device=dev)
    grid_out = torch.zeros((four.nu, four.half_nv), dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream()

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        plan.degrid(grid_in, out=vis_out)
        if ev is not None:
            ev[1].record(stream)
        plan.grid(vis_in, out=grid_out, accumulate=False)
        if ev is not None:
            ev[2].record(stream)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()

    # per-kernel timing (events on the launching stream)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    clocks = ClockSampler(local)
    clocks.start()
    ranks.barrier()
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    torch.cuda.synchronize()
    ranks.barrier()
    clk = clocks.stop()
    total_ms = t_start.elapsed_time(t_end)
    deg_ms = sum(e[0].elapsed_time(e[1]) for e in evs) / args.steps
    grd_ms = sum(e[1].elapsed_time(e[2]) for e in evs) / args.steps
    total_ms = ranks.max(total_ms)
    ms_per_step = total_ms / args.steps
    value = whole_job_rate(world, nvis, ms_per_step * 1e-3)

    # roofline of the dominant kernel: algorithmic bytes = N*(8 B coords + 8 B vis) + G
    G = four.nu * four.half_nv * 8
    alg_bytes = nvis * 16 + G
    dominant = GRID_KERNEL if grd_ms >= deg_ms else DEGRID_KERNEL
    dom_ms = max(grd_ms, deg_ms)
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
    traffic = TRAFFIC.get(dominant)

    # end to end through the C ABI host-buffer entry points, pinned complex128 host buffers
    grid_h = torch.empty((four.nu, four.half_nv), dtype=torch.complex128, pin_memory=True)
    grid_h.copy_(grid_in.cpu().to(torch.complex128))
    vis_h = torch.empty(nvis, dtype=torch.complex128, pin_memory=True)
    vis_h.copy_(vis_in.cpu().to(torch.complex128))
    vis_o = torch.empty(nvis, dtype=torch.complex128, pin_memory=True)
    grid_o = torch.empty((four.nu, four.half_nv), dtype=torch.complex128, pin_memory=True)
    L = N.lib()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def e2e_step():
        N.check(L.lentils_degrid_host(plan.handle, ctypes.c_void_p(grid_h.data_ptr()),
                                      ctypes.c_void_p(vis_o.data_ptr()), 0, sp))
        N.check(L.lentils_grid_host(plan.handle, ctypes.c_void_p(vis_h.data_ptr()),
                                    ctypes.c_void_p(grid_o.data_ptr()), 0, sp))

    for _ in range(2):
        e2e_step()
    e2e_steps = max(3, min(args.steps, 20))
    torch.cuda.synchronize()
    ranks.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = ranks.max((time.perf_counter() - t0) / e2e_steps)
    ranks.barrier()
    e2e_value = whole_job_rate(world, nvis, e2e_s)
    h2d = G * 2 + nvis * 16
    d2h = nvis * 16 + G * 2
    dropin = None if args.no_dropin else time_dropin(four, uvw, grid_h, vis_h, ranks)
    del grid_h, vis_h, vis_o, grid_o

    # accuracy of the timed outputs against the FP64 operator on the same inputs
    parity = fp64_parity(plan, grid_in, vis_in, vis_out, grid_out)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(),
            "gpu_launches": 2 * args.steps,
            "kernels_ms": {DEGRID_KERNEL: deg_ms, GRID_KERNEL: grd_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "kernel": dominant,
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "pair_frac": 2 * alg_bytes / ((deg_ms + grd_ms) * 1e-3) / 1e9 / peak,
                         "fp32_taps": fp32_taps_roofline(nvis, deg_ms, grd_ms)},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3,
                    "api": "lentils_degrid_host + lentils_grid_host (pinned c128, row order)"},
            "parity": parity,
            "e2e_dropin": dropin,
            "plan": {"build_s": plan_s, "items": st["nitems"], "tile": st["tile"],
                     "heaviest_tile_vis": st["heaviest_tile_vis"]},
            "clocks": clk,
        }
        if not args.no_deflect:
            line["deflect"] = run_deflect_bench(peak, cpu=not args.no_cpu_baseline)
        if not args.no_cg:
            line["cg"] = run_cg_bench(cpu=not (args.no_cpu_baseline or args.no_cpu_cg))
        if not args.no_sweep:
            line["sweep"] = run_sweep_bench(peak, args.sweep_samples)
        if not args.no_unet:
            line["unet"] = run_unet_bench()
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(four, uvw)
        print(json.dumps(line))
    ranks.close()
    return 0


def fp32_taps_roofline(nvis, deg_ms, grd_ms):
    """The tap arithmetic of both kernels against the nominal FP32 rate: each visibility is
    (2w)^2 complex-by-real multiply-adds per direction (4 FLOP each), weights not counted."""
    flop = 4 * (2 * WSUP) ** 2
    out = {"flop_per_vis": flop, "peak_tflops": FP32_PEAK_TFLOPS,
           "peak_source": "nominal: 152 SMs x 128 FP32 FMA/clock x 2 FLOP x 2.07 GHz"}
    for name, ms in (("degrid", deg_ms), ("grid", grd_ms)):
        t = nvis * flop / (ms * 1e-3) / 1e12
        out[name] = {"achieved_tflops": t, "frac": t / FP32_PEAK_TFLOPS}
    return out


def fp64_parity(plan, grid_in, vis_in, vis_out, grid_out):
    """Relative L2 of the timed FP32 outputs (the last step's degrid and grid, all 1e7
    visibilities and the whole half-plane grid) against the FP64 operator (lentils_degrid64 /
    lentils_grid64: FP64 coordinates, weights and accumulation, pinned to the oracle at this
    size by tests/test_gridding_gpu.py::test_full_size_fp32_vs_oracle) on the same inputs."""
    import torch

    def rel(a, b):
        a = a.to(torch.complex128).reshape(-1)
        b = b.reshape(-1)
        return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
    v64 = plan.degrid64(grid_in.to(torch.complex128))
    e_deg = rel(vis_out, v64)
    del v64
    g64 = plan.grid64(vis_in.to(torch.complex128))
    e_grid = rel(grid_out, g64)
    del g64
    torch.cuda.synchronize()
    return {"degrid_rel_l2": e_deg, "grid_rel_l2": e_grid, "bar": 1e-5,
            "against": "FP64 degrid/grid on the GPU (lentils_degrid64/lentils_grid64) of the "
                       "same inputs, all 1e7 visibilities",
            "accumulation": "plain FP32 (register runs over cell pairs, warp-private shared "
                            "tiles, float2 global atomics)"}


def time_dropin(four, uvw, grid_h, vis_h, ranks, steps=5):
    """The reference's own call path: grid_cpu FORWARD then ADJOINT with the reference's
    by-value structs and host complex128 buffers, as GriddingOperator._matrixfree_forward /
    _transpose make them (fourier_operators.py:85-93: fresh numpy zeros for each output), the
    uv binning kept by the drop-in's plan cache after the first call. Also with page-locked
    buffers (torch pinned tensors), which the kernels read and write directly."""
    import numpy as np
    import torch
    from lentils_gb300 import _native as N
    from lentils_gb300.spaces import VisibilitySpace
    L = N.lib()
    vs = VisibilitySpace(channels=[1.0], uvcoords=uvw)
    gs = N.FourierSpaceC(four.nu, four.nv, four.half_nv, 1, 1, four.du, four.dv, four.gcx,
                         four.gcy, None)
    g_np, v_np = grid_h.numpy().copy(), vis_h.numpy().copy()
    nvis = v_np.size

    def call(vis, grid, direction):
        L.grid_cpu(vs, ctypes.c_void_p(vis), gs, ctypes.c_void_p(grid), WSUP, BETA, direction)
        N.check_last()

    def pageable():
        v = np.zeros(nvis, dtype=np.complex128)
        call(v.ctypes.data, g_np.ctypes.data, 0)
        g = np.zeros(g_np.shape, dtype=np.complex128)
        call(v_np.ctypes.data, g.ctypes.data, 1)

    vo = torch.zeros(nvis, dtype=torch.complex128, pin_memory=True)
    go = torch.zeros(g_np.shape, dtype=torch.complex128, pin_memory=True)

    def pinned():
        vo.zero_()
        call(vo.data_ptr(), grid_h.data_ptr(), 0)
        go.zero_()
        call(vis_h.data_ptr(), go.data_ptr(), 1)

    out = {"api": "grid_cpu(FORWARD) + grid_cpu(ADJOINT), reference structs and signature",
           "unit": UNIT, "cache_mode": 1}
    t0 = time.perf_counter()
    pageable()  # first call: binning (plan cache miss)
    out["first_call_s"] = time.perf_counter() - t0
    for name, fn in (("pageable", pageable), ("pinned", pinned)):
        fn()
        ranks.barrier()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        dt = ranks.max((time.perf_counter() - t0) / steps)
        out[name] = {"value": whole_job_rate(ranks.world, nvis, dt), "ms_per_step": dt * 1e3}
    out["note"] = ("pageable: fresh numpy zeros per output, staged through device copies "
                   "(the reference caller's buffers); pinned: outputs zeroed on the host, kernels "
                   "address the page-locked buffers directly")
    L.lentils_dropin_cache_clear()
    return out


def run_deflect_bench(peak, cpu=True, steps=10, warmup=3):
    """PEMD + external-shear deflection (the CG workload's lens: b=1.2", q=0.7, gamma=2,
    shear 0.05 at 20 deg) in FP32 on the GPU: the 512^2 pixel grid of one image (262,144
    points, L2-resident, one launch) and 256 such grids offset by sub-pixel shifts (6.7e7
    points, 1.07 GB streamed) -- the roofline case, 16 algorithmic bytes per point (8 B in,
    8 B out). Error of the FP32 output against the FP64 path (lentils_deflect_f64io, pinned to
    the compiled reference by tests/test_deflect_gpu.py). Beside it the reference's serial
    deflect_points on the host (FP64, one thread as shipped)."""
    import numpy as np
    import torch
    from lentils_gb300 import _native as N
    from lentils_gb300 import workloads as WL
    lenses = np.ascontiguousarray(WL.lens_model().setup_raytracing(WL.Z_SRC))
    L = N.lib()
    half = 0.5 * WL.IMG * WL.PIX
    c = -half + WL.PIX * (np.arange(WL.IMG) + 0.5)
    pts = np.stack(np.meshgrid(c, c, indexing="ij"), axis=-1).reshape(-1, 2)
    s = torch.cuda.current_stream()
    sp = ctypes.c_void_p(s.cuda_stream)
    lp = ctypes.c_void_p(lenses.ctypes.data)
    out = {"workload": "PEMD b=1.2 q=0.7 gamma=2 + shear (0.05, 20 deg); 512^2 pixel centres "
                       "(0.01\") per image", "bytes_per_point": 16}
    shifts = np.random.default_rng(SEED + 5).uniform(-0.5, 0.5, (256, 2)) * WL.PIX
    for name, nimg in (("one_image", 1), ("256_images", 256)):
        p = pts[None] if nimg == 1 else pts[None] + shifts[:, None, :]
        p32 = torch.as_tensor(p.reshape(-1, 2).astype(np.float32)).cuda()
        o32 = torch.empty_like(p32)
        n = p32.shape[0]
        for _ in range(warmup):
            N.check(L.lentils_deflect_f32(lp, len(lenses), ctypes.c_void_p(p32.data_ptr()),
                                          ctypes.c_void_p(o32.data_ptr()), n, sp))
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(s)
        for _ in range(steps):
            N.check(L.lentils_deflect_f32(lp, len(lenses), ctypes.c_void_p(p32.data_ptr()),
                                          ctypes.c_void_p(o32.data_ptr()), n, sp))
        ev[1].record(s)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / steps
        achieved = 16.0 * n / (ms * 1e-3) / 1e9
        r = {"points": n, "ms_per_launch": ms, "mpts_per_s": n / (ms * 1e-3) / 1e6,
             "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                          "frac": achieved / peak}}
        # error against the FP64 path on the same (FP32-rounded) input points
        p64 = p32.double()
        o64 = torch.empty_like(p64)
        N.check(L.lentils_deflect_f64io(lp, len(lenses), ctypes.c_void_p(p64.data_ptr()),
                                        ctypes.c_void_p(o64.data_ptr()), n, sp))
        torch.cuda.synchronize()
        a32, a64 = (p64 - o32.double()), (p64 - o64)
        r["alpha_rel_l2_vs_fp64"] = float(torch.linalg.vector_norm(a32 - a64)
                                          / torch.linalg.vector_norm(a64))
        r["max_abs_err_arcsec"] = float((o32.double() - o64).abs().max())
        out[name] = r
        del p32, o32, p64, o64
    if cpu:
        O, _ = cpu_reference_lib()
        use_ref = O.ref_available()
        reps, t = 0, 0.0
        while t < 3.0:
            t0 = time.perf_counter()
            O.deflect(lenses, pts, use_ref=use_ref)
            t += time.perf_counter() - t0
            reps += 1
        out["cpu_baseline"] = {"value": reps * pts.shape[0] / t / 1e6, "unit": "Mpts/s",
                               "cores": 1, "kind": "reference" if use_ref else "port",
                               "sample": f"{reps} x 512^2 points, FP64, serial as shipped"}
    return out


# CG source inversion (512^2 image plane, 128^2 source grid, 2e6 visibilities, PEMD b=1.2",
# q=0.7, gamma=2.0 + external shear (0.05, 20 deg), lambda=1e-2 gradient prior, sigma=1).
def run_cg_bench(repeats=3, cpu=True):
    """CG source inversion to a true FP64 relative residual of 1e-6 (FP32 operator inside FP64
    iterative refinement, CUDA-graph inner iterations), three ways, each the best of `repeats`
    solves after a warm-up solve: plain Jacobi-PCG; flexible CG with Jacobi directions and an
    8-direction A-orthogonalisation window; the same with the learned preconditioner
    (committed weights, trained on the GPU by lentils_gb300.train_preconditioner, used with the
    deployment policy stored beside them)."""
    import ctypes
    import torch
    from lentils_gb300 import _native as N
    from lentils_gb300 import learned, workloads
    from lentils_gb300 import train_preconditioner as T
    from lentils_gb300.gridding import _ptr
    t0 = time.perf_counter()
    inv, _, geom = workloads.inversion()
    setup_s = time.perf_counter() - t0
    params, meta = T.load(T.DEFAULT_WEIGHTS)
    pol = T.deploy_policy(meta)
    net = learned.UNet(workloads.SRC, workloads.SRC, max_batch=1, params=params)
    net.set_jacobi_weight(pol["jacobi_weight"])
    inner_tol = 1e-3

    def learned_solve(target):
        return lambda tol: target.solve_flexible(net, tol=tol, inner_tol=inner_tol,
                                                 window=pol["window"],
                                                 net_every=pol["net_every"])
    runs = {
        "plain_jacobi_pcg": lambda tol: inv.solve(tol=tol, inner_tol=inner_tol),
        "jacobi_fcg8": lambda tol: inv.solve_flexible(None, tol=tol, inner_tol=inner_tol,
                                                      window=8),
        "learned_fcg8": learned_solve(inv),
    }
    out = {"workload": workloads.DESCRIPTION, "tol": 1e-6, "inner_tol": inner_tol,
           "setup_s": setup_s}
    for name, fn in runs.items():
        fn(1e-2)  # warm-up: graph capture, cuFFT plans, caches
        best = None
        for _ in range(repeats):
            _, info = fn(1e-6)
            if best is None or info["seconds"] < best["seconds"]:
                best = info
        out[name] = {"converged": best["converged"], "rel_residual_fp64": best["rel_residual"],
                     "outer": best["outer"], "inner_iterations": best["inner_total"],
                     "solve_s": best["seconds"]}
        if name == "learned_fcg8":
            out[name].update({"net_iterations": best["net_iterations"],
                              "fallback": best["fallback"], "policy": pol,
                              "training": {k: meta[k] for k in ("draws", "pairs", "steps",
                                                                "loss") if k in meta}})
    # the same inversion with the dirty-beam data term (the reference's production form)
    t1 = time.perf_counter()
    inv_b = workloads.inversion(nufft=inv.nufft, data_term="bcb")[0]
    out["bcb_setup_s"] = time.perf_counter() - t1
    runs_b = {
        "bcb_plain_jacobi_pcg": lambda tol: inv_b.solve(tol=tol, inner_tol=inner_tol),
        "bcb_jacobi_fcg8": lambda tol: inv_b.solve_flexible(None, tol=tol, inner_tol=inner_tol,
                                                            window=8),
        "bcb_learned_fcg8": learned_solve(inv_b),
    }
    for name, fn in runs_b.items():
        fn(1e-2)
        best = None
        for _ in range(repeats):
            _, info = fn(1e-6)
            if best is None or info["seconds"] < best["seconds"]:
                best = info
        out[name] = {"converged": best["converged"], "rel_residual_fp64": best["rel_residual"],
                     "outer": best["outer"], "inner_iterations": best["inner_total"],
                     "solve_s": best["seconds"]}
    p, lr = out["plain_jacobi_pcg"], out["learned_fcg8"]
    out["learned_vs_plain_time"] = p["solve_s"] / lr["solve_s"]
    out["learned_vs_plain_iterations"] = p["inner_iterations"] / max(1, lr["inner_iterations"])
    out["learned_vs_jacobi_fcg8_time"] = out["jacobi_fcg8"]["solve_s"] / lr["solve_s"]
    # per-iteration pieces, timed with events on the solver's stream
    s32 = torch.randn(inv.nsrc, device="cuda", dtype=torch.float32)
    s64 = s32.double()
    o32, o64 = torch.empty_like(s32), torch.empty_like(s64)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
    sp = ctypes.c_void_p(inv.stream.cuda_stream)
    L = N.lib()
    dinv, feat = inv.inv_diag32, learned.features(inv.inv_diag32)
    torch.cuda.synchronize()
    for _ in range(3):
        N.check(L.lentils_normal_op_apply(inv.handle, _ptr(s32), _ptr(o32), sp))
        N.check(L.lentils_unet_precondition(net.handle, _ptr(s32), _ptr(dinv), _ptr(feat),
                                            _ptr(o32), sp))
    ev[0].record(inv.stream)
    for _ in range(10):
        N.check(L.lentils_normal_op_apply(inv.handle, _ptr(s32), _ptr(o32), sp))
    ev[1].record(inv.stream)
    N.check(L.lentils_normal_op_apply64(inv.handle, _ptr(s64), _ptr(o64), sp))
    ev[2].record(inv.stream)
    N.check(L.lentils_normal_op_apply64(inv.handle, _ptr(s64), _ptr(o64), sp))
    ev[3].record(inv.stream)
    for _ in range(10):
        N.check(L.lentils_unet_precondition(net.handle, _ptr(s32), _ptr(dinv), _ptr(feat),
                                            _ptr(o32), sp))
    ev[4].record(inv.stream)
    torch.cuda.synchronize()  # the dirty-beam timing below must not overlap the work above
    spb = ctypes.c_void_p(inv_b.stream.cuda_stream)
    for _ in range(3):
        N.check(L.lentils_normal_op_apply(inv_b.handle, _ptr(s32), _ptr(o32), spb))
    ev[5].record(inv_b.stream)
    for _ in range(10):
        N.check(L.lentils_normal_op_apply(inv_b.handle, _ptr(s32), _ptr(o32), spb))
    ev[6].record(inv_b.stream)
    torch.cuda.synchronize()
    out.update({"matvec32_ms": ev[0].elapsed_time(ev[1]) / 10,
                "matvec64_ms": ev[2].elapsed_time(ev[3]),
                "precondition_ms": ev[3].elapsed_time(ev[4]) / 10,
                "bcb_matvec32_ms": ev[5].elapsed_time(ev[6]) / 10})
    out["gpu_fp64_jacobi_pcg"] = fp64_pcg(inv)
    out["bcb_gpu_fp64_jacobi_pcg"] = fp64_pcg(inv_b)
    out["gpu_mixed_jacobi_pcg"] = fp64_pcg(inv, operator32=True)
    out["bcb_gpu_mixed_jacobi_pcg"] = fp64_pcg(inv_b, operator32=True)
    lr = out["learned_fcg8"]["solve_s"]
    out["learned_vs_mixed_pcg_time"] = out["gpu_mixed_jacobi_pcg"]["solve_s"] / lr
    out["learned_vs_mixed_pcg_iterations"] = (out["gpu_mixed_jacobi_pcg"]["iterations"]
                                              / max(1, out["learned_fcg8"]["inner_iterations"]))
    if cpu:
        out["cpu_cg"] = cpu_cg_baseline(inv, geom)
    return out


def fp64_pcg(inv, tol=1e-6, maxiter=5000, operator32=False):
    """Plain Jacobi-PCG with FP64 vectors on the GPU (torch vector operations, no refinement
    loop, no restarts): the FP64 operator (lentils_normal_op_apply64) every iteration, or with
    operator32 the FP32 operator (lentils_normal_op_apply) on the FP32-rounded direction.
    Its iteration count is what CG needs without the conjugacy that FP32 inner vectors and
    restarts lose; the answer's true residual is recomputed with the FP64 operator."""
    import torch
    from lentils_gb300 import _native as N
    from lentils_gb300.gridding import _ptr
    L = N.lib()
    s = inv.stream
    sp = ctypes.c_void_p(s.cuda_stream)
    b = inv.b
    dinv = inv.inv_diag
    ap = torch.empty_like(b)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(s):
        x = torch.zeros_like(b)
        r = b.clone()
        z = dinv * r
        p = z.clone()
        rz = torch.dot(r, z)
        bn = float(torch.linalg.vector_norm(b))
        it = 0
        p32 = torch.empty(p.shape, dtype=torch.float32, device=p.device)
        ap32 = torch.empty_like(p32)
        while it < maxiter:
            if operator32:
                p32.copy_(p)
                N.check(L.lentils_normal_op_apply(inv.handle, _ptr(p32), _ptr(ap32), sp))
                ap.copy_(ap32)
            else:
                N.check(L.lentils_normal_op_apply64(inv.handle, _ptr(p), _ptr(ap), sp))
            alpha = rz / torch.dot(p, ap)
            x.add_(alpha * p)
            r.sub_(alpha * ap)
            it += 1
            if it % 10 == 0 and float(torch.linalg.vector_norm(r)) <= tol * bn:
                break
            z = dinv * r
            rz_new = torch.dot(r, z)
            p.mul_(rz_new / rz).add_(z)
            rz = rz_new
        N.check(L.lentils_normal_op_apply64(inv.handle, _ptr(x), _ptr(ap), sp))
        true_res = float(torch.linalg.vector_norm(b - ap)) / bn
    s.synchronize()
    return {"iterations": it, "solve_s": time.perf_counter() - t0, "rel_residual_fp64": true_res,
            "converged": true_res <= 1.5 * tol}


class _Budget(Exception):
    pass


def cpu_cg_baseline(inv, geom, budget_s=60.0):
    """The reference's CG on the host: scipy cg(rtol=1e-6) on the oracle's FP64 restatement of
    the normal equations of this inversion, as lentils/tests/solver_tests.py:77-114 runs it --
    the dirty-beam data term (data_base.py:115-172) with, in turn, the Jacobi preconditioner
    and the reference's own preconditioner (splu of reg + wtsum L^T L, solver_tests.py:103-106).
    FFTs and sparse products are single-threaded as in the reference (scipy defaults). The
    visibility-form operator (NUFFT degrid + grid of the 2e6 visibilities every iteration, the
    gridder on all host cores) is timed per application and scaled by the Jacobi iteration
    count, and says so."""
    import numpy as np
    import scipy.sparse.linalg as sla
    from lentils_gb300 import workloads as WL
    O, _ = cpu_reference_lib()
    vs, ims, srcs, uvw = geom
    img = O.ImageGeom((ims.nx, ims.ny), [(ims.xmin, ims.xmax), (ims.ymin, ims.ymax)])
    src = O.ImageGeom((srcs.nx, srcs.ny), [(srcs.xmin, srcs.xmax), (srcs.ymin, srcs.ymax)])
    pts = inv.lens.source_points.cpu().numpy().astype(np.float64)
    w = inv.weights_user
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    t0 = time.perf_counter()
    A, rhs, M, R = O.normal_operator_bcb(img, src, uvw, pts, w, WL.LAMBDA)
    b = rhs(inv.data_user)
    out = {"operator": "oracle FP64 restatement, dirty-beam data term", "tol": 1e-6,
           "fft_threads": 1, "setup_s": time.perf_counter() - t0,
           "setup_note": f"dirty beam and right-hand side by the C gridder on {cores} threads"}
    n = b.size
    Aop = sla.LinearOperator((n, n), matvec=A, dtype=np.float64)
    dinv = O.jacobi_inverse_diagonal(M, R, w)
    t0 = time.perf_counter()
    wsum = float(np.sum(np.abs(w)))
    lu = sla.splu((R + wsum * (M.T @ M)).tocsc())
    splu_s = time.perf_counter() - t0
    pcs = {"jacobi": sla.LinearOperator((n, n), matvec=lambda r: dinv * r, dtype=np.float64),
           "reference_splu": sla.LinearOperator((n, n), matvec=lu.solve, dtype=np.float64)}
    bn = float(np.linalg.norm(b))
    for name, pc in pcs.items():
        it = [0]
        t0 = time.perf_counter()

        def cb(_xk):
            it[0] += 1
            if time.perf_counter() - t0 > budget_s:
                raise _Budget()
        try:
            x, _ = sla.cg(Aop, b, rtol=1e-6, atol=0.0, maxiter=20000, M=pc, callback=cb)
            done = True
        except _Budget:
            x, done = None, False
        dt = time.perf_counter() - t0
        r = {"iterations": it[0], "solve_s": dt, "s_per_iteration": dt / max(1, it[0]),
             "cores": 1}
        if done:
            r["rel_residual_fp64"] = float(np.linalg.norm(b - A(x)) / bn)
        else:
            r["stopped"] = f"time budget {budget_s} s reached"
        if name == "reference_splu":
            r["factorisation_s"] = splu_s
        out[name] = r
    # the visibility-form operator per application (two CPU gridder passes of 2e6 vis)
    Av, _, _, _ = O.normal_operator(img, src, uvw, pts, w, WL.LAMBDA)
    xs = np.random.default_rng(SEED).normal(size=n)
    Av(xs)
    t0 = time.perf_counter()
    Av(xs)
    mv = time.perf_counter() - t0
    out["visibility_form"] = {"s_per_matvec": mv, "cores": cores,
                              "extrapolated_solve_s": mv * out["jacobi"]["iterations"],
                              "note": "per-application time x the Jacobi iteration count of the "
                                      "dirty-beam solve (the two forms agree to ~1e-6)"}
    return out


SWEEP_SEED = SEED + 3
SWEEP_FORM = 0  # lentils_sweep_create flags: the sweep kernel's item functions


def run_sweep_bench(peak, nsamples=256, steps=10, warmup=3, form=SWEEP_FORM):
    """Batched uneven lens-parameter sweep: 256 PEMD + shear samples from the priors, image
    sizes from {128, 256, 384, 512}^2 (0.02" pixels), visibility counts log-uniform in
    [1e5, 2e6] (uv density ~ 1/|uv| to 0.45 of Nyquist), per-sample KB width from the accuracy
    target 0.01 / sqrt(N_vis), tile and work-item size from the autotuner (JSON cache). One run
    = deflection of every pixel grid + degrid + grid of every sample in one persistent launch,
    replayed as a CUDA graph; timed with events on the sweep's stream. For comparison the same
    work as separate per-sample launches (deflection, degrid, grid: three launches a sample)."""
    import numpy as np
    import torch
    from lentils_gb300.sweep import BatchedSweep, draw_samples
    samples = draw_samples(np.random.default_rng(SWEEP_SEED), nsamples)
    t0 = time.perf_counter()
    sw = BatchedSweep(samples, form=form)
    setup_s = time.perf_counter() - t0
    if sw.tuner.tuned:
        try:
            sw.tuner.save()
        except OSError:
            pass
    st = sw.stats()
    s = sw.stream
    for _ in range(warmup):
        sw.run(use_graph=True)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    s.synchronize()
    ev[0].record(s)
    for _ in range(steps):
        sw.run(use_graph=True)
    ev[1].record(s)
    s.synchronize()
    ms = ev[0].elapsed_time(ev[1]) / steps
    # the same work launched per sample
    from lentils_gb300.lens_models import deflect_points
    from lentils_gb300.sweep import _lens_array
    pts = [torch.as_tensor(sw.pixel_points(k), dtype=torch.float32).cuda()
           for k in range(len(samples))]
    lens = [_lens_array(x.lenses) for x in samples]

    def per_sample():
        with torch.cuda.stream(s):
            for k in range(len(samples)):
                deflect_points(lens[k], pts[k], stream=s)
                sw.plans[k].degrid(sw.grid_in[k], sw.vis_out[k], stream=s)
                sw.plans[k].grid(sw.vis_in[k], sw.grid_out[k], stream=s)
    per_sample()
    s.synchronize()
    ev[0].record(s)
    per_sample()
    ev[1].record(s)
    s.synchronize()
    ms_sep = ev[0].elapsed_time(ev[1])
    widths = [x.info["w2"] for x in samples]
    tiles = [x.info["tile"] for x in samples]
    achieved = st["algorithmic_bytes"] / (ms * 1e-3) / 1e9
    return {"workload": f"{nsamples} PEMD+shear samples, images {{128..512}}^2, nvis log-uniform "
                        "[1e5, 2e6]; deflection + degrid + grid per sample in one persistent "
                        "launch (CUDA graph)",
            "seed": SWEEP_SEED, "total_vis": st["total_vis"], "total_pixels": st["total_pixels"],
            "ms_per_sweep": ms, "samples_per_s": nsamples / (ms * 1e-3),
            "mvis_per_s": st["total_vis"] / (ms * 1e-3) / 1e6,
            "note": "mvis_per_s = visibilities / (time of the whole sweep: degrid + grid of every "
                    "visibility and the deflections), the headline's convention",
            "per_sample_launches_ms": ms_sep, "speedup_vs_per_sample_launches": ms_sep / ms,
            "work_items": st["nwork"], "persistent_ctas": st["blocks"],
            "smem_bytes": st["smem_bytes"], "kb_width_counts": {"6": widths.count(6),
                                                                "8": widths.count(8)},
            "tile_counts": {str(t): tiles.count(t) for t in sorted(set(tiles))},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak,
                         "algorithmic_bytes_per_run": st["algorithmic_bytes"]},
            "kernel_form": form, "setup_s": setup_s, "autotuned_classes": sw.tuner.tuned}


def run_unet_bench(steps=20, warmup=3):
    """The learned preconditioner's network (128^2 source grid, 276,545 parameters, BF16 on the
    tcgen05 tensor cores): forward at batch 1 (as the solver applies it) and 32, one training
    step (forward, backward, Adam) at batch 32, and the preconditioner application (called from
    Python, and replayed from a CUDA graph as the solver applies it), with CUDA events on the
    current stream. Random weights and inputs (seeded); the forward FLOPs are
    2 * pixels * K * N summed over the convolutions."""
    import torch
    from lentils_gb300 import learned
    H = W = 128
    net = learned.UNet(H, W, max_batch=32, seed=3)
    g = torch.Generator(device="cuda").manual_seed(5)
    x, f, t = (torch.randn(32, H, W, device="cuda", generator=g) for _ in range(3))
    r = x[0].reshape(-1)
    d = torch.rand(H * W, device="cuda", generator=g) + 0.5
    ft = f[0].reshape(-1)
    s = torch.cuda.current_stream()

    def timed(fn, n):
        for _ in range(warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        for _ in range(n):
            fn()
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / n

    def graphed(fn, n):
        # the call captured once into a CUDA graph and replayed, as the solver applies it
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(warmup):
                fn()
        torch.cuda.current_stream().wait_stream(side)
        gr = torch.cuda.CUDAGraph()
        with torch.cuda.graph(gr):
            fn()
        return timed(gr.replay, n)

    fwd_flop = 0
    for ci, co, k, _, level in learned.LAYERS:
        npix = 32 * (H >> level) * (W >> level)
        fwd_flop += 2 * npix * k * k * ci * co
    out = {"workload": "U-Net 2->32->64->128->128 (3x3, 1x1 convolutions), 128^2 source grid, "
                       "BF16 tcgen05 GEMMs with FP32 accumulation; random weights and inputs",
           "forward_b1_ms": timed(lambda: net.forward(x[:1], f[:1]), steps),
           "forward_b32_ms": timed(lambda: net.forward(x, f), steps),
           "train_step_b32_ms": timed(lambda: net.train_step(x, f, t, 0.0), max(3, steps // 2)),
           "forward_b32_graph_ms": graphed(lambda: net.forward(x, f), steps),
           "train_step_b32_graph_ms": graphed(lambda: net.train_step(x, f, t, 0.0), max(3, steps // 2)),
           "precondition_ms": timed(lambda: net.precondition(r, d, ft), steps),
           "precondition_graph_ms": graphed(lambda: net.precondition(r, d, ft), steps),
           "forward_b32_gflop": fwd_flop / 1e9}
    out["forward_b32_tflops"] = fwd_flop / (out["forward_b32_ms"] * 1e-3) / 1e12
    out["train_step_b32_tflops"] = 3 * fwd_flop / (out["train_step_b32_ms"] * 1e-3) / 1e12
    if net.error_flag():
        raise RuntimeError("a tensor-core wait gave up in the U-Net section")
    return out


def _omp_threads(n):
    """Set the OpenMP thread count of this (calling) thread for the CPU gridder's parallel
    loops (libgomp, which the compiled gridder links)."""
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(n))
        return True
    except (OSError, AttributeError):
        return False


def cpu_baseline(four, uvw):
    """The reference's CPU gridder on all host cores over a bounded sample (~10 s), and on one
    thread over a smaller one (~5 s)."""
    O, use_ref = cpu_reference_lib()
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    cal = 20000
    rate = cal / time_cpu_gridder(O, use_ref, four, uvw, cal)[0]
    nsample = int(max(20000, min(2_000_000, rate * 10.0)))
    t = time_cpu_gridder(O, use_ref, four, uvw, nsample)[0]
    out = {"value": nsample / t / 1e6, "unit": UNIT, "cores": cores,
           "kind": "reference" if use_ref else "port",
           "sample": f"{nsample} random visibilities of the 1e7 set, full grid, degrid+grid"}
    if _omp_threads(1):
        try:
            cal1 = 4000
            rate1 = cal1 / time_cpu_gridder(O, use_ref, four, uvw, cal1)[0]
            n1 = int(max(4000, min(500_000, rate1 * 5.0)))
            t1 = time_cpu_gridder(O, use_ref, four, uvw, n1)[0]
            out["one_thread"] = {"value": n1 / t1 / 1e6, "unit": UNIT, "cores": 1,
                                 "sample": f"{n1} random visibilities, degrid+grid"}
        finally:
            _omp_threads(cores)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-cg", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--sweep-samples", type=int, default=256)
    ap.add_argument("--no-deflect", action="store_true")
    ap.add_argument("--no-dropin", action="store_true")
    ap.add_argument("--no-cpu-cg", action="store_true")
    ap.add_argument("--no-unet", action="store_true")
    ap.add_argument("--unet-only", action="store_true",
                    help="print only the U-Net section's JSON (for profiling its kernels)")
    args = ap.parse_args()
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    if args.impl == "reference":
        return run_reference(args)
    if args.unet_only:
        print(json.dumps({"unet": run_unet_bench(steps=args.steps, warmup=max(3, args.warmup))}))
        return 0
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
