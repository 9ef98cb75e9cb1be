#!/usr/bin/env python
"""Benchmark of the GB300 wave path: the batched FWI gradient.

One step = one misfit gradient (forward with checkpoints + checkpointed
adjoint) of the fwi1024 workload: 1024 x 1024 grid, 2000 time steps, 64 shots
along the surface in one batched call, 1024 receivers, order 8 + 20-cell
sponge, checkpoints every 45 steps (BF16), seeded synthetic layered + anomaly
models (no dataset exists for this path).

Metric: counted cell-updates per second, forward + adjoint: 2 x shots x
interior cells x steps per gradient (recomputed forward steps are not
counted). Algorithmic bytes: 16 B per forward update, 20 B per adjoint update
(16 B + the stored L u read for the imaging term), i.e. 36 B per (cell, step)
pair; "% HBM" = those bytes / time / measured HBM copy bandwidth.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload fwi1024|fwd2048|fwi384_3d|batch8|vd1024|temporal|fmc_tfm]

The other workloads (not the headline) print the same JSON line for:
  fwd2048    2D forward, 2048^2, 4000 steps, one shot (16 B per update);
  fwi384_3d  3D FWI gradient, 384^3, 1500 steps, 16 shots in two sequential
             groups of 8, BF16 checkpoints every 39 (18 B per counted update);
  batch8     8 models 512^2..1536^2, 1000..3000 steps, 128 shots, one
             graph-captured batch gradient (18 B per counted update);
  vd1024     the fwi1024 models with densities, (kappa, rho) gradient;
  temporal   the padded_step drop-in problem of the reference's temporal
             driver (8000 x 16000, order 2, Dirichlet): one step = one
             wfd_temporal_step launch (8 updates), 2 B per update (each
             launch reads and writes both levels once); the eight-launch
             wfd_step2d_order2 and wfd_step2d_exact rates are reported beside it;
  fmc_tfm    the ultrasonic plate pipeline: full matrix capture (32 elements
             on a 512^2 plate, order 8, 2.5 traversals), analytic signal and
             total focusing onto 512^2 pixels; value = capture cell-updates/s,
             the per-stage times beside it.

Multi-GPU (torchrun, one process per GPU): the survey holds 64 shots per rank
(weak scaling); neuralmech_gb300.shard.distributed_misfit_gradient gives each
rank its contiguous block of 64 and sums the gradients and misfits with one
all-reduce per step.

--impl reference times the reference's CPU path for this workload on the host
cores: the FP64 C++/OpenMP restatement in oracle/ (the reference's own solver
package is not installable here and its in-tree kernels are GPU-only), on a
bounded sample of each step.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_PATH = os.path.join(ROOT, "profiles", "dram_traffic.txt")
FALLBACK_HBM_GBS = 6800.0
METRIC = "Gcell-updates/s fwd+adj (% HBM peak); FWI grad shots/s batched vs plain, 1 GPU"
UNIT = "Gcell-updates/s"
# algorithmic bytes per cell-update, per kernel phase: u_n, u_{n-1} and m read,
# u_{n+1} written; the recompute adds the L u write unless the levels u_k
# themselves are kept (the 2D one-step default), the adjoint the L u or u_k read
ALG_BYTES = {"forward": 16.0, "recompute": 20.0, "adjoint": 20.0}


def alg_bytes(grid, phase: str) -> float:
    ustore = grid.ndim == 2 and grid.lap_store == "auto"
    return 16.0 if (phase == "recompute" and ustore) else ALG_BYTES[phase]


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scale", type=float, default=1.0, help="shrink grid and steps (testing only)")
    ap.add_argument("--plain-shots", type=int, default=4)
    ap.add_argument("--cpu-sample-steps", type=int, default=200)
    ap.add_argument("--no-extras", action="store_true", help="skip e2e, plain and CPU legs")
    ap.add_argument("--timeline", action="store_true",
                    help="batch8: device occupancy of one replay from the CUDA activity trace")
    ap.add_argument("--once", action="store_true",
                    help="run one gradient and exit (the command profiled by ncu)")
    ap.add_argument("--nt", type=int, default=0, help="override the number of time steps (profiling)")
    ap.add_argument("--shots", type=int, default=0, help="use the first N shots (profiling)")
    ap.add_argument("--ckpt-every", type=int, default=0, help="override the checkpoint interval (profiling)")
    ap.add_argument("--field-format", default="fp32", choices=["fp32", "fp16", "i16"],
                    help="fwd2048: storage of the wavefields (arithmetic stays FP32)")
    ap.add_argument("--adjoint", default="checkpoint", choices=["checkpoint", "reconstruct"],
                    help="how the gradient obtains the forward levels")
    ap.add_argument("--tile-rows", type=int, default=0, choices=[0, 16, 32],
                    help="fwd2048: 2D tile height of the one-step kernel (0: the library default)")
    ap.add_argument("--step-block", type=int, default=0, choices=[0, 1, 2],
                    help="time steps per launch of the forward and the recompute (0: two for the "
                         "fwi1024 gradient, whose summed two-step forward is the faster one; one elsewhere)")
    ap.add_argument("--group-shots", type=int, default=8,
                    help="fwi384_3d: shots per sequential group (0: all 16 at once)")
    ap.add_argument("--level-store-frac", type=float, default=0.8,
                    help="fraction of the GPU's memory for the forward levels the adjoint keeps "
                         "instead of recomputing them (0: recompute all but the last segment)")
    ap.add_argument("--level-format", default="fp32", choices=["fp32", "bfp16"],
                    help="kept forward levels of the fwi1024 gradient: FP32, or block floating point "
                         "(2.25 B per cell: more levels kept in the same budget, each encoded by the "
                         "forward and decoded by the adjoint; the same time on this workload)")
    ap.add_argument("--update", default="auto", choices=["auto", "leapfrog", "summed"],
                    help="forward update form (auto: summed for a gradient's forward, leapfrog otherwise)")
    ap.add_argument("--workload", default="fwi1024",
                    choices=["fwi1024", "fwd2048", "fwi384_3d", "batch8", "vd1024", "temporal", "fmc_tfm"])
    return ap.parse_args()


def peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def traffic_per_update():
    """ncu DRAM bytes per cell-update per phase kernel (profiles/dram_traffic.txt)."""
    out = {}
    try:
        with open(TRAFFIC_PATH) as f:
            for line in f:
                line = line.split("#", 1)[0].strip()
                if "=" in line:
                    k, v = (x.strip() for x in line.split("=", 1))
                    out[k] = float(v)
    except OSError:
        pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(scale: float, nt: int = 0, shots: int = 0):
    from neuralmech_gb300 import Grid
    from neuralmech_gb300.synth import workload as wl
    w = wl("fwi1024", scale=scale)
    if nt:
        g = w.grid
        w.grid = Grid(g.shape, g.spacing, g.dt, nt, order=g.order, sponge=g.sponge,
                      ckpt_every=min(g.ckpt_every, nt), ckpt_format=g.ckpt_format)
        w.wavelet = w.wavelet[:nt].copy()
    if shots:
        w.src, w.rec = w.src[:shots].copy(), w.rec[:shots].copy()
    return w


def weak_survey(wavelet, src, rec, observed_block, world: int, rank: int):
    """The survey of a weak-scaling run on `world` ranks: the single-GPU
    survey's shots once per rank (the same geometry, block r belongs to rank
    r, as shard_range splits them). Returns full-survey (wavelet, src, rec,
    observed) tensors; of `observed` only this rank's block is filled, the
    only block this rank reads."""
    import torch
    from neuralmech_gb300.shard import shard_range
    n = observed_block.shape[0]
    total = n * world
    if wavelet.dim() == 1:
        wavelet = wavelet.reshape(1, -1)
    wav_all = wavelet.expand(total, *wavelet.shape[1:]).contiguous() if wavelet.shape[0] == 1 else \
        wavelet.repeat(world, *([1] * (wavelet.dim() - 1)))
    src_all = src.repeat(world, *([1] * (src.dim() - 1)))
    rec_all = rec.repeat(world, *([1] * (rec.dim() - 1))) if rec.dim() == 3 else rec
    obs_all = torch.zeros((total,) + tuple(observed_block.shape[1:]), dtype=observed_block.dtype,
                          device=observed_block.device)
    sl = shard_range(total, rank, world)
    assert sl.stop - sl.start == n
    obs_all[sl] = observed_block
    return wav_all, src_all, rec_all, obs_all


def kept_segments(g) -> int:
    """Segments whose forward levels the adjoint keeps (the last one at least)."""
    K = g.ckpt_every or int(np.ceil(np.sqrt(g.nt)))
    nseg = -(-g.nt // K)
    return min(nseg, max(1, (g.store_levels - 2) // K))


def counted_updates(w) -> float:
    R = w.grid.order // 2
    interior = int(np.prod([n - 2 * R for n in w.grid.shape]))
    return 2.0 * w.nshot * interior * w.grid.nt, interior


def cpu_gradient_sample(w, steps: int, nshot: int = 1):
    """FP64 oracle gradient of the first `nshot` shots over `steps` time steps
    of the workload's grid: (counted updates, seconds, description)."""
    import oracle
    from neuralmech_gb300 import Grid, sponge_profiles
    oracle.build()
    g = w.grid
    sub = Grid(g.shape, g.spacing, g.dt, steps, order=g.order, sponge=g.sponge,
               ckpt_every=min(g.ckpt_every or 45, steps))
    gz, _, gx = sponge_profiles(sub)
    p3 = lambda p: np.stack([p[..., 0], 0 * p[..., 0], p[..., 1]], -1).astype(np.int32)
    wav = np.broadcast_to(w.wavelet[:steps], (nshot, steps)).astype(np.float64)[:, :, None].copy()
    geo = oracle.Geometry(vel=w.vel.astype(np.float64), wavelet=wav, src=p3(w.src[:nshot]),
                          rec=p3(w.rec[:nshot]), dt=float(np.float32(g.dt)),
                          h=(g.spacing[0], 1.0, g.spacing[1]), order=g.order,
                          sponge=(gz.astype(np.float64), None, gx.astype(np.float64)),
                          ckpt_every=sub.ckpt_every)
    obs = np.zeros((nshot, steps, w.rec.shape[1]))
    t0 = time.perf_counter()
    oracle.gradient(geo, obs)
    dt = time.perf_counter() - t0
    R = g.order // 2
    interior = int(np.prod([n - 2 * R for n in g.shape]))
    desc = (f"FP64 C++/OpenMP oracle gradient (forward + checkpointed adjoint), {nshot} shot, "
            f"{g.shape[0]}x{g.shape[1]} grid, {steps} of {g.nt} steps")
    return 2.0 * nshot * interior * steps, dt, desc


def numpy_fd_step_legs(steps: int = 1000):
    """The reference's NumPy CPU path, fd_step (projects/18_simple_wave_fd/
    2D_wave_cupy.py:54-62), timed on the fwd256 workload (256^2, dx 10 m,
    layered + anomaly model, 1000 steps) on one core (NumPy elementwise work is
    single-threaded): as written (order 2, constant wave speed = the model's
    maximum, Dirichlet ring) and in its slice form at order 8 with the velocity
    field and the 20-cell sponge. Forward cell-updates per second."""
    from oracle import numpy_ref
    from neuralmech_gb300 import sponge_profiles
    from neuralmech_gb300.synth import workload as wl
    w = wl("fwd256")
    g = w.grid
    n = g.shape[0]
    steps = min(steps, g.nt)
    src = tuple(int(c) for c in w.src[0, 0])
    out = {}
    vmax = float(w.vel.max())
    gz, _, gx = sponge_profiles(g)
    gfield = (gz[:, None] * gx[None, :]).astype(np.float32)
    wfield = (w.vel.astype(np.float32) * np.float32(g.dt)) ** 2
    for name, R in (("order2_as_written", 1), ("order8_sponge_slices", 4)):
        u0 = np.zeros((n, n), np.float32)
        u1 = np.zeros((n, n), np.float32)
        t0 = time.perf_counter()
        for k in range(steps):
            if R == 1:
                numpy_ref.fd_step_order2(u0, u1, u0, np.float32(g.dt), np.float32(g.spacing[1]),
                                         np.float32(g.spacing[0]), np.float32(vmax))
            else:
                numpy_ref.fd_step(u0, u1, u0, wfield, g.spacing, order=8, g=gfield)
            u0[src] += w.wavelet[k]
            u0, u1 = u1, u0
        dt = time.perf_counter() - t0
        inner = (n - 2 * R) ** 2
        out[name] = {"value": inner * steps / dt / 1e9, "unit": "Gcell-updates/s (forward)", "cores": 1,
                     "kind": "port",
                     "sample": f"fwd256: {n}^2, {steps} steps, one shot, NumPy FP32 on one core"
                               + (" (fd_step as written, cp -> np: order 2, wave speed = model max)" if R == 1
                                  else " (the same slice form at order 8, velocity field, 20-cell sponge)")}
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    w = workload(args.scale, args.nt, args.shots)
    cores = os.cpu_count()
    steps = max(10, int(args.cpu_sample_steps * args.scale)) if args.scale < 1 else args.cpu_sample_steps
    for _ in range(args.warmup):
        cpu_gradient_sample(w, steps)
    tot_u, tot_t, desc = 0.0, 0.0, ""
    for _ in range(args.steps):
        u, t, desc = cpu_gradient_sample(w, steps)
        tot_u += u
        tot_t += t
    value = tot_u / tot_t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": tot_t / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(w, args),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": desc + " per step", "numpy_fd_step": numpy_fd_step_legs()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def config_of(w, args):
    g = w.grid
    return {"workload": (f"fwi1024: 2D FWI gradient, {g.shape[0]}x{g.shape[1]}, {g.nt} steps, "
                         f"{w.nshot} shots in one batched call, {w.rec.shape[1]} receivers, order {g.order}, "
                         f"20-cell sponge, checkpoints every {g.ckpt_every} ({g.ckpt_format})"),
            "grid": list(g.shape), "nt": g.nt, "nshot": w.nshot, "nrec": int(w.rec.shape[1]),
            "ckpt_every": g.ckpt_every, "ckpt_format": g.ckpt_format, "order": g.order,
            "store_levels": g.store_levels, "level_format": g.level_format, "step_block": g.step_block,
            "adjoint": g.adjoint,
            "update": g.update, "kept_segments": kept_segments(g),
            "l2": "inputs larger than L2 (multi-GB state and checkpoints per step)",
            "parallelism": f"{args.gpus} GPU(s), shots batched per GPU, gradient all-reduce"}


def order2_pairs(dev, grids=((256, 256), (2048, 2048), (8000, 16000)), reps=None):
    """The reference's own order-2 step kernels (projects/18_simple_wave_fd/
    step2D_wave.cu, built for sm_103a with --use_fast_math as its drivers build
    them; oracle/ref_gpu.cpp) beside this library's drop-ins on the same grids
    and inputs: G updates/s of each and ours / reference.
      padded_step x 8   vs wfd_step2d_order2 x 8 (and wfd_step2d_exact x 8)
      temporal_step     vs wfd_temporal_step_fast (and wfd_temporal_step)
      mixed_step x 8    vs wfd_step2d_mixed_fast x 8 (and wfd_step2d_mixed x 8; FP16 storage)
    Grids: fwd256's and fwd2048's sizes and the temporal driver's 8000 x 16000
    (2D_wave_cuda_temporal.py:26), the drivers' Gaussian pulse, unit wave
    speed, dt at 0.95 of the order-2 bound; launches as the drivers launch
    them (ours on the same stream, one call per launch)."""
    import torch

    from neuralmech_gb300 import step2d_order2
    from neuralmech_gb300.wavefd import (step2d_exact, step2d_mixed, step2d_mixed_fast, temporal_step,
                                         temporal_step_fast)
    from oracle import ref
    if not ref.gpu_available():
        return {"unavailable": "the reference's GPU module files were not built (they need its sources)"}
    out = {}
    for N, M in grids:
        Mp = (M + 32) // 32 * 32  # (the FP16 drop-in needs M_padded > M)
        dx, dy = 1.0 / (N - 1), 2.0 / (M - 1)
        dt = 0.95 * min(dx, dy) / math.sqrt(2)
        x = torch.linspace(0, 1, N, device=dev)[:, None]
        y = torch.linspace(0, 2, M, device=dev)[None, :]
        u = torch.zeros((N, Mp), device=dev)
        u[:, :M] = torch.exp(-(x - 0.5) ** 2 / (2 * 0.02 ** 2)) * torch.exp(-(y - 0.5) ** 2 / (2 * 0.02 ** 2))
        args = (1.0, dt, dx, dy, N, M)
        inner = (N - 2) * (M - 2)
        n = reps or max(5, min(200, int(4e8 // (N * M))))
        bufs = [u.clone(), u.clone(), torch.zeros_like(u), torch.zeros_like(u)]
        hb = [u.half(), u.half()]

        def eight(fn, a, b):
            def go():
                p, q = a, b
                for _ in range(8):
                    p = fn(p, q, p, *args)
                    p, q = q, p
            return go

        def pair_launch(fn):
            k = {"k": 0}

            def go():
                i0, i1, o0, o1 = (0, 1, 2, 3) if k["k"] % 2 == 0 else (2, 3, 0, 1)
                fn(bufs[i0], bufs[i1], bufs[o0], bufs[o1], *args)
                k["k"] += 1
            return go

        def rate(go):
            for _ in range(2):
                go()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(n):
                go()
            e1.record()
            torch.cuda.synchronize()
            return 8 * inner * n / (e0.elapsed_time(e1) / 1e3) / 1e9

        ref.MODE["build"] = "fast"
        r = {
            "padded_step x8 (reference, fast math)": rate(eight(ref.padded_step_gpu, bufs[0], bufs[1])),
            "wfd_step2d_order2 x8": rate(eight(step2d_order2, bufs[0], bufs[1])),
            "wfd_step2d_exact x8": rate(eight(step2d_exact, bufs[0], bufs[1])),
            "temporal_step (reference, fast math)": rate(pair_launch(ref.temporal_step_gpu)),
            "wfd_temporal_step_fast": rate(pair_launch(temporal_step_fast)),
            "wfd_temporal_step": rate(pair_launch(temporal_step)),
            "mixed_step x8 (reference, fast math)": rate(eight(ref.mixed_step_gpu, hb[0], hb[1])),
            "wfd_step2d_mixed_fast x8": rate(eight(step2d_mixed_fast, hb[0], hb[1])),
            "wfd_step2d_mixed x8": rate(eight(step2d_mixed, hb[0], hb[1])),
        }
        r["ratio padded"] = r["wfd_step2d_order2 x8"] / r["padded_step x8 (reference, fast math)"]
        r["ratio temporal"] = r["wfd_temporal_step_fast"] / r["temporal_step (reference, fast math)"]
        r["ratio mixed"] = r["wfd_step2d_mixed_fast x8"] / r["mixed_step x8 (reference, fast math)"]
        out[f"{N}x{M}"] = {k: round(v, 2) for k, v in r.items()}
        del bufs, hb, u
        torch.cuda.empty_cache()
    out["unit"] = "G cell-updates/s (8 order-2 updates per timed call)"
    return out


def l2_copy_gbs(dev, mb: int = 32) -> float:
    """Copy bandwidth of a buffer that stays in L2 (32 MB read + 32 MB written
    per copy, 129 MB L2), measured live: the roofline of an L2-resident
    stencil such as fwd2048's."""
    import torch
    n = mb * 2**20 // 4
    a = torch.randn(n, device=dev)
    b = torch.empty_like(a)
    for _ in range(20):
        b.copy_(a)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(1000):
        b.copy_(a)
    e1.record()
    torch.cuda.synchronize()
    return 2.0 * n * 4 * 1000 / (e0.elapsed_time(e1) / 1e3) / 1e9


def multistep_pairs(dev, cases=((2048, 2048, 4000), (8000, 16000, 64)), reps=3):
    """The wave path's forward at orders 2 and 4, one step per launch against
    K steps per launch in a register window (step_block 8 at order 2, 4 at
    order 4): one shot, a 20-cell sponge, the velocity of fwd2048's model
    class (1500..3500 m/s layers), a source near the top and a receiver on
    every column of row 5. G cell-updates/s of each and the ratio."""
    import dataclasses

    import torch

    from neuralmech_gb300 import Grid, wave_forward
    from neuralmech_gb300.synth import layered, ricker
    out = {}
    for nz, nx, nt in cases:
        v = layered((nz, nx), [0, nz // 3, 2 * nz // 3], [1500.0, 2500.0, 3500.0]).astype(np.float32)
        dx = 10.0
        vel = torch.from_numpy(v).to(dev)
        src = torch.tensor([[[5, nx // 2]]], dtype=torch.int32)
        rec = torch.from_numpy(np.stack([np.full(nx - 8, 5), np.arange(4, nx - 4)], -1)[None].astype(np.int32))
        for order, K in ((2, 8), (4, 4)):
            dt = 0.4 * dx / 3500.0
            wav = torch.from_numpy(ricker(15.0, nt, dt).astype(np.float32)).reshape(1, nt, 1).to(dev)
            g = Grid((nz, nx), (dx, dx), dt, nt, order=order, sponge=20)
            R = order // 2
            upd = (nz - 2 * R) * (nx - 2 * R) * nt
            r = {}
            for sb in (1, K):
                gg = dataclasses.replace(g, step_block=sb)
                wave_forward(vel, wav, src, rec, gg, check=False)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(reps):
                    wave_forward(vel, wav, src, rec, gg, check=False)
                e1.record()
                torch.cuda.synchronize()
                r[f"{sb} step{'s' if sb > 1 else ''} per launch"] = round(upd * reps / (e0.elapsed_time(e1) / 1e3) / 1e9, 1)
            vals = list(r.values())
            r["ratio"] = round(vals[1] / vals[0], 2)
            out[f"order {order}, {nz}x{nx}, {nt} steps"] = r
    out["unit"] = "G cell-updates/s (one shot, receivers on a row)"
    return out


def secondary_legs(dev):
    """Short legs of the other configurations, in the default run: the fwd2048
    forward (2048^2, 4000 steps, one shot, order 8, sponge), the order-2
    drop-ins beside the reference's own kernels on the temporal driver's
    8000 x 16000 grid, and the wave path's multi-step forward at orders 2
    and 4 beside one step per launch."""
    import torch

    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300.synth import workload as wl
    out = {}
    w = wl("fwd2048")
    args = (torch.from_numpy(w.vel).to(dev), torch.from_numpy(w.wavelet).to(dev), torch.from_numpy(w.src),
            torch.from_numpy(w.rec))
    for _ in range(3):
        wave_forward(*args, w.grid, check=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        wave_forward(*args, w.grid, check=False)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 5
    R = w.grid.order // 2
    rate = (2048 - 2 * R) ** 2 * w.grid.nt / (ms / 1e3) / 1e9
    l2 = l2_copy_gbs(dev)
    out["fwd2048_forward"] = {"value": rate, "unit": "Gcell-updates/s", "ms_per_run": ms,
                              "config": "2048^2, 4000 steps, 1 shot, 2048 receivers, order 8, 20-cell sponge",
                              "fields": "u_n, u_{n-1}, m: 3 x 16.8 MB, resident in L2 across steps",
                              "alg_gbs": rate * 16.0, "l2_copy_gbs": l2, "alg_frac_of_l2_copy": rate * 16.0 / l2}
    out["order2_pairs"] = order2_pairs(dev, grids=((8000, 16000),))
    out["multistep"] = multistep_pairs(dev)
    return out


def _wl_temporal(args, dev):
    """The order-2 drop-ins on the reference temporal driver's grid, with the
    reference's own kernels beside them."""
    import torch

    from neuralmech_gb300.wavefd import temporal_step_fast
    N, M = 8000, 16000  # 2D_wave_cuda_temporal.py:26
    Mp = (M + 31) // 32 * 32
    dx, dy = 1.0 / (N - 1), 2.0 / (M - 1)
    dt = 0.95 * min(dx, dy) / math.sqrt(2)
    x = torch.linspace(0, 1, N, device=dev)[:, None]
    y = torch.linspace(0, 2, M, device=dev)[None, :]
    u0 = torch.zeros((N, Mp), device=dev)
    u0[:, :M] = torch.exp(-(x - 0.5) ** 2 / (2 * 0.02 ** 2)) * torch.exp(-(y - 0.5) ** 2 / (2 * 0.02 ** 2))
    bufs = [u0, u0.clone(), torch.empty_like(u0), torch.empty_like(u0)]
    state = {"k": 0}

    def step():  # two pairs of arrays, swapped every launch, as 2D_wave_cuda_temporal.py does
        a, b = (0, 1) if state["k"] % 2 == 0 else (2, 3)
        c, d = (2, 3) if state["k"] % 2 == 0 else (0, 1)
        temporal_step_fast(bufs[a], bufs[b], bufs[c], bufs[d], 1.0, dt, dx, dy, N, M)
        state["k"] += 1

    inner = (N - 2) * (M - 2)
    extra = {"pairs": order2_pairs(dev), "multistep": multistep_pairs(dev)}
    updates, bpu = 8.0 * inner, 16.0 / 8
    cfg = {"workload": f"temporal: wfd_temporal_step_fast, {N} x {M} (M_padded {Mp}), order 2, Dirichlet, "
                       "8 updates per launch; bytes: both levels read and written once per launch",
           "l2": "inputs larger than L2 (4 x 512 MB)"}
    return dict(step=step, updates=updates, bpu=bpu, cfg=cfg, extra=extra, graph_kernels=0)


def _wl_fmc_tfm(args, dev):
    """Full matrix capture, analytic signal and TFM on the plate driver's sizes."""
    import torch

    extra, graph_kernels = {}, 0
    from neuralmech_gb300 import Grid
    from neuralmech_gb300.cuwave_compat import sineburst, stable_dt
    from neuralmech_gb300.imaging import analytic_signal, full_matrix_capture, tfm
    n, E, c = 512, 32, 1.0  # projects/18_fwi/plate.py:19-32
    h = 1.0 / (n - 3)
    dt0 = 0.9 * stable_dt((h, h), c, 8)
    nt = math.ceil(2.5 / dt0) + 1
    dt = 2.5 / (nt - 1)
    grid = Grid((n, n), (h, h), dt, nt, order=8, sponge=0)
    cols = np.round(np.linspace(0.1, 0.9, E) * (n - 1)).astype(np.int32)
    el_cells = np.stack([np.full(E, 4, np.int32), cols], axis=1)       # (z, x): the top edge
    el_xy = np.stack([cols * h, np.full(E, 4 * h)], axis=1)            # (x, y) in plate units
    vel = torch.full((n, n), c, device=dev)
    rng = np.random.default_rng(0)
    for _ in range(4):  # circular slow voids (synthetic stand-ins for the plate's voids)
        zc, xc, r = rng.uniform(0.3, 0.8) * n, rng.uniform(0.3, 0.7) * n, rng.uniform(0.02, 0.05) * n
        zz, xx = torch.meshgrid(torch.arange(n, device=dev), torch.arange(n, device=dev), indexing="ij")
        vel[(zz - zc) ** 2 + (xx - xc) ** 2 < r * r] = 0.5 * c
    wav = torch.from_numpy(sineburst(np.arange(nt) * dt, 1.0, 20.0, 2)).to(dev)
    px = torch.linspace(0, 1, 512, device=dev)
    X, Y = torch.meshgrid(px, px, indexing="ij")
    t0 = 2 / (2 * 20.0)
    stage_ms = {"capture": [], "analytic": [], "tfm": []}
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def step():
        evs[0].record()
        traces = full_matrix_capture(vel, wav, el_cells, grid)          # (E, nt, E)
        evs[1].record()
        hs = analytic_signal(traces.permute(0, 2, 1).contiguous())       # (E, E, nt)
        evs[2].record()
        tfm(hs, el_xy, t0, dt, c, X, Y)
        evs[3].record()
        torch.cuda.synchronize()
        for k, name in enumerate(("capture", "analytic", "tfm")):
            stage_ms[name].append(evs[k].elapsed_time(evs[k + 1]))
    R = 4
    updates, bpu = float(E) * (n - 2 * R) ** 2 * nt, 16.0
    extra["stage_ms"] = stage_ms  # averaged over the timed calls below
    cfg = {"workload": f"fmc_tfm: full matrix capture, {E} elements on a {n}^2 plate, {nt} steps, order 8, "
                       "4 slow voids; analytic signal; TFM onto 512^2 pixels with reciprocity",
           "pixels": 512 * 512, "traces": E * E, "samples": nt}
    return dict(step=step, updates=updates, bpu=bpu, cfg=cfg, extra=extra, graph_kernels=graph_kernels)


def _wl_batch8(args, dev):
    """Eight uneven models in one graph-captured batch gradient."""
    import dataclasses

    import torch

    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300.batch import BatchFWI
    from neuralmech_gb300.synth import workload as wl

    extra = {}
    models = []
    for w in wl("batch8"):
        v = torch.from_numpy(w.vel).to(dev)
        wav = torch.from_numpy(w.wavelet).to(dev)
        src, rec = torch.from_numpy(w.src), torch.from_numpy(w.rec)
        obs = wave_forward(torch.from_numpy(w.vel_true).to(dev), wav, src, rec, w.grid)
        models.append(dict(vel=v, wavelet=wav, src=src, rec=rec, observed=obs, grid=w.grid))
    budget = args.level_store_frac * torch.cuda.get_device_properties(dev).total_memory
    batch = BatchFWI(models, autotune=True, level_budget=budget)
    # wfd_batch_run adds the kernels of each replay to wfd_kernel_launches itself
    graph_kernels = 0
    extra["graph_kernels_per_replay"] = batch.graph_kernels
    step = batch.run
    if args.timeline:
        # the same batch with a tenth of the steps (the same grids, kernels and
        # graph structure): its activity trace fits the profiler's buffers
        short = []
        for m in models:
            nt = max(10, m["grid"].nt // 10)
            g = dataclasses.replace(m["grid"], nt=nt, ckpt_every=0, store_levels=0)
            wav = m["wavelet"][..., :nt] if torch.as_tensor(m["wavelet"]).dim() == 1 else m["wavelet"][:, :nt]
            short.append(dict(m, grid=g, wavelet=wav, observed=m["observed"][:, :nt].contiguous()))
        sb = BatchFWI(short, autotune=True)
        extra["timeline"] = kernel_timeline(sb.run)
        extra["timeline"]["batch"] = "batch8 models with a tenth of their steps, one graph replay"
        se = BatchFWI(short, autotune=True, graph=False)
        extra["timeline_eager"] = kernel_timeline(se.run)
        extra["timeline_eager"]["batch"] = "the same batch launched eagerly on its streams"
        del sb, se
    updates, bpu = batch.cell_updates, 18.0
    cfg = {"workload": "batch8: 8 models 512^2..1536^2, 1000..3000 steps, 128 shots, Ricker 10..25 Hz, "
                       "one graph-captured batch gradient (streams per model), autotuned kernels, "
                       f"kept forward levels in {args.level_store_frac:.0%} of the GPU's memory",
           "models": [[list(m.call.grid.shape), m.call.grid.nt, m.call.problem.nshot] for m in batch.models],
           "configs": batch.configs,
           "store_levels": [m.call.grid.store_levels for m in batch.models]}
    return dict(step=step, updates=updates, bpu=bpu, cfg=cfg, extra=extra, graph_kernels=graph_kernels)


def kernel_timeline(step):
    """Device-side occupancy of one call of `step` from the CUDA activity
    trace (torch.profiler / CUPTI): the kernels' [start, end) intervals, their
    union (time with at least one kernel running), and the gaps between
    consecutive kernel activity (launch gaps, graph-edge latency). Returns the
    busy fraction of the span and the gap statistics."""
    import torch
    from torch.profiler import ProfilerActivity, profile
    step()
    torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CPU, ProfilerActivity.CUDA]) as prof:
        step()
        torch.cuda.synchronize()
    iv, kinds = [], {}
    for e in prof.profiler.kineto_results.events():  # raw activity records (graph kernels included)
        kind = str(e.device_type())
        kinds[kind] = kinds.get(kind, 0) + 1
        if "CUDA" not in kind:
            continue
        name = e.name().lower()
        if "memcpy" in name or "memset" in name:
            continue
        t0, dur = e.start_ns(), e.duration_ns()
        if dur > 0:
            iv.append((t0 / 1e3, (t0 + dur) / 1e3))
    if not iv:  # the aggregated events, where the raw records hold no device activity
        for e in prof.events():
            if "CUDA" in str(e.device_type) and e.time_range.elapsed_us() > 0:
                iv.append((float(e.time_range.start), float(e.time_range.end)))
    if not iv:
        return {"unavailable": "no CUDA kernel activity recorded", "records": kinds}
    iv.sort()
    busy, gaps, cur_s, cur_e = 0.0, [], iv[0][0], iv[0][1]
    for s0, e0 in iv[1:]:
        if s0 > cur_e:
            busy += cur_e - cur_s
            gaps.append(s0 - cur_e)
            cur_s, cur_e = s0, e0
        else:
            cur_e = max(cur_e, e0)
    busy += cur_e - cur_s
    span = iv[-1][1] - iv[0][0]
    gaps.sort()
    return {"kernels": len(iv), "span_ms": span / 1e3, "busy_ms": busy / 1e3, "busy_frac": busy / span,
            "gaps": len(gaps), "gap_total_ms": sum(gaps) / 1e3,
            "gap_median_us": gaps[len(gaps) // 2] if gaps else 0.0, "gap_max_us": gaps[-1] if gaps else 0.0}


def _wl_grid(args, dev):
    """vd1024 / fwd2048 / fwi384_3d: one grid, one library call per step."""
    import dataclasses

    import torch

    from neuralmech_gb300 import levels_for_budget, misfit_gradient, wave_forward
    from neuralmech_gb300.synth import workload as wl

    extra, graph_kernels = {}, 0
    w = wl("fwi1024" if args.workload == "vd1024" else args.workload, scale=args.scale)
    if args.shots:
        w.src = w.src[:args.shots].copy()
        if w.wavelet.ndim == 2:
            w.wavelet = w.wavelet[:args.shots].copy()
        if w.rec.ndim == 3:
            w.rec = w.rec[:args.shots].copy()
    g = w.grid
    if args.nt:
        g = dataclasses.replace(g, nt=args.nt, ckpt_every=min(g.ckpt_every or args.nt, args.nt))
        w.wavelet = w.wavelet[..., :args.nt]
    if args.ckpt_every:
        g = dataclasses.replace(g, ckpt_every=args.ckpt_every)
    g = dataclasses.replace(g, update=args.update)
    v = torch.from_numpy(w.vel).to(dev)
    wav = torch.from_numpy(w.wavelet).to(dev)
    src, rec = torch.from_numpy(w.src), torch.from_numpy(w.rec)
    R = g.order // 2
    interior = float(np.prod([n - 2 * R for n in g.shape]))
    if args.workload == "vd1024":
        # the fwi1024 models with Gardner densities rho = 310 v^0.25 and kappa = rho v^2
        from neuralmech_gb300.wavefd import vd_forward, vd_misfit_gradient
        if args.level_store_frac > 0:
            budget = args.level_store_frac * torch.cuda.get_device_properties(dev).total_memory
            g = dataclasses.replace(g, store_levels=levels_for_budget(g, w.nshot, budget))
        rho_of = lambda v: 310.0 * np.power(v.astype(np.float64), 0.25)
        r0, r1 = rho_of(w.vel), rho_of(w.vel_true)
        kap = torch.from_numpy((r0 * w.vel.astype(np.float64) ** 2).astype(np.float32)).to(dev)
        rho = torch.from_numpy(r0.astype(np.float32)).to(dev)
        obs = vd_forward(torch.from_numpy((r1 * w.vel_true.astype(np.float64) ** 2).astype(np.float32)).to(dev),
                         torch.from_numpy(r1.astype(np.float32)).to(dev), wav, src, rec, g)
        step = lambda: vd_misfit_gradient(kap, rho, wav, src, rec, obs, g, check=False)
        updates, bpu = 2.0 * w.nshot * interior * g.nt, 18.0
        cfg = {"workload": f"vd1024: 2D variable-density FWI gradient (kappa, rho) {g.shape[0]}^2, {g.nt} steps, "
                           f"{w.nshot} shots, {w.rec.shape[1]} receivers, order 8 staggered, 20-cell sponge, "
                           f"Gardner densities, BF16 checkpoints every {g.ckpt_every}",
               "store_levels": g.store_levels}
    elif args.workload == "fwd2048":
        g = dataclasses.replace(g, field_format=args.field_format, tile_rows=args.tile_rows,
                                step_block=(args.step_block or 1) if args.field_format == "fp32" else 1)
        step = lambda: wave_forward(v, wav, src, rec, g, check=False)
        updates, bpu = w.nshot * interior * g.nt, 16.0
        cfg = {"workload": f"fwd2048: 2D forward {g.shape[0]}^2, {g.nt} steps, 1 shot, "
                           f"{w.rec.shape[1]} receivers, order 8, 20-cell sponge",
               "field_format": g.field_format, "step_block": g.step_block, "tile_rows": g.tile_rows or 32}
        extra["l2_copy_gbs"] = l2_copy_gbs(dev)  # the fields stay in L2: its copy bandwidth is the roofline
        if g.field_format != "fp32":  # the storage error against the FP32 forward
            ref = wave_forward(v, wav, src, rec, dataclasses.replace(g, field_format="fp32"))
            got = step()
            cfg["traces_rel_l2_vs_fp32"] = float((got - ref).norm() / ref.norm())
    else:
        g = dataclasses.replace(g, group_shots=args.group_shots)
        obs = wave_forward(torch.from_numpy(w.vel_true).to(dev), wav, src, rec, g)
        step = lambda: misfit_gradient(v, wav, src, rec, obs, g, check=False)
        updates, bpu = 2.0 * w.nshot * interior * g.nt, 18.0
        cfg = {"workload": f"fwi384_3d: 3D FWI gradient {g.shape[0]}^3, {g.nt} steps, {w.nshot} shots "
                           f"in groups of {args.group_shots or w.nshot}, {w.rec.shape[1]} receivers per shot, "
                           f"BF16 checkpoints every {g.ckpt_every}", "update": g.update}
    return dict(step=step, updates=updates, bpu=bpu, cfg=cfg, extra=extra, graph_kernels=graph_kernels)


WORKLOADS = {"temporal": _wl_temporal, "fmc_tfm": _wl_fmc_tfm, "batch8": _wl_batch8}


def run_other(args):
    """Every workload but fwi1024: the kernel-level JSON line (no e2e leg)."""
    import torch

    from neuralmech_gb300 import _lib

    dev = torch.device("cuda", 0)
    lib = _lib.load()
    wk = WORKLOADS.get(args.workload, _wl_grid)(args, dev)
    step, updates, bpu, cfg = wk["step"], wk["updates"], wk["bpu"], wk["cfg"]
    extra, graph_kernels = wk["extra"], wk["graph_kernels"]
    if args.once:  # one step, no timing: the command profiled by ncu
        step()
        torch.cuda.synchronize()
        print(json.dumps({"once": args.workload, "config": cfg}), flush=True)
        return 0
    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    n0 = lib.wfd_kernel_launches()
    clocks.start()
    e0.record()
    for _ in range(args.steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1) / args.steps
    hbm, src_kind = peaks()
    gbs = updates * bpu / (ms / 1e3) / 1e9
    line = {"metric": METRIC, "value": updates / (ms / 1e3) / 1e9, "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": cfg,
            "hbm_alg_gbs": gbs, "hbm_frac_measured": gbs / hbm, "peak_source": src_kind, "clocks": clk,
            "gpu_launches": int(lib.wfd_kernel_launches() - n0) + graph_kernels * args.steps}
    if "l2_copy_gbs" in extra:
        extra["alg_frac_of_l2_copy"] = gbs / extra["l2_copy_gbs"]
    if "stage_ms" in extra:
        extra["stage_ms"] = {k: sum(v[-args.steps:]) / args.steps for k, v in extra["stage_ms"].items()}
    line.update(extra)
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "fwi1024":
        return run_other(args)

    import torch
    import torch.distributed as dist

    import dataclasses

    from neuralmech_gb300 import _lib, levels_for_budget, misfit_gradient, wave_forward
    from neuralmech_gb300.wavefd import Grid

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)
    lib = _lib.load()

    w = workload(args.scale, args.nt, args.shots)
    w.grid = dataclasses.replace(w.grid, step_block=args.step_block or 2, adjoint=args.adjoint, update=args.update)
    w.grid = dataclasses.replace(w.grid, level_format=args.level_format)
    if args.level_store_frac > 0:  # kept forward levels instead of recomputed ones
        budget = args.level_store_frac * torch.cuda.get_device_properties(dev).total_memory
        w.grid = dataclasses.replace(w.grid, store_levels=levels_for_budget(w.grid, w.nshot, budget))
    g = w.grid
    vel = torch.from_numpy(w.vel).to(dev)
    wav = torch.from_numpy(w.wavelet).to(dev)
    src = torch.from_numpy(w.src)
    rec = torch.from_numpy(w.rec)
    observed = wave_forward(torch.from_numpy(w.vel_true).to(dev), wav, src, rec, g)
    if world > 1:  # the survey of all ranks, sharded by shot block
        from neuralmech_gb300.shard import distributed_misfit_gradient
        survey = weak_survey(wav, src, rec, observed, world, rank)

    def step():
        if world > 1:
            return distributed_misfit_gradient(vel, *survey, g,
                                               compute=lambda *a: misfit_gradient(*a, check=False))
        return misfit_gradient(vel, wav, src, rec, observed, g, check=False)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # warm-up; the first call also checks the device status word (bounded TMA
    # waits, positions), the timed calls skip that synchronising read
    misfit_gradient(vel, wav, src, rec, observed, g, check=True)
    if args.once:
        torch.cuda.synchronize()
        return 0
    for _ in range(max(args.warmup - 1, 0)):
        step()
    barrier()

    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    launches0 = lib.wfd_kernel_launches()
    _lib.check(lib.wfd_profile_begin(), "wfd_profile_begin")
    barrier()
    clocks.start()
    e0.record(stream)
    for _ in range(args.steps):
        J, grad = step()
    e1.record(stream)
    barrier()
    clk = clocks.stop()
    phases = _lib.PhaseTimes()
    _lib.check(lib.wfd_profile_end(ctypes.byref(phases)), "wfd_profile_end")
    launches = lib.wfd_kernel_launches() - launches0
    ms = e0.elapsed_time(e1) / args.steps
    t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t)
    if not torch.isfinite(grad).all() or not np.isfinite(float(J)):
        raise RuntimeError("non-finite gradient or misfit in the timed region")
    misfit_gradient(vel, wav, src, rec, observed, g, check=True)  # status after the timed region

    updates, interior = counted_updates(w)
    value = updates * world / (ms / 1e3) / 1e9
    hbm, peak_src = peaks()
    alg_gbs = updates * 18.0 / (ms / 1e3) / 1e9  # 36 B per (cell, step) pair

    # roofline of the dominant kernel (largest device-time phase)
    names = ["forward", "recompute", "adjoint"]
    share = {n: phases.ms[i] for i, n in enumerate(names)}
    dom = max(share, key=share.get)
    i = names.index(dom)
    per_launch_ms = phases.ms[i] / max(1, phases.launches[i])
    bytes_per_launch = alg_bytes(g, dom) * w.nshot * interior
    achieved = bytes_per_launch / (per_launch_ms / 1e3) / 1e9
    tr = traffic_per_update().get(f"{dom}_bytes_per_cell_update")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                "traffic": None if tr is None else tr * w.nshot * interior,
                "kernel": f"step2d_kernel ({dom} phase)", "peak_source": peak_src,
                "alg_bytes_per_launch": bytes_per_launch, "ms_per_launch": per_launch_ms}
    if phases.ms[1] > 0 and kept_segments(g) >= 2:
        # the library recomputes each segment on a second stream beside the adjoint
        # of the segment after it: both phases' launch times include the other's
        # share of DRAM, and the phase times overlap in wall time
        roofline["concurrent_with"] = "recompute" if dom == "adjoint" else "adjoint"

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded layered + Gaussian anomaly models)",
        "config": config_of(w, args), "roofline": roofline, "clocks": clk, "gpu_launches": int(launches),
        "shots_per_s": w.nshot * world / (ms / 1e3),
        "hbm_alg_gbs": alg_gbs, "hbm_frac_measured": alg_gbs / hbm, "hbm_frac_8tbs": alg_gbs / 8000.0,
        "phase_ms_per_step": {n: phases.ms[k] / args.steps for k, n in enumerate(names)},
        "phase_share": {n: phases.ms[k] / max(1e-9, sum(phases.ms)) for k, n in enumerate(names)},
    }

    if not args.no_extras:
        # end to end through the public API, host buffers, copies inside the timed region
        host = {"vel": torch.from_numpy(w.vel).pin_memory(), "wav": torch.from_numpy(w.wavelet).pin_memory(),
                "obs": observed.cpu().pin_memory()}
        grad_h = torch.empty(g.shape, dtype=torch.float32).pin_memory()
        J_h = torch.empty((), dtype=torch.float64).pin_memory()
        h2d = sum(x.numel() * x.element_size() for x in host.values()) + src.numel() * 4 + rec.numel() * 4
        d2h = grad_h.numel() * 4 + 8

        # the observed traces (most of the bytes) go up on a second stream while
        # the forward runs; the call waits for them only before the residual.
        # The inputs the forward needs are copied first, so that the model's
        # copy cannot queue behind the traces' on a shared copy engine.
        copy_stream = torch.cuda.Stream(device=dev)
        ob = torch.empty(host["obs"].shape, dtype=torch.float32, device=dev)
        ob_ready = torch.cuda.Event()
        src_h, rec_h = src.pin_memory(), rec.pin_memory()

        def e2e_step():
            v = host["vel"].to(dev, non_blocking=True)
            wv = host["wav"].to(dev, non_blocking=True)
            s_d, r_d = src_h.to(dev, non_blocking=True), rec_h.to(dev, non_blocking=True)
            copy_stream.wait_stream(torch.cuda.current_stream(dev))  # the previous step's reads of ob
            with torch.cuda.stream(copy_stream):
                ob.copy_(host["obs"], non_blocking=True)
                ob_ready.record(copy_stream)
            J2, g2 = misfit_gradient(v, wv, s_d, r_d, ob, g, check=False, observed_ready=ob_ready)
            if world > 1:
                dist.all_reduce(g2)
                dist.all_reduce(J2)
            grad_h.copy_(g2, non_blocking=True)
            J_h.copy_(J2, non_blocking=True)

        e2e_step()
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        barrier()
        ms_e2e = e0.elapsed_time(e1) / args.steps
        t = torch.tensor([ms_e2e], device=dev)
        if world > 1:
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_e2e = float(t)
        line["e2e"] = {"value": updates * world / (ms_e2e / 1e3) / 1e9, "unit": UNIT,
                       "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h), "ms_per_step": ms_e2e}

        # plain: one shot per call (per-shot forward/adjoint, one launch per step)
        P = min(args.plain_shots, w.nshot)
        # the batched call's level budget too (one shot's levels all fit: nothing is recomputed)
        gp = Grid(g.shape, g.spacing, g.dt, g.nt, order=g.order, sponge=g.sponge, ckpt_every=g.ckpt_every,
                  ckpt_format=g.ckpt_format, shots_per_cta=1)
        if args.level_store_frac > 0:
            gp = dataclasses.replace(gp, store_levels=levels_for_budget(gp, 1, budget))
        misfit_gradient(vel, wav, src[:1], rec[:1], observed[:1].contiguous(), gp, check=False)
        barrier()
        e0.record(stream)
        for s in range(P):
            misfit_gradient(vel, wav, src[s:s + 1], rec[s:s + 1], observed[s:s + 1].contiguous(), gp, check=False)
        e1.record(stream)
        barrier()
        plain_sps = P / (e0.elapsed_time(e1) / 1e3)
        line["plain_shots_per_s"] = plain_sps
        line["batched_vs_plain"] = line["shots_per_s"] / world / plain_sps

        if rank == 0 and world == 1:
            steps = args.cpu_sample_steps if args.scale >= 1 else max(10, int(args.cpu_sample_steps * args.scale))
            u, tcpu, desc = cpu_gradient_sample(w, steps)
            line["cpu_baseline"] = {"value": u / tcpu / 1e9, "unit": UNIT, "cores": os.cpu_count(),
                                    "kind": "port", "sample": desc, "numpy_fd_step": numpy_fd_step_legs()}
            line["secondary"] = secondary_legs(dev)

    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
