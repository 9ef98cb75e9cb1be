"""Empirical autotuner of the 2D kernel configuration.

For a problem key (architecture, grid shape, order, shots) it times a short
forward (`steps` time steps) for every candidate:
  * one step per launch: tile_rows (16 or 32) x shots_per_cta (1, 2, 4, ...
    up to 32 and the shot count);
  * two steps per launch (step_block 2, 120 x 32 tiles) x shots_per_cta
    (automatic, 1, 2, 4, ...).

For the forward of a gradient (``for_gradient``) whose grid asks for the
summed update form ("auto" or "summed"), the candidates are timed in that
form (both kernels have it): the leapfrog form's accumulated rounding is
what a gradient from small residuals cannot afford.

It keeps the fastest, and caches the choice in a JSON file (default
``~/.cache/neuralmech_gb300/autotune.json``, or ``$WAVEFD_AUTOTUNE_CACHE``).
The candidate timings use CUDA events on the current stream after one warm-up
launch per candidate. 3D problems have a fixed tile (64 x 16 columns marching
64 planes, one shot per CTA) and are not tuned.
"""
from __future__ import annotations

import dataclasses
import json
import os
import threading

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("WAVEFD_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "neuralmech_gb300", "autotune.json"))


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path, data):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def problem_key(arch: str, shape, order: int, nshot: int, summed: bool = False) -> str:
    return f"{arch}|{'x'.join(map(str, shape))}|o{order}|s{nshot}" + ("|summed" if summed else "")


def candidates(nshot: int, summed: bool = False):
    spcs = [s for s in (1, 2, 4, 8, 16, 32) if s <= max(1, nshot)]
    if nshot <= 32 and nshot not in spcs:
        spcs.append(nshot)
    one = [{"tile_rows": tr, "shots_per_cta": s, "step_block": 1} for tr in (32, 16) for s in spcs]
    two = [{"tile_rows": 0, "shots_per_cta": s, "step_block": 2} for s in [0] + spcs]
    return one + two


def summed_for(grid, for_gradient: bool) -> bool:
    """Whether the forward that the tuned configuration serves runs in the
    summed form (FP32 fields, lap_store auto, checkpoint adjoint; the
    same rule as the library's WFD_UPDATE_AUTO)."""
    avail = grid.field_format == "fp32" and grid.lap_store == "auto" and grid.adjoint == "checkpoint"
    return avail and (grid.update == "summed" or (grid.update == "auto" and for_gradient))


def select(timings: dict) -> dict:
    """The fastest candidate of {json(candidate): seconds}."""
    best = min(timings, key=timings.get)
    return json.loads(best)


def tune(grid, nshot: int, vel=None, steps: int = 16, device=None, path: str | None = None,
         timer=None, refresh: bool = False, for_gradient: bool = False) -> dict:
    """Best {tile_rows, shots_per_cta, step_block} for `grid` with `nshot` shots (2D).

    `timer(config) -> seconds` replaces the GPU timing (used by tests)."""
    if grid.ndim != 2:
        return {"tile_rows": 0, "shots_per_cta": 0, "step_block": 0}
    import torch
    path = path or cache_path()
    arch = "cpu-timer" if timer else torch.cuda.get_device_name(device)
    summed = summed_for(grid, for_gradient)
    key = problem_key(arch, grid.shape, grid.order, nshot, summed)
    with _lock:
        cache = _load(path)
        if key in cache and not refresh:
            return cache[key]["best"]
    if timer is None:
        timer = _gpu_timer(dataclasses.replace(grid, update="summed" if summed else "leapfrog"), nshot, vel,
                           steps, device)
    timings = {json.dumps(c, sort_keys=True): float(timer(c)) for c in candidates(nshot, summed)}
    best = select(timings)
    with _lock:
        cache = _load(path)
        cache[key] = {"best": best, "timings_s": timings, "steps": steps}
        _store(path, cache)
    return best


def _gpu_timer(grid, nshot, vel, steps, device):
    import torch

    from .wavefd import wave_forward
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    nz, nx = grid.shape
    if vel is None:
        vel = torch.full((nz, nx), 2000.0, device=dev)
    R = grid.order // 2
    g = dataclasses.replace(grid, nt=steps, group_shots=0)
    src = torch.tensor([[[max(R, nz // 8), nx // 2]]] * nshot, dtype=torch.int32)
    rec = torch.tensor([[[max(R, nz // 8), x] for x in range(R, nx - R, max(1, (nx - 2 * R) // 64))]] * nshot,
                       dtype=torch.int32)
    wav = torch.zeros((nshot, steps), device=dev)

    def timer(cfg):
        gc = dataclasses.replace(g, **cfg)
        wave_forward(vel, wav, src, rec, gc, check=False)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        wave_forward(vel, wav, src, rec, gc, check=False)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    return timer


def tuned(grid, nshot: int, **kw):
    """`grid` with tile_rows / shots_per_cta / step_block replaced by the tuned choice."""
    best = tune(grid, nshot, **kw)
    return dataclasses.replace(grid, **best) if grid.ndim == 2 else grid
