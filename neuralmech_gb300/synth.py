"""Seeded synthetic inputs of the wave workloads (no dataset is involved).

Velocity models are horizontal layers plus Gaussian anomalies
v *= 1 +/- 0.1 exp(-r^2 / (2 sigma^2)), centre and sign drawn from the seed;
layer depths and sigmas are given for a 256-cell grid and scale with the grid.
The wavelet is a Ricker r(t) = (1 - 2 pi^2 f^2 tau^2) exp(-pi^2 f^2 tau^2),
tau = t - 1.5 / f. The time step is dt = CFL dx / v_max (CFL 0.5 in 2D, 0.45
in 3D, inside the order-8 bounds 0.5547 and 0.4529).

Presets (``workload(name)``):
  fwd256     2D forward, 256^2, dx 10 m, 1000 steps, source (x 128, z 5),
             256 receivers on row 5, 3 layers 1500/2500/3500 m/s at depths
             0/90/170, one anomaly sigma 20
  fwd2048    the same generator scaled to 2048^2, 4000 steps, 2048 receivers
  fwi1024    2D FWI gradient, 1024^2, 2000 steps, 64 shots along the surface,
             1024 receivers, true model layers + 3 anomalies, initial model the
             true one Gaussian-smoothed (sigma 30 cells), checkpoints every 45
  batch8     8 models, 128 shots, square grids U{512..1536 step 64}, steps
             U{1000..3000}, Ricker f U[10, 25] Hz
  fwi384_3d  3D FWI gradient, 384^3, 1500 steps, 16 shots on the top surface,
             64 x 64 receivers each, 4 layers 1500-4000 m/s + 2 blobs,
             checkpoints every 39 (BF16)
Every preset takes ``scale`` (grid and step counts multiplied by it) so the
tests can run the same generator at small sizes.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .wavefd import Grid


def ricker(freq: float, nt: int, dt: float, t0: float | None = None) -> np.ndarray:
    t0 = 1.5 / freq if t0 is None else t0
    t = np.arange(nt) * dt - t0
    a = (math.pi * freq * t) ** 2
    return ((1.0 - 2.0 * a) * np.exp(-a)).astype(np.float32)


def layered(shape, depths, velocities) -> np.ndarray:
    """Horizontal layers: velocity[i] from depth cell depths[i] down (z axis 0)."""
    v = np.empty(shape, dtype=np.float64)
    z = np.arange(shape[0])
    prof = np.full(shape[0], velocities[0], dtype=np.float64)
    for d, c in zip(depths, velocities):
        prof[z >= d] = c
    v[...] = prof.reshape((-1,) + (1,) * (len(shape) - 1))
    return v


def add_anomalies(v: np.ndarray, rng, count: int, sigma: float, amp: float = 0.1,
                  margin: float = 0.15) -> np.ndarray:
    """Multiply v by 1 +/- amp exp(-r^2/2 sigma^2) at `count` seeded centres."""
    grids = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in v.shape], indexing="ij")
    out = v.copy()
    for _ in range(count):
        c = [rng.uniform(margin * n, (1 - margin) * n) for n in v.shape]
        sign = 1.0 if rng.random() < 0.5 else -1.0
        r2 = sum((g - ci) ** 2 for g, ci in zip(grids, c))
        out *= 1.0 + sign * amp * np.exp(-r2 / (2.0 * sigma**2))
    return out


def gaussian_smooth(v: np.ndarray, sigma: float) -> np.ndarray:
    """Separable Gaussian blur (reflecting edges), sigma in cells."""
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(v, sigma=sigma, mode="nearest")


@dataclass
class Workload:
    name: str
    grid: Grid
    vel: np.ndarray           # model the traces are computed in (float32)
    wavelet: np.ndarray       # (nt,) or (nshot, nt)
    src: np.ndarray           # (nshot, nsrc, ndim) int32
    rec: np.ndarray           # (nshot, nrec, ndim) or (nrec, ndim)
    vel_true: np.ndarray | None = None  # FWI: model of the observed data
    seed: int = 0

    @property
    def nshot(self) -> int:
        return self.src.shape[0]


def _surface_line(n: int, count: int, lo: int, hi: int) -> np.ndarray:
    return np.rint(np.linspace(lo, hi, count)).astype(np.int32)


def fwd2d(n: int = 256, nt: int = 1000, seed: int = 0, dx: float = 10.0, order: int = 8,
          freq: float = 15.0, cfl: float = 0.5, nrec: int | None = None, name: str = "fwd256") -> Workload:
    rng = np.random.default_rng(seed)
    s = n / 256.0
    v = layered((n, n), [0, round(90 * s), round(170 * s)], [1500.0, 2500.0, 3500.0])
    v = add_anomalies(v, rng, 1, 20 * s).astype(np.float32)
    dt = cfl * dx / float(v.max())
    grid = Grid((n, n), (dx, dx), dt, nt, order=order, sponge=20)
    R = order // 2
    src = np.array([[[5, min(max(n // 2, R), n - R - 1)]]], dtype=np.int32)
    nrec = n if nrec is None else nrec
    rec = np.stack([np.full(nrec, 5), _surface_line(n, nrec, R, n - R - 1)], axis=-1).astype(np.int32)
    return Workload(name, grid, v, ricker(freq, nt, dt), src, rec[None], seed=seed)


def fwi2d(n: int = 1024, nt: int = 2000, nshot: int = 64, nrec: int = 1024, seed: int = 0,
          dx: float = 10.0, freq: float = 15.0, cfl: float = 0.5, ckpt_every: int = 45,
          order: int = 8, name: str = "fwi1024") -> Workload:
    rng = np.random.default_rng(seed)
    s = n / 256.0
    base = layered((n, n), [0, round(90 * s), round(170 * s)], [1500.0, 2500.0, 3500.0])
    true = add_anomalies(base, rng, 3, 20 * s)
    init = gaussian_smooth(true, 30 * s / 4)  # sigma 30 cells at n = 1024
    vmax = float(max(true.max(), init.max()))
    dt = cfl * dx / vmax
    grid = Grid((n, n), (dx, dx), dt, nt, order=order, sponge=20, ckpt_every=ckpt_every)
    R = order // 2
    xs = _surface_line(n, nshot, R + 16, n - R - 17)
    src = np.stack([np.full(nshot, 5), xs], axis=-1).astype(np.int32)[:, None, :]
    rec = np.stack([np.full(nrec, 5), _surface_line(n, nrec, R, n - R - 1)], axis=-1).astype(np.int32)
    return Workload(name, grid, init.astype(np.float32), ricker(freq, nt, dt), src, rec[None].repeat(nshot, 0),
                    vel_true=true.astype(np.float32), seed=seed)


def fwi3d(n: int = 384, nt: int = 1500, nshot: int = 16, nrec_side: int = 64, seed: int = 0,
          dx: float = 10.0, freq: float = 15.0, cfl: float = 0.45, ckpt_every: int = 39,
          order: int = 8, name: str = "fwi384_3d") -> Workload:
    rng = np.random.default_rng(seed)
    s = n / 256.0
    base = layered((n, n, n), [0, round(60 * s), round(120 * s), round(190 * s)],
                   [1500.0, 2300.0, 3100.0, 4000.0])
    true = add_anomalies(base, rng, 2, 20 * s)
    init = gaussian_smooth(true, 30 * s / 4)
    vmax = float(max(true.max(), init.max()))
    dt = cfl * dx / vmax
    grid = Grid((n, n, n), (dx, dx, dx), dt, nt, order=order, sponge=20, ckpt_every=ckpt_every,
                ckpt_format="bf16")
    R = order // 2
    side = int(math.ceil(math.sqrt(nshot)))
    pos = _surface_line(n, side, R + n // 8, n - R - 1 - n // 8)
    sy, sx = np.meshgrid(pos, pos, indexing="ij")
    src = np.stack([np.full(side * side, 5), sy.ravel(), sx.ravel()], axis=-1)[:nshot].astype(np.int32)[:, None, :]
    rl = _surface_line(n, nrec_side, R, n - R - 1)
    ry, rx = np.meshgrid(rl, rl, indexing="ij")
    rec = np.stack([np.full(rl.size**2, 5), ry.ravel(), rx.ravel()], axis=-1).astype(np.int32)
    return Workload(name, grid, init.astype(np.float32), ricker(freq, nt, dt), src,
                    rec[None].repeat(nshot, 0), vel_true=true.astype(np.float32), seed=seed)


def batch_models(nmodels: int = 8, nshot: int = 128, sizes=(512, 1536, 64), steps=(1000, 3000),
                 freqs=(10.0, 25.0), seed: int = 0, dx: float = 10.0, cfl: float = 0.5,
                 order: int = 8, ckpt_every: int = 0, ckpt_format: str = "bf16"):
    """Uneven batch: nmodels seeded layered+anomaly models of random square size
    and step count, shots split as evenly as possible; each entry a Workload
    with its own observed-data model (vel_true) and smoothed start model."""
    rng = np.random.default_rng(seed)
    lo, hi, step = sizes
    counts = [nshot // nmodels + (1 if i < nshot % nmodels else 0) for i in range(nmodels)]
    out = []
    for i in range(nmodels):
        n = int(rng.choice(np.arange(lo, hi + 1, step)))
        nt = int(rng.integers(steps[0], steps[1] + 1))
        f = float(rng.uniform(*freqs))
        w = fwi2d(n=n, nt=nt, nshot=counts[i], nrec=n, seed=seed * 1000 + i, dx=dx, freq=f, cfl=cfl,
                  ckpt_every=ckpt_every, order=order, name=f"batch{i}")
        g = w.grid
        w.grid = Grid(g.shape, g.spacing, g.dt, g.nt, order=g.order, sponge=g.sponge,
                      ckpt_every=ckpt_every, ckpt_format=ckpt_format)
        out.append(w)
    return out


def workload(name: str, scale: float = 1.0, seed: int = 0, **kw):
    """The named preset, optionally shrunk (grid and steps times `scale`)."""
    sc = lambda v, m=16: max(m, int(round(v * scale)))
    if name == "fwd256":
        return fwd2d(n=sc(256, 32), nt=sc(1000), seed=seed, name=name, **kw)
    if name == "fwd2048":
        return fwd2d(n=sc(2048, 32), nt=sc(4000), seed=seed, name=name, **kw)
    if name == "fwi1024":
        return fwi2d(n=sc(1024, 32), nt=sc(2000), seed=seed, name=name, **kw)
    if name == "fwi384_3d":
        return fwi3d(n=sc(384, 24), nt=sc(1500), seed=seed, name=name, **kw)
    if name == "batch8":
        return batch_models(seed=seed, **kw)
    raise KeyError(name)
