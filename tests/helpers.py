"""Shared test builders: small seeded problems run both through the product
(neuralmech_gb300, on the GPU) and through the FP64 oracle (on the CPU)."""
from __future__ import annotations

import numpy as np

from neuralmech_gb300 import Grid, sponge_profiles
from neuralmech_gb300.synth import add_anomalies, layered, ricker


def small_problem(shape=(60, 150), nshot=3, nsrc=1, nrec=17, nt=120, order=8, sponge=10,
                  seed=0, dx=10.0, cfl=0.45, freq=25.0, ckpt_every=0, ckpt_format="fp32",
                  lap_store="auto", spc=0, src_scale=1.0, tile_rows=0, step_block=0):
    rng = np.random.default_rng(seed)
    nd = len(shape)
    n0 = shape[0]
    v = layered(shape, [0, n0 // 3, 2 * n0 // 3], [1500.0, 2200.0, 3000.0])
    v = add_anomalies(v, rng, 2, max(2.0, min(shape) / 8)).astype(np.float32)
    h = (dx,) * nd
    dt = cfl * dx / float(v.max())
    grid = Grid(tuple(shape), h, dt, nt, order=order, sponge=sponge, ckpt_every=ckpt_every,
                ckpt_format=ckpt_format, lap_store=lap_store, shots_per_cta=spc, src_scale=src_scale,
                tile_rows=tile_rows, step_block=step_block)
    R = order // 2
    lo = [R] * nd
    hi = [n - R - 1 for n in shape]
    src = np.stack([rng.integers(l, h_ + 1, size=(nshot, nsrc)) for l, h_ in zip(lo, hi)], axis=-1)
    rec = np.stack([rng.integers(l, h_ + 1, size=(nshot, nrec)) for l, h_ in zip(lo, hi)], axis=-1)
    wav = np.stack([ricker(freq * (1 + 0.1 * s), nt, dt) for s in range(nshot)])
    wav = np.repeat(wav[:, :, None], nsrc, axis=2) * rng.uniform(0.5, 1.5, size=(nshot, 1, nsrc))
    return grid, v, wav.astype(np.float32), src.astype(np.int32), rec.astype(np.int32)


def oracle_geometry(oracle, grid, v, wav, src, rec):
    """The same problem as an oracle.Geometry (positions widened to (z, y, x))."""
    def p3(p):
        if p.shape[-1] == 3:
            return p
        return np.stack([p[..., 0], np.zeros_like(p[..., 0]), p[..., 1]], axis=-1)

    gz, gy, gx = sponge_profiles(grid)
    sp = tuple(None if g is None else g.astype(np.float64) for g in (gz, gy, gx))
    h = grid.spacing if grid.ndim == 3 else (grid.spacing[0], 1.0, grid.spacing[1])
    return oracle.Geometry(vel=v.astype(np.float64), wavelet=wav.astype(np.float64),
                           src=p3(src).astype(np.int32), rec=p3(rec).astype(np.int32),
                           dt=float(np.float32(grid.dt)), h=h, order=grid.order, sponge=sp,
                           src_scale=grid.src_scale, ckpt_every=grid.ckpt_every)


def vd_operator(kappa, rho, c):
    """kappa Lb of the variable-density step as a dense matrix on a unit grid,
    assembled term by term from its definition (rows and columns of the cells
    outside the fixed ring of R cells): F = b_half D u at the half points,
    b_half the mean of the two cells' b = 1/rho, Lb u = D F on each axis,
    (D f)_j = sum_k c_k (f_{j+k} - f_{j-k+1}), fields and b zero outside."""
    nz, nx = kappa.shape
    R = len(c)
    b = 1.0 / rho
    idx = {}
    for z in range(R, nz - R):
        for x in range(R, nx - R):
            idx[(z, x)] = len(idx)
    A = np.zeros((len(idx), len(idx)))

    def bcell(z, x):
        return b[z, x] if 0 <= z < nz and 0 <= x < nx else 0.0

    for (z, x), row in idx.items():
        for axis in (0, 1):
            step = (1, 0) if axis == 0 else (0, 1)
            pos = z if axis == 0 else x

            def cell(q):
                return (q, x) if axis == 0 else (z, q)
            for k in range(1, R + 1):
                for sgn, j in ((1.0, pos + k - 1), (-1.0, pos - k)):  # F at j + 1/2
                    bh = 0.5 * (bcell(*cell(j)) + bcell(*cell(j + 1)))
                    for m in range(1, R + 1):
                        for s2, q in ((1.0, j + m), (-1.0, j - m + 1)):
                            col = idx.get(cell(q))
                            if col is not None:
                                A[row, col] += kappa[z, x] * sgn * c[k - 1] * bh * s2 * c[m - 1]
    return A
