"""GPU parity of the variable-density path (2D staggered conservative
operator, kappa and rho) against the FP64 oracle, through the C ABI:
  * traces: 1e-5 relative L2 (FP32 stencil against FP64);
  * gradient w.r.t. kappa, rho and the wavelets: 1e-4 with FP32 checkpoints
    (recomputed and kept segments), 1e-2 with BF16 checkpoints (measured
    5.6e-3: the rounding of the restored levels, as in the constant-density
    path);
  * order 2 with constant density equals the constant-density path's
    5-point step (1e-5).
"""
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _vd_problem(order=8, shape=(72, 200), nshot=3, nt=120, seed=0, ckpt_every=0, ckpt_format="fp32", nrec=25):
    from neuralmech_gb300 import Grid
    from neuralmech_gb300.synth import ricker
    rng = np.random.default_rng(seed)
    nz, nx = shape
    rho = np.full(shape, 1000.0)
    c = np.full(shape, 1500.0)
    rho[nz // 2:, :] = 1800.0
    c[nz // 2:, :] = 2500.0
    zz, xx = np.mgrid[0:nz, 0:nx]
    blob = (zz - 0.35 * nz) ** 2 + (xx - 0.6 * nx) ** 2 < (0.12 * nz) ** 2
    rho[blob] = 2600.0  # a dense inclusion: a sharp density interface
    c[blob] = 3000.0
    c *= 1 + 0.02 * rng.standard_normal(shape)
    kappa = (rho * c * c).astype(np.float32)
    rho = rho.astype(np.float32)
    dx = 10.0
    dt = 0.4 * dx / float(c.max())
    grid = Grid(shape, (dx, dx), dt, nt, order=order, sponge=10, ckpt_every=ckpt_every, ckpt_format=ckpt_format)
    R = order // 2
    src = np.stack([rng.integers(R, nz - R, (nshot, 1)), rng.integers(R, nx - R, (nshot, 1))], -1)
    rec = np.stack([rng.integers(R, nz - R, (nshot, nrec)), rng.integers(R, nx - R, (nshot, nrec))], -1)
    wav = np.stack([ricker(25.0 * (1 + 0.1 * s), nt, dt) for s in range(nshot)])[:, :, None].astype(np.float32)
    return grid, kappa, rho, wav, src.astype(np.int32), rec.astype(np.int32)


def _geom(orc, grid, kappa, rho, wav, src, rec):
    from neuralmech_gb300 import sponge_profiles
    gz, _, gx = sponge_profiles(grid)
    p3 = lambda p: np.stack([p[..., 0], 0 * p[..., 0], p[..., 1]], -1).astype(np.int32)
    return orc.VdGeometry(kappa.astype(np.float64), rho.astype(np.float64), wav.astype(np.float64), p3(src), p3(rec),
                          float(np.float32(grid.dt)), grid.spacing, order=grid.order,
                          sponge=(gz.astype(np.float64), gx.astype(np.float64)))


@pytest.mark.parametrize("order", [2, 4, 8])
def test_vd_forward_matches_oracle(cuda, orc, order):
    from neuralmech_gb300.wavefd import vd_forward
    grid, kappa, rho, wav, src, rec = _vd_problem(order=order, shape=(66, 190) if order != 4 else (53, 141))
    t = vd_forward(torch.from_numpy(kappa).to(cuda), torch.from_numpy(rho).to(cuda), torch.from_numpy(wav).to(cuda),
                   torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.vd_forward(_geom(orc, grid, kappa, rho, wav, src, rec))
    err = rel_l2(t.cpu().numpy(), ref)
    print(f"order {order}: traces rel L2 {err:.2e}")
    assert err < 1e-5


@pytest.mark.parametrize("order,ckpt,levels,fmt,tol", [
    (8, 0, 0, "fp32", 1e-4),
    (4, 13, 0, "fp32", 1e-4),
    (8, 17, 10 ** 6, "fp32", 1e-4),
    (8, 11, 0, "bf16", 1e-2),
])
def test_vd_gradient_matches_oracle(cuda, orc, order, ckpt, levels, fmt, tol):
    from neuralmech_gb300.wavefd import vd_forward, vd_misfit_gradient
    grid, kappa, rho, wav, src, rec = _vd_problem(order=order, ckpt_every=ckpt, ckpt_format=fmt, seed=3)
    grid = dataclasses.replace(grid, store_levels=levels)
    geo = _geom(orc, grid, kappa, rho, wav, src, rec)
    obs = orc.vd_forward(dataclasses.replace(geo, kappa=geo.kappa * 1.04)).astype(np.float32)
    J, gk, gr, gw = vd_misfit_gradient(torch.from_numpy(kappa).to(cuda), torch.from_numpy(rho).to(cuda),
                                       torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec),
                                       torch.from_numpy(obs).to(cuda), grid, want_wavelet=True)
    Jr, gkr, grr, gwr, _ = orc.vd_gradient(geo, obs)
    e = (rel_l2(gk.cpu().numpy(), gkr), rel_l2(gr.cpu().numpy(), grr), rel_l2(gw.cpu().numpy(), gwr))
    print(f"order {order} ckpt {ckpt} levels {levels} {fmt}: misfit {abs(J.item() - Jr) / Jr:.1e}, "
          f"grad kappa / rho / wavelet rel L2 {e}")
    assert abs(J.item() - Jr) / Jr < 2e-4
    assert max(e) < tol


def test_vd_constant_density_order2_is_the_scalar_step(cuda):
    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300.wavefd import vd_forward
    grid, kappa, rho, wav, src, rec = _vd_problem(order=2)
    rho = np.full_like(rho, 1700.0)
    vel = np.sqrt(kappa / rho).astype(np.float32)
    args = (torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec), grid)
    t_vd = vd_forward(torch.from_numpy(kappa).to(cuda), torch.from_numpy(rho).to(cuda), *args)
    t_sc = wave_forward(torch.from_numpy(vel).to(cuda), *args)
    assert rel_l2(t_vd.cpu().numpy(), t_sc.cpu().numpy()) < 1e-5
