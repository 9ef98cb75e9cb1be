"""The reconstruction adjoint (time reversal from the last two levels, the
damped frame restored from per-step copies, no checkpoints) against the FP64
oracle gradient, for the constant- and the variable-density operator, with a
sponge and without one (a Dirichlet plate, where reversal needs no copies at
all). FP32 reversal accumulates rounding over the steps; measured 2-14e-6 on the
gradients and 3-4e-5 on the wavelet gradients, bounds 1e-4 / 2e-4."""
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import oracle_geometry, small_problem

pytestmark = pytest.mark.gpu


def _observed(orc, grid, v, wav, src, rec, seed=7):
    rng = np.random.default_rng(seed)
    vt = (v * (1 + 0.05 * rng.standard_normal(v.shape).clip(-2, 2))).astype(np.float32)
    return orc.forward(oracle_geometry(orc, grid, vt, wav, src, rec)).astype(np.float32)


@pytest.mark.parametrize("order,sponge,nt", [(8, 10, 150), (2, 0, 120), (4, 12, 200)])
def test_reconstruct_gradient_matches_oracle(cuda, orc, order, sponge, nt):
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(80, 210), nshot=3, nt=nt, order=order, sponge=sponge, seed=12)
    obs = _observed(orc, grid, v, wav, src, rec)
    g = dataclasses.replace(grid, adjoint="reconstruct")
    J, gv, gw = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                                torch.from_numpy(rec), torch.from_numpy(obs).to(cuda), g, want_wavelet=True)
    Jr, gr, gwr, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    e = (rel_l2(gv.cpu().numpy(), gr), rel_l2(gw.cpu().numpy(), gwr))
    print(f"order {order} sponge {sponge} nt {nt}: misfit {abs(J.item() - Jr) / Jr:.1e}, gradient / wavelet {e}")
    assert abs(J.item() - Jr) / Jr < 2e-4
    assert e[0] < 1e-4 and e[1] < 2e-4


def test_reconstruct_variable_density(cuda, orc):
    from test_vd_gpu import _geom, _vd_problem
    from neuralmech_gb300.wavefd import vd_misfit_gradient
    grid, kappa, rho, wav, src, rec = _vd_problem(order=8, seed=5)
    geo = _geom(orc, grid, kappa, rho, wav, src, rec)
    obs = orc.vd_forward(dataclasses.replace(geo, kappa=geo.kappa * 1.04)).astype(np.float32)
    g = dataclasses.replace(grid, adjoint="reconstruct")
    J, gk, gr = vd_misfit_gradient(torch.from_numpy(kappa).to(cuda), torch.from_numpy(rho).to(cuda),
                                   torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec),
                                   torch.from_numpy(obs).to(cuda), g)
    Jr, gkr, grr, _, _ = orc.vd_gradient(geo, obs)
    e = (rel_l2(gk.cpu().numpy(), gkr), rel_l2(gr.cpu().numpy(), grr))
    print(f"variable density, reconstruction: misfit {abs(J.item() - Jr) / Jr:.1e}, kappa / rho {e}")
    assert max(e) < 1e-4


def test_reconstruct_autograd_path(cuda, orc):
    """wave_forward (checkpointed forward keeping frames) + backward through
    torch.autograd with the reconstruction adjoint equals the fused call."""
    from neuralmech_gb300 import misfit_gradient, wave_forward
    grid, v, wav, src, rec = small_problem(shape=(60, 170), nshot=2, nt=90, seed=4)
    g = dataclasses.replace(grid, adjoint="reconstruct")
    obs = torch.from_numpy(_observed(orc, grid, v, wav, src, rec)).to(cuda)
    vel = torch.from_numpy(v).to(cuda).requires_grad_(True)
    t = wave_forward(vel, torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec), g)
    (0.5 * ((t - obs) ** 2).sum()).backward()
    _, gf = misfit_gradient(vel.detach(), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                            torch.from_numpy(rec), obs, g)
    assert rel_l2(vel.grad.cpu().numpy(), gf.cpu().numpy()) < 1e-5
