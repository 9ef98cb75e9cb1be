"""A seeded sweep of small problems against the FP64 oracle, to cover
combinations that the targeted tests take one at a time:
  * 2D and 3D grids of random, mostly odd sizes (tile seams, partial tiles,
    partial z chunks);
  * orders 2, 4 and 8;
  * no sponge, a uniform sponge, or per-face widths;
  * 1 to 4 shots with 1 to 3 sources at random interior cells and 1 to 30
    receivers within reach of the first source (duplicates allowed);
  * the leapfrog and summed update forms;
  * one or two steps per launch (2D);
  * shot groups, checkpoint intervals from 1 step to the whole run, FP32 and
    BF16 checkpoints.

Each case checks the forward traces (1e-5 relative L2, FP32 against FP64),
the misfit (2e-4) and the velocity gradient. The gradient bound is 2e-4
with FP32 checkpoints and 5e-3 with BF16 ones; these are the bounds of the
targeted gradient tests. Two more sweeps cover the variable-density path
(both adjoints, kept levels) and the reconstruction adjoint of the
constant-density path (sponges with Dirichlet faces).
"""
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import oracle_geometry, small_problem

pytestmark = pytest.mark.gpu


def _cases(n2=16, n3=8, seed=20261204):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n2 + n3):
        ndim = 2 if i < n2 else 3
        order = int(rng.choice([2, 4, 8]))
        R = order // 2
        lo = 2 * R + 8
        if ndim == 2:
            shape = (int(rng.integers(lo, 121)), int(rng.integers(lo, 331)))
        else:
            shape = tuple(int(rng.integers(lo, 49)) for _ in range(3))
        kind = int(rng.integers(0, 3))
        if kind == 0:
            sponge = 0
        elif kind == 1:
            sponge = int(rng.integers(2, max(3, min(shape) // 4)))
        else:
            sponge = [(int(rng.integers(0, max(1, n // 5))), int(rng.integers(0, max(1, n // 5)))) for n in shape]
        nt = int(rng.integers(50, 101))  # the 25 Hz Ricker wavelet peaks at step 40
        case = dict(ndim=ndim, shape=shape, order=order, sponge=sponge, nt=nt,
                    nshot=int(rng.integers(1, 5)), nsrc=int(rng.integers(1, 4)), nrec=int(rng.integers(1, 31)),
                    update=str(rng.choice(["auto", "leapfrog", "summed"])),
                    step_block=int(rng.choice([1, 2])) if ndim == 2 else 1,
                    group_shots=int(rng.choice([0, 0, 2])),
                    ckpt_every=int(rng.choice([0, 1, int(rng.integers(2, nt + 1)), nt])),
                    ckpt_format=str(rng.choice(["fp32", "fp32", "bf16"])), seed=1000 + i)
        out.append(case)
    return out


CASES = _cases()


def _ids(c):
    return (f"{c['ndim']}d-{'x'.join(map(str, c['shape']))}-o{c['order']}-nt{c['nt']}-{c['update']}"
            f"-sb{c['step_block']}-{c['ckpt_format']}")


def _near_sources(rec, src, grid, seed):
    """Receivers moved to within reach of each shot's first source: at most
    0.3 (nt - 35) cells away per axis (waves travel at most 0.45 cells per
    step), inside the interior."""
    rng = np.random.default_rng(seed + 2)
    R = grid.order // 2
    reach = max(3, int(0.3 * (grid.nt - 35)))
    out = src[:, :1, :] + rng.integers(-reach, reach + 1, size=rec.shape)
    hi = np.array(grid.shape) - R - 1
    return np.clip(out, R, hi).astype(np.int32)


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_sweep_matches_oracle(cuda, orc, case):
    from neuralmech_gb300 import misfit_gradient, wave_forward
    grid, v, wav, src, rec = small_problem(shape=case["shape"], nshot=case["nshot"], nsrc=case["nsrc"],
                                           nrec=case["nrec"], nt=case["nt"], order=case["order"],
                                           sponge=case["sponge"], seed=case["seed"],
                                           ckpt_every=case["ckpt_every"], ckpt_format=case["ckpt_format"],
                                           step_block=case["step_block"])
    grid = dataclasses.replace(grid, update=case["update"], group_shots=case["group_shots"])
    rec = _near_sources(rec, src, grid, case["seed"])
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    geo = oracle_geometry(orc, grid, v, wav, src, rec)
    ref = orc.forward(geo)
    traces = wave_forward(*args, grid).cpu().numpy()
    assert np.abs(ref).max() > 0
    assert rel_l2(traces, ref) < 1e-5

    # observed data: the oracle's traces in a 5%-perturbed model
    rng = np.random.default_rng(case["seed"] + 1)
    vt = (v * (1 + 0.05 * rng.standard_normal(v.shape).clip(-2, 2))).astype(np.float32)
    obs = orc.forward(oracle_geometry(orc, grid, vt, wav, src, rec)).astype(np.float32)
    J, g = misfit_gradient(*args, torch.from_numpy(obs).to(cuda), grid)
    Jr, gr, _, _ = orc.gradient(geo, obs)
    assert abs(J.item() - Jr) / Jr < 2e-4
    tol = 2e-4 if case["ckpt_format"] == "fp32" else 5e-3
    err = rel_l2(g.cpu().numpy(), gr)
    print(f"{_ids(case)}: gradient rel L2 {err:.2e}")
    assert err < tol


def _vd_cases(n=8, seed=20261205):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        order = int(rng.choice([2, 4, 8]))
        lo = 2 * (order // 2) + 24  # room for the 10-cell sponge of the builder
        nt = int(rng.integers(60, 131))
        out.append(dict(order=order, shape=(int(rng.integers(lo, 101)), int(rng.integers(lo, 261))), nt=nt,
                        nshot=int(rng.integers(1, 4)), nrec=int(rng.integers(1, 26)),
                        ckpt_every=int(rng.choice([0, int(rng.integers(1, nt + 1))])),
                        ckpt_format=str(rng.choice(["fp32", "fp32", "bf16"])),
                        store_levels=int(rng.choice([0, 10 ** 6])),
                        adjoint="reconstruct" if i % 3 == 2 else "checkpoint", seed=2000 + i))
    return out


VD_CASES = _vd_cases()


def _vd_ids(c):
    return (f"vd-{c['shape'][0]}x{c['shape'][1]}-o{c['order']}-nt{c['nt']}-{c['adjoint']}-{c['ckpt_format']}"
            f"-levels{int(c['store_levels'] > 0)}")


@pytest.mark.parametrize("case", VD_CASES, ids=[_vd_ids(c) for c in VD_CASES])
def test_sweep_variable_density_matches_oracle(cuda, orc, case):
    """The variable-density (kappa, rho) path over random sizes, orders,
    checkpoint intervals and formats, kept levels and both adjoints: traces
    (1e-5), misfit (2e-4) and the kappa, rho and wavelet gradients (1e-4, and
    1e-2 with BF16 checkpoints, the bounds of the targeted tests)."""
    from test_vd_gpu import _geom, _vd_problem
    from neuralmech_gb300.wavefd import vd_forward, vd_misfit_gradient
    grid, kappa, rho, wav, src, rec = _vd_problem(order=case["order"], shape=case["shape"], nshot=case["nshot"],
                                                  nt=case["nt"], seed=case["seed"], ckpt_every=case["ckpt_every"],
                                                  ckpt_format=case["ckpt_format"], nrec=case["nrec"])
    grid = dataclasses.replace(grid, store_levels=case["store_levels"], adjoint=case["adjoint"])
    rec = _near_sources(rec, src, grid, case["seed"])
    geo = _geom(orc, grid, kappa, rho, wav, src, rec)
    t = (torch.from_numpy(kappa).to(cuda), torch.from_numpy(rho).to(cuda), torch.from_numpy(wav).to(cuda),
         torch.from_numpy(src), torch.from_numpy(rec))
    ref = orc.vd_forward(geo)
    assert np.abs(ref).max() > 0
    assert rel_l2(vd_forward(*t, grid).cpu().numpy(), ref) < 1e-5
    obs = orc.vd_forward(dataclasses.replace(geo, kappa=geo.kappa * 1.04)).astype(np.float32)
    J, gk, gr, gw = vd_misfit_gradient(*t, torch.from_numpy(obs).to(cuda), grid, want_wavelet=True)
    Jr, gkr, grr, gwr, _ = orc.vd_gradient(geo, obs)
    e = (rel_l2(gk.cpu().numpy(), gkr), rel_l2(gr.cpu().numpy(), grr), rel_l2(gw.cpu().numpy(), gwr))
    print(f"{_vd_ids(case)}: kappa / rho / wavelet gradient rel L2 {e}")
    assert abs(J.item() - Jr) / Jr < 2e-4
    tol = 1e-2 if case["ckpt_format"] == "bf16" and case["adjoint"] == "checkpoint" else 1e-4
    assert max(e) < tol


def _recon_cases(n=6, seed=20261206):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        order = int(rng.choice([2, 4, 8]))
        lo = 2 * (order // 2) + 8
        kind = int(rng.integers(0, 3))
        shape = (int(rng.integers(lo, 101)), int(rng.integers(lo, 261)))
        sponge = 0 if kind == 0 else (int(rng.integers(3, 13)) if kind == 1 else
                                      [(int(rng.integers(0, 9)), int(rng.integers(0, 9))) for _ in range(2)])
        out.append(dict(order=order, shape=shape, sponge=sponge, nt=int(rng.integers(60, 161)),
                        nshot=int(rng.integers(1, 4)), nrec=int(rng.integers(1, 31)), seed=3000 + i))
    return out


RECON_CASES = _recon_cases()


@pytest.mark.parametrize("case", RECON_CASES,
                         ids=[f"recon-{c['shape'][0]}x{c['shape'][1]}-o{c['order']}-nt{c['nt']}" for c in RECON_CASES])
def test_sweep_reconstruction_adjoint_matches_oracle(cuda, orc, case):
    """The reconstruction adjoint (time reversal, no checkpoints) of the
    constant-density path over random sizes, orders and sponges: misfit
    (2e-4), velocity and wavelet gradients (1e-4 / 2e-4, the targeted test's
    bounds)."""
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=case["shape"], nshot=case["nshot"], nrec=case["nrec"],
                                           nt=case["nt"], order=case["order"], sponge=case["sponge"],
                                           seed=case["seed"])
    grid = dataclasses.replace(grid, adjoint="reconstruct")
    rec = _near_sources(rec, src, grid, case["seed"])
    rng = np.random.default_rng(case["seed"] + 1)
    vt = (v * (1 + 0.05 * rng.standard_normal(v.shape).clip(-2, 2))).astype(np.float32)
    obs = orc.forward(oracle_geometry(orc, grid, vt, wav, src, rec)).astype(np.float32)
    J, gv, gw = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                                torch.from_numpy(rec), torch.from_numpy(obs).to(cuda), grid, want_wavelet=True)
    Jr, gr, gwr, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    e = (rel_l2(gv.cpu().numpy(), gr), rel_l2(gw.cpu().numpy(), gwr))
    print(f"recon {case['shape']} order {case['order']} nt {case['nt']}: gradient / wavelet rel L2 {e}")
    assert abs(J.item() - Jr) / Jr < 2e-4
    assert e[0] < 1e-4 and e[1] < 2e-4
