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
targeted gradient tests.
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
