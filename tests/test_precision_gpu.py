"""Precision at the benchmark's scale: the fwi1024 grid and time axis
(1024 x 1024, 2000 steps, order 8, 20-cell sponge, checkpoints every 45) for
two of its 64 shots, against the FP64 oracle.

* Forward traces: 1e-5 relative L2 (the trace tolerance of this path against
  the reference solver).
* Gradient: 1e-3 relative L2, the bound on the FWI gradient against an FP64
  oracle. On this workload the residuals are about 1.1e-4 of the traces (the
  2000-step record ends before the deep reflections return), so the gradient
  sees the FP32 trace error magnified about 10^4 times. The leapfrog update
  u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1} puts the rounding of two stored
  levels of size |u| into the velocity u_n - u_{n-1} at every step; its
  gradient misses the bound (about 4.4e-3, asserted here as a documented
  miss). The summed form of the same recursion (state u_n and the increment
  d_n, the default for the forward of a gradient) keeps the increment's own
  rounding and meets it, with FP32, BF16 and int16 checkpoints alike: every
  segment but the last is recomputed from a checkpoint here (store_levels 0).
  The benchmark's configuration, two steps per launch (whose summed kernel
  forms L u in the centre-weight form), meets it too (4.7e-4), and so it does
  with every level kept in block floating point (level_format "bfp16").
"""
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import oracle_geometry

pytestmark = pytest.mark.gpu


def test_fwi1024_two_shots_against_fp64(cuda, orc):
    from neuralmech_gb300 import misfit_gradient, synth, wave_forward
    w = synth.workload("fwi1024")
    sel = [0, 63]
    src, rec = w.src[sel], w.rec[sel]
    wav = np.repeat(w.wavelet[None], 2, 0).astype(np.float32)
    g = w.grid
    assert g.store_levels == 0 and g.update == "auto"
    obs = orc.forward(oracle_geometry(orc, g, w.vel_true, wav[:, :, None], src, rec)).astype(np.float32)
    geo = oracle_geometry(orc, g, w.vel, wav[:, :, None], src, rec)
    Jr, gr, _, tr_ref = orc.gradient(geo, obs)
    args = (torch.from_numpy(w.vel).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    e_tr = {}
    for form in ("leapfrog", "summed"):
        tr = wave_forward(*args, dataclasses.replace(g, update=form)).cpu().numpy()
        e_tr[form] = rel_l2(tr, tr_ref)
    errs, e_J = {}, {}
    for form, fmt, sb in (("auto", "fp32", 1), ("auto", "i16", 1), ("auto", "bf16", 1), ("auto", "bf16", 2),
                          ("leapfrog", "bf16", 1)):
        J, gv = misfit_gradient(*args, torch.from_numpy(obs).to(cuda),
                                dataclasses.replace(g, ckpt_format=fmt, update=form, step_block=sb))
        key = (form, fmt) if sb == 1 else (form, fmt, "two steps per launch")
        errs[key] = rel_l2(gv.cpu().numpy(), gr)
        e_J[key] = abs(float(J) - Jr) / Jr
    # every level kept in block floating point (level_format "bfp16"): no
    # segment recomputed, the adjoint's u_k rounded to 2^-15 of their 4-cell block
    key = ("auto", "bf16", "two steps per launch", "bfp16 levels")
    J, gv = misfit_gradient(*args, torch.from_numpy(obs).to(cuda),
                            dataclasses.replace(g, ckpt_format="bf16", step_block=2, store_levels=10 ** 6,
                                                level_format="bfp16"))
    errs[key] = rel_l2(gv.cpu().numpy(), gr)
    e_J[key] = abs(float(J) - Jr) / Jr
    print(f"fwi1024 (2 shots): traces rel L2 {e_tr}; gradient rel L2 {errs}; misfit rel {e_J}")
    assert e_tr["leapfrog"] < 1e-5 and e_tr["summed"] < 1e-5
    assert e_tr["summed"] < 0.5 * e_tr["leapfrog"]
    for key in (("auto", "fp32"), ("auto", "i16"), ("auto", "bf16"), ("auto", "bf16", "two steps per launch"),
                ("auto", "bf16", "two steps per launch", "bfp16 levels")):
        assert errs[key] <= 1e-3, key
        assert e_J[key] <= 5e-3, key
    # the leapfrog form's floor: the documented miss of the 1e-3 bound
    assert 1e-3 < errs[("leapfrog", "bf16")] < 1e-2
