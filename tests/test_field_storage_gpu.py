"""Reduced-precision field storage (a forward-only mode of the 2D wave path):
FP16 and block-scaled int16 levels with FP32 arithmetic, against the FP32
forward on the same problem. The error is measured as the reference measures
its mixed and scaled steps (2D_wave_cuda_scaled.py:121-126: relative L2 to
single precision), on the traces and on the final wavefield."""
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import small_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("order", [2, 4, 8])
def test_forward_storage_error(cuda, order):
    from neuralmech_gb300.wavefd import wave_forward, wave_forward_final
    grid, v, wav, src, rec = small_problem(shape=(90, 270), nshot=3, nt=160, order=order, nsrc=2,
                                           nrec=30, seed=31)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    t32, u32 = wave_forward_final(*args, grid)
    errs = {}
    for fmt in ("fp16", "i16"):
        g = dataclasses.replace(grid, field_format=fmt)
        t, u = wave_forward_final(*args, g)
        assert torch.equal(t, wave_forward(*args, g))  # the traces-only call is the same computation
        errs[fmt] = (rel_l2(t.cpu().numpy(), t32.cpu().numpy()), rel_l2(u.cpu().numpy(), u32.cpu().numpy()))
    print(f"order {order}: relative L2 to FP32 (traces, final field): {errs}")
    assert errs["fp16"][0] < 2e-2 and errs["fp16"][1] < 2e-2
    assert errs["i16"][0] < 2e-3 and errs["i16"][1] < 2e-3
    assert errs["i16"][0] < errs["fp16"][0]


def test_reduced_precision_is_forward_only(cuda):
    from neuralmech_gb300 import misfit_gradient
    from neuralmech_gb300._lib import WaveFDError
    from neuralmech_gb300.wavefd import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(40, 130), nshot=1, nt=30, seed=2)
    g = dataclasses.replace(grid, field_format="fp16")
    vel = torch.from_numpy(v).to(cuda).requires_grad_(True)
    with pytest.raises(ValueError):
        wave_forward(vel, torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec), g)
    obs = torch.zeros((1, 30, rec.shape[1]), device=cuda)
    with pytest.raises(WaveFDError):
        misfit_gradient(vel.detach(), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                        torch.from_numpy(rec), obs, g)
