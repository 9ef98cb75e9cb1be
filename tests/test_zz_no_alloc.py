"""The allocation-free forward entry point, wfd_forward_static.

Callers that cannot allocate device memory use it: a host framework that owns
the whole device pool, a plugin that receives only its input and output
buffers, a loop that cannot afford cudaMalloc's implicit synchronisation. It
runs the same forward as wfd_forward but keeps its scratch in the library's
64 MiB static device array. These tests call it through the C ABI and compare
its traces with those of wfd_forward (workspace from the caller) on two calls
in a row with different inputs, so a call that saw the previous call's leftover
scratch would fail. Tolerance: 1e-6 relative L2 (the same kernels run on the
same inputs; only the scratch address differs).

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import small_problem

pytestmark = pytest.mark.gpu


def _static_forward(call):
    """Traces from wfd_forward_static for a prepared call."""
    from neuralmech_gb300 import _lib
    from neuralmech_gb300.wavefd import _ptr, _stream
    lib = _lib.load()
    p = call.problem
    traces = torch.full((p.nshot, p.nt, p.nrec), float("nan"), device=call.vel.device)
    gz, gy, gx = call.sponges
    rc = lib.wfd_forward_static(ctypes.byref(p), _ptr(call.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                                _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec), _ptr(traces),
                                _stream())
    _lib.check(rc, "wfd_forward_static")
    torch.cuda.synchronize()
    return traces


def test_static_forward_matches_workspace_forward(cuda):
    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300.wavefd import _prepare
    cases = [dict(shape=(64, 200), nshot=3, nt=80, seed=0, order=8),
             dict(shape=(45, 150), nshot=2, nt=60, seed=1, order=4, sponge=6)]
    for kw in cases:  # two calls in a row on different grids and inputs
        grid, v, wav, src, rec = small_problem(**kw)
        vel = torch.from_numpy(v).to(cuda)
        w = torch.from_numpy(wav).to(cuda)
        ref = wave_forward(vel, w, torch.from_numpy(src), torch.from_numpy(rec), grid)
        got = _static_forward(_prepare(vel, w, torch.from_numpy(src), torch.from_numpy(rec), grid))
        assert torch.isfinite(got).all()
        assert np.abs(ref.cpu().numpy()).max() > 0
        assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-6


def test_static_forward_rejects_oversized_problem(cuda):
    from neuralmech_gb300 import Grid, _lib
    from neuralmech_gb300.wavefd import _prepare
    grid = Grid((4096, 4096), (10.0, 10.0), 1e-3, 4)  # 2 x 64 MiB of wavefields alone
    vel = torch.full((4096, 4096), 2000.0, device=cuda)
    call = _prepare(vel, torch.zeros(4, device=cuda), [[10, 10]], [[10, 20]], grid)
    lib = _lib.load()
    from neuralmech_gb300.wavefd import _ptr, _stream
    rc = lib.wfd_forward_static(ctypes.byref(call.problem), _ptr(call.vel), None, None, None,
                                _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec), None, _stream())
    assert rc == _lib.WFD_ERR_WORKSPACE
    assert "64 MiB" in lib.wfd_last_error().decode()
