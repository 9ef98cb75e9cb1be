"""The allocation-free forward entry point, wfd_forward_static.

Callers that cannot allocate device memory use it: a host framework that owns
the whole device pool, a plugin that receives only its input and output
buffers, a loop that cannot afford cudaMalloc's implicit synchronisation. It
runs the same forward as wfd_forward but keeps its scratch in the library's
64 MiB static device array. These tests call it through the C ABI and compare
its traces with those of wfd_forward (workspace from the caller) on two calls
in a row with different inputs, so a call that saw the previous call's leftover
scratch would fail. Tolerance: 1e-6 relative L2 (the same kernels run on the
same inputs; only the scratch address differs). They also check that a call
allocates no device memory, cover 2D and 3D grids, shot groups (which reuse
the array group after group), two steps per launch and int16 field storage,
and read a device-side error back through wfd_forward_static_status.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it.
"""
import ctypes
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import small_problem

pytestmark = pytest.mark.gpu


def _static_forward(call, traces=None):
    """Traces from wfd_forward_static for a prepared call."""
    from neuralmech_gb300 import _lib
    from neuralmech_gb300.wavefd import _ptr, _stream
    lib = _lib.load()
    p = call.problem
    if traces is None:
        traces = torch.full((p.nshot, p.nt, p.nrec), float("nan"), device=call.vel.device)
    gz, gy, gx = call.sponges
    rc = lib.wfd_forward_static(ctypes.byref(p), _ptr(call.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                                _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec), _ptr(traces),
                                _stream())
    _lib.check(rc, "wfd_forward_static")
    torch.cuda.synchronize()
    return traces


def _static_status():
    from neuralmech_gb300 import _lib
    from neuralmech_gb300.wavefd import _stream
    return _lib.load().wfd_forward_static_status(_stream())


def _both(cuda, grid, v, wav, src, rec):
    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300.wavefd import _prepare
    vel = torch.from_numpy(v).to(cuda)
    w = torch.from_numpy(wav).to(cuda)
    ref = wave_forward(vel, w, torch.from_numpy(src), torch.from_numpy(rec), grid)
    got = _static_forward(_prepare(vel, w, torch.from_numpy(src), torch.from_numpy(rec), grid))
    return ref, got


def test_static_forward_matches_workspace_forward(cuda):
    cases = [dict(shape=(64, 200), nshot=3, nt=80, seed=0, order=8),
             dict(shape=(45, 150), nshot=2, nt=60, seed=1, order=4, sponge=6)]
    for kw in cases:  # two calls in a row on different grids and inputs
        ref, got = _both(cuda, *small_problem(**kw))
        assert torch.isfinite(got).all()
        assert np.abs(ref.cpu().numpy()).max() > 0
        assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-6
        assert _static_status() == 0


@pytest.mark.parametrize("kind", ["3d", "groups", "two_step", "i16"])
def test_static_forward_other_paths(cuda, kind):
    """3D, shot groups (the array reused group after group), two steps per
    launch (four field buffers) and int16 field storage: each twice in a row
    against wfd_forward."""
    kw = {"3d": dict(shape=(24, 20, 36), nshot=2, nt=40, order=8, sponge=4),
          "groups": dict(shape=(48, 160), nshot=5, nt=50, order=8),
          "two_step": dict(shape=(50, 170), nshot=3, nt=41, order=8, step_block=2),
          "i16": dict(shape=(50, 170), nshot=2, nt=45, order=4)}[kind]
    for seed in (0, 1):
        grid, v, wav, src, rec = small_problem(seed=seed, **kw)
        if kind == "groups":
            grid = dataclasses.replace(grid, group_shots=2)
        if kind == "i16":
            grid = dataclasses.replace(grid, field_format="i16")
        ref, got = _both(cuda, grid, v, wav, src, rec)
        assert torch.isfinite(got).all()
        assert rel_l2(got.cpu().numpy(), ref.cpu().numpy()) <= 1e-6, (kind, seed)
        assert _static_status() == 0


def test_static_forward_allocates_nothing(cuda):
    """Once the kernels of a problem have run (lazy module loading may take
    device memory at a kernel's first launch), a further call changes neither
    the device's free memory nor PyTorch's reserved pool."""
    from neuralmech_gb300.wavefd import _prepare
    grid, v, wav, src, rec = small_problem(shape=(64, 200), nshot=3, nt=80, seed=4)
    call = _prepare(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                    torch.from_numpy(rec), grid)
    traces = torch.empty((3, 80, rec.shape[-2]), device=cuda)
    _static_forward(call, traces)  # warm-up
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    first = traces.clone()
    _static_forward(call, traces)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_reserved() == reserved0
    assert torch.equal(first, traces)


def test_static_forward_reports_device_errors(cuda):
    """A receiver outside the interior is refused on the device (its samples
    are not written); the call itself returns 0 and the status accessor
    reports WFD_ERR_POSITION once, then 0."""
    from neuralmech_gb300 import _lib
    from neuralmech_gb300.wavefd import _prepare
    grid, v, wav, src, rec = small_problem(shape=(48, 150), nshot=2, nt=30, seed=3)
    rec = rec.copy()
    rec[1, 2] = [1, 70]  # inside the grid, inside the fixed ring of 4 cells
    call = _prepare(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                    torch.from_numpy(rec), grid)
    assert _static_status() == 0
    _static_forward(call)
    assert _static_status() == _lib.WFD_ERR_POSITION
    assert _static_status() == 0


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
