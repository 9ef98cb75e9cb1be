"""The reference's own step kernels (projects/18_simple_wave_fd/step2D_wave.cu),
compiled from its sources for sm_103a and run on the GPU (oracle/ref_gpu.cpp),
against this library's drop-ins on the same inputs:

  * built with IEEE division and no fused multiply-adds (the arithmetic of
    the expression as written, operation by operation), padded_step,
    shared_step, basic_step, coalesced_step, mixed_step, scaled_step and
    temporal_step give the same bits as wfd_step2d_exact, wfd_step2d_mixed,
    wfd_step2d_scaled and wfd_temporal_step;
  * built with --use_fast_math, as the reference's drivers build them,
    padded_step and temporal_step agree with wfd_step2d_order2 and
    wfd_temporal_step_fast to 1e-5 relative L2 (approximate division and
    contracted products against the IEEE or pre-divided forms), mixed_step
    with wfd_step2d_mixed and wfd_step2d_mixed_fast to 2e-3 (FP16 storage: a
    different rounding of one value moves it by an FP16 ulp).

Skipped where the module files were not built (they need the reference
sources at build time)."""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    from oracle import ref as r
    if not r.gpu_available():
        pytest.skip("the reference's GPU module is not built here")
    return r


def _pulse(N, M, Mp, dev):
    """The drivers' Gaussian initial condition on [0, 1] x [0, 2] (FP32)."""
    x = torch.linspace(0, 1, N, device=dev)[:, None]
    y = torch.linspace(0, 2, M, device=dev)[None, :]
    u = torch.zeros((N, Mp), device=dev)
    u[:, :M] = torch.exp(-(x - 0.4) ** 2 / (2 * 0.05 ** 2)) * torch.exp(-(y - 0.7) ** 2 / (2 * 0.05 ** 2))
    dx, dy = 1.0 / (N - 1), 2.0 / (M - 1)
    dt = 0.95 * min(dx, dy) / math.sqrt(2)
    args = (1.0, float(np.float32(dt)), float(np.float32(dx)), float(np.float32(dy)))
    return u, args


def _run(step, u, args, N, M, n):
    a, b = u.clone(), u.clone()
    for _ in range(n):  # the drivers' rotation: u0 = step(u0, u1, u0); swap
        a = step(a, b, a, *args, N, M)
        a, b = b, a
    return b


@pytest.mark.parametrize("N,M,Mp", [(300, 700, 704), (129, 333, 352)])
def test_padded_and_shared_step_bitwise(cuda, ref, N, M, Mp):
    from neuralmech_gb300.wavefd import step2d_exact
    u, args = _pulse(N, M, Mp, cuda)
    ref.MODE["build"] = "ieee"
    mine = _run(step2d_exact, u, args, N, M, 20)
    for fn in (ref.padded_step_gpu, ref.shared_step_gpu):
        theirs = _run(fn, u, args, N, M, 20)
        assert torch.equal(mine, theirs), fn.__name__


def test_basic_and_coalesced_step_bitwise(cuda, ref):
    from neuralmech_gb300.wavefd import step2d_exact
    N, M = 201, 333  # unpadded rows: M_padded = M, odd
    u, args = _pulse(N, M, M, cuda)
    ref.MODE["build"] = "ieee"
    mine = _run(step2d_exact, u, args, N, M, 15)
    for fn in (ref.basic_step_gpu, ref.coalesced_step_gpu):
        assert torch.equal(mine, _run(fn, u, args, N, M, 15)), fn.__name__


def test_mixed_step_bitwise_and_fast(cuda, ref):
    from neuralmech_gb300.wavefd import step2d_mixed
    N, M, Mp = 300, 701, 704
    u, args = _pulse(N, M, Mp, cuda)
    h = u.half()
    ref.MODE["build"] = "ieee"
    mine = _run(step2d_mixed, h, args, N, M, 20)
    assert torch.equal(mine, _run(ref.mixed_step_gpu, h, args, N, M, 20))
    ref.MODE["build"] = "fast"
    fast = _run(ref.mixed_step_gpu, h, args, N, M, 20)
    assert rel_l2(mine.float().cpu().numpy(), fast.float().cpu().numpy()) < 2e-3
    from neuralmech_gb300.wavefd import step2d_mixed_fast
    mine_fast = _run(step2d_mixed_fast, h, args, N, M, 20)
    assert rel_l2(mine_fast.float().cpu().numpy(), fast.float().cpu().numpy()) < 2e-3


def test_scaled_step_bitwise(cuda, ref):
    """scaled_step (int16 + one FP32 scale per 32 values, warp shuffles) run
    from the reference's source, against wfd_step2d_scaled, over 20 steps."""
    from neuralmech_gb300.wavefd import step2d_scaled
    from oracle.numpy_ref import scaled_encode
    N, M, Mp = 300, 700, 704  # M_padded a multiple of 64 (whole warps of pairs)
    u, args = _pulse(N, M, Mp, cuda)
    q, s = scaled_encode(u.cpu().numpy())
    lv = lambda: [torch.from_numpy(q.copy()).to(cuda), torch.from_numpy(s.copy()).to(cuda)]
    ref.MODE["build"] = "ieee"
    out = {}
    for name in ("mine", "ref"):
        a, b = lv(), lv()
        for _ in range(20):
            if name == "mine":
                step2d_scaled(a[0], a[1], b[0], b[1], a[0], a[1], *args, N, M)
            else:
                ref.scaled_step_gpu(a[0], a[1], b[0], b[1], a[0], a[1], *args, N, M)
            a, b = b, a
        out[name] = b
    assert torch.equal(out["mine"][0], out["ref"][0])
    assert torch.equal(out["mine"][1], out["ref"][1])


@pytest.mark.parametrize("N,M,Mp", [(500, 1000, 1024), (77, 301, 320)])
def test_temporal_step_bitwise_and_fast(cuda, ref, N, M, Mp):
    from neuralmech_gb300.wavefd import temporal_step, temporal_step_fast
    u, args = _pulse(N, M, Mp, cuda)
    out = {}
    for name, fn, build in (("mine", temporal_step, None), ("fast", temporal_step_fast, None),
                            ("ref_ieee", ref.temporal_step_gpu, "ieee"), ("ref_fast", ref.temporal_step_gpu, "fast")):
        if build:
            ref.MODE["build"] = build
        a0, a1 = u.clone(), u.clone()
        b0, b1 = torch.zeros_like(u), torch.zeros_like(u)
        for k in range(3):  # the driver's two pairs of arrays, swapped every launch
            fn(a0, a1, b0, b1, *args, N, M)
            a0, a1, b0, b1 = b0, b1, a0, a1
        out[name] = a1
    assert torch.equal(out["mine"], out["ref_ieee"])
    assert rel_l2(out["ref_fast"][:, :M].cpu().numpy(), out["mine"][:, :M].cpu().numpy()) < 1e-5
    assert rel_l2(out["fast"][:, :M].cpu().numpy(), out["mine"][:, :M].cpu().numpy()) < 1e-5


def test_padded_step_fast_math_against_order2(cuda, ref):
    """padded_step as the drivers build it (--use_fast_math) against the
    generic kernel's drop-in (pre-divided weights): 1e-5 over 40 steps."""
    from neuralmech_gb300 import step2d_order2
    N, M, Mp = 400, 900, 928
    u, args = _pulse(N, M, Mp, cuda)
    ref.MODE["build"] = "fast"
    theirs = _run(ref.padded_step_gpu, u, args, N, M, 40)
    mine = _run(step2d_order2, u, args, N, M, 40)
    assert rel_l2(mine[:, :M].cpu().numpy(), theirs[:, :M].cpu().numpy()) < 1e-5
