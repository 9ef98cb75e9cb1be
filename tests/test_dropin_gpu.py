"""GPU parity of the reduced-precision and 1D drop-ins (through the C ABI)
against golden vectors of the reference kernels:
  * wfd_step2d_mixed vs mixed_step (FP16 storage), and
  * wfd_step1d vs step1D, golden vectors from the reference sources built for
    the CPU (tests/golden/make_golden.py): value for value, both being IEEE
    evaluations of the reference's expression in its operation order;
  * wfd_step2d_scaled vs the NumPy restatement of scaled_step (int16 + one
    FP32 scale per 32 values): value for value.
Then the storage error after many steps against the FP32 step, measured as
2D_wave_cuda_scaled.py:121-126 measures it (relative L2 to single precision).
"""
import math
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, ROOT, rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(ROOT, "tests", "golden")


def _params(p):
    N, M, MP, steps = (int(v) for v in p[:4])
    c, dt, dx, dy = (float(np.float32(v)) for v in p[4:])
    return N, M, MP, steps, c, dt, dx, dy


@pytest.mark.parametrize("case", [0, 1])
def test_mixed_step_golden(cuda, case):
    from neuralmech_gb300.wavefd import step2d_mixed
    g = np.load(os.path.join(GOLDEN, "mixed_step.npz"))
    N, M, MP, steps, c, dt, dx, dy = _params(g[f"c{case}_params"])
    a = torch.from_numpy(g[f"c{case}_u0"]).to(cuda)
    b = a.clone()
    for t in range(steps):
        a = step2d_mixed(a, b, a, c, dt, dx, dy, N, M)  # in place, as 2D_wave_cuda_mixed.py
        a, b = b, a
        key = f"c{case}_step{t}"
        if key in g.files:
            got = b.cpu().numpy()
            assert np.array_equal(got.view(np.uint16), g[key].view(np.uint16)), (t, np.abs(got.astype(np.float32) - g[key].astype(np.float32)).max())


@pytest.mark.parametrize("case", [0, 1])
def test_scaled_step_golden(cuda, case):
    from neuralmech_gb300.wavefd import step2d_scaled
    g = np.load(os.path.join(GOLDEN, "scaled_step.npz"))
    N, M, MP, steps, c, dt, dx, dy = _params(g[f"c{case}_params"])
    q = torch.from_numpy(g[f"c{case}_q0"]).to(cuda)
    s = torch.from_numpy(g[f"c{case}_s0"]).to(cuda)
    a, b = (q, s), (q.clone(), s.clone())
    for t in range(steps):
        a = step2d_scaled(a[0], a[1], b[0], b[1], a[0], a[1], c, dt, dx, dy, N, M)
        a, b = b, a
        key = f"c{case}_step{t}"
        if key + "_q" in g.files:
            assert np.array_equal(b[0].cpu().numpy(), g[key + "_q"]), t
            assert np.array_equal(b[1].cpu().numpy(), g[key + "_s"]), t


def test_step1d_golden(cuda):
    from neuralmech_gb300.wavefd import step1d
    g = np.load(os.path.join(GOLDEN, "step1d.npz"))
    N, c, dt, dx = g["params"]
    c, dt, dx = (float(np.float32(v)) for v in (c, dt, dx))
    a = torch.from_numpy(g["u0"]).to(cuda)
    b = a.clone()
    for t in range(25):
        a = step1d(a, b, a, c, dt, dx)
        a, b = b, a
        if f"step{t}" in g.files:
            assert np.array_equal(b.cpu().numpy(), g[f"step{t}"]), t


def test_storage_error_against_fp32(cuda):
    """FP16 and block-int16 storage against the FP32 step after 100 / 400 steps
    of a Gaussian pulse (the reference's measurement, 2D_wave_cuda_scaled.py:121-126)."""
    from neuralmech_gb300.wavefd import step2d_mixed, step2d_order2, step2d_scaled
    from oracle import numpy_ref as nr
    N, M, MP = 256, 250, 256
    dx, dy = 1.0 / (N - 1), 1.0 / (M - 1)
    c = 1.0
    dt = float(np.float32(0.95 * min(dx, dy) / c / math.sqrt(2)))
    x = np.linspace(0, 1, N)[:, None]
    y = np.linspace(0, 1, M)[None, :]
    u = np.zeros((N, MP), np.float32)
    u[:, :M] = np.exp(-((x - 0.4) ** 2 + (y - 0.55) ** 2) / (2 * 0.05**2))
    u[0] = u[-1] = 0
    u[:, 0] = 0
    u[:, M - 1:] = 0
    f = [torch.from_numpy(u).to(cuda), torch.from_numpy(u).to(cuda)]
    h = [torch.from_numpy(u.astype(np.float16)).to(cuda) for _ in range(2)]
    q, s = nr.scaled_encode(u)
    qs = [(torch.from_numpy(q).to(cuda), torch.from_numpy(s).to(cuda)) for _ in range(2)]
    errs = {}
    for t in range(400):
        f[0] = step2d_order2(f[0], f[1], f[0], c, dt, dx, dy, N, M)
        h[0] = step2d_mixed(h[0], h[1], h[0], c, dt, dx, dy, N, M)
        qs[0] = step2d_scaled(qs[0][0], qs[0][1], qs[1][0], qs[1][1], qs[0][0], qs[0][1], c, dt, dx, dy, N, M)
        f.reverse(), h.reverse(), qs.reverse()
        if t + 1 in (100, 400):
            ref = f[1][:, :M].double()
            dec = (qs[1][1].repeat_interleave(32, dim=1) * qs[1][0].float())[:, :M].double()
            errs[t + 1] = (float((h[1][:, :M].double() - ref).norm() / ref.norm()),
                           float((dec - ref).norm() / ref.norm()))
    print("relative L2 to FP32 (fp16, int16) after 100 / 400 steps:", errs)
    for fp16, int16 in errs.values():
        assert fp16 < 2e-2 and int16 < 2e-3
        assert int16 < fp16


def test_temporal_step_matches_golden_bitwise(cuda):
    """wfd_temporal_step: one launch = eight padded_step updates, two launches
    = sixteen; v0 = u_{n+7}, v1 = u_{n+8} equal the reference's host build bit
    for bit on every written cell, and the padding columns stay untouched."""
    from neuralmech_gb300.wavefd import temporal_step
    g = np.load(os.path.join(GOLDEN, "temporal_step.npz"))
    for ci in range(3):
        N, M, MP, c, dt, dx, dy = g[f"c{ci}_params"]
        N, M = int(N), int(M)
        args = (float(np.float32(c)), float(np.float32(dt)), float(np.float32(dx)), float(np.float32(dy)), N, M)
        u0 = torch.from_numpy(g[f"c{ci}_u0"]).to(cuda)
        u1 = torch.from_numpy(g[f"c{ci}_u1"]).to(cuda)
        v0 = torch.full_like(u0, 7.0)
        v1 = torch.full_like(u0, 7.0)
        temporal_step(u0, u1, v0, v1, *args)
        if f"c{ci}_after8_v0" in g:
            assert np.array_equal(v0.cpu().numpy()[:, :M], g[f"c{ci}_after8_v0"][:, :M]), ci
            assert np.array_equal(v1.cpu().numpy()[:, :M], g[f"c{ci}_after8_v1"][:, :M]), ci
            assert torch.all(v0[:, M:] == 7.0) and torch.all(v1[:, M:] == 7.0)
        w0, w1 = torch.empty_like(u0), torch.empty_like(u0)
        temporal_step(v0, v1, w0, w1, *args)
        assert np.array_equal(w0.cpu().numpy()[:, :M], g[f"c{ci}_after16_v0"][:, :M]), ci
        assert np.array_equal(w1.cpu().numpy()[:, :M], g[f"c{ci}_after16_v1"][:, :M]), ci


def test_step2d_exact_matches_padded_step_bitwise(cuda):
    """wfd_step2d_exact with M_padded: padded_step's host build value for value
    over the golden runs (in-place rotation), padding columns untouched."""
    from neuralmech_gb300.wavefd import step2d_exact
    g = np.load(os.path.join(GOLDEN, "padded_step.npz"))
    for ci in range(2):
        N, M, MP, steps, c, dt, dx, dy = g[f"c{ci}_params"]
        N, M, steps = int(N), int(M), int(steps)
        a = torch.from_numpy(g[f"c{ci}_u0"]).to(cuda)
        b = torch.from_numpy(g[f"c{ci}_u1"]).to(cuda)
        for t in range(steps):
            a = step2d_exact(a, b, a, float(np.float32(c)), float(np.float32(dt)), float(np.float32(dx)),
                             float(np.float32(dy)), N, M)
            a, b = b, a
            if f"c{ci}_step{t}" in g:
                assert np.array_equal(b.cpu().numpy(), g[f"c{ci}_step{t}"]), (ci, t)


def test_step2d_exact_matches_basic_and_coalesced_step(cuda):
    """Unpadded rows (M_padded = M, odd M: rows not 16-byte aligned):
    basic_step's and coalesced_step's host builds value for value."""
    from neuralmech_gb300.wavefd import step2d_exact
    g = np.load(os.path.join(GOLDEN, "basic_step.npz"))
    for ci in range(2):
        N, M, steps, c, dt, dx, dy = g[f"c{ci}_params"]
        N, M, steps = int(N), int(M), int(steps)
        a = torch.from_numpy(g[f"c{ci}_u0"]).to(cuda)
        b = a.clone()
        for _ in range(steps):
            a = step2d_exact(a, b, a, float(np.float32(c)), float(np.float32(dt)), float(np.float32(dx)),
                             float(np.float32(dy)), N, M)
            a, b = b, a
        got = b.cpu().numpy()
        assert np.array_equal(got, g[f"c{ci}_basic_last"]) and np.array_equal(got, g[f"c{ci}_coalesced_last"])


def test_temporal_step_many_tiles_bitwise(cuda):
    """A grid of several CTA waves (1000 x 3000): two launches equal sixteen
    padded_step updates restated in PyTorch FP32 (one rounded operation per
    term, the kernel's order), value for value."""
    from neuralmech_gb300.wavefd import temporal_step
    N, M = 1000, 3000
    Mp = (M + 31) // 32 * 32
    f = np.float32
    dx, dy = f(1.0 / (N - 1)), f(2.0 / (M - 1))
    dt = f(0.95 * min(dx, dy) / math.sqrt(2))
    k = torch.tensor(dt * dt * f(1.0) * f(1.0), device=cuda)
    dx2, dy2 = torch.tensor(dx * dx, device=cuda), torch.tensor(dy * dy, device=cuda)
    g = torch.Generator(device="cpu").manual_seed(5)
    u0 = torch.zeros((N, Mp))
    u0[:, :M] = torch.rand((N, M), generator=g) - 0.5
    u1 = u0.clone()
    u1[:, :M] += 0.01 * (torch.rand((N, M), generator=g) - 0.5)
    u0, u1 = u0.to(cuda), u1.to(cuda)

    def padded(a, b):  # the in-place padded_step update of a from b
        c = b[1:-1, 1:M - 1]
        two = 2.0 * c
        li = (b[:-2, 1:M - 1] - two) + b[2:, 1:M - 1]
        lj = (b[1:-1, :M - 2] - two) + b[1:-1, 2:M]
        a[1:-1, 1:M - 1] = (-a[1:-1, 1:M - 1] + two) + k * (li / dx2 + lj / dy2)
        return a

    a, b = u0.clone(), u1.clone()
    for _ in range(16):
        a = padded(a, b)
        a, b = b, a
    v0, v1 = torch.empty_like(u0), torch.empty_like(u0)
    w0, w1 = torch.empty_like(u0), torch.empty_like(u0)
    args = (1.0, float(dt), float(dx), float(dy), N, M)
    temporal_step(u0, u1, v0, v1, *args)
    temporal_step(v0, v1, w0, w1, *args)
    assert torch.equal(w0[:, :M], a[:, :M]) and torch.equal(w1[:, :M], b[:, :M])


@pytest.mark.parametrize("N,M,Mp", [(3, 3, 4), (5, 7, 8), (9, 150, 152), (40, 145, 148)])
def test_temporal_step_equals_eight_exact_steps(cuda, N, M, Mp):
    """Small and ragged grids (one interior cell, grids smaller than the
    staged window, M not a multiple of the tile): one temporal_step launch
    equals eight step2d_exact launches value for value, boundary included."""
    from neuralmech_gb300.wavefd import step2d_exact, temporal_step
    g = torch.Generator(device="cpu").manual_seed(N * 1000 + M)
    u0 = torch.zeros((N, Mp))
    u0[:, :M] = torch.rand((N, M), generator=g) - 0.5
    u1 = u0.clone()
    u1[:, :M] += 0.05 * (torch.rand((N, M), generator=g) - 0.5)
    u0, u1 = u0.to(cuda), u1.to(cuda)
    args = (1.0, 0.004, 0.01, 0.012, N, M)
    a, b = u0.clone(), u1.clone()
    for _ in range(8):
        a = step2d_exact(a, b, a, *args)
        a, b = b, a
    v0, v1 = torch.full_like(u0, 3.0), torch.full_like(u0, 3.0)
    temporal_step(u0, u1, v0, v1, *args)
    assert torch.equal(v0[:, :M], a[:, :M]) and torch.equal(v1[:, :M], b[:, :M])
    assert torch.all(v0[:, M:] == 3.0) and torch.all(v1[:, M:] == 3.0)


def test_step2d_exact_single_interior_cell(cuda):
    """N = M = 3: exactly one updated cell, equal to the expression in FP32."""
    from neuralmech_gb300.wavefd import step2d_exact
    f = np.float32
    u0 = np.arange(12, dtype=f).reshape(3, 4) / f(7)
    u1 = (np.arange(12, dtype=f).reshape(3, 4) ** 2) / f(50)
    args = (1.0, 0.004, 0.01, 0.012, 3, 3)
    got = step2d_exact(torch.from_numpy(u0).to(cuda), torch.from_numpy(u1).to(cuda),
                       torch.from_numpy(u0.copy()).to(cuda), *args).cpu().numpy()
    k = f(0.004) * f(0.004) * f(1.0) * f(1.0)
    two = f(2) * u1[1, 1]
    li = (u1[0, 1] - two) + u1[2, 1]
    lj = (u1[1, 0] - two) + u1[1, 2]
    want = (-u0[1, 1] + two) + k * (li / (f(0.01) * f(0.01)) + lj / (f(0.012) * f(0.012)))
    expect = u0.copy()
    expect[1, 1] = want
    assert np.array_equal(got, expect)


def test_temporal_step_rejects_overlapping_outputs(cuda):
    from neuralmech_gb300 import _lib
    from neuralmech_gb300.wavefd import temporal_step
    u = torch.zeros((20, 64), device=cuda)
    with pytest.raises(_lib.WaveFDError):
        temporal_step(u, u.clone(), u, torch.zeros_like(u), 1.0, 1e-3, 0.1, 0.1, 20, 60)



@pytest.mark.parametrize("N,M,Mp", [(3, 3, 4), (5, 7, 8), (9, 150, 152), (40, 145, 148), (77, 301, 304),
                                    (700, 1500, 1504)])
def test_temporal_step_fast_tracks_exact(cuda, N, M, Mp):
    """wfd_temporal_step_fast (pre-divided weights, the window in registers):
    within 1e-6 relative L2 of the exact drop-in after three launches, on
    grids smaller than one window (boundary path only), ragged edges and
    several waves of interior windows; the padding columns stay untouched.
    On unpadded rows (M_padded = M, which the exact drop-in does not take) it
    gives the same values as on the padded ones."""
    from neuralmech_gb300.wavefd import temporal_step, temporal_step_fast
    g = torch.Generator(device="cpu").manual_seed(N * 7 + M)
    x = torch.linspace(0, 1, N)[:, None]
    y = torch.linspace(0, 2, M)[None, :]
    u = torch.zeros((N, Mp))
    u[:, :M] = torch.exp(-((x - 0.45) ** 2 + (y - 0.8) ** 2) / (2 * 0.1 ** 2)) + \
        0.01 * (torch.rand((N, M), generator=g) - 0.5)
    u = u.to(cuda)
    dx, dy = 1.0 / max(N - 1, 1), 2.0 / max(M - 1, 1)
    args = (1.0, 0.9 * min(dx, dy) / math.sqrt(2), dx, dy, N, M)
    out = {}
    for name, fn in (("exact", temporal_step), ("fast", temporal_step_fast)):
        a0, a1 = u.clone(), (u * 0.999).clone()
        b0, b1 = torch.full_like(u, 3.0), torch.full_like(u, 3.0)
        for _ in range(3):
            fn(a0, a1, b0, b1, *args)
            a0, a1, b0, b1 = b0, b1, a0, a1
        out[name] = (a0, a1)
    for lev in (0, 1):
        e, f = out["exact"][lev], out["fast"][lev]
        assert torch.isfinite(f).all()
        assert rel_l2(f[:, :M].cpu().numpy(), e[:, :M].cpu().numpy()) < 1e-6
        assert torch.equal(f[:, M:], e[:, M:])
        # the fixed boundary keeps its values exactly
        assert torch.equal(f[0, :M], e[0, :M]) and torch.equal(f[-1, :M], e[-1, :M])
        assert torch.equal(f[:, 0], e[:, 0]) and torch.equal(f[:, M - 1], e[:, M - 1])
    a0, a1 = u[:, :M].contiguous(), (u * 0.999)[:, :M].contiguous()
    b0, b1 = torch.zeros_like(a0), torch.zeros_like(a0)
    for _ in range(3):  # the fast form on unpadded rows: the same values
        temporal_step_fast(a0, a1, b0, b1, *args)
        a0, a1, b0, b1 = b0, b1, a0, a1
    assert torch.equal(a1, out["fast"][1][:, :M]) and torch.equal(a0, out["fast"][0][:, :M])


@pytest.mark.parametrize("N,M,Mp", [(3, 3, 8), (9, 150, 152), (300, 701, 704), (257, 1024, 1032)])
def test_mixed_fast_tracks_exact(cuda, N, M, Mp):
    """wfd_step2d_mixed_fast (pre-divided weights, 8 values per thread) against
    the value-for-value FP16 drop-in over 30 in-place steps: within 2e-3
    relative L2 (an FP16 rounding here and there), the boundary and the
    padding untouched."""
    from neuralmech_gb300.wavefd import step2d_mixed, step2d_mixed_fast
    x = torch.linspace(0, 1, N)[:, None]
    y = torch.linspace(0, 2, M)[None, :]
    u = torch.zeros((N, Mp))
    u[:, :M] = torch.exp(-((x - 0.45) ** 2 + (y - 0.8) ** 2) / (2 * 0.1 ** 2))
    u = u.half().to(cuda)
    dx, dy = 1.0 / max(N - 1, 1), 2.0 / max(M - 1, 1)
    args = (1.0, 0.9 * min(dx, dy) / math.sqrt(2), dx, dy, N, M)
    out = {}
    for name, fn in (("exact", step2d_mixed), ("fast", step2d_mixed_fast)):
        a, b = u.clone(), (u * 0.999).clone()
        b[:, M:] = 7.0
        a[:, M:] = 7.0
        for _ in range(30):
            a = fn(a, b, a, *args)
            a, b = b, a
        out[name] = b
    e, f = out["exact"].float(), out["fast"].float()
    assert torch.isfinite(f).all()
    assert rel_l2(f[:, :M].cpu().numpy(), e[:, :M].cpu().numpy()) < 2e-3
    assert torch.equal(f[:, M:], e[:, M:]) and bool((f[:, M:] == 7.0).all())
    assert torch.equal(f[0], e[0]) and torch.equal(f[-1], e[-1])
    assert torch.equal(f[:, 0], e[:, 0]) and torch.equal(f[:, M - 1], e[:, M - 1])
