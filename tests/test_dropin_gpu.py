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

from conftest import ROOT

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
