"""Fields of more than 2^31 cells: 130 identical shots of 4096^2 (2D) or 256^3
(3D) cells, 2.18e9 cells per field, so the last shots sit past every 32-bit
offset. Every shot sees the same model, wavelet, source and receivers:
  * the forward traces of the last shot equal those of the first and those
    of a one-shot call bit for bit (the same kernels on the same values; only
    the shot offset differs), and the first shot matches the FP64 oracle
    (1e-5);
  * the 2D misfit gradient of the 130 shots equals 130 times the one-shot
    gradient (1e-5: the shots' terms are summed by atomics in another order).
About 20 GB of device memory for a forward and 100 GB for the gradient;
skipped when the device has less free memory.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import oracle_geometry

pytestmark = pytest.mark.gpu

NSHOT = 130


def _setup(cuda, shape, need_gb):
    if torch.cuda.mem_get_info(cuda)[0] < need_gb * 2**30:
        pytest.skip(f"needs about {need_gb} GB of free device memory")
    from neuralmech_gb300 import Grid
    from neuralmech_gb300.synth import ricker
    nd = len(shape)
    c, h = 2000.0, 10.0
    dt = 0.4 * h / c
    nt = 8
    grid = Grid(shape, (h,) * nd, dt, nt, order=8, sponge=0, ckpt_every=4)
    vel = np.full(shape, c, dtype=np.float32)
    mid = [n // 2 for n in shape]
    src = np.array([[mid]], dtype=np.int32)
    rec = np.array([[[m + (2 if k == nd - 1 else 0) for k, m in enumerate(mid)],
                     [m + (3 if k == 0 else 0) for k, m in enumerate(mid)]]], dtype=np.int32)
    wav = (1.0 + ricker(60.0, nt, dt)).astype(np.float32)[None, :, None]  # nonzero from step 0
    return grid, vel, wav, src, rec


def _many(a, n=NSHOT):
    return np.repeat(a, n, axis=0)


@pytest.mark.parametrize("shape", [(4096, 4096), (256, 256, 256)])
def test_forward_beyond_2_31_cells(cuda, orc, shape):
    from neuralmech_gb300 import wave_forward
    grid, vel, wav, src, rec = _setup(cuda, shape, 40)
    assert NSHOT * int(np.prod(shape)) > 2**31
    v = torch.from_numpy(vel).to(cuda)
    one = wave_forward(v, torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec), grid)
    many = wave_forward(v, torch.from_numpy(_many(wav)).to(cuda), torch.from_numpy(_many(src)),
                        torch.from_numpy(_many(rec)), grid)
    assert many.shape[0] == NSHOT
    assert torch.count_nonzero(one) > 0
    assert torch.equal(many[-1], many[0])
    assert torch.equal(many[0], one[0])
    ref = orc.forward(oracle_geometry(orc, grid, vel, wav, src, rec))
    assert rel_l2(one.cpu().numpy(), ref) < 1e-5


def test_gradient_beyond_2_31_cells(cuda):
    from neuralmech_gb300 import misfit_gradient
    grid, vel, wav, src, rec = _setup(cuda, (4096, 4096), 120)
    v = torch.from_numpy(vel).to(cuda)
    obs1 = torch.zeros((1, grid.nt, rec.shape[1]), device=cuda)  # residual = the traces themselves
    J1, g1 = misfit_gradient(v, torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec),
                             obs1, grid)
    Jn, gn = misfit_gradient(v, torch.from_numpy(_many(wav)).to(cuda), torch.from_numpy(_many(src)),
                             torch.from_numpy(_many(rec)), obs1.expand(NSHOT, -1, -1).contiguous(), grid)
    assert float(J1) > 0
    assert abs(float(Jn) - NSHOT * float(J1)) <= 1e-9 * NSHOT * float(J1)
    assert rel_l2(gn.cpu().numpy(), NSHOT * g1.cpu().numpy()) < 1e-5
