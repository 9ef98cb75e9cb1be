"""Full matrix capture + TFM imaging (the consumer of the wave path's traces).

CPU: the Hilbert kernel reproduces scipy.signal.hilbert; the NumPy restatement
of the reference kernel agrees with the reference's array form on data where
they coincide.
GPU: the analytic signal vs scipy (1e-5 relative L2), TFM vs the reference
kernel restated in FP64 (1e-4 relative L2: the kernel forms sample times of
several hundred in FP32, as the reference's FP32 kernel does, so the
interpolation weights carry ~1e-5 relative error), and an end-to-end image of
a point scatterer whose peak lands within a few cells of the scatterer.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2


def test_hilbert_kernel_matches_scipy():
    from scipy.signal import hilbert

    from neuralmech_gb300.imaging import hilbert_kernel
    rng = np.random.default_rng(0)
    for nt in (16, 17, 200, 257):
        x = rng.standard_normal(nt)
        g = hilbert_kernel(nt).astype(np.float64)
        Hx = np.array([sum(x[k] * g[(n - k) % nt] for k in range(nt)) for n in range(nt)])
        assert rel_l2(Hx, np.imag(hilbert(x))) < 1e-6


def test_tfm_restatements_agree():
    from oracle.tfm_ref import tfm_array_form, tfm_kernel_semantics
    rng = np.random.default_rng(1)
    E, nt = 6, 300
    a = rng.standard_normal((E, E, nt)) + 1j * rng.standard_normal((E, E, nt))
    h = a + a.transpose(1, 0, 2)  # reciprocal FMC
    el = np.stack([np.linspace(0.1, 0.9, E), np.zeros(E)], axis=1)
    x, y = np.meshgrid(np.linspace(0, 1, 17), np.linspace(0.05, 0.5, 13), indexing="ij")
    c, dt, t0 = 1.0, 0.01, 0.02
    ref = tfm_array_form(h, el, t0, dt, c, x, y).ravel()
    kern = tfm_kernel_semantics(h, el[:, 0], el[:, 1], t0, dt, c, x, y, reciprocity=True)
    full = tfm_kernel_semantics(h, el[:, 0], el[:, 1], t0, dt, c, x, y, reciprocity=False)
    assert rel_l2(kern, full) < 1e-12  # reciprocity is exact on symmetric data
    assert rel_l2(kern, ref) < 1e-12   # no pair reaches the end of the traces here


@pytest.mark.gpu
def test_analytic_signal_matches_scipy(cuda):
    from scipy.signal import hilbert

    from neuralmech_gb300.imaging import analytic_signal
    rng = np.random.default_rng(2)
    x = rng.standard_normal((3, 5, 1000)).astype(np.float32)
    h = analytic_signal(torch.from_numpy(x).to(cuda)).cpu().numpy()
    ref = hilbert(x.astype(np.float64), axis=-1)
    assert rel_l2(h, ref) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("E,reciprocity", [(8, True), (16, False), (32, True), (5, True)])
def test_tfm_matches_reference_kernel(cuda, E, reciprocity):
    from oracle.tfm_ref import tfm_kernel_semantics

    from neuralmech_gb300.imaging import tfm
    rng = np.random.default_rng(E)
    nt = 400
    a = (rng.standard_normal((E, E, nt)) + 1j * rng.standard_normal((E, E, nt))).astype(np.complex64)
    h = a + a.transpose(1, 0, 2)
    el = np.stack([np.linspace(0.1, 0.9, E), np.full(E, 1.0)], axis=1).astype(np.float32)
    x, y = np.meshgrid(np.linspace(0, 1, 41), np.linspace(0, 1, 37), indexing="ij")
    c, dt, t0 = 1.0, 0.005, 0.02
    img = tfm(torch.from_numpy(h).to(cuda), el, t0, dt, c, x, y, reciprocity=reciprocity)
    ref = tfm_kernel_semantics(h.astype(np.complex128), el[:, 0].astype(np.float64), el[:, 1].astype(np.float64),
                               t0, dt, c, x.astype(np.float32), y.astype(np.float32), reciprocity=reciprocity)
    assert rel_l2(img.cpu().numpy().ravel(), ref) < 1e-4


@pytest.mark.gpu
def test_fmc_tfm_images_a_point_scatterer(cuda):
    """Full matrix capture with and without a small high-velocity inclusion;
    the TFM image of the scattered field peaks at the inclusion."""
    from neuralmech_gb300 import Grid
    from neuralmech_gb300.imaging import analytic_signal, full_matrix_capture, tfm
    from neuralmech_gb300.synth import ricker
    n, h = 160, 1.0
    c = 1.0
    dt = 0.4 * h / 1.5
    nt = 480  # the echo of the inclusion returns near step 340
    grid = Grid((n, n), (h, h), dt, nt, order=8, sponge=20)
    E = 16
    xs = np.linspace(30, 130, E).round().astype(int)
    elements = np.stack([np.full(E, 24), xs], axis=1)  # (z, x) cells on a line
    f = 0.08
    wav = ricker(f, nt, dt)
    vel0 = torch.full((n, n), c, device=cuda)
    vel1 = vel0.clone()
    zt, xt = 60, 75
    vel1[zt - 2:zt + 3, xt - 2:xt + 3] = 1.5
    sc = full_matrix_capture(vel1, wav, elements, grid) - full_matrix_capture(vel0, wav, elements, grid)
    assert sc.abs().max() > 1e-3
    hs = analytic_signal(sc.transpose(1, 2).contiguous())   # (E, E, nt): emitter, receiver, time
    zz, xx = np.meshgrid(np.arange(34, 120, 1.0), np.arange(20, 140, 1.0), indexing="ij")
    # element coordinates (x, y) = (x cell, z cell); the wavelet injected at step n
    # shows in trace sample n, so its peak sits at sample 1.5 / (f dt)
    el_xy = np.stack([elements[:, 1], elements[:, 0]], axis=1).astype(np.float32)
    t0 = 1.5 / f
    img = tfm(hs, el_xy, t0, dt, c, xx, zz).cpu().numpy()
    iz, ix = np.unravel_index(np.argmax(img), img.shape)
    assert abs(zz[iz, ix] - (zt - 2)) <= 3 and abs(xx[iz, ix] - xt) <= 3, (zz[iz, ix], xx[iz, ix])
