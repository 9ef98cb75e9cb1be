"""Full matrix capture and total focusing method imaging on the GPU.

The consumer side of the wave path in projects/18_fwi:
  * ``full_matrix_capture``: every element of an array fires once while all
    elements listen. These are the shots of one batched ``wave_forward``, and
    the traces come out (emitter, step, receiver) (plate.py:62-64);
  * ``analytic_signal``: x + i H[x] along time, the periodic discrete Hilbert
    transform of scipy.signal.hilbert (2D_tfm.py:37), by the library's own
    circular-convolution kernel;
  * ``tfm``: delay and sum of the analytic traces onto pixels
    (tfm.py:12-36), one thread per pixel.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .wavefd import Grid, _ptr, _require_cuda, _stream, wave_forward


def hilbert_kernel(nt: int) -> np.ndarray:
    """Circular-convolution kernel g of the periodic discrete Hilbert
    transform: g = ifft(-i sign(k)), sign 0 at k = 0 and (even nt) at nt/2."""
    k = np.arange(nt)
    sgn = np.zeros(nt)
    half = nt // 2
    sgn[1:(nt + 1) // 2] = 1.0
    sgn[half + 1:] = -1.0
    if nt % 2 == 1:
        sgn[(nt + 1) // 2:] = -1.0
    g = np.fft.ifft(-1j * sgn).real
    del k
    return g.astype(np.float32)


def analytic_signal(traces: torch.Tensor) -> torch.Tensor:
    """complex64 analytic signal of FP32 CUDA traces along the last axis."""
    _require_cuda(traces, "traces")
    x = traces.to(torch.float32).contiguous()
    nt = x.shape[-1]
    g = torch.from_numpy(hilbert_kernel(nt)).to(x.device)
    out = torch.empty(x.shape + (2,), dtype=torch.float32, device=x.device)
    _lib.check(_lib.load().wfd_analytic_signal(_ptr(x), x.numel() // nt, nt, _ptr(g), _ptr(out), _stream()),
               "wfd_analytic_signal")
    return torch.view_as_complex(out)


def tfm(h: torch.Tensor, elements, t0: float, dt: float, c: float, x, y, reciprocity: bool = True):
    """Image |sum_e sum_r h_er(t0 + (|p - x_e| + |p - x_r|) / c)| on the pixel
    grid (x, y).

    h: (E, E, nt) complex64 CUDA analytic traces (emitter, receiver, sample);
    elements: (E, 2) coordinates (x, y) in the units of x, y and c * dt."""
    _require_cuda(h, "h")
    if h.dtype != torch.complex64 or h.dim() != 3 or h.shape[0] != h.shape[1]:
        raise ValueError("h must be a (E, E, nt) complex64 tensor")
    dev = h.device
    hr = torch.view_as_real(h.contiguous()).contiguous()
    el = torch.as_tensor(elements, dtype=torch.float32, device=dev)
    xe = el[:, 0].contiguous()
    ye = el[:, 1].contiguous()
    xp = torch.as_tensor(x, dtype=torch.float32, device=dev)
    shape = xp.shape
    xp = xp.reshape(-1).contiguous()
    yp = torch.as_tensor(y, dtype=torch.float32, device=dev).reshape(-1).contiguous()
    image = torch.empty(xp.numel(), dtype=torch.float32, device=dev)
    E, _, nt = h.shape
    _lib.check(_lib.load().wfd_tfm(_ptr(hr), E, _ptr(xe), _ptr(ye), nt, float(dt), float(t0), float(c),
                                   _ptr(xp), _ptr(yp), xp.numel(), int(reciprocity), _ptr(image),
                                   _stream()), "wfd_tfm")
    return image.reshape(shape)


def full_matrix_capture(vel: torch.Tensor, wavelet, elements, grid: Grid) -> torch.Tensor:
    """(E, nt, E) traces: element e fires the wavelet, all E elements record.

    elements: (E, 2) integer cells (z, x) inside the interior."""
    el = torch.as_tensor(elements, dtype=torch.int32)
    E = el.shape[0]
    src = el[:, None, :]                              # shot e: one source at element e
    rec = el[None, :, :].expand(E, E, 2).contiguous()  # every shot: all elements listen
    w = torch.as_tensor(wavelet, dtype=torch.float32, device=vel.device)
    if w.dim() == 1:
        w = w.view(1, -1).expand(E, -1).contiguous()
    return wave_forward(vel, w, src, rec, grid)
