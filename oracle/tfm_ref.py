"""The reference's total focusing method restated on NumPy (FP64).

TEST INFRASTRUCTURE ONLY (checker).

``tfm_kernel_semantics`` follows the CUDA kernel of
projects/18_fwi/tfm.py:12-36:
  * upper triangle r >= e with weight 2 off the diagonal (reciprocity);
  * linear interpolation between samples k and k + 1;
  * pairs whose k reaches nt - 1 skipped.

``tfm_array_form`` follows the array version tfm.py:39-53: every ordered
pair; k clamped to nt - 2 and the sample masked when k >= nt - 2.

The analytic signal of the reference is scipy.signal.hilbert (2D_tfm.py:37);
the tests call scipy directly.
"""
from __future__ import annotations

import numpy as np


def tfm_kernel_semantics(h, xe, ye, t0, dt, c, xp, yp, reciprocity=True):
    h = np.asarray(h)
    E, _, nt = h.shape
    xp = np.asarray(xp, dtype=np.float64).ravel()
    yp = np.asarray(yp, dtype=np.float64).ravel()
    tau = np.stack([np.hypot(xp - xe[e], yp - ye[e]) / c for e in range(E)])  # (E, P)
    s = np.zeros(xp.size, dtype=np.complex128)
    for e in range(E):
        for r in range(e if reciprocity else 0, E):
            t = (t0 + tau[e] + tau[r]) / dt
            k = t.astype(np.int64)
            ok = k < nt - 1
            kk = np.where(ok, k, 0)
            scale = 2.0 if (reciprocity and r > e) else 1.0
            w = (t - k) * scale
            v = scale - w
            val = v * h[e, r, kk] + w * h[e, r, kk + 1]
            s += np.where(ok, val, 0.0)
    return np.abs(s)


def tfm_array_form(h, elements, t0, dt, c, x, y):
    h = np.asarray(h)
    E, _, nt = h.shape
    tau = [np.hypot(x - ex, y - ey) / c for ex, ey in elements]
    s = np.zeros(np.shape(x), dtype=np.complex128)
    for e in range(E):
        for r in range(E):
            t = (t0 + tau[e] + tau[r]) / dt
            k = np.minimum(t.astype(np.int32), nt - 2)
            w = t - k
            s += ((1 - w) * h[e, r, k] + w * h[e, r, k + 1]) * (k < nt - 2)
    return np.abs(s)
