"""The reference's CPU path for one wave step, in NumPy array slices.

TEST INFRASTRUCTURE ONLY (checker and timed CPU baseline).

``fd_step_order2`` restates ``fd_step`` of
projects/18_simple_wave_fd/2D_wave_cupy.py:54-62 with ``cp`` replaced by
``np``: the 5-point Laplacian on the interior, the outer ring untouched, in the
reference's own operation order. ``fd_step`` generalises the same slice form
to space order 2R, a per-cell ``w = v^2 dt^2`` and the sponge factor ``g``:
``u2 = g (2 u1 + w Lap u1) - g^2 u0`` on the interior. NumPy elementwise
operations run on one core.
"""
from __future__ import annotations

import numpy as np


def fd_step_order2(u0, u1, u2, dt, dx, dy, wavespeed):
    """2D_wave_cupy.py:54-62 on NumPy (FP32 arrays stay FP32)."""
    laplacian_x = (u1[:-2, 1:-1] - 2 * u1[1:-1, 1:-1] + u1[2:, 1:-1]) / dx**2
    laplacian_y = (u1[1:-1, :-2] - 2 * u1[1:-1, 1:-1] + u1[1:-1, 2:]) / dy**2
    u2[1:-1, 1:-1] = (
        -u0[1:-1, 1:-1]
        + 2 * u1[1:-1, 1:-1]
        + dt**2 * wavespeed**2 * (laplacian_x + laplacian_y)
    )
    return u2


def weights(order: int) -> np.ndarray:
    """Central second-derivative weights a_0..a_R on a unit grid (closed form)."""
    from math import factorial

    R = order // 2
    a = np.zeros(R + 1)
    for k in range(1, R + 1):
        a[k] = 2.0 * (1 if k % 2 else -1) * factorial(R) ** 2 / (k * k * factorial(R - k) * factorial(R + k))
    a[0] = -2.0 * a[1:].sum()
    return a


def fd_step(u0, u1, u2, w, h, order=8, g=None):
    """One interior update of order ``order`` on 2D or 3D arrays, slice form.

    ``w`` (same shape as u, or scalar) is v^2 dt^2; ``h`` is (dz, dx) in 2D or
    (dz, dy, dx) in 3D; ``g`` the per-cell sponge factor (None = 1). The ring of
    R cells is left untouched, as ``fd_step_order2`` leaves its ring of 1.
    """
    R = order // 2
    a = weights(order)
    nd = u1.ndim
    inner = tuple(slice(R, n - R) for n in u1.shape)
    lap = sum(a[0] / hh**2 for hh in h) * u1[inner]
    for axis in range(nd):
        for k in range(1, R + 1):
            lo = list(inner)
            hi = list(inner)
            n = u1.shape[axis]
            lo[axis] = slice(R - k, n - R - k)
            hi[axis] = slice(R + k, n - R + k)
            lap = lap + a[k] / h[axis] ** 2 * (u1[tuple(lo)] + u1[tuple(hi)])
    wi = w[inner] if np.ndim(w) else w
    if g is None:
        u2[inner] = 2 * u1[inner] + wi * lap - u0[inner]
    else:
        gi = g[inner]
        u2[inner] = gi * (2 * u1[inner] + wi * lap) - gi * gi * u0[inner]
    return u2
