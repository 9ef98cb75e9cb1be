"""The reference's CPU path for one wave step, in NumPy array slices.

TEST INFRASTRUCTURE ONLY (parity reference and timed CPU baseline).

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


def _update_order2(u0, u1c, il, ir, jl, jr, k, dx2, dy2):
    """-u0 + 2 u1 + k ((il - 2u1 + ir)/dx2 + (jl - 2u1 + jr)/dy2), FP32, the
    operation order of step2D_wave.cu:108-113 and 162-167."""
    two = np.float32(2) * u1c
    li = (il - two) + ir
    lj = (jl - two) + jr
    return (-u0 + two) + k * (li / dx2 + lj / dy2)


def scaled_step(q0, s0, q1, s1, c, dt, dx, dy, N, M):
    """scaled_step (projects/18_simple_wave_fd/step2D_wave.cu:128-183) restated
    on NumPy: int16 fields q [N][Mp] with one FP32 scale per 32 values of a row,
    s [N][Mp/32], u = s q. Returns (q2, s2) for rows 1..N-2 (rows 0 and N-1 are
    copied from q0/s0, which the in-place driver passes as q2/s2). The
    reference's shuffles only move decoded neighbour values between threads:
    here each neighbour is decoded with its own block's scale, as they are."""
    f32 = np.float32
    Mp = q1.shape[1]
    k = f32(dt) * f32(dt) * f32(c) * f32(c)
    dx2, dy2 = f32(dx) * f32(dx), f32(dy) * f32(dy)
    u0 = np.repeat(s0, 32, axis=1) * q0.astype(f32)
    u1 = np.repeat(s1, 32, axis=1) * q1.astype(f32)
    zero = np.zeros((N, 1), f32)
    jl = np.concatenate([zero, u1[:, :-1]], axis=1)  # j - 1 (0 at j = 0)
    jr = np.concatenate([u1[:, 1:], zero], axis=1)   # j + 1 (0 past M_padded)
    q2, s2 = q0.copy(), s0.copy()
    v = _update_order2(u0[1:-1], u1[1:-1], u1[:-2], u1[2:], jl[1:-1], jr[1:-1], k, dx2, dy2)
    j = np.arange(Mp)[None, :]
    v = np.where((j == 0) | (j >= M - 1), f32(0), v).astype(f32)
    m = np.abs(v).reshape(N - 2, Mp // 32, 32).max(axis=2)
    with np.errstate(divide="ignore"):
        inv = np.where(m > 0, f32(32767) / np.where(m > 0, m, f32(1)), f32(0)).astype(f32)
    q2[1:-1] = np.rint(v * np.repeat(inv, 32, axis=1)).astype(np.int16)
    s2[1:-1] = (m / f32(32767)).astype(f32)
    return q2, s2


def scaled_encode(u):
    """A field [N][Mp] as (q, s): per 32-value block, s = max|u| / 32767 and
    q = rint(u * 32767 / max|u|) (the encoding of step2D_wave.cu:175-182)."""
    f32 = np.float32
    N, Mp = u.shape
    m = np.abs(u).reshape(N, Mp // 32, 32).max(axis=2).astype(f32)
    m = np.where(m < f32(2.0**-100), f32(0), m)  # (32767 / m must stay finite: such blocks encode as 0)
    inv = np.where(m > 0, f32(32767) / np.where(m > 0, m, f32(1)), f32(0)).astype(f32)
    return np.rint(u.astype(f32) * np.repeat(inv, 32, axis=1)).astype(np.int16), (m / f32(32767)).astype(f32)
