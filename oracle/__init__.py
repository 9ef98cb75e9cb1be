"""FP64 CPU oracle for the finite-difference acoustic wave path.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package, and only as the
reference results of the parity checks or the timed CPU baseline. The product (``neuralmech_gb300``) never
imports it and has no CPU fallback.

Contents:
  * ``liboracle.so`` (``oracle.cpp``): C++/OpenMP FP64 forward modelling,
    single step and exact checkpointed misfit gradient;
  * ``numpy_ref``: the reference's array-slice step
    (projects/18_simple_wave_fd/2D_wave_cupy.py:54-62) on NumPy, generalised to
    space order 2R, a velocity field and the sponge;
  * ``ref``: the reference's own CUDA C step kernels
    (projects/18_simple_wave_fd/step2D_wave.cu, step1D_wave.cu) compiled for the
    CPU into ``_ref/libstepref.so`` by ``Makefile.ref``; present only where the
    reference sources were available at build time.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (seconds)."""
    src = os.path.join(HERE, "oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


class _Problem(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32), ("order", ctypes.c_int32),
        ("nz", ctypes.c_int32), ("ny", ctypes.c_int32), ("nx", ctypes.c_int32),
        ("nshot", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("nsrc", ctypes.c_int32), ("nrec", ctypes.c_int32),
        ("ckpt_every", ctypes.c_int32),
        ("dt", ctypes.c_double), ("dz", ctypes.c_double), ("dy", ctypes.c_double),
        ("dx", ctypes.c_double), ("src_scale", ctypes.c_double),
    ]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        d = ctypes.POINTER(ctypes.c_double)
        i32 = ctypes.POINTER(ctypes.c_int32)
        P = ctypes.POINTER(_Problem)
        _lib.orc_fd_coeffs.argtypes = [ctypes.c_int, d]
        _lib.orc_step.argtypes = [P, d, ctypes.c_double, d, d, d, d, d, d]
        _lib.orc_forward.argtypes = [P, d, d, d, d, d, i32, i32, d, d]
        _lib.orc_gradient.argtypes = [P, d, d, d, d, d, i32, i32, d, d, d, d, d]
        _lib.orc_stag_coeffs.argtypes = [ctypes.c_int, d]
        _lib.orc_vd_forward.argtypes = [P, d, d, d, d, d, i32, i32, d, d]
        _lib.orc_vd_gradient.argtypes = [P, d, d, d, d, d, i32, i32, d, d, d, d, d, d]
        for f in (_lib.orc_fd_coeffs, _lib.orc_step, _lib.orc_forward, _lib.orc_gradient):
            f.restype = ctypes.c_int
    return _lib


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def fd_coeffs(order: int) -> np.ndarray:
    """Second-derivative weights a_0..a_R of space order ``order`` (unit grid)."""
    a = np.zeros(5)
    if lib().orc_fd_coeffs(order, _dp(a)) != 0:
        raise ValueError(f"unsupported order {order}")
    return a[: order // 2 + 1].copy()


@dataclass
class Geometry:
    """Inputs of one oracle run (all arrays NumPy; converted to FP64 here)."""
    vel: np.ndarray            # (nz, nx) or (nz, ny, nx)
    wavelet: np.ndarray        # (nshot, nt, nsrc)
    src: np.ndarray            # (nshot, nsrc, 3) int (z, y, x)
    rec: np.ndarray            # (nshot, nrec, 3) int
    dt: float
    h: tuple                   # (dz, dy, dx); dy ignored in 2D
    order: int = 8
    sponge: tuple | None = None  # (gz, gy, gx) 1D profiles, None entries = 1
    src_scale: float = 1.0
    ckpt_every: int = 0


def _problem(g: Geometry) -> _Problem:
    ndim = g.vel.ndim
    shape = g.vel.shape
    nz, nx = shape[0], shape[-1]
    ny = shape[1] if ndim == 3 else 1
    nshot, nt, nsrc = g.wavelet.shape
    return _Problem(ndim, g.order, nz, ny, nx, nshot, nt, nsrc, g.rec.shape[1],
                    g.ckpt_every, g.dt, g.h[0], g.h[1], g.h[2], g.src_scale)


def _profiles(g: Geometry):
    if g.sponge is None:
        return None, None, None
    return tuple(None if p is None else np.ascontiguousarray(p, dtype=np.float64) for p in g.sponge)


def forward(g: Geometry, want_final: bool = False):
    """Traces (nshot, nt, nrec) in FP64; optionally the final fields."""
    p = _problem(g)
    vel = np.ascontiguousarray(g.vel, dtype=np.float64)
    wav = np.ascontiguousarray(g.wavelet, dtype=np.float64)
    src = np.ascontiguousarray(g.src, dtype=np.int32)
    rec = np.ascontiguousarray(g.rec, dtype=np.int32)
    gz, gy, gx = _profiles(g)
    traces = np.zeros((p.nshot, p.nt, p.nrec))
    final = np.zeros((p.nshot,) + g.vel.shape) if want_final else None
    rc = lib().orc_forward(ctypes.byref(p), _dp(vel), _dp(gz), _dp(gy), _dp(gx), _dp(wav),
                           _ip(src), _ip(rec), _dp(traces), _dp(final))
    if rc != 0:
        raise ValueError(f"orc_forward failed ({rc}): positions must be interior")
    return (traces, final) if want_final else traces


def gradient(g: Geometry, observed: np.ndarray):
    """(misfit, grad_vel, grad_wavelet, traces) in FP64."""
    p = _problem(g)
    vel = np.ascontiguousarray(g.vel, dtype=np.float64)
    wav = np.ascontiguousarray(g.wavelet, dtype=np.float64)
    src = np.ascontiguousarray(g.src, dtype=np.int32)
    rec = np.ascontiguousarray(g.rec, dtype=np.int32)
    obs = np.ascontiguousarray(observed, dtype=np.float64)
    gz, gy, gx = _profiles(g)
    grad = np.zeros(g.vel.shape)
    gwav = np.zeros(wav.shape)
    traces = np.zeros((p.nshot, p.nt, p.nrec))
    J = ctypes.c_double(0.0)
    rc = lib().orc_gradient(ctypes.byref(p), _dp(vel), _dp(gz), _dp(gy), _dp(gx), _dp(wav),
                            _ip(src), _ip(rec), _dp(obs), _dp(grad), _dp(gwav), _dp(traces),
                            ctypes.byref(J))
    if rc != 0:
        raise ValueError(f"orc_gradient failed ({rc}): positions must be interior")
    return J.value, grad, gwav, traces


def step(order: int, h: tuple, uo, uc, un, w=None, w_const: float = 0.0, sponge=None):
    """One FP64 interior update in place on ``un`` (2D or 3D dense arrays).

    ``w`` is v^2 dt^2 per cell (or ``w_const`` everywhere)."""
    ndim = uc.ndim
    nz, nx = uc.shape[0], uc.shape[-1]
    ny = uc.shape[1] if ndim == 3 else 1
    p = _Problem(ndim, order, nz, ny, nx, 1, 1, 0, 0, 0, 1.0, h[0], h[1], h[2], 1.0)
    gz, gy, gx = (None, None, None) if sponge is None else sponge
    for a in (uo, uc, un):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    rc = lib().orc_step(ctypes.byref(p), _dp(w), w_const, _dp(gz), _dp(gy), _dp(gx),
                        _dp(uo), _dp(uc), _dp(un))
    assert rc == 0
    return un


def stag_coeffs(order: int) -> np.ndarray:
    """Staggered first-derivative weights c_1..c_R of order ``order`` (unit grid)."""
    c = np.zeros(5)
    if lib().orc_stag_coeffs(order, _dp(c)) != 0:
        raise ValueError(f"unsupported order {order}")
    return c[1: order // 2 + 1].copy()


@dataclass
class VdGeometry:
    """Inputs of one variable-density oracle run (2D; kappa, rho per cell)."""
    kappa: np.ndarray          # (nz, nx) bulk modulus
    rho: np.ndarray            # (nz, nx) density
    wavelet: np.ndarray        # (nshot, nt, nsrc)
    src: np.ndarray            # (nshot, nsrc, 3) int (z, 0, x)
    rec: np.ndarray            # (nshot, nrec, 3) int
    dt: float
    h: tuple                   # (dz, dx)
    order: int = 8
    sponge: tuple | None = None  # (gz, gx)
    src_scale: float = 1.0


def _vd_args(g: VdGeometry):
    nz, nx = g.kappa.shape
    nshot, nt, nsrc = g.wavelet.shape
    p = _Problem(2, g.order, nz, 1, nx, nshot, nt, nsrc, g.rec.shape[1], 0, g.dt, g.h[0], 1.0, g.h[1],
                 g.src_scale)
    f = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
    gz, gx = (None, None) if g.sponge is None else g.sponge
    return (p, f(g.kappa), f(g.rho), f(gz), f(gx), f(g.wavelet), np.ascontiguousarray(g.src, dtype=np.int32),
            np.ascontiguousarray(g.rec, dtype=np.int32))


def vd_forward(g: VdGeometry, want_final: bool = False):
    """Variable-density traces (nshot, nt, nrec) in FP64; optionally the final fields."""
    p, kap, rho, gz, gx, wav, src, rec = _vd_args(g)
    traces = np.zeros((p.nshot, p.nt, p.nrec))
    final = np.zeros((p.nshot,) + g.kappa.shape) if want_final else None
    rc = lib().orc_vd_forward(ctypes.byref(p), _dp(kap), _dp(rho), _dp(gz), _dp(gx), _dp(wav), _ip(src), _ip(rec),
                              _dp(traces), _dp(final))
    if rc != 0:
        raise ValueError(f"orc_vd_forward failed ({rc})")
    return (traces, final) if want_final else traces


def vd_gradient(g: VdGeometry, observed: np.ndarray):
    """(misfit, grad_kappa, grad_rho, grad_wavelet, traces) in FP64."""
    p, kap, rho, gz, gx, wav, src, rec = _vd_args(g)
    obs = np.ascontiguousarray(observed, dtype=np.float64)
    gk, gr, gw = np.zeros(g.kappa.shape), np.zeros(g.kappa.shape), np.zeros(wav.shape)
    traces = np.zeros((p.nshot, p.nt, p.nrec))
    J = ctypes.c_double(0.0)
    rc = lib().orc_vd_gradient(ctypes.byref(p), _dp(kap), _dp(rho), _dp(gz), _dp(gx), _dp(wav), _ip(src), _ip(rec),
                               _dp(obs), _dp(gk), _dp(gr), _dp(gw), _dp(traces), ctypes.byref(J))
    if rc != 0:
        raise ValueError(f"orc_vd_gradient failed ({rc})")
    return J.value, gk, gr, gw, traces
