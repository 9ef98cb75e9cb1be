"""ctypes access to the reference's own step kernels built for the CPU.

TEST INFRASTRUCTURE ONLY. ``_ref/libstepref.so`` is compiled by
``Makefile.ref`` straight from projects/18_simple_wave_fd/step2D_wave.cu and
step1D_wave.cu through ``ref_shim.h``; it exists only where the reference
sources were present at build time. ``available()`` tells whether it does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libstepref.so")
REFERENCE = os.environ.get("WAVEFD_REFERENCE", "/root/reference")

_lib = None


def build() -> bool:
    """Build _ref/libstepref.so when the reference sources are present."""
    src = os.path.join(REFERENCE, "projects", "18_simple_wave_fd", "step2D_wave.cu")
    if not os.path.exists(src):
        return os.path.exists(LIB_PATH)
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), f"REFERENCE={REFERENCE}"],
                   check=True, cwd=os.path.dirname(HERE))
    return True


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise FileNotFoundError(LIB_PATH)
        _lib = ctypes.CDLL(LIB_PATH)
        f = ctypes.POINTER(ctypes.c_float)
        u16 = ctypes.POINTER(ctypes.c_uint16)
        F, I = ctypes.c_float, ctypes.c_int
        _lib.ref_padded_step.argtypes = [f, f, f, F, F, F, F, I, I, I]
        _lib.ref_coalesced_step.argtypes = [f, f, f, F, F, F, F, I, I]
        _lib.ref_basic_step.argtypes = [f, f, f, F, F, F, F, I, I]
        _lib.ref_mixed_step.argtypes = [u16, u16, u16, F, F, F, F, I, I, I]
        _lib.ref_step1d.argtypes = [f, f, f, F, F, F, I]
    return _lib


def _fp(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def padded_step(u0, u1, u2, c, dt, dx, dy, N, M):
    """step2D_wave.cu:59-81 on (N, M_padded) FP32 arrays; u2 may alias u0."""
    lib().ref_padded_step(_fp(u0), _fp(u1), _fp(u2), c, dt, dx, dy, N, M, u1.shape[1])
    return u2


def coalesced_step(u0, u1, u2, c, dt, dx, dy):
    N, M = u1.shape
    lib().ref_coalesced_step(_fp(u0), _fp(u1), _fp(u2), c, dt, dx, dy, N, M)
    return u2


def basic_step(u0, u1, u2, c, dt, dx, dy):
    N, M = u1.shape
    lib().ref_basic_step(_fp(u0), _fp(u1), _fp(u2), c, dt, dx, dy, N, M)
    return u2


def mixed_step(u0, u1, u2, c, dt, dx, dy, N, M):
    """step2D_wave.cu:85-124 on float16 arrays of shape (N, M_padded)."""
    p = lambda a: a.view(np.uint16).ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
    lib().ref_mixed_step(p(u0), p(u1), p(u2), c, dt, dx, dy, N, M, u1.shape[1])
    return u2


def step1d(u0, u1, u2, c, dt, dx):
    lib().ref_step1d(_fp(u0), _fp(u1), _fp(u2), c, dt, dx, u1.shape[0])
    return u2
