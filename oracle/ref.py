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


# ---------------------------------------------------------------- the reference's kernels on the GPU
# _ref/step2D_wave.cubin: step2D_wave.cu built for sm_103a with --use_fast_math
# (Makefile.ref, where the reference sources are); librefgpu.so (ref_gpu.cpp)
# loads it with the CUDA driver API. Launch shapes are those of the reference's
# drivers, restated at each call below.
GPU_LIB_PATH = os.path.join(HERE, "librefgpu.so")
CUBIN_PATH = os.path.join(HERE, "_ref", "step2D_wave.cubin")            # --use_fast_math
CUBIN_IEEE_PATH = os.path.join(HERE, "_ref", "step2D_wave_ieee.cubin")  # IEEE, no FMA

_gpu = None
_handles = {}


def gpu_build() -> bool:
    """Build librefgpu.so (own source, needs the CUDA headers and driver
    library) and, where the reference sources are present, the cubin."""
    subprocess.run(["make", "-s", "-C", HERE, "librefgpu.so"], check=True)
    build()
    return gpu_available()


def gpu_available() -> bool:
    return all(os.path.exists(p) for p in (GPU_LIB_PATH, CUBIN_PATH, CUBIN_IEEE_PATH))


def _gpu_lib():
    global _gpu
    if _gpu is None:
        if not gpu_available():
            raise FileNotFoundError(f"{GPU_LIB_PATH} or {CUBIN_PATH} missing")
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the primary context, current on this thread
        lib = ctypes.CDLL(GPU_LIB_PATH)
        lib.refgpu_load.argtypes = [ctypes.c_char_p]
        lib.refgpu_error.restype = ctypes.c_char_p
        lib.refgpu_launch.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                      ctypes.c_uint, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        for key, path in (("fast", CUBIN_PATH), ("ieee", CUBIN_IEEE_PATH)):
            h = lib.refgpu_load(path.encode())
            if h < 0:
                raise RuntimeError(lib.refgpu_error().decode())
            _handles[key] = h
        _gpu = lib
    return _gpu


# which build the calls below use: "fast" (--use_fast_math, as the drivers) or
# "ieee" (IEEE division, no fused multiply-adds)
MODE = {"build": "fast"}


def _gpu_launch(name, grid, block, args):
    """args: CUDA tensors (passed as device pointers), Python floats (FP32)
    and ints (int32), in the kernel's parameter order."""
    import torch
    hold = []
    for a in args:
        if isinstance(a, torch.Tensor):
            assert a.is_cuda and a.is_contiguous()
            hold.append(ctypes.c_void_p(a.data_ptr()))
        elif isinstance(a, int):
            hold.append(ctypes.c_int(a))
        else:
            hold.append(ctypes.c_float(a))
    ptrs = (ctypes.c_void_p * len(hold))(*[ctypes.cast(ctypes.pointer(h), ctypes.c_void_p) for h in hold])
    lib = _gpu_lib()
    stream = torch.cuda.current_stream().cuda_stream
    h = _handles[MODE["build"]]
    if lib.refgpu_launch(h, name.encode(), grid[0], grid[1], block[0], block[1], ptrs, ctypes.c_void_p(stream)) != 0:
        raise RuntimeError(lib.refgpu_error().decode())


def padded_step_gpu(u0, u1, u2, c, dt, dx, dy, N, M):
    """padded_step with the launch of 2D_wave_cuda_padding.py:62-76: blocks of
    128 x 4 threads over (M_padded, N)."""
    Mp = u1.shape[1]
    _gpu_launch("padded_step", ((Mp + 127) // 128, (N + 3) // 4), (128, 4), (u0, u1, u2, c, dt, dx, dy, N, M, Mp))
    return u2


def mixed_step_gpu(u0, u1, u2, c, dt, dx, dy, N, M):
    """mixed_step (float16 tensors) with the launch of 2D_wave_cuda_mixed.py:63-75:
    one thread per pair of points."""
    Mp = u1.shape[1]
    _gpu_launch("mixed_step", ((Mp // 2 + 127) // 128, (N + 3) // 4), (128, 4), (u0, u1, u2, c, dt, dx, dy, N, M, Mp))
    return u2


def scaled_step_gpu(q0, s0, q1, s1, q2, s2, c, dt, dx, dy, N, M):
    """scaled_step (int16 levels q with FP32 scales s per 32 values) with the
    launch of 2D_wave_cuda_scaled.py:76-91."""
    Mp = q1.shape[1]
    _gpu_launch("scaled_step", ((Mp // 2 + 127) // 128, (N + 3) // 4), (128, 4),
                (q0, s0, q1, s1, q2, s2, c, dt, dx, dy, N, M, Mp))


def temporal_step_gpu(u0, u1, v0, v1, c, dt, dx, dy, N, M):
    """temporal_step (eight steps per launch) with the launch of
    2D_wave_cuda_temporal.py:60-75: 128 x 4 threads, tiles of 112 x 32
    updated points."""
    Mp = u1.shape[1]
    _gpu_launch("temporal_step", ((M + 111) // 112, (N + 31) // 32), (128, 4),
                (u0, u1, v0, v1, c, dt, dx, dy, N, M, Mp))


def shared_step_gpu(u0, u1, u2, c, dt, dx, dy, N, M):
    """shared_step with the launch of 2D_wave_cuda_shared.py:62-75."""
    Mp = u1.shape[1]
    _gpu_launch("shared_step", ((Mp + 127) // 128, (N + 3) // 4), (128, 4), (u0, u1, u2, c, dt, dx, dy, N, M, Mp))
    return u2


def basic_step_gpu(u0, u1, u2, c, dt, dx, dy, N, M):
    """basic_step on unpadded (N, M) rows with the launch of
    2D_wave_cuda_basic.py:58-66: blocks of 4 x 128 threads, x along i."""
    _gpu_launch("basic_step", ((N + 3) // 4, (M + 127) // 128), (4, 128), (u0, u1, u2, c, dt, dx, dy, N, M))
    return u2


def coalesced_step_gpu(u0, u1, u2, c, dt, dx, dy, N, M):
    """coalesced_step on unpadded (N, M) rows with the launch of
    2D_wave_cuda_coalesced.py:58-66: blocks of 128 x 4 threads, x along j."""
    _gpu_launch("coalesced_step", ((M + 127) // 128, (N + 3) // 4), (128, 4), (u0, u1, u2, c, dt, dx, dy, N, M))
    return u2
