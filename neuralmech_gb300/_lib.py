"""ctypes binding of libwavefd.so (include/wavefd.h).

The library is the product path: there is no CPU or PyTorch fallback. If the
shared object is missing it is built with nvcc when available; if that is not
possible, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwavefd.so")

WFD_OK = 0
WFD_ERR_INVALID = -1
WFD_ERR_WORKSPACE = -2
WFD_ERR_CUDA = -3
WFD_ERR_UNSTABLE = -4
WFD_ERR_POSITION = -5
WFD_ERR_TIMEOUT = -6
WFD_ERR_STATE = -7

# Every symbol include/wavefd.h declares.
EXPORTS = (
    "wfd_strerror", "wfd_last_error", "wfd_version", "wfd_workspace_bytes", "wfd_forward",
    "wfd_backward", "wfd_misfit_gradient", "wfd_status", "wfd_sum_sq", "wfd_step2d_order2",
    "wfd_kernel_launches", "wfd_profile_begin", "wfd_profile_end", "wfd_forward_static",
    "wfd_forward_static_status",
    "wfd_analytic_signal", "wfd_tfm", "wfd_forward_final", "wfd_step2d_mixed", "wfd_step2d_mixed_fast", "wfd_step2d_scaled",
    "wfd_temporal_step", "wfd_temporal_step_fast", "wfd_step2d_exact", "wfd_misfit_gradient_overlap",
    "wfd_step1d", "wfd_vd_workspace_bytes", "wfd_vd_forward", "wfd_vd_forward_final", "wfd_vd_misfit_gradient",
    "wfd_batch_plan", "wfd_batch_run", "wfd_batch_launches", "wfd_batch_free",
)


class PhaseTimes(ctypes.Structure):
    """Mirror of ``wfd_phase_times``: forward, recompute, adjoint."""
    _fields_ = [("ms", ctypes.c_double * 3), ("launches", ctypes.c_int64 * 3)]


class Problem(ctypes.Structure):
    """Mirror of ``wfd_problem`` (include/wavefd.h)."""
    _fields_ = [
        ("ndim", ctypes.c_int32), ("order", ctypes.c_int32),
        ("nz", ctypes.c_int32), ("ny", ctypes.c_int32), ("nx", ctypes.c_int32),
        ("nshot", ctypes.c_int32), ("nt", ctypes.c_int32),
        ("nsrc", ctypes.c_int32), ("nrec", ctypes.c_int32),
        ("ckpt_every", ctypes.c_int32), ("ckpt_format", ctypes.c_int32),
        ("lap_store", ctypes.c_int32), ("shots_per_cta", ctypes.c_int32),
        ("group_shots", ctypes.c_int32), ("tile_rows", ctypes.c_int32),
        ("step_block", ctypes.c_int32), ("store_levels", ctypes.c_int32),
        ("field_format", ctypes.c_int32), ("adjoint_mode", ctypes.c_int32), ("recon_band", ctypes.c_int32),
        ("dt", ctypes.c_float), ("dz", ctypes.c_float), ("dy", ctypes.c_float),
        ("dx", ctypes.c_float), ("src_scale", ctypes.c_float), ("vmax", ctypes.c_float),
        ("update_form", ctypes.c_int32), ("level_format", ctypes.c_int32),
    ]


class BatchItem(ctypes.Structure):
    """Mirror of ``wfd_batch_item`` (include/wavefd.h): one wfd_misfit_gradient call."""
    _fields_ = [("problem", ctypes.POINTER(Problem))] + [
        (n, ctypes.c_void_p) for n in ("vel", "sponge_z", "sponge_y", "sponge_x", "wavelet", "src", "rec",
                                       "observed", "traces", "grad_vel", "grad_wavelet", "misfit", "workspace")
    ] + [("workspace_bytes", ctypes.c_size_t)]


class WaveFDError(RuntimeError):
    """A libwavefd call returned a negative status."""

    def __init__(self, status: int, where: str, detail: str):
        super().__init__(f"{where}: {detail} (status {status})")
        self.status = status


_lib = None
_lock = threading.Lock()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libwavefd.so (building it in-tree first if it is missing)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH) and build_if_missing:
            from .build import build
            build()
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with "
                              "`python -m neuralmech_gb300.build` (needs nvcc)")
        lib = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER(Problem)
        vp, f, i32, d = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p
        sz = ctypes.c_size_t
        lib.wfd_strerror.argtypes = [ctypes.c_int]
        lib.wfd_strerror.restype = ctypes.c_char_p
        lib.wfd_last_error.argtypes = []
        lib.wfd_last_error.restype = ctypes.c_char_p
        lib.wfd_version.argtypes = []
        lib.wfd_workspace_bytes.argtypes = [P, ctypes.c_int, ctypes.POINTER(sz)]
        lib.wfd_forward.argtypes = [P, f, f, f, f, f, i32, i32, f, ctypes.c_int, vp, sz, vp]
        lib.wfd_backward.argtypes = [P, f, f, f, f, f, i32, i32, f, f, f, vp, sz, vp]
        lib.wfd_misfit_gradient.argtypes = [P, f, f, f, f, f, i32, i32, f, f, f, f, d, vp, sz, vp]
        lib.wfd_misfit_gradient_overlap.argtypes = [P, f, f, f, f, f, i32, i32, f, vp, f, f, f, d, vp, sz, vp]
        lib.wfd_status.argtypes = [vp, vp]
        lib.wfd_sum_sq.argtypes = [f, ctypes.c_int64, d, vp]
        lib.wfd_step2d_order2.argtypes = [f, f, f, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                          ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
        lib.wfd_forward_static.argtypes = [P, f, f, f, f, f, i32, i32, f, vp]
        lib.wfd_forward_static_status.argtypes = [vp]
        lib.wfd_forward_final.argtypes = [P, f, f, f, f, f, i32, i32, f, f, vp, sz, vp]
        lib.wfd_analytic_signal.argtypes = [f, ctypes.c_int64, ctypes.c_int, f, f, vp]
        F, I = ctypes.c_float, ctypes.c_int
        lib.wfd_tfm.argtypes = [f, I, f, f, I, F, F, F, f, f, I, I, f, vp]
        lib.wfd_step2d_mixed.argtypes = [vp, vp, vp, F, F, F, F, I, I, I, vp]
        lib.wfd_step2d_mixed_fast.argtypes = [vp, vp, vp, F, F, F, F, I, I, I, vp]
        lib.wfd_temporal_step.argtypes = [vp, vp, vp, vp, F, F, F, F, I, I, I, vp]
        lib.wfd_temporal_step_fast.argtypes = [vp, vp, vp, vp, F, F, F, F, I, I, I, vp]
        lib.wfd_step2d_exact.argtypes = [vp, vp, vp, F, F, F, F, I, I, I, vp]
        lib.wfd_step2d_scaled.argtypes = [vp, f, vp, f, vp, f, F, F, F, F, I, I, I, vp]
        lib.wfd_step1d.argtypes = [f, f, f, F, F, F, I, vp]
        lib.wfd_vd_workspace_bytes.argtypes = [P, ctypes.c_int, ctypes.POINTER(sz)]
        lib.wfd_vd_forward.argtypes = [P, f, f, f, f, f, i32, i32, f, vp, sz, vp]
        lib.wfd_vd_forward_final.argtypes = [P, f, f, f, f, f, i32, i32, f, f, vp, sz, vp]
        lib.wfd_vd_misfit_gradient.argtypes = [P, f, f, f, f, f, i32, i32, f, f, f, f, f, d, vp, sz, vp]
        lib.wfd_kernel_launches.argtypes = []
        lib.wfd_kernel_launches.restype = ctypes.c_uint64
        lib.wfd_batch_plan.argtypes = [ctypes.POINTER(BatchItem), ctypes.c_int, vp, ctypes.POINTER(vp)]
        lib.wfd_batch_run.argtypes = [vp, vp]
        lib.wfd_batch_launches.argtypes = [vp]
        lib.wfd_batch_launches.restype = ctypes.c_uint64
        lib.wfd_batch_free.argtypes = [vp]
        lib.wfd_profile_begin.argtypes = []
        lib.wfd_profile_end.argtypes = [ctypes.POINTER(PhaseTimes)]
        for name in EXPORTS:
            if name not in ("wfd_strerror", "wfd_last_error", "wfd_kernel_launches", "wfd_batch_launches"):
                getattr(lib, name).restype = ctypes.c_int
        _lib = lib
        return lib


def check(status: int, where: str) -> None:
    if status != WFD_OK:
        lib = load()
        detail = lib.wfd_last_error().decode() or lib.wfd_strerror(status).decode()
        raise WaveFDError(status, where, detail)
