"""GB300-native finite-difference acoustic wave path (drop-in for the
wave-solver call of cmpmech/neuralmech's 18_simple_wave_fd / 18_fwi drivers).

Host side: Python over PyTorch tensors. Device side: hand-written sm_103a CUDA
kernels in libwavefd.so behind the C ABI of include/wavefd.h.
"""
from . import autotune
from .wavefd import (Grid, fd_weights, levels_for_budget, misfit_gradient, sponge_profile,
                     sponge_profiles, stable_dt, step2d_order2, sum_sq, wave_forward, workspace_bytes)

__all__ = ["autotune", "Grid", "fd_weights", "levels_for_budget", "misfit_gradient", "sponge_profile", "sponge_profiles",
           "stable_dt", "step2d_order2", "sum_sq", "wave_forward", "workspace_bytes"]
