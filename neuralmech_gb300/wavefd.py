"""Python host API of the GB300 finite-difference acoustic wave path.

PyTorch tensors in, PyTorch tensors out; every call goes through the C ABI of
libwavefd.so (include/wavefd.h) on the current CUDA stream. There is no CPU
path: tensors must live on a CUDA device.

Mapping to the reference (cmpmech/neuralmech):
  * ``step2d_order2``  <- padded_step, projects/18_simple_wave_fd/step2D_wave.cu:59-81
    as driven by 2D_wave_cuda_padding.py:66-76 (same arguments, u2 may alias u0);
  * ``wave_forward``   <- cuwave ``measure(sim, sources, indicator, sensors)``
    (projects/18_fwi/plate.py:62-64): one forward per shot, traces stacked
    (shot, step, receiver); differentiable through ``torch.autograd``;
  * ``misfit_gradient`` <- cuwave ``misfit_gradient(sim, sources, gamma, sensors,
    observed) -> (cost, gradient)`` (projects/18_fwi/2D_fwi.py:40), here with
    respect to the velocity (and optionally the wavelets);
  * ``stable_dt``      <- cuwave ``stable_dt(dx, c, order)`` (projects/18_fwi/helper.py:52).

Discretisation (shared with the FP64 oracle):
  u_{n+1} = g (2 u_n + (v dt)^2 L u_n + src_scale w_n) - g^2 u_{n-1}
on the interior; the outer ring of order/2 cells stays 0; L is the central
Laplacian of space order 2, 4 or 8; g the product of the per-axis
exponential (Cerjan) sponge profiles; traces[s, n, r] = u_{n+1}(rec[s, r]).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib


# ---------------------------------------------------------------- descriptors
CKPT_FORMATS = {"fp32": 0, "bf16": 1, "i16": 2}
LAP_STORES = {"auto": 0, "bf16": 1, "fp32": 2}
FIELD_FORMATS = {"fp32": 0, "fp16": 1, "i16": 2}
ADJOINT_MODES = {"checkpoint": 0, "reconstruct": 1}
UPDATE_FORMS = {"auto": 0, "leapfrog": 1, "summed": 2}
LEVEL_FORMATS = {"fp32": 0, "bfp16": 1}


@dataclass(frozen=True)
class Grid:
    """Simulation descriptor (the role of cuwave's ``ScalarWave``).

    shape    (nz, nx) or (nz, ny, nx) cells
    spacing  (dz, dx) or (dz, dy, dx)
    dt, nt   time step and number of steps
    order    space order (2, 4, 8)
    sponge   sponge width in cells: one int for every face, or one
             (low, high) pair per axis
    sponge_strength  alpha W of the taper exp(-(alpha d)^2), d the depth into
             the layer (1 .. W); 0.3 gives the classic Cerjan wall factor 0.914
    ckpt_every   steps between checkpoints of the adjoint (0 = ceil(sqrt(nt)))
    ckpt_format  checkpoint snapshots: "fp32", "bf16" or "i16" (int16 with one
             FP32 scale per 32 cells)
    lap_store    what the adjoint keeps of each recomputed step for its imaging
             term: "auto" (2D one-step kernel: the level u_k, which the
             recompute writes anyway, with L u_k formed by the adjoint; else
             FP32 L u_k), "fp32" or "bf16" (L u_k stored in that type)
    shots_per_cta  shots one CTA walks through per step (0 = automatic)
    group_shots  run the shots of a misfit gradient (or of a forward without
             autograd) in sequential groups of this many, sharing one workspace
             sized for a group (0 = all at once)
    tile_rows    2D tile height, 16 or 32 rows (0 = 32)
    step_block   2D time steps per kernel launch, 1 or 2 (0 = 1); for a
             forward (no gradient) with the leapfrog update and FP32 fields
             also 8 at order 2 or 4 at order 4 (a register window per CTA)
    store_levels levels the adjoint's workspace may hold (lap_store "auto"):
             the forward keeps the levels of its last (store_levels - 2) // K
             segments and only the earlier ones are recomputed (0: the last
             segment only); see levels_for_budget()
    level_format how those kept levels are stored: "fp32" (4 B per cell) or
             "bfp16" (block floating point: int16 mantissas and one exponent
             byte per 4 cells along x, 2.25 B per cell, each value within 2^-15
             of its block's largest; about 1.8x the kept levels in the same
             memory; 2D, step_block 2, the summed forward)
    field_format storage of the wavefields in a forward without gradient (2D):
             "fp32", "fp16" or "i16" (int16 with one FP32 scale per 32 cells
             along x); arithmetic is FP32 in every format
    adjoint      how the gradient obtains the forward levels (2D): "checkpoint"
             (checkpoints, kept levels, recomputed segments) or "reconstruct"
             (time reversal from the last two levels; the sponge frame of every
             level is saved by the forward instead of checkpoints)
    update       how the forward evaluates the update: "leapfrog" (u_{n+1} over
             u_{n-1}, 16 B per update), "summed" (state u_n and the increment
             d_n = u_n - u_{n-1}, d_{n+1} = g^2 d_n - (1 - g)^2 u_n + g m L u_n,
             u_{n+1} = u_n + d_{n+1}: the FP32 rounding of the increment is no
             longer that of |u|, so a misfit gradient whose residuals are much
             smaller than the traces keeps its accuracy; 20 B per update, 10
             with step_block 2 in 2D; 2D and 3D, FP32 fields, lap_store "auto",
             checkpoint adjoint) or
             "auto" (summed for the forward of a gradient where available,
             leapfrog otherwise)
    """
    shape: tuple
    spacing: tuple
    dt: float
    nt: int
    order: int = 8
    sponge: object = 20
    sponge_strength: float = 0.3
    src_scale: float = 1.0
    ckpt_every: int = 0
    ckpt_format: str = "bf16"
    lap_store: str = "auto"
    shots_per_cta: int = 0
    group_shots: int = 0
    tile_rows: int = 0
    step_block: int = 0
    store_levels: int = 0
    field_format: str = "fp32"
    adjoint: str = "checkpoint"
    update: str = "auto"
    level_format: str = "fp32"

    @property
    def ndim(self) -> int:
        return len(self.shape)

    def sponge_widths(self):
        if isinstance(self.sponge, int):
            return [(self.sponge, self.sponge)] * self.ndim
        w = [tuple(p) for p in self.sponge]
        if len(w) != self.ndim:
            raise ValueError("sponge needs one (low, high) pair per axis")
        return w


def fd_weights(order: int) -> np.ndarray:
    """Central second-derivative weights a_0..a_R of space order ``order``."""
    R = order // 2
    a = np.zeros(R + 1)
    for k in range(1, R + 1):
        a[k] = 2.0 * (1 if k % 2 else -1) * math.factorial(R) ** 2 / (
            k * k * math.factorial(R - k) * math.factorial(R + k))
    a[0] = -2.0 * a[1:].sum()
    return a


def levels_for_budget(grid: Grid, nshot: int, budget_bytes: float) -> int:
    """store_levels that fit `budget_bytes` of kept levels in the grid's
    level_format (nshot fields of the grid, rows padded to 8 cells; "bfp16":
    2-byte mantissas plus one exponent byte per 4 cells, exponent rows padded
    to 16 bytes)."""
    nx = grid.shape[-1]
    ld = (nx + 7) // 8 * 8
    rows = int(np.prod(grid.shape[:-1]))
    if grid.level_format == "bfp16":
        per = nshot * rows * (2 * ld + (ld // 4 + 15) // 16 * 16)
    else:
        per = 4 * nshot * rows * ld
    return max(0, int(budget_bytes // per))


def stable_dt(spacing, vmax: float, order: int = 8) -> float:
    """Largest stable leapfrog step: vmax dt sqrt(sum_axis S / h^2) <= 2,
    S = |a_0| + 2 sum |a_k| (0.5547 h / vmax in 2D, 0.4529 in 3D, order 8)."""
    a = fd_weights(order)
    S = abs(a[0]) + 2 * np.abs(a[1:]).sum()
    return 2.0 / (vmax * math.sqrt(S * sum(1.0 / h**2 for h in spacing)))


def sponge_profile(n: int, low: int, high: int, strength: float = 0.3) -> np.ndarray:
    """1D exponential sponge factors g[0..n-1] (1 in the interior)."""
    g = np.ones(n, dtype=np.float64)
    for w, idx in ((low, lambda d: w - d), (high, lambda d: n - 1 - (w - d))):
        if w <= 0:
            continue
        a = strength / w
        for d in range(1, w + 1):
            i = idx(d)
            if 0 <= i < n:
                g[i] = math.exp(-(a * d) ** 2)
    return g.astype(np.float32)


def sponge_profiles(grid: Grid):
    """(gz, gy, gx) FP32 profiles (gy None in 2D); None where the width is 0."""
    widths = grid.sponge_widths()
    prof = []
    for n, (lo, hi) in zip(grid.shape, widths):
        prof.append(None if lo == 0 and hi == 0 else sponge_profile(n, lo, hi, grid.sponge_strength))
    if grid.ndim == 2:
        return prof[0], None, prof[1]
    return tuple(prof)


def _problem(grid: Grid, nshot: int, nsrc: int, nrec: int, vmax: float) -> _lib.Problem:
    if grid.ndim == 2:
        nz, nx = grid.shape
        ny = 1
        dz, dx = grid.spacing
        dy = 1.0
    else:
        nz, ny, nx = grid.shape
        dz, dy, dx = grid.spacing
    return _lib.Problem(grid.ndim, grid.order, nz, ny, nx, nshot, grid.nt, nsrc, nrec,
                        grid.ckpt_every, CKPT_FORMATS[grid.ckpt_format], LAP_STORES[grid.lap_store],
                        grid.shots_per_cta, grid.group_shots, grid.tile_rows, grid.step_block, grid.store_levels,
                        FIELD_FORMATS[grid.field_format], ADJOINT_MODES[grid.adjoint],
                        max(max(w) for w in grid.sponge_widths()) if grid.adjoint == "reconstruct" else 0,
                        grid.dt, dz, dy, dx, grid.src_scale, vmax, UPDATE_FORMS[grid.update],
                        LEVEL_FORMATS[grid.level_format])


# ---------------------------------------------------------------- argument prep
def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _require_cuda(t: torch.Tensor, name: str):
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (no CPU path)")


def _positions(pos, nshot: int, ndim: int, device) -> torch.Tensor:
    """(nshot, n, 3) int32 (z, y, x) from (n, ndim) or (nshot, n, ndim)."""
    p = torch.as_tensor(pos, device=device)
    if p.dim() == 2:
        p = p.unsqueeze(0).expand(nshot, -1, -1)
    if p.dim() != 3 or p.shape[0] != nshot or p.shape[2] != ndim:
        raise ValueError(f"positions must be (n, {ndim}) or ({nshot}, n, {ndim})")
    p = p.to(torch.int32)
    if ndim == 2:
        p = torch.stack([p[..., 0], torch.zeros_like(p[..., 0]), p[..., 1]], dim=-1)
    return p.contiguous()


def _wavelet(w, nshot: int, nt: int, nsrc: int, device) -> torch.Tensor:
    """(nshot, nt, nsrc) FP32 from (nt,), (nshot, nt) or (nshot, nt, nsrc)."""
    w = torch.as_tensor(w, device=device, dtype=torch.float32)
    if w.dim() == 1:
        w = w.view(1, -1, 1).expand(nshot, -1, nsrc)
    elif w.dim() == 2:
        w = w.unsqueeze(-1).expand(-1, -1, nsrc)
    if tuple(w.shape) != (nshot, nt, nsrc):
        raise ValueError(f"wavelet must broadcast to ({nshot}, {nt}, {nsrc})")
    return w.contiguous()


@dataclass
class _Call:
    grid: Grid
    problem: _lib.Problem
    vel: torch.Tensor
    wavelet: torch.Tensor
    src: torch.Tensor
    rec: torch.Tensor
    sponges: tuple = field(default_factory=tuple)


def _prepare(vel, wavelet, src, rec, grid: Grid, nshot=None) -> _Call:
    _require_cuda(vel, "vel")
    if tuple(vel.shape) != tuple(grid.shape):
        raise ValueError(f"vel has shape {tuple(vel.shape)}, grid {grid.shape}")
    vel = vel.detach().to(torch.float32).contiguous()
    dev = vel.device
    src_t = torch.as_tensor(src)
    if nshot is None:
        nshot = src_t.shape[0] if src_t.dim() == 3 else 1
    srcp = _positions(src, nshot, grid.ndim, dev)
    recp = _positions(rec, nshot, grid.ndim, dev)
    wav = _wavelet(wavelet, nshot, grid.nt, srcp.shape[1], dev)
    vmax = float(vel.max())
    prob = _problem(grid, nshot, srcp.shape[1], recp.shape[1], vmax)
    gz, gy, gx = sponge_profiles(grid)
    sp = tuple(None if g is None else torch.from_numpy(g).to(dev) for g in (gz, gy, gx))
    return _Call(grid, prob, vel, wav, srcp, recp, sp)


def workspace_bytes(grid: Grid, nshot: int, nsrc: int, nrec: int, with_gradient: bool) -> int:
    lib = _lib.load()
    n = ctypes.c_size_t(0)
    _lib.check(lib.wfd_workspace_bytes(ctypes.byref(_problem(grid, nshot, nsrc, nrec, 0.0)),
                                       int(with_gradient), ctypes.byref(n)), "wfd_workspace_bytes")
    return n.value


def _workspace(c: _Call, with_gradient: bool) -> torch.Tensor:
    lib = _lib.load()
    n = ctypes.c_size_t(0)
    _lib.check(lib.wfd_workspace_bytes(ctypes.byref(c.problem), int(with_gradient), ctypes.byref(n)),
               "wfd_workspace_bytes")
    ws = torch.empty(n.value + 256, dtype=torch.uint8, device=c.vel.device)
    off = (-ws.data_ptr()) % 256
    return ws[off:off + n.value]


def _status(ws: torch.Tensor, where: str):
    _lib.check(_lib.load().wfd_status(_ptr(ws), _stream()), where)


# ---------------------------------------------------------------- autograd
class _WaveForward(torch.autograd.Function):
    """Traces from (vel, wavelet); backward = the hand-written adjoint."""

    @staticmethod
    def forward(ctx, vel, wavelet, call: _Call, check: bool):
        lib = _lib.load()
        call.problem.group_shots = 0  # the checkpointed forward keeps every shot's state
        ws = _workspace(call, True)
        c = call
        traces = torch.empty((c.problem.nshot, c.problem.nt, c.problem.nrec),
                             dtype=torch.float32, device=vel.device)
        gz, gy, gx = c.sponges
        _lib.check(lib.wfd_forward(ctypes.byref(c.problem), _ptr(c.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                                   _ptr(c.wavelet), _ptr(c.src), _ptr(c.rec), _ptr(traces), 1,
                                   _ptr(ws), ws.numel(), _stream()), "wfd_forward")
        if check:
            _status(ws, "wfd_forward")
        ctx.call = call
        ctx.ws = ws
        ctx.check = check
        ctx.wavelet_shape = wavelet.shape
        return traces

    @staticmethod
    def backward(ctx, dtraces):
        lib = _lib.load()
        c = ctx.call
        if ctx.ws is None:  # a second backward: redo the checkpointed forward first
            ctx.ws = _workspace(c, True)
            gz, gy, gx = c.sponges
            _lib.check(lib.wfd_forward(ctypes.byref(c.problem), _ptr(c.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                                       _ptr(c.wavelet), _ptr(c.src), _ptr(c.rec), None, 1,
                                       _ptr(ctx.ws), ctx.ws.numel(), _stream()), "wfd_forward")
        ws = ctx.ws
        dtraces = dtraces.to(torch.float32).contiguous()
        grad_vel = torch.empty_like(c.vel)
        want_wav = ctx.needs_input_grad[1]
        grad_wav = torch.empty_like(c.wavelet) if want_wav else None
        gz, gy, gx = c.sponges
        _lib.check(lib.wfd_backward(ctypes.byref(c.problem), _ptr(c.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                                    _ptr(c.wavelet), _ptr(c.src), _ptr(c.rec), _ptr(dtraces),
                                    _ptr(grad_vel), _ptr(grad_wav), _ptr(ws), ws.numel(), _stream()),
                   "wfd_backward")
        if ctx.check:
            _status(ws, "wfd_backward")
        ctx.ws = None
        gw = None
        if want_wav:
            gw = grad_wav
            shape = ctx.wavelet_shape
            if len(shape) == 1:
                gw = gw.sum(dim=(0, 2))
            elif len(shape) == 2:
                gw = gw.sum(dim=2)
        return (grad_vel if ctx.needs_input_grad[0] else None), gw, None, None


# ---------------------------------------------------------------- public API
def wave_forward(vel: torch.Tensor, wavelet, src, rec, grid: Grid, *, check: bool = True):
    """Traces (nshot, nt, nrec) of every shot through the velocity ``vel``.

    vel      (nz, nx) / (nz, ny, nx) CUDA tensor (m/s); differentiable
    wavelet  (nt,), (nshot, nt) or (nshot, nt, nsrc); differentiable
    src, rec (n, ndim) shared by all shots or (nshot, n, ndim) integer cells
             (z, x) / (z, y, x), inside the interior (>= order/2 from every edge)
    check    synchronise and raise on device-side errors (bad positions, timeouts)
    """
    wav_t = torch.as_tensor(wavelet, device=vel.device)
    nshot = None
    s = torch.as_tensor(src)
    if s.dim() == 3:
        nshot = s.shape[0]
    elif wav_t.dim() >= 2:
        nshot = wav_t.shape[0]
    call = _prepare(vel, wav_t.detach(), src, rec, grid, nshot)
    if torch.is_grad_enabled() and (vel.requires_grad or wav_t.requires_grad):
        if grid.field_format != "fp32":
            raise ValueError("reduced-precision field storage is a forward-only mode: use fp32 for gradients")
        return _WaveForward.apply(vel, wav_t, call, check)
    lib = _lib.load()
    ws = _workspace(call, False)
    p = call.problem
    traces = torch.empty((p.nshot, p.nt, p.nrec), dtype=torch.float32, device=vel.device)
    gz, gy, gx = call.sponges
    _lib.check(lib.wfd_forward(ctypes.byref(p), _ptr(call.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                               _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec), _ptr(traces), 0,
                               _ptr(ws), ws.numel(), _stream()), "wfd_forward")
    if check:
        _status(ws, "wfd_forward")
    return traces


def wave_forward_final(vel: torch.Tensor, wavelet, src, rec, grid: Grid, *, check: bool = True):
    """(traces, u_final): the forward plus the last wavefield u_nt of every
    shot, shaped (nshot,) + grid.shape (no autograd)."""
    wav_t = torch.as_tensor(wavelet, device=vel.device)
    s = torch.as_tensor(src)
    nshot = s.shape[0] if s.dim() == 3 else (wav_t.shape[0] if wav_t.dim() >= 2 else None)
    call = _prepare(vel, wav_t, src, rec, grid, nshot)
    call.problem.group_shots = 0
    p = call.problem
    ws = _workspace(call, False)
    traces = torch.empty((p.nshot, p.nt, p.nrec), dtype=torch.float32, device=vel.device)
    final = torch.empty((p.nshot,) + tuple(grid.shape), dtype=torch.float32, device=vel.device)
    gz, gy, gx = call.sponges
    _lib.check(_lib.load().wfd_forward_final(ctypes.byref(p), _ptr(call.vel), _ptr(gz), _ptr(gy), _ptr(gx),
                                             _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec),
                                             _ptr(traces), _ptr(final), _ptr(ws), ws.numel(), _stream()),
               "wfd_forward_final")
    if check:
        _status(ws, "wfd_forward_final")
    return traces, final


def misfit_gradient(vel: torch.Tensor, wavelet, src, rec, observed: torch.Tensor, grid: Grid, *,
                    want_wavelet: bool = False, want_traces: bool = False, check: bool = True,
                    observed_ready: torch.cuda.Event | None = None):
    """(misfit, grad_vel[, grad_wavelet][, traces]) in one library call.

    misfit = 1/2 sum (traces - observed)^2, accumulated in FP64 on the GPU
    (a 0-d float64 tensor); grad_vel has vel's shape (0 on the fixed ring).
    observed_ready: an event recorded after the (asynchronous) copy that fills
    ``observed``; the call waits for it only after the forward, so the copy
    overlaps the forward (``observed`` must then be a contiguous float32
    tensor, read in place)."""
    wav_t = torch.as_tensor(wavelet, device=vel.device)
    nshot = observed.shape[0]
    call = _prepare(vel, wav_t, src, rec, grid, nshot)
    _require_cuda(observed, "observed")
    p = call.problem
    if tuple(observed.shape) != (p.nshot, p.nt, p.nrec):
        raise ValueError(f"observed must be ({p.nshot}, {p.nt}, {p.nrec})")
    if observed_ready is not None and (observed.dtype != torch.float32 or not observed.is_contiguous()):
        raise ValueError("with observed_ready, observed must be a contiguous float32 tensor")
    obs = observed.to(torch.float32).contiguous()
    ws = _workspace(call, True)
    grad = torch.empty_like(call.vel)
    gwav = torch.empty_like(call.wavelet) if want_wavelet else None
    traces = torch.empty_like(obs) if want_traces else None
    misfit = torch.zeros((), dtype=torch.float64, device=vel.device)
    _misfit_gradient_into(call, obs, ws, grad, misfit, gwav, traces, observed_ready)
    if check:
        _status(ws, "wfd_misfit_gradient")
    out = [misfit, grad]
    if want_wavelet:
        out.append(gwav)
    if want_traces:
        out.append(traces)
    return tuple(out)


def _misfit_gradient_into(call: _Call, obs, ws, grad, misfit, gwav=None, traces=None, observed_ready=None):
    """wfd_misfit_gradient into caller buffers on the current stream (no
    allocation, no synchronisation: safe inside CUDA-graph capture)."""
    gz, gy, gx = call.sponges
    lib = _lib.load()
    head = (ctypes.byref(call.problem), _ptr(call.vel), _ptr(gz), _ptr(gy), _ptr(gx), _ptr(call.wavelet),
            _ptr(call.src), _ptr(call.rec), _ptr(obs))
    tail = (_ptr(traces), _ptr(grad), _ptr(gwav), _ptr(misfit), _ptr(ws), ws.numel(), _stream())
    if observed_ready is None:
        _lib.check(lib.wfd_misfit_gradient(*head, *tail), "wfd_misfit_gradient")
    else:
        _lib.check(lib.wfd_misfit_gradient_overlap(*head, observed_ready._as_parameter_, *tail),
                   "wfd_misfit_gradient_overlap")


def sum_sq(x: torch.Tensor) -> torch.Tensor:
    """FP64 sum of squares of an FP32 CUDA tensor (gradient norms)."""
    _require_cuda(x, "x")
    x = x.to(torch.float32).contiguous()
    out = torch.zeros((), dtype=torch.float64, device=x.device)
    _lib.check(_lib.load().wfd_sum_sq(_ptr(x), x.numel(), _ptr(out), _stream()), "wfd_sum_sq")
    return out


def _check_fields(dtype, names_tensors, dim):
    for n, t in names_tensors:
        _require_cuda(t, n)
        if t.dtype != dtype or not t.is_contiguous() or t.dim() != dim:
            raise ValueError(f"{n} must be a contiguous {dim}D {dtype} tensor")


def step2d_mixed(u0, u1, u2, wavespeed: float, dt: float, dx: float, dy: float, N: int, M: int):
    """mixed_step (step2D_wave.cu:85-124): the padded_step update on (N, M_padded)
    float16 CUDA tensors, FP32 arithmetic; u2 may be u0."""
    _check_fields(torch.float16, (("u0", u0), ("u1", u1), ("u2", u2)), 2)
    _lib.check(_lib.load().wfd_step2d_mixed(_ptr(u0), _ptr(u1), _ptr(u2), wavespeed, dt, dx, dy,
                                            N, M, u1.shape[1], _stream()), "wfd_step2d_mixed")
    return u2


def step2d_mixed_fast(u0, u1, u2, wavespeed: float, dt: float, dx: float, dy: float, N: int, M: int):
    """mixed_step's update on (N, M_padded) float16 tensors with pre-divided
    weights and FMAs (within an FP16 rounding of the reference's fast-math
    build); M_padded a multiple of 8; u2 may be u0."""
    _check_fields(torch.float16, (("u0", u0), ("u1", u1), ("u2", u2)), 2)
    _lib.check(_lib.load().wfd_step2d_mixed_fast(_ptr(u0), _ptr(u1), _ptr(u2), wavespeed, dt, dx, dy,
                                                 N, M, u1.shape[1], _stream()), "wfd_step2d_mixed_fast")
    return u2


def step2d_exact(u0, u1, u2, wavespeed: float, dt: float, dx: float, dy: float, N: int, M: int):
    """padded_step / shared_step (M_padded = u1.shape[1]) or basic_step /
    coalesced_step (M_padded = M) evaluated as the reference kernels evaluate
    them, value for value; (N, M_padded) float32 CUDA tensors, u2 may be u0."""
    _check_fields(torch.float32, (("u0", u0), ("u1", u1), ("u2", u2)), 2)
    _lib.check(_lib.load().wfd_step2d_exact(_ptr(u0), _ptr(u1), _ptr(u2), wavespeed, dt, dx, dy,
                                            N, M, u1.shape[1], _stream()), "wfd_step2d_exact")
    return u2


def temporal_step(u0, u1, v0, v1, wavespeed: float, dt: float, dx: float, dy: float, N: int, M: int):
    """temporal_step (step2D_wave.cu:244-304): eight padded_step updates in one
    launch; from u0 = u_{n-1}, u1 = u_n ((N, M_padded) float32 CUDA tensors)
    v0 receives u_{n+7} and v1 u_{n+8}. v0, v1 must be separate tensors."""
    _check_fields(torch.float32, (("u0", u0), ("u1", u1), ("v0", v0), ("v1", v1)), 2)
    _lib.check(_lib.load().wfd_temporal_step(_ptr(u0), _ptr(u1), _ptr(v0), _ptr(v1), wavespeed, dt, dx, dy,
                                             N, M, u1.shape[1], _stream()), "wfd_temporal_step")
    return v0, v1


def temporal_step_fast(u0, u1, v0, v1, wavespeed: float, dt: float, dx: float, dy: float, N: int, M: int):
    """temporal_step's eight updates with pre-divided weights and fused
    multiply-adds (no division per cell): within FP32 rounding of the
    reference expression, as the reference's --use_fast_math build is."""
    _check_fields(torch.float32, (("u0", u0), ("u1", u1), ("v0", v0), ("v1", v1)), 2)
    _lib.check(_lib.load().wfd_temporal_step_fast(_ptr(u0), _ptr(u1), _ptr(v0), _ptr(v1), wavespeed, dt, dx, dy,
                                                  N, M, u1.shape[1], _stream()), "wfd_temporal_step_fast")
    return v0, v1


def step2d_scaled(q0, s0, q1, s1, q2, s2, wavespeed: float, dt: float, dx: float, dy: float, N: int,
                  M: int):
    """scaled_step (step2D_wave.cu:128-183): the padded_step update on int16
    fields q (N, M_padded) with one float32 scale per 32 values, s (N, M_padded / 32),
    u = s q; (q2, s2) may be (q0, s0)."""
    _check_fields(torch.int16, (("q0", q0), ("q1", q1), ("q2", q2)), 2)
    _check_fields(torch.float32, (("s0", s0), ("s1", s1), ("s2", s2)), 2)
    if s1.shape[1] * 32 != q1.shape[1]:
        raise ValueError("s must have M_padded / 32 columns")
    _lib.check(_lib.load().wfd_step2d_scaled(_ptr(q0), _ptr(s0), _ptr(q1), _ptr(s1), _ptr(q2), _ptr(s2),
                                             wavespeed, dt, dx, dy, N, M, q1.shape[1], _stream()),
               "wfd_step2d_scaled")
    return q2, s2


def step1d(u0, u1, u2, wavespeed: float, dt: float, dx: float):
    """step1D (step1D_wave.cu:4-17) on (N,) float32 CUDA tensors; u2 may be u0."""
    _check_fields(torch.float32, (("u0", u0), ("u1", u1), ("u2", u2)), 1)
    _lib.check(_lib.load().wfd_step1d(_ptr(u0), _ptr(u1), _ptr(u2), wavespeed, dt, dx, u1.shape[0],
                                      _stream()), "wfd_step1d")
    return u2


def step2d_order2(u0, u1, u2, wavespeed: float, dt: float, dx: float, dy: float, N: int, M: int):
    """padded_step (step2D_wave.cu:59-81): u2 <- -u0 + 2u1 + dt^2 c^2 Lap(u1) on
    rows 1..N-2, columns 1..M-2 of (N, M_padded) FP32 CUDA tensors; u2 may be u0."""
    for t, n in ((u0, "u0"), (u1, "u1"), (u2, "u2")):
        _require_cuda(t, n)
        if t.dtype != torch.float32 or not t.is_contiguous() or t.dim() != 2:
            raise ValueError(f"{n} must be a contiguous 2D float32 tensor")
    _lib.check(_lib.load().wfd_step2d_order2(_ptr(u0), _ptr(u1), _ptr(u2), wavespeed, dt, dx, dy,
                                             N, M, u1.shape[1], _stream()), "wfd_step2d_order2")
    return u2


# ---------------------------------------------------------------- variable density
def _vd_prepare(kappa, rho, wavelet, src, rec, grid: Grid, nshot=None):
    if grid.ndim != 2:
        raise ValueError("variable density is 2D")
    _require_cuda(rho, "rho")
    if tuple(rho.shape) != tuple(grid.shape):
        raise ValueError(f"rho has shape {tuple(rho.shape)}, grid {grid.shape}")
    rho = rho.detach().to(torch.float32).contiguous()
    call = _prepare(kappa, torch.as_tensor(wavelet, device=kappa.device), src, rec, grid, nshot)
    call.problem.vmax = vd_vmax(call.vel, rho, grid.order, grid.spacing)
    return call, rho


def _stag_weights(R: int) -> list:
    """Staggered first-derivative weights c_1..c_R (unit grid): the
    Lagrange-product form, exact on polynomials up to degree 2R - 1."""
    c = []
    for k in range(1, R + 1):
        v = 1.0 / (2 * k - 1)
        for m in range(1, R + 1):
            if m != k:
                a, b = (2 * m - 1) ** 2, (2 * k - 1) ** 2
                v *= a / (a - b)
        c.append(v)
    return c


def vd_vmax(kappa: torch.Tensor, rho: torch.Tensor, order: int, spacing=(1.0, 1.0)) -> float:
    """The speed that bounds the variable-density operator for the CFL check
    (vmax dt sqrt(S (1/dz^2 + 1/dx^2)) <= 2, S = 4 (sum |c_k|)^2).

    Row i of kappa Lb along one axis is kappa_i sum_k c_k (F_{i+k-1/2} -
    F_{i-k+1/2}) with F = b_half D u, b_half the mean of two cells' b = 1/rho.
    Its absolute sum is at most kappa_i 2 sum|c| B_i, B_i = sum_k |c_k|
    (b_{i+k-1/2} + b_{i-k+1/2}), which bounds the spectral radius
    (Gershgorin). vmax^2 = max_i kappa_i (B_i^z / dz^2 + B_i^x / dx^2) /
    (2 sum|c| (1/dz^2 + 1/dx^2)): max kappa / rho in a smooth medium, larger
    where 1/rho jumps (air beside a solid), where a cell's stiffness meets its
    neighbour's large 1/rho and the step's stability follows that product."""
    R = order // 2
    c = _stag_weights(R)
    csum = sum(abs(v) for v in c)
    b = 1.0 / rho.detach().double()
    kap = kappa.detach().double()
    dz, dx = float(spacing[0]), float(spacing[-1])

    def B(f):  # along the last axis of f
        n = f.shape[-1]
        fp = torch.nn.functional.pad(f, (R + 1, R + 1))   # b zero outside the grid
        bh = 0.5 * (fp[..., :-1] + fp[..., 1:])           # bh[.., q] = b at q - R - 1/2
        out = torch.zeros_like(f)
        for k in range(1, R + 1):
            # half points i + k - 1/2 and i - k + 1/2 are q = i + k + R and q = i - k + R + 1
            out += abs(c[k - 1]) * (bh[..., k + R:k + R + n] + bh[..., R + 1 - k:R + 1 - k + n])
        return out

    row = kap * (B(b.t()).t() / dz ** 2 + B(b) / dx ** 2)
    return float(torch.sqrt(row.max() / (2.0 * csum * (1.0 / dz ** 2 + 1.0 / dx ** 2))))


def _vd_workspace(call: _Call, with_gradient: bool) -> torch.Tensor:
    lib = _lib.load()
    n = ctypes.c_size_t(0)
    _lib.check(lib.wfd_vd_workspace_bytes(ctypes.byref(call.problem), int(with_gradient), ctypes.byref(n)),
               "wfd_vd_workspace_bytes")
    ws = torch.empty(n.value + 256, dtype=torch.uint8, device=call.vel.device)
    off = (-ws.data_ptr()) % 256
    return ws[off:off + n.value]


def vd_forward(kappa: torch.Tensor, rho: torch.Tensor, wavelet, src, rec, grid: Grid, *, check: bool = True):
    """Traces (nshot, nt, nrec) of the variable-density acoustic medium
    p_tt = kappa div(grad p / rho) + s (2D, staggered order-`grid.order`
    operator; kappa, rho (nz, nx) CUDA tensors)."""
    call, rho = _vd_prepare(kappa, rho, wavelet, src, rec, grid)
    p = call.problem
    ws = _vd_workspace(call, False)
    traces = torch.empty((p.nshot, p.nt, p.nrec), dtype=torch.float32, device=kappa.device)
    gz, _, gx = call.sponges
    _lib.check(_lib.load().wfd_vd_forward(ctypes.byref(p), _ptr(call.vel), _ptr(rho), _ptr(gz), _ptr(gx),
                                          _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec), _ptr(traces),
                                          _ptr(ws), ws.numel(), _stream()), "wfd_vd_forward")
    if check:
        _status(ws, "wfd_vd_forward")
    return traces


def vd_forward_final(kappa: torch.Tensor, rho: torch.Tensor, wavelet, src, rec, grid: Grid, *,
                     check: bool = True):
    """(traces, u_final): vd_forward plus the last field u_nt of every shot,
    shaped (nshot,) + grid.shape (no autograd)."""
    call, rho = _vd_prepare(kappa, rho, wavelet, src, rec, grid)
    p = call.problem
    ws = _vd_workspace(call, False)
    traces = torch.empty((p.nshot, p.nt, p.nrec), dtype=torch.float32, device=kappa.device)
    final = torch.empty((p.nshot,) + tuple(grid.shape), dtype=torch.float32, device=kappa.device)
    gz, _, gx = call.sponges
    _lib.check(_lib.load().wfd_vd_forward_final(ctypes.byref(p), _ptr(call.vel), _ptr(rho), _ptr(gz), _ptr(gx),
                                                _ptr(call.wavelet), _ptr(call.src), _ptr(call.rec), _ptr(traces),
                                                _ptr(final), _ptr(ws), ws.numel(), _stream()),
               "wfd_vd_forward_final")
    if check:
        _status(ws, "wfd_vd_forward_final")
    return traces, final


def vd_misfit_gradient(kappa: torch.Tensor, rho: torch.Tensor, wavelet, src, rec, observed: torch.Tensor,
                       grid: Grid, *, want_wavelet: bool = False, want_traces: bool = False, check: bool = True):
    """(misfit, dJ/dkappa, dJ/drho[, dJ/dwavelet][, traces]) of the
    variable-density medium, misfit = 1/2 sum (traces - observed)^2 (FP64)."""
    call, rho = _vd_prepare(kappa, rho, wavelet, src, rec, grid, observed.shape[0])
    p = call.problem
    _require_cuda(observed, "observed")
    if tuple(observed.shape) != (p.nshot, p.nt, p.nrec):
        raise ValueError(f"observed must be ({p.nshot}, {p.nt}, {p.nrec})")
    obs = observed.to(torch.float32).contiguous()
    ws = _vd_workspace(call, True)
    gk = torch.empty_like(call.vel)
    gr = torch.empty_like(call.vel)
    gwav = torch.empty_like(call.wavelet) if want_wavelet else None
    traces = torch.empty_like(obs) if want_traces else None
    misfit = torch.zeros((), dtype=torch.float64, device=kappa.device)
    gz, _, gx = call.sponges
    _lib.check(_lib.load().wfd_vd_misfit_gradient(
        ctypes.byref(p), _ptr(call.vel), _ptr(rho), _ptr(gz), _ptr(gx), _ptr(call.wavelet), _ptr(call.src),
        _ptr(call.rec), _ptr(obs), _ptr(traces), _ptr(gk), _ptr(gr), _ptr(gwav), _ptr(misfit), _ptr(ws),
        ws.numel(), _stream()), "wfd_vd_misfit_gradient")
    if check:
        _status(ws, "wfd_vd_misfit_gradient")
    out = [misfit, gk, gr]
    if want_wavelet:
        out.append(gwav)
    if want_traces:
        out.append(traces)
    return tuple(out)
