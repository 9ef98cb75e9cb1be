"""cuwave-shaped adapter: the reference drivers' call sequence on this library.

projects/18_fwi (plate.py, helper.py, 2D_fwi.py) and projects/16_neuralopt
drive the pip package cuwave through a small surface:
  ScalarWave(Nx, dx, N, dt, threads, precision, space_order, wavespeed, density),
  line, shots, point_source, Sensors, sineburst, stable_dt, simulate, measure,
  misfit, misfit_gradient, resample, Adam, grid_coords, interior_slice, circle,
  box, nodes, threshold, energy, response, response_gradient,
  reconstruction_sensitivity, reconstruction_nodes,
  ScalarWave.parametrization_jacobian; and,
  for the absorbing layer of projects/0_conceptual_figures/4_analog_rnn.py:
  73,95-97, pad_for_sponge and sponge.
This module offers the same names and call shapes over PyTorch tensors, with
every time step in the library's CUDA kernels. cuwave's own equations are
not available (the package is absent), so the choices below are this
module's own. They are written here so callers can check parity:

* Material indicator gamma (the reference's "indicator", 1 = solid, ~1e-4 =
  void; plate.py:36,54-59, helper.py:30-43). It scales the stiffness at
  constant density: c(x) = wavespeed * sqrt(gamma(x)). misfit_gradient returns
  d misfit / d gamma = d misfit / d c * wavespeed / (2 sqrt(gamma)).
* Grid. The nodes of ScalarWave((nx, ny), (dx, dy)) sit at x = -dx + i dx
  (helper.py:240-242: one ghost node outside [0, L] on each side). The library's
  order-2R stencil holds a ring of R cells fixed, so the adapter pads R - 1
  more ghost nodes on every side; the physical nodes, the array on the plate
  edge included, are then updated. Indicators are read where the reference
  drivers put them, in [:nx, :ny] of an array of shape Nx or larger
  (helper.py:76-77, 2D_fwi.py:34), and their edge values extend into the
  margin. Gradients come back in the indicator's shape and place. Nx_padded
  rounds each axis up to a multiple of 8. ScalarWave also takes 3D grids
  (nx, ny, nz), as projects/8_physics_drivers/waveND.py does with DIM = 3;
  AcousticWave is 2D.
* Coordinates map to the nearest node, as cuwave's point sources and sensors
  do. Source and Sensors hold node numbers as cuwave does (check.py:54): an
  array (D, n), node 0 the ghost node at -dx; the library's grid index is the
  node number plus the margin. Source.signal is the source term f of
  u_tt = c^2 Lap u + f: point_source divides the signal by the cell volume
  dx dy (projects/9_structural_optimization/README.md:87), and dt^2 f is
  added per step.
* sineburst(t, A, f, cycles) is a Hann-windowed tone burst
  A sin(2 pi f t) sin^2(pi f t / cycles) on 0 <= t <= cycles / f.
* Array axes follow the reference (x first); they map onto the library's
  (z, x) axes unchanged.
* Absorbing layer. pad_for_sponge(resolution, dx, thickness) pads every
  face by ceil(thickness / dx) cells; sponge(sim, field, width, beta) returns
  the layer for ScalarWave.damping. The library damps with the product of
  per-axis factors g (u_{n+1} = g (2 u_n + m L u_n) - g^2 u_{n-1}),
  g = exp(-(a d)^2) at depth d of the layer's W cells and a = s / W. beta is
  read as the reference states it, the peak damping d dt / 2m at the wall: a
  centred damping term of that size shrinks the amplitude per step by
  sqrt((1 - beta) / (1 + beta)), and s is chosen so the wall factor
  exp(-s^2) equals it. A plain int is a width with the library's default
  strength.
* AcousticWave(..., rho1, rho2, kappa1, kappa2): the two-phase medium
  u_tt = kappa div(grad u / rho) + f of projects/8_physics_drivers/
  waveND.py:52-65. Like cuwave (1_benchmark_2D/README.md:141-144) it
  interpolates 1/rho and 1/kappa linearly in the indicator (0: rho1, kappa1;
  1: rho2, kappa2), and source samples are scaled by the indicator at their
  node, so that nothing is injected into a hole. misfit_gradient returns
  d misfit / d gamma through kappa, rho and the source scaling.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field

import numpy as np
import torch

from .wavefd import Grid, misfit_gradient as _misfit_gradient, stable_dt as _stable_dt, wave_forward
from .wavefd import vd_forward, vd_forward_final, vd_misfit_gradient, vd_vmax, wave_forward_final


@dataclass(frozen=True)
class Sponge:
    """An absorbing layer: (low, high) widths in cells per axis and the
    strength s of the factor exp(-(s d / W)^2)."""
    widths: tuple
    strength: float


def pad_for_sponge(resolution, dx, thickness: float, faces=None):
    """(Nx, width, origin, region): the grid of `resolution` nodes padded by a
    layer of `thickness` (length units) on every face, or on `faces` only,
    given as (axis, side) pairs with side 0 (low) or 1 (high). width is the
    layer's (low, high) cells per axis, origin the first node of the region of
    interest, region its index slices."""
    res = tuple(int(n) for n in resolution)
    cells = tuple(int(math.ceil(thickness / h - 1e-9)) for h in dx)
    on = set(faces) if faces is not None else {(a, sd) for a in range(len(res)) for sd in (0, 1)}
    width = tuple((cells[a] if (a, 0) in on else 0, cells[a] if (a, 1) in on else 0) for a in range(len(res)))
    Nx = tuple(n + lo + hi for n, (lo, hi) in zip(res, width))
    origin = tuple(lo for lo, _ in width)
    region = tuple(slice(o, o + n) for o, n in zip(origin, res))
    return Nx, width, origin, region


def sponge(sim, field, width, beta: float, faces=None) -> "Sponge":
    """The absorbing layer for ``ScalarWave.damping`` (see the module notes):
    `width` as pad_for_sponge returns it, or one int for every face; `beta`
    the peak damping d dt / 2m at the wall; `field` (the reference passes an
    array of ones of Nx_padded) only has to cover the grid."""
    if field is not None and any(f < n for f, n in zip(tuple(field.shape), sim.Nx)):
        raise ValueError("field does not cover the grid")
    if not 0.0 < beta < 1.0:
        raise ValueError("beta must lie in (0, 1)")
    nd = len(sim.Nx)
    w = [(int(width), int(width))] * nd if isinstance(width, (int, np.integer)) else [tuple(map(int, p)) for p in width]
    if faces is not None:
        on = set(faces)
        w = [(lo if (a, 0) in on else 0, hi if (a, 1) in on else 0) for a, (lo, hi) in enumerate(w)]
    wall = math.sqrt((1.0 - beta) / (1.0 + beta))
    return Sponge(tuple(w), math.sqrt(-math.log(wall)))


def circle(coords, center, radius: float) -> torch.Tensor:
    """Mask of the nodes within `radius` of `center` (grid_coords arrays;
    fwi_penalization.py:92, cylinder_snapshots.py:37)."""
    d2 = sum((torch.as_tensor(x).double() - float(c)) ** 2 for x, c in zip(coords, center))
    return d2 <= float(radius) ** 2


def box(coords, center, size) -> torch.Tensor:
    """Mask of the nodes with |x_d - center_d| <= size_d / 2 on every axis
    (topopt_acoustic2D.py:144-147)."""
    m = None
    for x, c, w in zip(coords, center, size):
        inside = (torch.as_tensor(x).double() - float(c)).abs() <= 0.5 * float(w)
        m = inside if m is None else m & inside
    return m


def nodes(mask) -> np.ndarray:
    """(D, n) numbers of the masked nodes, the layout of Source and Sensors
    node arrays (topopt_acoustic2D.py:144 passes it as the sensors)."""
    idx = torch.nonzero(torch.as_tensor(mask).bool().cpu(), as_tuple=False)
    return idx.T.numpy().astype(np.int32)


def threshold(field, level: float):
    """1 where field > level, else 0, in the field's type (analog_rnn_train.py:179)."""
    f = torch.as_tensor(field)
    return (f > level).to(f.dtype)


def interior_slice(sim) -> tuple:
    """Index slices of the nodes on [0, L] along each axis (the ghost node
    at each end left out), for an indicator or a simulate() field indexed
    from node 0 (2D_fwi.py:47, 1_benchmark_2D/forward/wave.py:109)."""
    return tuple(slice(1, n - 1) for n in sim.Nx)


def grid_coords(Nx, dx, dtype=None, device="cuda"):
    """Node coordinates of a ScalarWave grid, one array per axis
    (x_i = -dx + i dx, the ghost node first), indexed like the fields."""
    axes = [torch.arange(n, dtype=torch.float64) * h - h for n, h in zip(Nx, dx)]
    mesh = torch.meshgrid(*axes, indexing="ij")
    dt_ = dtype if isinstance(dtype, torch.dtype) else torch.float32
    return tuple(m.to(device=device, dtype=dt_) for m in mesh)


@dataclass
class ScalarWave:
    """Simulation descriptor (cuwave.scalar.ScalarWave's arguments)."""
    Nx: tuple
    dx: tuple
    N: int
    dt: float
    threads: tuple = (4, 128)
    precision: str = "float32"
    space_order: int = 2
    wavespeed: float = 1.0
    density: float = 1.0
    damping: object = 0  # a sponge() layer, or its width in cells on every face (0: reflecting plate)
    device: str = "cuda"

    @property
    def dtype(self):
        return torch.float32

    @property
    def margin(self) -> int:
        return self.space_order // 2 - 1

    @property
    def grid_shape(self) -> tuple:
        return tuple(n + 2 * self.margin for n in self.Nx)

    @property
    def Nx_padded(self) -> tuple:
        return tuple((n + 7) // 8 * 8 for n in self.grid_shape)

    def grid(self) -> Grid:
        if isinstance(self.damping, Sponge):
            return Grid(self.grid_shape, tuple(self.dx), self.dt, self.N, order=self.space_order,
                        sponge=[tuple(w) for w in self.damping.widths],
                        sponge_strength=self.damping.strength, src_scale=1.0)
        return Grid(self.grid_shape, tuple(self.dx), self.dt, self.N, order=self.space_order,
                    sponge=int(self.damping), src_scale=1.0)

    def node(self, coord) -> tuple:
        """Number of the nearest node of a physical coordinate (node i sits at
        x = -dx + i dx, node 0 the ghost node), as Source and Sensors hold it."""
        return tuple(int(round(c / h)) + 1 for c, h in zip(coord, self.dx))

    @property
    def interior(self) -> tuple:
        """Index slices of the Nx nodes on the library's grid."""
        return tuple(slice(self.margin, self.margin + n) for n in self.Nx)

    def extend(self, indicator) -> torch.Tensor:
        """gamma on the library's grid: read from [:nx, :ny(, :nz)] of the
        indicator, edge values extended into the margin."""
        g = torch.as_tensor(indicator, device=self.device, dtype=torch.float32)
        nd = len(self.Nx)
        if nd not in (2, 3):
            raise ValueError(f"{nd}-dimensional grids are not supported (2 or 3)")
        if g.dim() != nd or any(a < n for a, n in zip(g.shape, self.Nx)):
            raise ValueError(f"indicator of shape {tuple(g.shape)} does not cover {self.Nx}")
        g = g[tuple(slice(0, n) for n in self.Nx)]
        m = self.margin
        if m:
            g = torch.nn.functional.pad(g[None, None], (m, m) * nd, mode="replicate")[0, 0]
        return g

    def velocity(self, indicator) -> torch.Tensor:
        """c = wavespeed sqrt(gamma) on the library's grid."""
        return self.wavespeed * torch.sqrt(self.extend(indicator).clamp_min(0.0))

    def parametrization_jacobian(self, indicator):
        """(d mass / d gamma, d stiff / d gamma) in the indicator's shape
        (analog_rnn_train.py:136). This adapter's scalar medium has mass 1
        and stiffness gamma (c^2 = wavespeed^2 stiff / mass): (0, 1)."""
        g = torch.as_tensor(indicator, device=self.device, dtype=torch.float32)
        return torch.zeros_like(g), torch.ones_like(g)


def stable_dt(dx, c: float, order: int) -> float:
    return _stable_dt(tuple(dx), c, order)


def sineburst(t, amplitude: float, frequency: float, cycles: float) -> np.ndarray:
    t = np.asarray(t, dtype=np.float64)
    on = (t >= 0) & (t <= cycles / frequency)
    s = amplitude * np.sin(2 * math.pi * frequency * t) * np.sin(math.pi * frequency * t / cycles) ** 2
    return np.where(on, s, 0.0).astype(np.float32)


def line(a, b, n: int) -> np.ndarray:
    """n points evenly spaced from a to b."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return a[None, :] + np.linspace(0.0, 1.0, n)[:, None] * (b - a)[None, :]


def _host(a) -> np.ndarray:
    return a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)


@dataclass
class Source:
    """A source as cuwave holds one (check.py:54): `nodes` (D, nsrc), the node
    numbers it drives along each axis (node 0 the ghost node at -dx), and
    `signal` (N, nsrc), the source term f of u_tt = c^2 Lap u + f at those
    nodes. The step's dt^2 is applied when the library is called."""
    nodes: np.ndarray
    signal: np.ndarray


def point_source(sim: ScalarWave, coords, signal) -> Source:
    """Sources at the nodes nearest `coords`, the signal divided by the cell
    volume (projects/9_structural_optimization/README.md:87)."""
    coords = np.atleast_2d(np.asarray(coords, dtype=np.float64))
    nodes = np.array([sim.node(c) for c in coords], dtype=np.int32).reshape(-1, len(sim.Nx)).T
    sig = np.asarray(signal, dtype=np.float64).reshape(sim.N, -1)
    if sig.shape[1] == 1 and nodes.shape[1] > 1:
        sig = np.repeat(sig, nodes.shape[1], axis=1)
    return Source(nodes, sig / float(np.prod(sim.dx)))


class _SourceList(list):
    def __getitem__(self, i):
        r = super().__getitem__(i)
        return _SourceList(r) if isinstance(i, slice) else r


def shots(sim: ScalarWave, coords, signal):
    """One point source per coordinate (every element fires once)."""
    return _SourceList(point_source(sim, c, signal) for c in np.asarray(coords))


@dataclass
class Sensors:
    sim: ScalarWave
    coords: np.ndarray
    nodes: np.ndarray = field(init=False)

    def __post_init__(self):
        """nodes (D, nsensors): node numbers, laid out as Source.nodes."""
        nd = len(self.sim.Nx)
        pts = np.atleast_2d(np.asarray(self.coords, dtype=np.float64))
        self.nodes = np.array([self.sim.node(c) for c in pts], dtype=np.int32).reshape(-1, nd).T

    def traces(self, um):
        """The sensor traces (N, nsensors) of a simulate() record
        (4_analog_rnn.py:128): the record already holds them."""
        return um

    def objective(self, objective):
        """`objective` applied to the sensor traces of a record, for
        response_gradient (analog_rnn_train.py:143)."""
        return lambda um: objective(self.traces(um))


def _grid_points(sim, nodes) -> np.ndarray:
    """(D, n) node numbers -> (n, D) int32 indices on the library's grid."""
    a = _host(nodes).astype(np.int64).reshape(len(sim.Nx), -1)
    return (a.T + sim.margin).astype(np.int32)


def _grid_signal(sim, source) -> np.ndarray:
    """(N, nsrc) source samples added per step: dt^2 f, FP32."""
    return (np.asarray(_host(source.signal), dtype=np.float64).reshape(sim.N, -1) * (sim.dt * sim.dt)).astype(np.float32)


def _batch(sim, sources, sensors):
    """The library's arrays for a list of shots: positions (nshot, nsrc, D),
    samples (nshot, N, nsrc) and receivers (nshot, nrec, D)."""
    srcs = list(sources) if isinstance(sources, (list, tuple)) else [sources]
    pts = [_grid_points(sim, s.nodes) for s in srcs]
    if any(len(q) != len(pts[0]) for q in pts):
        raise ValueError("every shot needs the same number of source points")
    src = np.stack(pts)
    wav = np.stack([_grid_signal(sim, s) for s in srcs])
    rec = np.repeat(_grid_points(sim, sensors.nodes)[None], len(srcs), axis=0)
    return src, wav, rec


def measure(sim: ScalarWave, sources, indicator, sensors: Sensors):
    """Records of every shot: a list of (N, nsensors) tensors (plate.py:62-64)."""
    src, wav, rec = _batch(sim, sources, sensors)
    vel = sim.velocity(indicator)
    tr = wave_forward(vel, torch.from_numpy(wav).to(vel.device), src, rec, sim.grid())
    return list(tr.unbind(0))


def simulate(sim: ScalarWave, source: Source, indicator, sensors=None, record_every: int | None = None):
    """One shot. Returns the final field u_N on the physical nodes (shape Nx)
    (2D_scalar_wave_forward_B_hai.py:30); with `sensors` (a Sensors, or
    their node array as the reference passes it) also the record um
    (N, nsensors); with `record_every` k also the frames u_0, u_k, u_2k, ...
    on the physical nodes (animate_bhai_waves.py:29, 4_analog_rnn.py:125-128):
    u, (u, um), (u, frames) or (u, um, frames). An AcousticWave runs the
    two-phase medium (waveND.py:52-65,94). The library forward starts
    from rest, so frame j is a forward of j k steps: frames cost
    O(N^2 / k) steps, meant for the few snapshots a figure takes."""
    if record_every is not None and int(record_every) < 1:
        raise ValueError(f"record_every must be at least 1 (got {record_every})")
    nd = len(sim.Nx)
    if sensors is None:
        s = Sensors(sim, np.zeros((0, nd)))
    elif isinstance(sensors, Sensors):
        s = sensors
    else:  # a node array (D, nsensors), as Sensors.nodes holds it
        s = Sensors(sim, np.zeros((0, nd)))
        s.nodes = _host(sensors).astype(np.int32).reshape(nd, -1)
    acoustic = isinstance(sim, AcousticWave)
    if acoustic:  # the two-phase medium on the variable-density kernels
        kap, rho = sim.materials(indicator)
        source = _scaled_sources(sim, source, indicator)
    else:
        vel = sim.velocity(indicator)
    src, wav, rec = _batch(sim, source, s)
    rec_t = torch.from_numpy(rec) if rec.shape[1] > 0 else torch.zeros((1, 0, nd), dtype=torch.int32)
    wav_t = torch.from_numpy(wav).to(sim.device)
    grid = sim.grid()

    def run(g, w, r):
        return vd_forward_final(kap, rho, w, src, r, g) if acoustic else wave_forward_final(vel, w, src, r, g)

    traces, final = run(grid, wav_t, rec_t)

    def physical(f):
        return f[(0,) + sim.interior]

    u = physical(final)
    out = [u]
    if sensors is not None:
        out.append(traces[0])
    if record_every is not None:
        k = int(record_every)
        frames = [torch.zeros_like(u)]
        none = torch.zeros((1, 0, nd), dtype=torch.int32)
        for j in range(1, sim.N // k + 1):
            n = j * k
            if n == sim.N:
                frames.append(u)
                continue
            g = dataclasses.replace(grid, nt=n, ckpt_every=0)
            frames.append(physical(run(g, wav_t[:, :n], none)[1]))
        out.append(torch.stack(frames))
    return out[0] if len(out) == 1 else tuple(out)


def energy(sim):
    """The objective of topopt_acoustic2D.py:171: dt times the sum of the
    record's squares (the time-integrated squared field at the sensor nodes),
    returned with its derivative, (cost, dJ/d(record)), as the reference's
    objectives do (analog_rnn_fixture.py:106-121)."""
    dt = float(sim.dt)
    def objective(um):
        u = torch.as_tensor(um).detach().double()
        return dt * float((u ** 2).sum()), 2.0 * dt * u

    return objective


def _cost_and_cotangent(objective, um):
    """(cost, dJ/d(record)) of an objective that returns that pair, or of one
    that returns a differentiable scalar tensor (its derivative by autograd)."""
    x = um.detach().double().requires_grad_(True)
    out = objective(x)
    if isinstance(out, tuple):
        cost, cot = out
        return float(cost), torch.as_tensor(cot, dtype=torch.float64, device=um.device).detach()
    (cot,) = torch.autograd.grad(out, x)
    return float(out.detach()), cot


def response(sim, source, indicator, sensors, objective):
    """(cost, record) of one shot (topopt_acoustic2D.py:179,260); `sensors`
    a Sensors or a node array, `objective` as for response_gradient."""
    _, um = simulate(sim, source, indicator, sensors)
    out = objective(um)
    return float(out[0] if isinstance(out, tuple) else out), um


def response_gradient(sim, source, indicator, sensors, objective, adjoint=None):
    """(cost, d cost / d indicator) of one shot (topopt_acoustic2D.py:194-195).
    `objective` maps the record (N, nsensors) to (cost, dJ/d(record)), as the
    reference's objectives do, or to a differentiable scalar tensor. The
    gradient has the indicator's shape, nonzero in [:nx, :ny] only.
    `adjoint`: reconstruction_sensitivity runs the library's reconstruction
    adjoint (topopt_acoustic2D.py:195) and combines its mass and stiffness
    gradients with parametrization_jacobian; otherwise the checkpointed
    adjoint runs.

    ScalarWave: autograd through wave_forward (the library's adjoint behind
    torch.autograd) and c = wavespeed sqrt(gamma). AcousticWave: the
    variable-density misfit gradient with observed = record - s dJ/d(record),
    whose residual is s dJ/d(record), so its gradient is s times the
    objective's; s = max|record| / max|dJ/d(record)| keeps that residual at
    the record's scale in FP32."""
    if adjoint is reconstruction_sensitivity:
        J, grads, _, _ = reconstruction_sensitivity(sim, source, indicator, sensors, objective)
        d_mass, d_stiff = sim.parametrization_jacobian(indicator)
        return J, d_mass * grads["mass"] + d_stiff * grads["stiff"]
    sens = sensors
    if not isinstance(sens, Sensors):
        sens = Sensors(sim, np.zeros((0, len(sim.Nx))))
        sens.nodes = _host(sensors).astype(np.int32).reshape(len(sim.Nx), -1)
    gamma = torch.as_tensor(indicator, device=sim.device, dtype=torch.float32)
    if isinstance(sim, AcousticWave):
        record = acoustic_measure(sim, [source], gamma, sens)[0]
        J, cot = _cost_and_cotangent(objective, record)
        peak = float(cot.abs().max())
        if peak == 0.0:
            return J, torch.zeros_like(gamma)
        scale = max(float(record.abs().max()), 1e-30) / peak
        observed = (record.double() - scale * cot).float()
        _, grad = acoustic_misfit_gradient(sim, [source], gamma, sens, [observed])
        return J, grad / scale
    src, wav, rec = _batch(sim, source, sens)
    g = gamma.detach().clone().requires_grad_(True)
    record = wave_forward(sim.velocity(g), torch.from_numpy(wav).to(g.device), src, rec, sim.grid())[0]
    J, cot = _cost_and_cotangent(objective, record)
    record.backward(cot.to(record.dtype))
    return J, g.grad


def resample(record, dt_obs: float, dt: float, N: int):
    """Linear interpolation of a record (steps first) onto N steps of dt."""
    r = torch.as_tensor(record)
    t = torch.arange(N, dtype=torch.float64, device=r.device) * dt
    pos = (t / dt_obs).clamp(0, r.shape[0] - 1)
    k = pos.floor().long().clamp(max=r.shape[0] - 2)
    w = (pos - k).to(r.dtype).view(-1, *([1] * (r.dim() - 1)))
    return (1 - w) * r[k] + w * r[k + 1]


def misfit_gradient(sim: ScalarWave, sources, indicator, sensors: Sensors, observed):
    """(cost, d cost / d indicator) with cost = 1/2 sum over shots of
    |record - observed|^2 (2D_fwi.py:40). The gradient has the indicator's
    shape, nonzero in [:nx, :ny] only."""
    src, wav, rec = _batch(sim, sources, sensors)
    gamma = torch.as_tensor(indicator, device=sim.device, dtype=torch.float32)
    vel = sim.velocity(gamma)
    obs = torch.stack([torch.as_tensor(o, device=vel.device, dtype=torch.float32) for o in observed])
    J, gv = _misfit_gradient(vel, torch.from_numpy(wav).to(vel.device), src, rec, obs, sim.grid())
    # c = w sqrt(gamma): d cost / d gamma = d cost / d c * w^2 / (2 c)
    g_pad = gv * (sim.wavespeed ** 2) / (2.0 * vel.clamp_min(1e-6 * sim.wavespeed))
    out = torch.zeros_like(gamma)
    out[tuple(slice(0, n) for n in sim.Nx)] = g_pad[sim.interior]
    return J, out


def misfit(sim: ScalarWave, sources, indicator, sensors: Sensors, observed):
    records = measure(sim, sources, indicator, sensors)
    return sum(0.5 * float(((r.double() - torch.as_tensor(o, device=r.device).double()) ** 2).sum())
               for r, o in zip(records, observed))


class Adam:
    """Adam on a tensor parameter (2D_fwi.py:34-41: step(x, grad) -> new x)."""

    def __init__(self, lr: float = 0.1, betas=(0.9, 0.999), eps: float = 1e-8):
        self.lr, self.b1, self.b2, self.eps = lr, betas[0], betas[1], eps
        self.m = self.v = None
        self.t = 0

    def step(self, x: torch.Tensor, grad: torch.Tensor) -> torch.Tensor:
        if self.m is None:
            self.m = torch.zeros_like(grad)
            self.v = torch.zeros_like(grad)
        self.t += 1
        self.m.mul_(self.b1).add_(grad, alpha=1 - self.b1)
        self.v.mul_(self.b2).addcmul_(grad, grad, value=1 - self.b2)
        mh = self.m / (1 - self.b1 ** self.t)
        vh = self.v / (1 - self.b2 ** self.t)
        return x - self.lr * mh / (vh.sqrt() + self.eps)


@dataclass
class AcousticWave(ScalarWave):
    """Two-phase acoustic descriptor (cuwave.acoustic.AcousticWave's arguments)."""
    rho1: float = 1.204
    rho2: float = 2643.0
    kappa1: float = 1.419e5
    kappa2: float = 6.87e8

    def indicator(self, indicator) -> torch.Tensor:
        """gamma on the library's grid (the variable-density kernels are 2D)."""
        if len(self.Nx) != 2:
            raise ValueError("AcousticWave runs on 2D grids")
        return self.extend(indicator)

    def materials(self, indicator):
        """(kappa, rho) on the padded grid from 1/rho and 1/kappa linear in gamma."""
        g = self.indicator(indicator).double()
        inv_rho = (1 - g) / self.rho1 + g / self.rho2
        inv_kap = (1 - g) / self.kappa1 + g / self.kappa2
        return (1 / inv_kap).float(), (1 / inv_rho).float()

    def velocity(self, indicator) -> torch.Tensor:
        kap, rho = self.materials(indicator)
        return torch.sqrt(kap / rho)

    def parametrization_jacobian(self, indicator):
        """(d mass / d gamma, d stiff / d gamma) in the indicator's shape: the
        mass is 1/kappa and the stiffness 1/rho, both linear in gamma
        (1_benchmark_2D/README.md:141-144), so the derivatives are the
        constants 1/kappa2 - 1/kappa1 and 1/rho2 - 1/rho1."""
        g = torch.as_tensor(indicator, device=self.device, dtype=torch.float32)
        return (torch.full_like(g, 1.0 / self.kappa2 - 1.0 / self.kappa1),
                torch.full_like(g, 1.0 / self.rho2 - 1.0 / self.rho1))

    def max_speed(self, indicator) -> float:
        """The speed to give stable_dt for this medium: sqrt(kappa / rho) in
        a smooth medium, larger where 1/rho jumps between cells (air beside
        a solid), as the staggered step's stability requires."""
        kap, rho = self.materials(indicator)
        return vd_vmax(kap, rho, self.space_order, tuple(self.dx))


def _scaled_sources(sim: AcousticWave, sources, indicator):
    """Source signals times the indicator at each source node."""
    g = sim.indicator(indicator)
    srcs = list(sources) if isinstance(sources, (list, tuple)) else [sources]
    out = []
    for s in srcs:
        w = g.detach().cpu().numpy().astype(np.float64)[tuple(_grid_points(sim, s.nodes).T)]
        out.append(Source(s.nodes, np.asarray(_host(s.signal), dtype=np.float64) * w[None, :]))
    return _SourceList(out)


def acoustic_measure(sim: AcousticWave, sources, indicator, sensors: Sensors):
    kap, rho = sim.materials(indicator)
    src, wav, rec = _batch(sim, _scaled_sources(sim, sources, indicator), sensors)
    tr = vd_forward(kap, rho, torch.from_numpy(wav).to(kap.device), src, rec, sim.grid())
    return list(tr.unbind(0))


def _acoustic_parts(sim: AcousticWave, sources, gamma, sensors: Sensors, observed, grid):
    """The variable-density misfit gradient's parts on the library's grid (FP64):
    (J, dJ/dkappa, dJ/drho, the source term dJ/dgamma at the source nodes,
    kappa, rho)."""
    kap, rho = sim.materials(gamma)
    scaled = _scaled_sources(sim, sources, gamma)
    src, wav, rec = _batch(sim, scaled, sensors)
    obs = torch.stack([torch.as_tensor(o, device=kap.device, dtype=torch.float32) for o in observed])
    J, gk, gr, gw = vd_misfit_gradient(kap, rho, torch.from_numpy(wav).to(kap.device), src, rec, obs, grid,
                                       want_wavelet=True)
    # the source samples scale with gamma at their nodes: sum_n dJ/dw_n * signal_n
    g_src = torch.zeros_like(gk, dtype=torch.float64)
    srcs = list(sources) if isinstance(sources, (list, tuple)) else [sources]
    for si, s in enumerate(srcs):
        sig = torch.from_numpy(_grid_signal(sim, s)).to(kap.device).double()  # (N, nsrc), dt^2 f
        contrib = (gw[si].double() * sig).sum(0)
        for j, (a, b) in enumerate(_grid_points(sim, s.nodes)):
            g_src[a, b] += contrib[j]
    return J, gk.double(), gr.double(), g_src, kap, rho


def _to_indicator(sim, g_pad, gamma):
    """A field on the library's grid -> the indicator's shape (the Nx nodes)."""
    out = torch.zeros_like(gamma)
    out[tuple(slice(0, n) for n in sim.Nx)] = g_pad[sim.interior].to(out.dtype)
    return out


def acoustic_misfit_gradient(sim: AcousticWave, sources, indicator, sensors: Sensors, observed):
    """(cost, d cost / d indicator) for the two-phase medium."""
    gamma = torch.as_tensor(indicator, device=sim.device, dtype=torch.float32)
    J, gk, gr, g_src, kap, rho = _acoustic_parts(sim, sources, gamma, sensors, observed, sim.grid())
    # kappa = 1 / ((1-g)/k1 + g/k2): d kappa / d g = -kappa^2 (1/k2 - 1/k1); rho likewise
    dk = -kap.double() ** 2 * (1 / sim.kappa2 - 1 / sim.kappa1)
    dr = -rho.double() ** 2 * (1 / sim.rho2 - 1 / sim.rho1)
    return J, _to_indicator(sim, gk * dk + gr * dr + g_src, gamma)


def reconstruction_nodes(sim):
    """(nodes, count): the nodes whose values the reconstruction adjoint saves
    at every step (the frame of the grid where the sponge damps, as the
    library's reconstruction adjoint restores it), as a (D, n) array of node
    numbers (Source / Sensors numbering, margin nodes negative or beyond Nx),
    and n; analog_rnn_fixture.py:84 sizes its memory from it. A reflecting
    plate (no sponge) saves none."""
    grid = sim.grid()
    if len(sim.Nx) != 2:
        raise ValueError("the reconstruction adjoint runs on 2D grids")
    W = max(max(w) for w in grid.sponge_widths())
    nz, nx = grid.shape
    if W == 0:
        return np.zeros((2, 0), dtype=np.int32), 0
    z, x = np.meshgrid(np.arange(nz), np.arange(nx), indexing="ij")
    band = (z < W) | (z >= nz - W) | (x < W) | (x >= nx - W)
    pts = np.stack([z[band], x[band]]) - sim.margin
    return pts.astype(np.int32), int(pts.shape[1])


def reconstruction_sensitivity(sim, source, indicator, sensors, objective):
    """(loss, grads, record, None) of one shot with the reconstruction adjoint
    (analog_rnn_train.py:142; cuwave.sensitivity): the adjoint rebuilds the
    forward levels by running the step backwards from the last two, with the
    damped frame restored from per-step copies, instead of checkpoints.
    `sensors` is a node array (D, n) or a Sensors; `objective` maps the record
    (N, nsensors) to (cost, dJ/d(record)) or to a differentiable scalar.
    grads = {"mass": dJ/d mass, "stiff": dJ/d stiff} in the indicator's shape,
    for the parametrisation of parametrization_jacobian, so that
    d_mass * grads["mass"] + d_stiff * grads["stiff"] is dJ/d gamma:
      ScalarWave   mass 1, stiff gamma: dJ/d stiff = dJ/d gamma,
                   dJ/d mass = -gamma dJ/d gamma;
      AcousticWave mass 1/kappa, stiff 1/rho: dJ/d mass = -kappa^2 dJ/d kappa,
                   dJ/d stiff = -rho^2 dJ/d rho; the source samples scale with
                   gamma at their nodes (this adapter's choice), and that term
                   is added to dJ/d mass there, divided by d mass / d gamma.
    2D grids."""
    if len(sim.Nx) != 2:
        raise ValueError("the reconstruction adjoint runs on 2D grids")
    sens = sensors
    if not isinstance(sens, Sensors):
        sens = Sensors(sim, np.zeros((0, len(sim.Nx))))
        sens.nodes = _host(sensors).astype(np.int32).reshape(len(sim.Nx), -1)
    gamma = torch.as_tensor(indicator, device=sim.device, dtype=torch.float32)
    grid = dataclasses.replace(sim.grid(), adjoint="reconstruct")
    if isinstance(sim, AcousticWave):
        kap, rho = sim.materials(gamma)
        scaled = _scaled_sources(sim, [source], gamma)
        src, wav, rec = _batch(sim, scaled, sens)
        record = vd_forward(kap, rho, torch.from_numpy(wav).to(kap.device), src, rec, grid)[0]
        J, cot = _cost_and_cotangent(objective, record)
        peak = float(cot.abs().max())
        if peak == 0.0:
            z = torch.zeros_like(gamma)
            return J, {"mass": z, "stiff": z.clone()}, record, None
        # residual s dJ/d(record): observed = record - s cot (as response_gradient)
        scale = max(float(record.abs().max()), 1e-30) / peak
        observed = (record.double() - scale * cot).float()
        _, gk, gr, g_src, kap, rho = _acoustic_parts(sim, [source], gamma, sens, [observed], grid)
        d_mass = 1.0 / sim.kappa2 - 1.0 / sim.kappa1
        g_mass = (-kap.double() ** 2 * gk + g_src / d_mass) / scale
        g_stiff = (-rho.double() ** 2 * gr) / scale
        return J, {"mass": _to_indicator(sim, g_mass, gamma), "stiff": _to_indicator(sim, g_stiff, gamma)}, \
            record, None
    src, wav, rec = _batch(sim, source, sens)
    g = gamma.detach().clone().requires_grad_(True)
    record = wave_forward(sim.velocity(g), torch.from_numpy(wav).to(g.device), src, rec, grid)[0]
    J, cot = _cost_and_cotangent(objective, record)
    record.backward(cot.to(record.dtype))
    dg = g.grad
    return J, {"mass": -gamma * dg, "stiff": dg}, record.detach(), None
