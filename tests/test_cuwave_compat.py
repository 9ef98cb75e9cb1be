"""The cuwave-shaped adapter: the call sequences of projects/18_fwi,
8_physics_drivers (waveND, topopt_acoustic2D) and the analog-RNN drivers on
this library. CPU: node numbering and layout, sources, sensors, sponge and
geometry helpers, and response_gradient's chain rule with stand-ins for the
library calls. GPU: the FWI flow, indicator gradients against FP64 finite
differences, simulate's call forms against measure and the FP64 oracle (2D,
3D, two-phase), and the sponge's absorption."""
import math

import numpy as np
import pytest
import torch

from conftest import rel_l2


def test_geometry_and_helpers():
    from neuralmech_gb300 import cuwave_compat as cw
    sim = cw.ScalarWave((64, 80), (1 / 61, 1 / 77), 100, 1e-3, space_order=8)
    assert sim.margin == 3 and sim.grid_shape == (70, 86) and sim.Nx_padded == (72, 88)
    # node i sits at x = -dx + i dx (node 0 the ghost node); on the library's
    # grid it is index i + margin
    assert sim.node((0.0, 0.0)) == (1, 1)
    assert sim.node((1.0, 1.0)) == (62, 78)  # the last node on [0, L]
    R = 4
    assert sim.node((1.0, 1.0))[1] + sim.margin < sim.grid_shape[1] - R  # updated by the order-8 stencil
    pts = cw.line((0.1, 1.0), (0.9, 1.0), 5)
    assert pts.shape == (5, 2) and np.allclose(pts[:, 1], 1.0) and np.isclose(pts[2, 0], 0.5)
    t = np.linspace(0, 0.5, 1001)
    s = cw.sineburst(t, 2.0, 10.0, 2)
    assert np.all(s[t > 0.2] == 0) and np.abs(s).max() <= 2.0 and np.abs(s).max() > 1.5
    src = cw.point_source(sim, (0.5, 1.0), np.ones(100))
    assert src.nodes.shape == (2, 1) and np.allclose(src.signal, 1.0 / (1 / 61 * 1 / 77))
    # interior_slice: the nodes on [0, L], as the indicator and simulate() index them
    inner = cw.interior_slice(sim)
    assert inner == (slice(1, 63), slice(1, 79))
    x, y = cw.grid_coords(sim.Nx, sim.dx, device="cpu")
    assert abs(float(x[inner][0, 0])) < 1e-12 and abs(float(x[inner][-1, 0]) - 1.0) < 1e-6
    assert abs(float(y[inner][0, -1]) - 1.0) < 1e-6 and x[inner].shape == (62, 78)
    for bad in (0, -3):  # refused before any device work
        with pytest.raises(ValueError):
            cw.simulate(sim, src, np.ones(sim.Nx), record_every=bad)


def test_source_and_sensor_conventions():
    """Source(indices (D, nsrc), signal (N, nsrc)) built by hand, as check.py:54
    does, drives node n // 2 of each axis (the library's index n // 2 + margin)
    with dt^2 signal per step; point_source at a node's coordinate gives the
    same shot with the signal divided by the cell volume; Sensors and node
    arrays are (D, n), in 2D and 3D."""
    from neuralmech_gb300 import cuwave_compat as cw
    for Nx in ((40, 52), (20, 22, 24)):
        nd = len(Nx)
        dx = tuple(1.0 / (n - 3) for n in Nx)
        sim = cw.ScalarWave(Nx, dx, 30, 2e-3, space_order=8, device="cpu")
        sig = np.sin(np.arange(30.0))[:, None]
        hand = cw.Source(np.array([[n // 2] for n in Nx], dtype=np.int32), sig)
        sensors = cw.Sensors(sim, [tuple(0.25 for _ in Nx), tuple(0.5 for _ in Nx)])
        assert sensors.nodes.shape == (nd, 2)
        src, wav, rec = cw._batch(sim, hand, sensors)
        assert src.shape == (1, 1, nd) and tuple(src[0, 0]) == tuple(n // 2 + sim.margin for n in Nx)
        assert wav.dtype == np.float32 and np.allclose(wav[0, :, 0], sig[:, 0] * 2e-3 ** 2, rtol=1e-6, atol=0)
        assert tuple(rec[0, 1]) == tuple(k + sim.margin for k in sim.node((0.5,) * nd))
        coord = tuple((n // 2 - 1) * h for n, h in zip(Nx, dx))
        ps = cw.point_source(sim, coord, sig[:, 0])
        s2, w2, _ = cw._batch(sim, ps, sensors)
        assert np.array_equal(s2, src)
        assert np.allclose(w2 * np.prod(dx), wav, rtol=1e-6, atol=0)


def test_geometry_masks_and_nodes():
    """circle, box, nodes and threshold on grid_coords: the masks select the
    nodes inside the shape; nodes gives their (D, n) numbers, usable as
    sensors (node i at x = -dx + i dx)."""
    from neuralmech_gb300 import cuwave_compat as cw
    sim = cw.ScalarWave((43, 53), (1 / 40, 1 / 50), 10, 1e-3, space_order=4, device="cpu")
    x, y = cw.grid_coords(sim.Nx, sim.dx, device="cpu")
    disc = cw.circle((x, y), (0.5, 0.5), 0.1)
    assert disc.shape == sim.Nx and bool(disc[21, 26]) and not bool(disc[21, 40])
    assert abs(int(disc.sum()) - math.pi * 0.1 ** 2 / (sim.dx[0] * sim.dx[1])) < 0.1 * int(disc.sum())
    rect = cw.box((x, y), (0.5, 0.5), (0.21, 0.11))  # edges between nodes
    assert int(rect.sum()) == 9 * 5  # x = 0.4 .. 0.6 (9 nodes), y = 0.46 .. 0.54 (5 nodes)
    n = cw.nodes(rect)
    assert n.shape == (2, 45) and n.dtype == np.int32
    assert np.allclose(x[n[0], n[1]].numpy(), x[rect].numpy()) and (np.abs(x[n[0], n[1]].numpy() - 0.5) <= 0.105).all()
    src, wav, rec = cw._batch(sim, cw.point_source(sim, (0.5, 0.5), np.ones(10)), type("S", (), {"nodes": n})())
    assert rec.shape == (1, 45, 2) and (rec[0] == n.T + sim.margin).all()
    t = cw.threshold(torch.tensor([0.2, 0.5, 0.7]), 0.5)
    assert t.tolist() == [0.0, 0.0, 1.0] and t.dtype == torch.float32


def test_response_gradient_chain(monkeypatch):
    """response_gradient's host logic with differentiable stand-ins for the
    library calls. ScalarWave: the gradient through c = wavespeed sqrt(gamma)
    and the indicator's margin extension matches central differences of the
    objective. AcousticWave: with a linear record M gamma, the scaled misfit
    residual returns M^T dJ/d(record)."""
    from neuralmech_gb300 import cuwave_compat as cw
    n, N = 20, 12
    dx = (1 / (n - 3),) * 2
    sim = cw.ScalarWave((n, n), dx, N, 1e-3, space_order=4, wavespeed=1.5, device="cpu")
    src = cw.point_source(sim, (0.5, 0.5), np.linspace(0.0, 1.0, N))
    sensors = cw.Sensors(sim, cw.line((0.2, 0.3), (0.8, 0.3), 3))
    rng = np.random.default_rng(0)

    def fake_forward(vel, wav, src_, rec_, grid):  # smooth, nonlinear in vel
        assert tuple(vel.shape) == grid.shape
        r = torch.as_tensor(rec_)[0].long()
        v = vel[r[:, 0], r[:, 1]]
        t = torch.arange(grid.nt, dtype=vel.dtype)[:, None]
        return (torch.sin(v[None, :] * (1 + t)) * vel.mean() + wav[0, :, :1] * v[None, :] ** 2)[None]

    monkeypatch.setattr(cw, "wave_forward", fake_forward)
    gamma = torch.from_numpy(rng.uniform(0.5, 1.0, sim.Nx_padded).astype(np.float32))
    obj = cw.energy(sim)
    J, grad = cw.response_gradient(sim, src, gamma, sensors, sensors.objective(obj))
    assert grad.shape == gamma.shape and float(grad[n:, :].abs().max()) == 0.0
    # the same objective as a differentiable scalar (autograd for dJ/d(record))
    J2, grad2 = cw.response_gradient(sim, src, gamma, sensors.nodes, lambda um: sim.dt * (um ** 2).sum())
    assert abs(J2 - J) < 1e-12 * abs(J) and torch.allclose(grad2, grad, rtol=1e-6, atol=0)
    d = torch.zeros_like(gamma)
    d[:n, :n] = torch.from_numpy(rng.standard_normal((n, n)).astype(np.float32))
    eps = 1e-2

    def Jof(gm):
        s_, w_, r_ = cw._batch(sim, src, sensors)
        return obj(fake_forward(sim.velocity(gm).double(), torch.from_numpy(w_).double(), s_, r_, sim.grid())[0])[0]

    fd = (Jof(gamma + eps * d) - Jof(gamma - eps * d)) / (2 * eps)
    an = float((grad.double() * d.double()).sum())
    assert abs(fd - an) < 1e-2 * abs(fd), (fd, an)

    ac = cw.AcousticWave((n, n), dx, N, 1e-3, space_order=4, device="cpu")
    M = torch.from_numpy(rng.standard_normal((N * 3, n * n)))

    def rec_of(gm):
        return (M @ torch.as_tensor(gm)[:n, :n].double().reshape(-1)).reshape(N, 3).float()

    def fake_measure(sim_, sources, gm, sens):
        return [rec_of(gm)]

    def fake_misfit_gradient(sim_, sources, gm, sens, observed):
        res = (rec_of(gm) - observed[0]).double().reshape(-1)
        g = torch.zeros(tuple(torch.as_tensor(gm).shape), dtype=torch.float64)
        g[:n, :n] = (M.T @ res).reshape(n, n)
        return 0.5 * float((res ** 2).sum()), g.float()

    monkeypatch.setattr(cw, "acoustic_measure", fake_measure)
    monkeypatch.setattr(cw, "acoustic_misfit_gradient", fake_misfit_gradient)
    gm = torch.from_numpy(rng.uniform(0.0, 1.0, (n, n)).astype(np.float32))
    Ja, ga = cw.response_gradient(ac, src, gm, sensors.nodes, obj)
    um = rec_of(gm).double()
    want = (M.T @ (2 * ac.dt * um).reshape(-1)).reshape(n, n)
    assert abs(Ja - float(ac.dt * (um ** 2).sum())) < 1e-9 * abs(Ja)
    assert rel_l2(ga.double().numpy(), want.numpy()) < 1e-5


def test_sponge_helpers():
    """pad_for_sponge / sponge / grid_coords (4_analog_rnn.py:73,95-97;
    plate.py:56): widths from the thickness, the region inside, a wall factor
    that matches the stated peak damping, and node coordinates."""
    import dataclasses
    import math
    from neuralmech_gb300 import cuwave_compat as cw
    Nx, width, origin, region = cw.pad_for_sponge((100, 80), (0.01, 0.02), 0.1)
    assert width == ((10, 10), (5, 5)) and Nx == (120, 90) and origin == (10, 5)
    assert region == (slice(10, 110), slice(5, 85))
    Nx1, width1, origin1, _ = cw.pad_for_sponge((100, 80), (0.01, 0.02), 0.1, faces=[(0, 1), (1, 0)])
    assert width1 == ((0, 10), (5, 0)) and Nx1 == (110, 85) and origin1 == (0, 5)
    sim = cw.ScalarWave(Nx, (0.01, 0.02), 50, 1e-4, space_order=8)
    layer = cw.sponge(sim, torch.ones(sim.Nx_padded), width, 0.1)
    assert math.isclose(math.exp(-layer.strength ** 2), math.sqrt(0.9 / 1.1), rel_tol=1e-12)
    g = dataclasses.replace(sim, damping=layer).grid()
    assert g.sponge == [(10, 10), (5, 5)] and g.sponge_strength == layer.strength
    assert dataclasses.replace(sim, damping=7).grid().sponge == 7
    with pytest.raises(ValueError):
        cw.sponge(sim, torch.ones(10, 10), width, 0.1)  # field does not cover the grid
    with pytest.raises(ValueError):
        cw.sponge(sim, None, width, 1.5)
    x, y = cw.grid_coords((4, 3), (0.5, 1.0), device="cpu")
    assert x.shape == (4, 3) and torch.allclose(x[:, 0], torch.tensor([-0.5, 0.0, 0.5, 1.0]))
    assert torch.allclose(y[0], torch.tensor([-1.0, 0.0, 1.0]))


def test_resample_and_adam():
    from neuralmech_gb300 import cuwave_compat as cw
    r = torch.arange(10, dtype=torch.float32)[:, None].repeat(1, 3)
    assert torch.allclose(cw.resample(r, 1.0, 1.0, 10), r)
    half = cw.resample(r, 1.0, 0.5, 19)
    assert torch.allclose(half[:, 0], torch.arange(19, dtype=torch.float32) / 2)
    opt = cw.Adam(lr=0.1)
    x = torch.zeros(3)
    x = opt.step(x, torch.tensor([1.0, -2.0, 0.0]))
    assert torch.allclose(x, torch.tensor([-0.1, 0.1, 0.0]), atol=1e-6)


def _plate(cuda, order=4, n=72, N=260, E=8):
    from neuralmech_gb300 import cuwave_compat as cw
    L = 1.0
    dx = (L / (n - 3), L / (n - 3))
    dt = 0.9 * cw.stable_dt(dx, 1.0, order)
    sim = cw.ScalarWave((n, n), dx, N, dt, space_order=order, wavespeed=1.0, density=1.0)
    t = np.arange(N) * dt
    elements = cw.line((0.1, L), (0.9, L), E)
    sources = cw.shots(sim, elements, cw.sineburst(t, 1.0, 12.0, 2))
    sensors = cw.Sensors(sim, elements)
    gamma_true = torch.ones(sim.Nx_padded, device=cuda)
    xx, yy = np.meshgrid(np.arange(n) * dx[0] - dx[0], np.arange(n) * dx[1] - dx[1], indexing="ij")
    void = (xx - 0.5) ** 2 + (yy - 0.55) ** 2 < 0.08 ** 2
    gamma_true[:n, :n][torch.from_numpy(void).to(cuda)] = 1e-4
    return cw, sim, sources, sensors, gamma_true


@pytest.mark.gpu
def test_plate_fwi_flow(cuda):
    """plate.py + 2D_fwi.py on the adapter: measure with the void, then Adam on
    the indicator from gamma = 1 lowers the misfit."""
    cw, sim, sources, sensors, gamma_true = _plate(cuda)
    observed = cw.measure(sim, sources, gamma_true, sensors)
    assert len(observed) == 8 and observed[0].shape == (sim.N, 8)
    gamma = torch.ones(sim.Nx_padded, device=cuda)
    opt = cw.Adam(lr=0.05)
    costs = []
    for _ in range(6):
        cost, grad = cw.misfit_gradient(sim, sources[::2], gamma, sensors, observed[::2])
        assert grad.shape == gamma.shape and torch.isfinite(grad).all()
        assert torch.count_nonzero(grad[sim.Nx[0]:]) == 0
        costs.append(float(cost))
        gamma = torch.clamp(opt.step(gamma, grad), 1e-3, 1.0)
    assert costs[-1] < 0.9 * costs[0], costs
    c2 = cw.misfit(sim, sources[::2], gamma, sensors, observed[::2])
    assert np.isfinite(c2)


@pytest.mark.gpu
def test_indicator_gradient_finite_difference(cuda, orc):
    """d misfit / d gamma of the adapter (GPU) against central differences of
    the same misfit computed by the FP64 oracle on the adapter's own grid,
    positions and scaled wavelets. (FP32 traces bound the gradient's precision
    by the residual-to-data ratio; the observed model differs by 10 % so that
    the residuals are not a cancellation of nearly equal traces.)"""
    cw, sim, sources, sensors, _ = _plate(cuda, order=8, N=220)
    gamma = torch.ones(sim.Nx_padded, device=cuda) * 0.8
    g_obs = gamma.clone()
    g_obs[30:40, 30:45] *= 1.1
    shots = sources[:3]
    observed = cw.measure(sim, shots, g_obs, sensors)
    cost, grad = cw.misfit_gradient(sim, shots, gamma, sensors, observed)

    src, wav, rec = cw._batch(sim, shots, sensors)
    p3 = lambda p: np.stack([p[..., 0], 0 * p[..., 0], p[..., 1]], -1).astype(np.int32)
    obs = torch.stack(observed).cpu().numpy().astype(np.float64)

    def J(gm):
        v = sim.velocity(gm).cpu().numpy().astype(np.float64)
        geo = orc.Geometry(vel=v, wavelet=wav.astype(np.float64), src=p3(src), rec=p3(rec),
                           dt=float(np.float32(sim.dt)), h=(sim.dx[0], 1.0, sim.dx[1]), order=8,
                           sponge=None, src_scale=1.0)
        return 0.5 * float(((orc.forward(geo) - obs) ** 2).sum())

    # gradient test along the steepest-descent direction: <g, d> = |g||d|, no
    # cancellation between cells of opposite sign in the projection
    d = 1e-3 * grad / grad.abs().max()
    fd = (J(gamma + d) - J(gamma - d)) / 2
    an = float((grad.double() * d.double()).sum())
    assert abs(fd - an) < 2e-3 * abs(fd), (fd, an)


@pytest.mark.gpu
def test_sponge_absorbs(cuda):
    """A pulse in a padded plate: with the sponge layer the field left after
    it has crossed the plate several times is far smaller than with
    reflecting edges."""
    import dataclasses
    from neuralmech_gb300 import cuwave_compat as cw
    Nx, width, origin, region = cw.pad_for_sponge((81, 81), (1 / 78, 1 / 78), 0.15)
    dx = (1 / 78, 1 / 78)
    dt = 0.5 * cw.stable_dt(dx, 1.0, 8)
    N = int(3.0 / dt)
    sim = cw.ScalarWave(Nx, dx, N, dt, space_order=8)
    t = np.arange(N) * dt
    src = cw.point_source(sim, ((origin[0] + 40) * dx[0] - dx[0], (origin[1] + 40) * dx[1] - dx[1]),
                          cw.sineburst(t, 1.0, 8.0, 2))
    gamma = torch.ones(sim.Nx_padded, device=cuda)
    plain = cw.simulate(sim, src, gamma)
    damped = cw.simulate(dataclasses.replace(sim, damping=cw.sponge(sim, gamma, width, 0.1)), src, gamma)
    e_plain = float((plain[region] ** 2).sum())
    e_damped = float((damped[region] ** 2).sum())
    assert np.isfinite(e_damped) and e_damped < 0.05 * e_plain


@pytest.mark.gpu
def test_simulate_frames_and_node_sensors(cuda):
    """simulate(..., sensors=sensors.nodes, record_every=k) returns
    (u, um, frames) as the analog-RNN drivers unpack it: um equals the record
    with a Sensors object, frame j equals the final field of a j k-step run,
    the last frame is u; Sensors.traces(um) is the record."""
    import dataclasses
    cw, sim, sources, sensors, gamma_true = _plate(cuda, N=120)
    u, um = cw.simulate(sim, sources[3], gamma_true, sensors)
    u2, um2, frames = cw.simulate(sim, sources[3], gamma_true, sensors=sensors.nodes, record_every=40)
    assert torch.equal(u2, u) and torch.equal(um2, um) and torch.equal(sensors.traces(um2), um2)
    assert frames.shape == (4,) + tuple(sim.Nx) and torch.all(frames[0] == 0) and torch.equal(frames[3], u)
    short = dataclasses.replace(sim, N=80)
    src80 = cw.Source(sources[3].nodes, sources[3].signal[:80])
    assert rel_l2(frames[2].cpu().numpy(), cw.simulate(short, src80, gamma_true).cpu().numpy()) < 1e-6
    u3, snaps = cw.simulate(sim, sources[3], gamma_true, record_every=60)
    assert torch.equal(u3, u) and snaps.shape[0] == 3


@pytest.mark.gpu
def test_simulate_3d_against_oracle(cuda, orc):
    """waveND.py with DIM = 3: ScalarWave on a cube, a point source at the
    origin, simulate() with sensors and frames. The final field and the
    record match the FP64 oracle run on the adapter's grid and positions."""
    from neuralmech_gb300 import cuwave_compat as cw
    n, N, order = 28, 60, 4
    dx = (1.0 / (n - 3),) * 3
    dt = 0.9 * cw.stable_dt(dx, 0.5, order)
    sim = cw.ScalarWave((n,) * 3, dx, N, dt, (4, 4, 64), space_order=order, wavespeed=0.5, density=1.0)
    t = np.arange(N) * dt
    source = cw.point_source(sim, (0.0, 0.0, 0.0), cw.sineburst(t, 1e3, 8.0, 2))
    sensors = cw.Sensors(sim, cw.line((0.2, 0.5, 0.3), (0.8, 0.5, 0.3), 5))
    indicator = torch.ones(sim.Nx_padded, device=cuda)
    indicator[10:16, 10:16, 10:16] = 0.25
    u, um, frames = cw.simulate(sim, source, indicator, sensors=sensors, record_every=20)
    assert u.shape == (n,) * 3 and um.shape == (N, 5) and frames.shape == (4,) + (n,) * 3
    assert torch.equal(frames[3], u)

    src, wav, rec = cw._batch(sim, source, sensors)
    geo = orc.Geometry(vel=sim.velocity(indicator).cpu().numpy().astype(np.float64),
                       wavelet=wav.astype(np.float64), src=src, rec=rec, dt=float(np.float32(dt)),
                       h=tuple(dx), order=order, sponge=None, src_scale=1.0)
    tr, fin = orc.forward(geo, want_final=True)
    assert rel_l2(u.cpu().numpy(), fin[(0,) + sim.interior]) < 1e-5
    assert rel_l2(um.cpu().numpy(), tr[0]) < 1e-5


@pytest.mark.gpu
def test_simulate_acoustic_against_oracle(cuda, orc):
    """waveND.py with FORMULATION = "acoustic": simulate() on an AcousticWave
    runs the two-phase medium. Final field, record and frames against the FP64
    variable-density oracle on the adapter's grid, materials and signals."""
    import dataclasses
    from neuralmech_gb300 import cuwave_compat as cw
    n, N = 48, 600
    dx = (1.0 / (n - 3),) * 2
    sim = cw.AcousticWave((n, n), dx, N, 1.0, space_order=4, rho1=1.204, rho2=2643.0, kappa1=1.419e5, kappa2=6.87e8)
    gamma = torch.ones((n, n), device=cuda)
    gamma[20:30, 15:35] = 0.3  # an air-like pocket in the solid: 1/rho jumps 1500x at its walls
    # the walls set the step: a solid cell beside the pocket meets the air's 1/rho
    vmax = sim.max_speed(gamma)
    assert vmax > 10 * float(sim.velocity(gamma).max())
    dt = 0.8 * cw.stable_dt(dx, vmax, 4)
    sim = dataclasses.replace(sim, dt=dt)
    t = np.arange(N) * dt
    source = cw.point_source(sim, (0.43, 0.45), cw.sineburst(t, 1e3, 6.0 / (N * dt), 2))
    sensors = cw.Sensors(sim, cw.line((0.35, 0.55), (0.55, 0.55), 4))
    u, um, frames = cw.simulate(sim, source, gamma, sensors=sensors.nodes, record_every=200)
    assert u.shape == (n, n) and um.shape == (N, 4) and frames.shape == (4, n, n)
    assert torch.isfinite(u).all() and u.abs().max() > 0 and torch.equal(frames[3], u)

    kap, rho = (a.cpu().numpy().astype(np.float64) for a in sim.materials(gamma))
    src, wav, rec = cw._batch(sim, cw._scaled_sources(sim, source, gamma), sensors)
    p3 = lambda p: np.stack([p[..., 0], 0 * p[..., 0], p[..., 1]], -1).astype(np.int32)

    def oracle(nt):
        geo = orc.VdGeometry(kap, rho, wav[:, :nt].astype(np.float64), p3(src), p3(rec), float(np.float32(dt)),
                             tuple(dx), order=4)
        return orc.vd_forward(geo, want_final=True)

    # FP32 against FP64 over 600 steps across a 1500x jump of 1/rho: 1.8e-5
    # measured on the final field; 5e-5 leaves room for the rounding's spread
    tol = 5e-5
    tr, fin = oracle(N)
    assert rel_l2(u.cpu().numpy(), fin[(0,) + sim.interior]) < tol
    assert rel_l2(um.cpu().numpy(), tr[0]) < tol
    assert rel_l2(frames[2].cpu().numpy(), oracle(400)[1][(0,) + sim.interior]) < tol


@pytest.mark.gpu
def test_simulate_matches_measure(cuda):
    cw, sim, sources, sensors, gamma_true = _plate(cuda, N=120)
    u, record = cw.simulate(sim, sources[3], gamma_true, sensors)
    assert u.shape == sim.Nx and torch.isfinite(u).all() and u.abs().max() > 0
    ref = cw.measure(sim, sources[3:4], gamma_true, sensors)[0]
    assert rel_l2(record.cpu().numpy(), ref.cpu().numpy()) < 1e-6
    # the last recorded sample is the final field at the sensor nodes
    nodes = sensors.nodes  # (2, nsensors) node numbers index simulate()'s field directly
    assert rel_l2(u[nodes[0], nodes[1]].cpu().numpy(), record[-1].cpu().numpy()) < 1e-6


@pytest.mark.gpu
def test_acoustic_indicator_gradient(cuda, orc):
    """The two-phase AcousticWave adapter: d misfit / d gamma (through kappa,
    rho and the source scaling) against central differences of the same
    misfit computed by the FP64 variable-density oracle on the adapter's own
    padded grid, positions and signals, along the steepest-descent direction."""
    from neuralmech_gb300 import cuwave_compat as cw
    n, N, E = 60, 200, 6
    dx = (1.0 / (n - 3), 1.0 / (n - 3))
    dt = 0.8 * cw.stable_dt(dx, float(np.sqrt(6.87e8 / 2643.0)), 8)
    sim = cw.AcousticWave((n, n), dx, N, dt, space_order=8, rho1=1.204, rho2=2643.0, kappa1=1.419e5, kappa2=6.87e8)
    t = np.arange(N) * dt
    elements = cw.line((0.1, 1.0), (0.9, 1.0), E)
    sources = cw.shots(sim, elements, cw.sineburst(t, 1.0, 8.0 / (N * dt), 2))[:3]
    sensors = cw.Sensors(sim, elements)
    gamma = torch.full((n, n), 0.8, device=cuda)
    g_obs = gamma.clone()
    g_obs[20:32, 25:40] = 0.95
    observed = cw.acoustic_measure(sim, sources, g_obs, sensors)
    cost, grad = cw.acoustic_misfit_gradient(sim, sources, gamma, sensors, observed)
    assert torch.isfinite(grad).all() and grad.abs().max() > 0
    obs = torch.stack(observed).cpu().numpy().astype(np.float64)
    p3 = lambda p: np.stack([p[..., 0], 0 * p[..., 0], p[..., 1]], -1).astype(np.int32)

    def J(gm):
        kap, rho = (a.cpu().numpy().astype(np.float64) for a in sim.materials(gm))
        src, wav, rec = cw._batch(sim, cw._scaled_sources(sim, sources, gm), sensors)
        geo = orc.VdGeometry(kap, rho, wav.astype(np.float64), p3(src), p3(rec), float(np.float32(sim.dt)),
                             tuple(sim.dx), order=8)
        return 0.5 * float(((orc.vd_forward(geo) - obs) ** 2).sum())

    d = 1e-3 * grad / grad.abs().max()
    fd = (J(gamma + d) - J(gamma - d)) / 2
    an = float((grad.double() * d.double()).sum())
    print("acoustic adapter: fd", fd, "analytic", an)
    assert abs(fd - an) < 5e-3 * abs(fd), (fd, an)


def test_parametrization_jacobian():
    """parametrization_jacobian against central differences of the adapter's
    own parametrisation: AcousticWave mass 1/kappa and stiffness 1/rho from
    materials(); ScalarWave (0, 1) with stiffness gamma."""
    from neuralmech_gb300 import cuwave_compat as cw
    ac = cw.AcousticWave((12, 10), (0.1, 0.1), 5, 1e-3, space_order=4, device="cpu")
    g = torch.full((12, 10), 0.4, dtype=torch.float64)
    dm, ds = ac.parametrization_jacobian(g)
    h = 0.2  # (1/kappa and 1/rho are linear in gamma; materials() returns FP32)

    def inv(gm):
        k, r = ac.materials(gm)
        return 1 / k.double(), 1 / r.double()

    (mp, sp), (mm, sm) = inv(g + h), inv(g - h)
    fd_m = float(((mp - mm) / (2 * h)).mean())
    fd_s = float(((sp - sm) / (2 * h)).mean())
    assert abs(float(dm[0, 0]) - fd_m) < 1e-3 * abs(fd_m)
    assert abs(float(ds[0, 0]) - fd_s) < 1e-3 * abs(fd_s)
    sc = cw.ScalarWave((12, 10), (0.1, 0.1), 5, 1e-3, space_order=4, device="cpu")
    z, o = sc.parametrization_jacobian(torch.ones((12, 10)))
    assert float(z.abs().max()) == 0.0 and float((o - 1).abs().max()) == 0.0


def test_reconstruction_nodes_frame():
    """reconstruction_nodes: the frame of sponge-width cells along every edge
    of the library's grid, in node numbers; none for a reflecting plate."""
    from neuralmech_gb300 import cuwave_compat as cw
    sim = cw.ScalarWave((40, 30), (0.1, 0.1), 5, 1e-3, space_order=8, damping=6, device="cpu")
    nodes, n = cw.reconstruction_nodes(sim)
    nz, nx = sim.grid_shape
    assert n == nz * nx - (nz - 12) * (nx - 12) and nodes.shape == (2, n)
    assert nodes.min() == -sim.margin and nodes[0].max() == nz - 1 - sim.margin
    plate = cw.ScalarWave((40, 30), (0.1, 0.1), 5, 1e-3, space_order=8, device="cpu")
    assert cw.reconstruction_nodes(plate)[1] == 0


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["scalar", "acoustic"])
def test_reconstruction_sensitivity_matches_checkpoint_adjoint(cuda, kind, monkeypatch):
    """reconstruction_sensitivity (the library's reconstruction adjoint,
    analog_rnn_train.py:142) combined with parametrization_jacobian as the
    driver combines it equals response_gradient with the checkpointed
    adjoint, here with FP32 checkpoints (BF16 checkpoints alone move the
    checkpointed gradient by ~1e-3 on this plate), on a padded plate with a
    sponge; the record and loss agree too. Both are the exact discrete
    gradient in FP32: 1e-5 relative L2 (measured 3.5e-7 and 4.2e-7)."""
    import dataclasses
    from neuralmech_gb300 import cuwave_compat as cw
    grid_of = cw.ScalarWave.grid
    monkeypatch.setattr(cw.ScalarWave, "grid", lambda self: dataclasses.replace(grid_of(self), ckpt_format="fp32"))
    n, N = 56, 240
    Nx, width, origin, region = cw.pad_for_sponge((n, n), (1 / (n - 3), 1 / (n - 3)), 0.1)
    dx = (1 / (n - 3), 1 / (n - 3))
    if kind == "scalar":
        dt = 0.5 * cw.stable_dt(dx, 1.0, 8)
        sim = cw.ScalarWave(Nx, dx, N, dt, space_order=8)
    else:
        dt = 0.5 * cw.stable_dt(dx, float(np.sqrt(6.87e8 / 2643.0)), 8)
        sim = cw.AcousticWave(Nx, dx, N, dt, space_order=8, rho1=1.204, rho2=2643.0, kappa1=1.419e5,
                              kappa2=6.87e8)
    gamma = torch.full(sim.Nx_padded, 0.85, device=cuda)
    gamma[origin[0] + 20:origin[0] + 30, origin[1] + 15:origin[1] + 35] = 0.6
    sim = dataclasses.replace(sim, damping=cw.sponge(sim, gamma, width, 0.1))
    t = np.arange(N) * dt
    c0 = ((origin[0] + 8) * dx[0], (origin[1] + n // 2) * dx[1])
    src = cw.point_source(sim, c0, cw.sineburst(t, 1.0, 6.0 / (N * dt), 2))
    sensors = cw.Sensors(sim, [((origin[0] + 8) * dx[0], (origin[1] + k) * dx[1]) for k in range(5, n - 5, 6)])
    obj = sensors.objective(cw.energy(sim))
    J1, g1 = cw.response_gradient(sim, src, gamma, sensors.nodes, obj)
    J2, grads, um, _ = cw.reconstruction_sensitivity(sim, src, gamma, sensors.nodes, obj)
    d_mass, d_stiff = sim.parametrization_jacobian(gamma)
    g2 = d_mass * grads["mass"] + d_stiff * grads["stiff"]
    J3, g3 = cw.response_gradient(sim, src, gamma, sensors.nodes, obj, adjoint=cw.reconstruction_sensitivity)
    assert um.shape == (N, sensors.nodes.shape[1])
    assert abs(J1 - J2) <= 1e-5 * abs(J1) and abs(J3 - J2) <= 1e-12 * abs(J2)
    assert torch.isfinite(g2).all() and float(g1.abs().max()) > 0
    err = rel_l2(g2.cpu().numpy(), g1.cpu().numpy())
    print(f"reconstruction_sensitivity ({kind}) vs checkpointed adjoint: gradient rel L2 {err:.2e}")
    assert err < 1e-5
    assert rel_l2(g3.cpu().numpy(), g2.cpu().numpy()) < 1e-12
