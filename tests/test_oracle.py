"""CPU tests of the oracle: pinned against the reference's own kernels
(golden vectors from oracle/_ref, i.e. step2D_wave.cu / step1D_wave.cu compiled
for the CPU), cross-checked with the NumPy slice-form restatement, and its
adjoint gradient checked against finite differences in FP64."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_l2


def test_fd_weights_taylor(orc):
    """Order-2R weights are exact on polynomials up to degree 2R+1."""
    for order in (2, 4, 6, 8):
        a = orc.fd_coeffs(order)
        R = order // 2
        for deg in range(0, 2 * R + 2):
            # second derivative of x^deg at 0 from samples at k = -R..R (h = 1)
            f = lambda k: float(k) ** deg
            d2 = a[0] * f(0) + sum(a[k] * (f(k) + f(-k)) for k in range(1, R + 1))
            exact = 2.0 if deg == 2 else 0.0
            assert abs(d2 - exact) < 1e-9, (order, deg)
        # residual of the first neglected term is nonzero
        f = lambda k: float(k) ** (2 * R + 2)
        assert abs(a[0] * f(0) + sum(a[k] * (f(k) + f(-k)) for k in range(1, R + 1))) > 1e-3
    a8 = orc.fd_coeffs(8)
    assert abs(abs(a8[0]) + 2 * np.abs(a8[1:]).sum() - 6.5016) < 1e-4


def test_oracle_pinned_to_padded_step(orc):
    """The FP64 oracle in order-2, constant-speed, Dirichlet form reproduces the
    reference kernel padded_step (golden vectors) over several steps."""
    g = np.load(os.path.join(GOLDEN, "padded_step.npz"))
    for ci in range(2):
        N, M, MP, steps, c, dt, dx, dy = g[f"c{ci}_params"]
        N, M, steps = int(N), int(M), int(steps)
        a = g[f"c{ci}_u0"][:, :M].astype(np.float64)
        b = g[f"c{ci}_u1"][:, :M].astype(np.float64)
        f32 = lambda x: float(np.float32(x))
        w = (f32(c) * f32(dt)) ** 2
        for t in range(steps):
            orc.step(2, (f32(dx), 1.0, f32(dy)), a, b, a, w_const=w)
            a, b = b, a
            key = f"c{ci}_step{t}"
            if key in g:
                assert rel_l2(b, g[key][:, :M]) < 1e-5, (ci, t)


def test_numpy_fd_step_is_reference_bitwise():
    """The NumPy restatement of 2D_wave_cupy.py:54-62 equals padded_step's
    host build bit for bit on the first step (same operation order, FP32)."""
    from oracle import numpy_ref
    g = np.load(os.path.join(GOLDEN, "padded_step.npz"))
    N, M, MP, steps, c, dt, dx, dy = g["c0_params"]
    M = int(M)
    u0 = g["c0_u0"][:, :M].copy()
    u1 = g["c0_u1"][:, :M].copy()
    u2 = u0.copy()
    numpy_ref.fd_step_order2(u0, u1, u2, np.float32(dt), np.float32(dx), np.float32(dy), np.float32(c))
    assert rel_l2(u2, g["c0_step0"][:, :M]) < 1e-6


def test_temporal_golden_is_padded_restatement():
    """temporal_step's golden levels (eight and sixteen padded_step updates of
    the reference's host build) equal the NumPy restatement of the padded_step
    expression (oracle.numpy_ref._update_order2, FP32, the kernel's operation
    order) bit for bit, on every cell the steps update."""
    from oracle import numpy_ref
    g = np.load(os.path.join(GOLDEN, "temporal_step.npz"))
    f32 = np.float32
    for ci in range(3):
        N, M, MP, c, dt, dx, dy = g[f"c{ci}_params"]
        N, M = int(N), int(M)
        k = f32(dt) * f32(dt) * f32(c) * f32(c)
        dx2, dy2 = f32(dx) * f32(dx), f32(dy) * f32(dy)
        a, b = g[f"c{ci}_u0"].copy(), g[f"c{ci}_u1"].copy()
        for t in range(16):
            new = a.copy()
            new[1:-1, 1:M - 1] = numpy_ref._update_order2(
                a[1:-1, 1:M - 1], b[1:-1, 1:M - 1], b[:-2, 1:M - 1], b[2:, 1:M - 1], b[1:-1, :M - 2],
                b[1:-1, 2:M], k, dx2, dy2)
            a, b = b, new
            key = f"c{ci}_after{t + 1}_v0"
            if key in g:
                assert np.array_equal(a, g[key]) and np.array_equal(b, g[f"c{ci}_after{t + 1}_v1"]), (ci, t)


def test_step1d_golden_vs_oracle(orc):
    """step1D (step1D_wave.cu:4-17) as the 1-row special case of the oracle."""
    g = np.load(os.path.join(GOLDEN, "step1d.npz"))
    N, c, dt, dx = g["params"]
    N = int(N)
    # embed the 1D line as the middle row of a 3-row grid with no z coupling
    f32 = lambda x: float(np.float32(x))
    a = g["u0"].astype(np.float64)[None, :].repeat(3, 0)
    b = a.copy()
    for t in range(25):
        n = a.copy()
        orc.step(2, (1e30, 1.0, f32(dx)), a, b, n, w_const=(f32(c) * f32(dt)) ** 2)
        n[0] = n[1]
        n[2] = n[1]
        a, b = b, n
        if f"step{t}" in g:
            assert rel_l2(b[1], g[f"step{t}"]) < 1e-5


def test_mixed_step_golden_close_to_fp32(orc):
    """mixed_step (FP16 storage) stays within FP16 accuracy of the FP32 path."""
    g = np.load(os.path.join(GOLDEN, "mixed_step.npz"))
    p = np.load(os.path.join(GOLDEN, "padded_step.npz"))
    N, M, MP, steps, c, dt, dx, dy = g["c0_params"]
    M, steps = int(M), int(steps)
    last = f"c0_step{steps - 1}"
    assert rel_l2(g[last][:, :M].astype(np.float32), p[last][:, :M]) < 2e-2


@pytest.mark.parametrize("shape,order", [((20, 21, 22), 8), ((20, 21, 22), 4), ((20, 21, 22), 2),
                                         ((30, 37), 8), ((30, 37), 4), ((30, 37), 2)])
def test_numpy_generic_matches_oracle(orc, shape, order):
    """The oracle's constant-density step against the NumPy slice-form
    restatement: 2D and 3D, orders 2/4/8, unequal spacings, per-axis sponge."""
    from oracle import numpy_ref
    rng = np.random.default_rng(order + len(shape))
    u = [rng.standard_normal(shape) for _ in range(2)]
    w = rng.uniform(0.05, 0.2, shape)
    prof = [rng.uniform(0.8, 1, n) for n in shape]
    G = np.ones(shape)
    for axis, pr in enumerate(prof):
        G = G * pr.reshape([-1 if i == axis else 1 for i in range(len(shape))])
    h = (1.0, 1.1, 0.9) if len(shape) == 3 else (1.0, 0.9)
    a = u[0].copy()
    numpy_ref.fd_step(u[0], u[1], a, w, h, order=order, g=G)
    b = u[0].copy()
    sponge = tuple(prof) if len(shape) == 3 else (prof[0], None, prof[1])
    orc.step(order, h if len(shape) == 3 else (h[0], 1.0, h[1]), u[0], u[1], b, w=w, sponge=sponge)
    assert rel_l2(a, b) < 1e-14


def _tiny(orc, order=8, ndim=2, nshot=2, nt=70, seed=0, ckpt=0):
    from helpers import oracle_geometry, small_problem
    shape = (36, 52) if ndim == 2 else (20, 22, 24)
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=nshot, nt=nt, order=order, sponge=6,
                                           seed=seed, ckpt_every=ckpt, nrec=9)
    geo = oracle_geometry(orc, grid, v.astype(np.float64), wav, src, rec)
    rng = np.random.default_rng(seed + 1)
    vt = v * (1 + 0.03 * rng.standard_normal(v.shape))
    geo_t = oracle_geometry(orc, grid, vt, wav, src, rec)
    obs = orc.forward(geo_t)
    return geo, obs


@pytest.mark.parametrize("order,ndim,ckpt", [(8, 2, 0), (2, 2, 7), (4, 3, 5)])
def test_oracle_gradient_finite_differences(orc, order, ndim, ckpt):
    """The oracle's adjoint gradient vs central differences of its own FP64
    misfit (validates the adjoint derivation independently of the GPU)."""
    geo, obs = _tiny(orc, order=order, ndim=ndim, ckpt=ckpt, nt=60 if ndim == 2 else 40)
    J, g, gw, _ = orc.gradient(geo, obs)
    rng = np.random.default_rng(3)
    v0 = geo.vel.copy()
    for _ in range(3):
        d = rng.standard_normal(v0.shape)
        d *= 1e-4 * np.abs(v0).mean() / np.abs(d).max()
        Js = []
        for sgn in (1, -1):
            geo.vel = v0 + sgn * d
            Js.append(0.5 * ((orc.forward(geo) - obs) ** 2).sum())
        fd = (Js[0] - Js[1]) / 2
        an = float((g * d).sum())
        assert abs(fd - an) <= 1e-6 * abs(fd) + 1e-30, (fd, an)
    geo.vel = v0
    # wavelet gradient: the misfit is quadratic in the wavelet
    dw = rng.standard_normal(geo.wavelet.shape) * 1e-3
    w0 = geo.wavelet.copy()
    Js = []
    for sgn in (1, -1):
        geo.wavelet = w0 + sgn * dw
        Js.append(0.5 * ((orc.forward(geo) - obs) ** 2).sum())
    geo.wavelet = w0
    fd = (Js[0] - Js[1]) / 2
    assert abs(fd - float((gw * dw).sum())) <= 1e-8 * abs(fd)


def test_oracle_checkpoint_interval_invariance(orc):
    geo, obs = _tiny(orc, nt=50)
    res = []
    for k in (1, 7, 50, 0):
        geo.ckpt_every = k
        res.append(orc.gradient(geo, obs)[1])
    for r in res[1:]:
        assert rel_l2(r, res[0]) < 1e-13


def test_oracle_homogeneous_greens_function(orc):
    """Known answer: in a homogeneous 2D medium, far from the source and before
    any boundary reflection, the trace is the 2D Green's function of
    u_tt - c^2 Lap u = delta(x) delta(t), G = H(t - r/c) / (2 pi c^2 sqrt(t^2 - r^2/c^2)),
    convolved with the injected wavelet.
    With u_tt = c^2 Lap u + f, a discrete source adds w_n * dt^2 / h^2 per step.
    """
    from neuralmech_gb300.synth import ricker
    n, h, c = 401, 5.0, 2000.0
    dt = 0.4 * h / c
    nt = 300
    f = 20.0
    wav = ricker(f, nt, dt).astype(np.float64)
    sz, sx = 200, 200
    r_cells = 60
    geo = orc.Geometry(vel=np.full((n, n), c), wavelet=wav[None, :, None],
                       src=np.array([[[sz, 0, sx]]], dtype=np.int32),
                       rec=np.array([[[sz, 0, sx + r_cells]]], dtype=np.int32), dt=dt,
                       h=(h, 1.0, h), order=8, sponge=None, src_scale=dt * dt / (h * h))
    tr = orc.forward(geo)[0, :, 0]
    # trace_n = u(t_{n+1}); u(t) = 1/(2 pi c^2) int_0^acosh(ct/r) w(t - (r/c) cosh s) ds
    # (tau = (r/c) cosh s removes the 1/sqrt singularity of G)
    r = r_cells * h
    t = (np.arange(nt) + 1) * dt
    t0 = 1.5 / f

    def w(tt):
        a = (math.pi * f * (tt - t0)) ** 2
        return np.where(tt >= 0, (1 - 2 * a) * np.exp(-a), 0.0)

    ana = np.zeros(nt)
    for i, ti in enumerate(t):
        if ti * c > r:
            s = np.linspace(0.0, math.acosh(ti * c / r), 4001)
            ana[i] = np.trapezoid(w(ti - (r / c) * np.cosh(s)), s) / (2 * math.pi * c * c)
    win = (t > r / c) & (t < r / c + t0 + 2 / f)
    assert rel_l2(tr[win], ana[win]) < 0.05


def test_oracle_homogeneous_greens_function_3d(orc):
    """Known answer in 3D: in a homogeneous medium the point source of
    u_tt - c^2 Lap u = s(t) delta(x) radiates u(r, t) = s(t - r/c) / (4 pi c^2 r).
    A discrete source adds w_n dt^2 / h^3 per step; trace_n = u(t_{n+1}).
    Receivers on two axes, 30 cells out, before any boundary reflection."""
    from neuralmech_gb300.synth import ricker
    n, h, c = 161, 5.0, 2000.0
    dt = 0.3 * h / c
    nt, f = 300, 25.0
    wav = ricker(f, nt, dt).astype(np.float64)
    s0, r_cells = n // 2, 30
    geo = orc.Geometry(vel=np.full((n, n, n), c), wavelet=wav[None, :, None],
                       src=np.array([[[s0, s0, s0]]], dtype=np.int32),
                       rec=np.array([[[s0, s0, s0 + r_cells], [s0 + r_cells, s0, s0]]], dtype=np.int32),
                       dt=dt, h=(h, h, h), order=8, sponge=None, src_scale=dt * dt / h**3)
    tr = orc.forward(geo)[0]
    r = r_cells * h
    t = (np.arange(nt) + 1) * dt
    t0 = 1.5 / f
    a = (math.pi * f * (t - r / c - t0)) ** 2
    ana = np.where(t >= r / c, (1 - 2 * a) * np.exp(-a), 0.0) / (4 * math.pi * c * c * r)
    win = (t > r / c) & (t < r / c + t0 + 2 / f)
    for j in range(2):
        assert rel_l2(tr[win, j], ana[win]) < 0.03


def test_scaled_step_restatement_tracks_fp32():
    """The NumPy restatement of scaled_step (the golden source for
    wfd_step2d_scaled) stays within int16 quantisation of the FP32 slice step
    (pinned to padded_step above) on the same field, and its encoding round
    trips to 1/65534 of each block's largest magnitude."""
    from oracle import numpy_ref as nr
    N, M, MP = 48, 90, 128
    dx, dy = 1.0 / (N - 1), 2.0 / (M - 1)
    dt = 0.95 * min(dx, dy) / math.sqrt(2)
    f32 = np.float32
    x = np.linspace(0, 1, N)[:, None]
    y = np.linspace(0, 2, M)[None, :]
    u = np.zeros((N, MP), f32)
    u[:, :M] = np.exp(-((x - 0.5) ** 2 + (y - 0.9) ** 2) / (2 * 0.1**2))
    u[0] = u[-1] = 0
    u[:, 0] = 0
    u[:, M - 1:] = 0
    q, s = nr.scaled_encode(u)
    dec = np.repeat(s, 32, axis=1) * q
    blockmax = np.repeat(np.abs(u).reshape(N, MP // 32, 32).max(axis=2), 32, axis=1)
    assert np.all(np.abs(dec - u) <= blockmax / 65534 * 1.0001 + 1e-30)
    a, b = (q.copy(), s.copy()), (q.copy(), s.copy())
    fa, fb = u[:, :M].copy(), u[:, :M].copy()
    for _ in range(12):
        a = nr.scaled_step(a[0], a[1], b[0], b[1], 1.0, dt, dx, dy, N, M)
        a, b = b, a
        fa = nr.fd_step_order2(fa, fb, fa, f32(dt), f32(dx), f32(dy), f32(1.0))
        fa, fb = fb, fa
    got = (np.repeat(b[1], 32, axis=1) * b[0])[:, :M]
    assert np.linalg.norm(got - fb) / np.linalg.norm(fb) < 2e-4
    assert np.all(b[0][:, M - 1:] == 0) and np.all(b[0][1:-1, 0] == 0)


def test_staggered_weights_taylor(orc):
    """sum_k c_k (2k-1)^(2j+1) = 1 for j = 0 and 0 for 0 < j < R: exact first
    derivatives of the odd monomials up to degree 2R - 1 at the half point."""
    for order in (2, 4, 8):
        c = orc.stag_coeffs(order)
        R = order // 2
        for j in range(R):
            terms = [c[k - 1] * (2 * k - 1) ** (2 * j + 1) for k in range(1, R + 1)]
            assert abs(sum(terms) - (1.0 if j == 0 else 0.0)) < 1e-14 * sum(abs(t) for t in terms)


def _vd_case(orc, order, sponge=True, seed=0):
    rng = np.random.default_rng(seed)
    nz, nx, nt = 34, 46, 70
    kap = 2.0e9 * (1 + 0.2 * rng.random((nz, nx)))
    rho = 1000.0 * (1 + 0.5 * rng.random((nz, nx)))
    rho[10:16, 15:30] = 2600.0  # a dense inclusion: a sharp interface
    dt, h = 1e-4, (6.0, 5.0)
    wav = np.zeros((2, nt, 1))
    wav[:, :12, 0] = np.sin(0.5 * np.arange(12))[None] * np.array([[1.0], [0.7]])
    src = np.array([[[17, 0, 23]], [[12, 0, 9]]])
    rec = np.array([[[8, 0, 10], [22, 0, 36], [12, 0, 30]]] * 2)
    sp = None
    if sponge:
        from neuralmech_gb300 import sponge_profile
        sp = (sponge_profile(nz, 6, 6).astype(np.float64), sponge_profile(nx, 6, 6).astype(np.float64))
    return orc.VdGeometry(kap, rho, wav, src, rec, dt, h, order=order, sponge=sp)


def test_vd_constant_density_order2_is_the_scalar_step(orc):
    """At order 2 the staggered operator with constant rho is the 5-point
    Laplacian: the variable-density oracle equals the scalar one with v^2 = kappa/rho."""
    g = _vd_case(orc, 2)
    g.rho = np.full_like(g.rho, 1500.0)
    vel = np.sqrt(g.kappa / g.rho)
    t_vd = orc.vd_forward(g)
    gs = orc.Geometry(vel=vel, wavelet=g.wavelet, src=g.src, rec=g.rec, dt=g.dt, h=(g.h[0], 1.0, g.h[1]), order=2,
                      sponge=(g.sponge[0], None, g.sponge[1]))
    t_sc = orc.forward(gs)
    assert rel_l2(t_vd, t_sc) < 1e-12


@pytest.mark.parametrize("order,sponge", [(2, False), (4, False), (8, False), (4, True)])
def test_vd_operator_matches_assembled_matrix(orc, order, sponge):
    """The oracle's variable-density step applies the documented staggered
    operator and sponge: from u_1 = g w_0 (a point source on every interior
    cell, w_1 = 0), u_2 / g - 2 u_1 = dt^2 kappa Lb u_1, g = gz[z] gx[x], with
    kappa Lb assembled term by term as a matrix, on random kappa, rho with a
    100x jump of rho (and random sponge profiles)."""
    from helpers import vd_operator
    R, n, dt = order // 2, 16, 0.01
    rng = np.random.default_rng(order)
    kappa = rng.uniform(1.0, 3.0, (n, n))
    rho = rng.uniform(0.5, 2.0, (n, n))
    rho[:, n // 2:] *= 100.0
    cells = [(z, x) for z in range(R, n - R) for x in range(R, n - R)]
    src = np.array([[z, 0, x] for z, x in cells], dtype=np.int32)[None]
    amp = rng.standard_normal(len(cells))
    gz, gx = (rng.uniform(0.9, 1.0, n), rng.uniform(0.9, 1.0, n)) if sponge else (np.ones(n), np.ones(n))

    def final(nt):
        wav = np.zeros((1, nt, len(cells)))
        wav[0, 0, :] = amp
        geo = orc.VdGeometry(kappa, rho, wav, src, np.zeros((1, 0, 3), np.int32), dt, (1.0, 1.0), order=order,
                             sponge=(gz, gx) if sponge else None)
        return orc.vd_forward(geo, want_final=True)[1][0].ravel()

    idx = [z * n + x for z, x in cells]
    g = np.outer(gz, gx).ravel()[idx]
    u1, u2 = final(1), final(2)
    assert np.allclose(u1[idx], g * amp, rtol=1e-15, atol=0)
    rhs = dt * dt * (vd_operator(kappa, rho, orc.stag_coeffs(order)) @ u1[idx])
    assert np.abs(u2[idx] / g - 2 * u1[idx] - rhs).max() < 1e-11 * np.abs(rhs).max()


@pytest.mark.parametrize("order", [2, 8])
def test_vd_gradient_finite_differences(orc, order):
    """The variable-density adjoint gradient w.r.t. kappa and rho (every cell,
    the fixed ring included: rho there enters the boundary fluxes) against
    central differences of the FP64 misfit."""
    g = _vd_case(orc, order)
    obs = orc.vd_forward(orc.VdGeometry(**{**g.__dict__, "kappa": g.kappa * 1.03}))
    J, gk, gr, gw, _ = orc.vd_gradient(g, obs)
    rng = np.random.default_rng(4)
    for name, grad in (("kappa", gk), ("rho", gr)):
        base = getattr(g, name)
        d = rng.standard_normal(base.shape) * base
        eps = 1e-6

        def Jof(v):
            t = orc.vd_forward(orc.VdGeometry(**{**g.__dict__, name: v}))
            return 0.5 * ((t - obs) ** 2).sum()

        fd = (Jof(base + eps * d) - Jof(base - eps * d)) / (2 * eps)
        an = float((grad * d).sum())
        assert abs(fd - an) < 1e-6 * abs(fd), (name, fd, an)
    # wavelet gradient: one sample
    wav = g.wavelet.copy()
    eps = 1e-6
    wp, wm = wav.copy(), wav.copy()
    wp[1, 5, 0] += eps
    wm[1, 5, 0] -= eps
    Jp = 0.5 * ((orc.vd_forward(orc.VdGeometry(**{**g.__dict__, "wavelet": wp})) - obs) ** 2).sum()
    Jm = 0.5 * ((orc.vd_forward(orc.VdGeometry(**{**g.__dict__, "wavelet": wm})) - obs) ** 2).sum()
    assert abs((Jp - Jm) / (2 * eps) - gw[1, 5, 0]) < 1e-6 * abs(gw[1, 5, 0])


def test_scaled_golden_is_the_reference_kernel_and_restatement():
    """scaled_step.npz comes from the reference's own scaled_step run on the
    GPU (make_golden_gpu.py: its source built for sm_103a with IEEE division
    and no fused multiply-adds); the NumPy restatement that the GPU drop-in
    was written against gives the same int16 levels and scales, bit for bit."""
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import scaled_golden
    want = np.load(os.path.join(GOLDEN, "scaled_step.npz"))
    got = scaled_golden(write=False)
    assert sorted(got) == sorted(want.keys())
    for k in want.keys():
        assert np.array_equal(got[k], want[k]), k


def test_temporal_golden_is_the_reference_kernel():
    """The committed temporal_step levels (8 and 16 padded_step updates of the
    reference's CPU build) are what the reference's own temporal_step returns
    after one and two launches on the GPU: equal SHA-256 digests (recorded by
    make_golden_gpu.py from that GPU run)."""
    import json
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden_gpu import digest
    with open(os.path.join(GOLDEN, "ref_gpu_digests.json")) as f:
        ref = json.load(f)["temporal_step"]
    g = np.load(os.path.join(GOLDEN, "temporal_step.npz"))
    checked = 0
    for k in g.keys():
        if "_after" in k:
            assert digest(g[k]) == ref[k], k
            checked += 1
    assert checked >= 10
