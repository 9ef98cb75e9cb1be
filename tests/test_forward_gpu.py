"""GPU parity of the forward path: the padded_step shim against the reference's
own kernel (golden vectors), and the generic forward against the FP64 oracle.
Tolerances: 1e-5 relative L2 against padded_step (FP32 vs FP32, different
operation order); 1e-5 relative L2 against the FP64 oracle for FP32 traces.
A known answer without the oracle: the homogeneous 2D and 3D Green's
functions convolved with the Ricker wavelet (5% and 3%: numerical dispersion
and the discrete point source).
"""
import math
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, rel_l2
from helpers import oracle_geometry, small_problem

pytestmark = pytest.mark.gpu


def test_step2d_order2_matches_padded_step(cuda):
    from neuralmech_gb300 import step2d_order2
    g = np.load(os.path.join(GOLDEN, "padded_step.npz"))
    for ci in range(2):
        N, M, MP, steps, c, dt, dx, dy = g[f"c{ci}_params"]
        N, M, MP, steps = int(N), int(M), int(MP), int(steps)
        a = torch.from_numpy(g[f"c{ci}_u0"]).to(cuda)
        b = torch.from_numpy(g[f"c{ci}_u1"]).to(cuda)
        for t in range(steps):
            # the driver's in-place rotation: u0 = fd_step(u0, u1, u0); u1, u0 = u0, u1
            a = step2d_order2(a, b, a, float(np.float32(c)), float(np.float32(dt)),
                              float(np.float32(dx)), float(np.float32(dy)), N, M)
            a, b = b, a
            key = f"c{ci}_step{t}"
            if key in g:
                got = b.cpu().numpy()
                assert rel_l2(got[:, :M], g[key][:, :M]) < 1e-5, (ci, t)
                # padding columns and the ring are never written
                assert np.array_equal(got[:, M:], g[key][:, M:])
                assert np.array_equal(got[0], g[key][0]) and np.array_equal(got[-1], g[key][-1])


def test_step2d_order2_separate_output(cuda):
    from neuralmech_gb300 import step2d_order2
    g = np.load(os.path.join(GOLDEN, "padded_step.npz"))
    N, M, MP, steps, c, dt, dx, dy = g["c0_params"]
    N, M = int(N), int(M)
    u0 = torch.from_numpy(g["c0_u0"]).to(cuda)
    u1 = torch.from_numpy(g["c0_u1"]).to(cuda)
    u2 = torch.full_like(u0, 7.0)
    step2d_order2(u0, u1, u2, float(c), float(dt), float(dx), float(dy), N, M)
    got = u2.cpu().numpy()
    assert rel_l2(got[1:-1, 1:M - 1], g["c0_step0"][1:-1, 1:M - 1]) < 1e-5
    assert np.all(got[0] == 7.0) and np.all(got[:, 0] == 7.0) and np.all(got[:, M - 1:] == 7.0)


@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("shape,sponge,nshot,spc,rows", [
    ((60, 150), 10, 3, 0, 0),
    ((37, 131), 0, 2, 1, 16),
    ((100, 260), (5, 12), 5, 2, 0),
    ((100, 260), (5, 12), 5, 3, 16),
    ((33, 40), 6, 1, 0, 0),
])
def test_forward_matches_oracle(cuda, orc, order, shape, sponge, nshot, spc, rows):
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=nshot, order=order,
                                           sponge=sponge if isinstance(sponge, int) else [sponge, sponge],
                                           nt=90, spc=spc, seed=order + nshot, tile_rows=rows)
    traces = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                          torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert traces.shape == ref.shape
    assert np.isfinite(ref).all() and np.abs(ref).max() > 0
    assert rel_l2(traces.cpu().numpy(), ref) < 1e-5


def test_forward_many_sources_and_duplicates(cuda, orc):
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(70, 300), nshot=4, nsrc=5, nrec=40, nt=80)
    src[:, 1] = src[:, 0]  # two sources on one cell (atomic injection)
    rec[:, 3] = rec[:, 2]  # two receivers on one cell
    traces = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                          torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert rel_l2(traces.cpu().numpy(), ref) < 1e-5
    t = traces.cpu().numpy()
    assert np.array_equal(t[:, :, 2], t[:, :, 3])


def test_forward_positions_on_interior_edge(cuda, orc):
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(48, 140), nshot=1, nrec=4, nt=60)
    R = grid.order // 2
    src[0, 0] = [R, R]
    rec[0] = [[R, R], [47 - R, 139 - R], [R, 139 - R], [47 - R, R]]
    traces = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                          torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert rel_l2(traces.cpu().numpy(), ref) < 1e-5


def test_forward_rejects_ring_positions(cuda):
    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300._lib import WaveFDError
    grid, v, wav, src, rec = small_problem(shape=(40, 140), nshot=1, nt=10)
    rec[0, 0] = [1, 20]  # inside the fixed ring of order 8
    with pytest.raises(WaveFDError):
        wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                     torch.from_numpy(src), torch.from_numpy(rec), grid)


def test_forward_no_receivers_no_sources(cuda):
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(40, 140), nshot=2, nt=10)
    out = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                       torch.from_numpy(src), torch.zeros((2, 0, 2), dtype=torch.int32), grid)
    assert out.shape == (2, 10, 0)
    out = wave_forward(torch.from_numpy(v).to(cuda), torch.zeros((2, 10, 0), device=cuda),
                       torch.zeros((2, 0, 2), dtype=torch.int32), torch.from_numpy(rec), grid)
    assert torch.count_nonzero(out) == 0


@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("shape,nshot,sponge", [
    ((70, 20, 72), 2, 5),     # two z chunks, two x tiles, two y tiles
    ((30, 37, 41), 1, 0),     # odd sizes, one chunk
    ((67, 18, 70), 2, 4),     # a last chunk of 3 planes: an iteration of one plane
])
def test_forward_3d_matches_oracle(cuda, orc, order, shape, nshot, sponge):
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=nshot, order=order, sponge=sponge,
                                           nt=50, nrec=25, seed=order + 7)
    traces = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                          torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert np.abs(ref).max() > 0
    assert rel_l2(traces.cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("shape,nshot,nt,sponge", [
    ((70, 250), 3, 91, 8),    # odd step count: a one-step launch at the end
    ((40, 130), 2, 60, 0),
    ((100, 370), 4, 75, (5, 11)),
])
def test_forward_two_step_blocking(cuda, orc, order, shape, nshot, nt, sponge):
    """step_block=2 (two steps per launch, u_{n+1} kept in shared memory) against
    the FP64 oracle; sources and receivers sit on and around tile seams, where
    the injections of neighbouring tiles' extended regions must agree."""
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=nshot, nt=nt, order=order,
                                           sponge=sponge if isinstance(sponge, int) else [sponge, sponge],
                                           nsrc=3, nrec=20, step_block=2, seed=order * 3 + nshot)
    R = order // 2
    seams_x = [x for x in (116, 117, 119, 120, 121, 123, 124, 239, 240, 243) if R <= x < shape[1] - R]
    seams_z = [z for z in (28, 29, 31, 32, 33, 35, 36, 63, 64, 65) if R <= z < shape[0] - R]
    for s in range(nshot):
        for i in range(3):
            src[s, i] = [seams_z[(s + i) % len(seams_z)], seams_x[(2 * s + i) % len(seams_x)]]
        for i in range(min(10, rec.shape[1])):
            rec[s, i] = [seams_z[(i + s) % len(seams_z)], seams_x[(i * 3 + s) % len(seams_x)]]
    traces = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                          torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert np.abs(ref).max() > 0
    assert rel_l2(traces.cpu().numpy(), ref) < 1e-5


@pytest.mark.parametrize("ndim", [2, 3])
def test_homogeneous_greens_function(cuda, ndim):
    """Known answer, no oracle: the CUDA forward in a homogeneous medium against
    the analytic Green's function convolved with the Ricker wavelet, before
    any boundary reflection (numerical dispersion and the discrete point source
    bound the agreement).
      2D: u = 1/(2 pi c^2) int_0^acosh(ct/r) w(t - (r/c) cosh s) ds (< 5%);
      3D: u = w(t - r/c) / (4 pi c^2 r) (< 3%).
    A discrete source adds w_n dt^2 / h^ndim per step; traces[n] = u(t_{n+1})."""
    from neuralmech_gb300 import Grid, wave_forward
    from neuralmech_gb300.synth import ricker
    h, c, f, r_cells = 5.0, 2000.0, (20.0 if ndim == 2 else 25.0), (60 if ndim == 2 else 30)
    n = 401 if ndim == 2 else 161
    dt = (0.4 if ndim == 2 else 0.3) * h / c
    nt = 300
    s0 = n // 2
    grid = Grid((n,) * ndim, (h,) * ndim, dt, nt, order=8, sponge=0, src_scale=dt * dt / h**ndim)
    wav = torch.from_numpy(ricker(f, nt, dt).astype(np.float32)).reshape(1, nt, 1).to(cuda)
    src = np.full((1, 1, ndim), s0, dtype=np.int32)
    rec = np.full((1, 2, ndim), s0, dtype=np.int32)
    rec[0, 0, -1] += r_cells  # along x
    rec[0, 1, 0] += r_cells   # along z
    vel = torch.full((n,) * ndim, c, device=cuda)
    tr = wave_forward(vel, wav, torch.from_numpy(src), torch.from_numpy(rec), grid)[0].double().cpu().numpy()
    r = r_cells * h
    t = (np.arange(nt) + 1) * dt
    t0 = 1.5 / f

    def w(tt):
        a = (math.pi * f * (tt - t0)) ** 2
        return np.where(tt >= 0, (1 - 2 * a) * np.exp(-a), 0.0)

    if ndim == 3:
        ana = w(t - r / c) / (4 * math.pi * c * c * r)
    else:
        ana = np.zeros(nt)
        for i, ti in enumerate(t):
            if ti * c > r:
                sv = np.linspace(0.0, math.acosh(ti * c / r), 4001)
                ana[i] = np.trapezoid(w(ti - (r / c) * np.cosh(sv)), sv) / (2 * math.pi * c * c)
    win = (t > r / c) & (t < r / c + t0 + 2 / f)
    for j in range(2):
        err = rel_l2(tr[win, j], ana[win])
        print(f"{ndim}D Green's function, receiver {j}: rel L2 {err:.3e}")
        assert err < (0.05 if ndim == 2 else 0.03)


@pytest.mark.parametrize("order,shape,nshot,nt,sponge", [
    (2, (100, 600), 3, 77, 10),            # 3 x 5 windows, a last launch of 5 steps
    (4, (53, 487), 2, 61, [(6, 11), (4, 9)]),  # odd sizes, per-face sponge, a last launch of 1 step
    (2, (30, 250), 1, 40, 0),              # one window row, no sponge
    (4, (240, 260), 2, 33, 8),
])
def test_forward_register_window(cuda, orc, order, shape, nshot, nt, sponge):
    """step_block 8 (order 2) and 4 (order 4): K steps per launch in a register
    window, against the FP64 oracle (1e-5) and the one-step forward (traces
    and final level, 1e-6). Sources and receivers sit on and around the window
    seams (columns 240 k and 240 k +- 8, rows 24 k and 24 k +- 8), where a
    source joins up to four windows' halos."""
    import dataclasses
    from neuralmech_gb300 import wave_forward
    from neuralmech_gb300.wavefd import wave_forward_final
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=nshot, nt=nt, order=order, sponge=sponge,
                                           nsrc=3, nrec=40, seed=order * 5 + nshot)
    R = order // 2
    nz, nx = shape
    clampz = lambda z: int(min(max(z, R), nz - R - 1))
    clampx = lambda x: int(min(max(x, R), nx - R - 1))
    seams = [(24, 240), (16, 232), (32, 248), (23, 239), (47, 241), (8, 120)]
    for s in range(nshot):
        for i in range(3):
            z, x = seams[(s + i) % len(seams)]
            src[s, i] = [clampz(z), clampx(x)]
        for i in range(12):
            z, x = seams[i % len(seams)]
            rec[s, i] = [clampz(z + i // len(seams)), clampx(x + 2 * (i // len(seams)))]
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    gk = dataclasses.replace(grid, step_block=8 if order == 2 else 4)
    g1 = dataclasses.replace(grid, step_block=1)
    tk = wave_forward(*args, gk).cpu().numpy()
    t1 = wave_forward(*args, g1).cpu().numpy()
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert np.abs(ref).max() > 0
    assert rel_l2(tk, ref) < 1e-5
    assert rel_l2(tk, t1) < 1e-6
    fk = wave_forward_final(*args, gk)[1].cpu().numpy()
    f1 = wave_forward_final(*args, g1)[1].cpu().numpy()
    assert np.abs(f1).max() > 0
    assert rel_l2(fk, f1) < 1e-6


def test_forward_register_window_many_points(cuda, orc):
    """More than the 1024 sources and receivers a CTA links into its
    per-column lists (1100 sources in one window, 1500 receivers in one
    tile): the overflow entries take the scanning path, with the same results
    as one step per launch (1e-6) and the FP64 oracle (1e-5)."""
    import dataclasses
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(40, 250), nshot=1, nt=20, order=2, sponge=4, nsrc=1, nrec=1,
                                           seed=31)
    rng = np.random.default_rng(31)
    cells = rng.permutation(16 * 200)[:1500]  # distinct cells of tile (0, 0): rows 8..23, columns 20..219
    rec = np.stack([8 + cells // 200, 20 + cells % 200], -1)[None].astype(np.int32)
    src = np.stack([rng.integers(2, 38, 1100), rng.integers(2, 248, 1100)], -1)[None].astype(np.int32)
    wav = (np.repeat(wav[:, :, :1], 1100, axis=2) * rng.uniform(0.5, 1.5, (1, 1, 1100))).astype(np.float32)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    tk = wave_forward(*args, dataclasses.replace(grid, step_block=8)).cpu().numpy()
    t1 = wave_forward(*args, dataclasses.replace(grid, step_block=1)).cpu().numpy()
    ref = orc.forward(oracle_geometry(orc, grid, v, wav, src, rec))
    assert np.abs(ref).max() > 0
    assert rel_l2(tk, t1) < 1e-6
    assert rel_l2(tk, ref) < 1e-5
