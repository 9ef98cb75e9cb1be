"""GPU parity of the adjoint path (hand-written adjoint kernel behind
torch.autograd.Function, checkpointed recomputation).

Tolerances (relative L2 unless stated):
  * misfit vs the oracle's: 2e-4 relative (FP32 traces, residuals cancel);
  * velocity gradient vs the exact FP64 oracle gradient: 1e-4 with FP32
    checkpoints and FP32 Laplacian store, 2e-4 with block-scaled int16
    checkpoints, 5e-3 with BF16 checkpoints on this small case (one shot
    group, few segments; the benchmark-size error is stated separately);
  * wavelet gradient vs the oracle: 1e-4 (FP32 storage);
  * adjoint dot-product test <S w, y> = <w, S^T y>: 1e-5 relative difference;
  * central finite differences of the FP64 misfit along 8 seeded directions:
    1e-3 relative difference of the directional derivative, plus 1e-4 |g||d|
    for directions nearly orthogonal to the gradient.
"""
import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import oracle_geometry, small_problem

pytestmark = pytest.mark.gpu


def _observed(orc, grid, v, wav, src, rec, seed=7):
    """Observed data: the oracle's traces in a perturbed model."""
    rng = np.random.default_rng(seed)
    vt = (v * (1 + 0.05 * rng.standard_normal(v.shape).clip(-2, 2))).astype(np.float32)
    return orc.forward(oracle_geometry(orc, grid, vt, wav, src, rec)).astype(np.float32)


@pytest.mark.parametrize("order", [2, 8])
@pytest.mark.parametrize("shape,nshot,nt,ckpt,spc,rows", [
    ((60, 150), 3, 100, 0, 0, 0),
    ((41, 133), 2, 77, 10, 1, 16),
    ((70, 260), 4, 64, 64, 2, 0),
])
def test_gradient_matches_oracle_fp32(cuda, orc, order, shape, nshot, nt, ckpt, spc, rows):
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=nshot, nt=nt, order=order,
                                           ckpt_every=ckpt, spc=spc, seed=3, tile_rows=rows)
    obs = _observed(orc, grid, v, wav, src, rec)
    J, g, gw = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                               torch.from_numpy(src), torch.from_numpy(rec),
                               torch.from_numpy(obs).to(cuda), grid, want_wavelet=True)
    Jr, gr, gwr, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    assert abs(J.item() - Jr) / Jr < 2e-4
    assert rel_l2(g.cpu().numpy(), gr) < 1e-4
    assert rel_l2(gw.cpu().numpy(), gwr) < 1e-4


@pytest.mark.parametrize("fmt,lap_store,tol", [
    ("fp32", "auto", 1e-4),
    ("fp32", "fp32", 1e-4),
    ("i16", "auto", 2e-4),
    ("bf16", "auto", 5e-3),
    ("fp32", "bf16", 5e-3),
])
def test_gradient_checkpoint_formats(cuda, orc, fmt, lap_store, tol):
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(80, 200), nshot=3, nt=150, ckpt_every=12,
                                           ckpt_format=fmt, lap_store=lap_store, seed=5)
    obs = _observed(orc, grid, v, wav, src, rec)
    J, g = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                           torch.from_numpy(src), torch.from_numpy(rec),
                           torch.from_numpy(obs).to(cuda), grid)
    _, gr, _, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    err = rel_l2(g.cpu().numpy(), gr)
    print(f"checkpoint {fmt} lap_store={lap_store}: gradient rel L2 {err:.3e}")
    assert err < tol, err


@pytest.mark.parametrize("order,shape,nt,ckpt,rows,group", [
    (8, (90, 260), 100, 13, 0, 0),
    (4, (48, 136), 60, 60, 0, 2),
    (8, (64, 200), 75, 0, 16, 0),
])
def test_u_store_matches_lap_store(cuda, orc, order, shape, nt, ckpt, rows, group):
    """The u-store adjoint (levels u_k kept, L u_k formed in the adjoint
    kernel) against the stored-FP32-L u adjoint: with the leapfrog forward of
    both, the same arithmetic per cell, so the gradients agree to FP32
    summation-order noise (1e-6). The summed-form forward (the default of the
    u-store path) changes only the forward's rounding: within 1e-4 of both."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=shape, nshot=5, nt=nt, order=order, ckpt_every=ckpt,
                                           seed=21, tile_rows=rows)
    grid = dataclasses.replace(grid, group_shots=group, update="leapfrog")
    obs = _observed(orc, grid, v, wav, src, rec)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec), torch.from_numpy(obs).to(cuda))
    out = {}
    for store in ("auto", "fp32"):
        out[store] = misfit_gradient(*args, dataclasses.replace(grid, lap_store=store), want_wavelet=True)
    Ja, ga, gwa = out["auto"]
    Jf, gf, gwf = out["fp32"]
    assert abs(Ja.item() - Jf.item()) <= 1e-6 * abs(Jf.item())
    assert rel_l2(ga.cpu().numpy(), gf.cpu().numpy()) < 1e-6
    assert rel_l2(gwa.cpu().numpy(), gwf.cpu().numpy()) < 1e-6
    Js, gs, gws = misfit_gradient(*args, dataclasses.replace(grid, update="auto"), want_wavelet=True)
    assert abs(Js.item() - Jf.item()) <= 1e-5 * abs(Jf.item())
    assert rel_l2(gs.cpu().numpy(), gf.cpu().numpy()) < 1e-4
    assert rel_l2(gws.cpu().numpy(), gwf.cpu().numpy()) < 1e-4


@pytest.mark.parametrize("update,tol", [("leapfrog", 1e-6), ("auto", 2e-6)])
@pytest.mark.parametrize("nt,ckpt,levels", [(100, 13, 30), (100, 13, 10 ** 6), (61, 20, 45), (100, 10, 60),
                                             (101, 9, 50)])
def test_kept_levels_match_recompute(cuda, orc, nt, ckpt, levels, update, tol):
    """store_levels: the forward keeps the levels of its last segments and the
    adjoint recomputes only the others. With (100, 10, 60) and (101, 9, 50)
    the kept levels leave room for two sets of recompute slots, so the
    recompute of each segment runs on a second stream beside the adjoint of
    the segment after it, alternating between the sets. With FP32 checkpoints and the leapfrog
    forward the recompute reproduces the kept levels exactly, so the gradients
    agree to summation order (1e-6). With the summed forward (the default) the
    recompute restarts the leapfrog recursion from u_{k0-1} = u_k0 - d_k0, one
    rounding away from the forward's levels (2e-6). With BF16 checkpoints the
    kept levels are the exact forward ones, and the gradient is no further
    from the FP64 oracle than before."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(72, 210), nshot=4, nt=nt, ckpt_every=ckpt, seed=8)
    grid = dataclasses.replace(grid, update=update)
    obs = _observed(orc, grid, v, wav, src, rec)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec), torch.from_numpy(obs).to(cuda))
    _, gr, gwr, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    res = {}
    for fmt in ("fp32", "bf16"):
        for lv in (0, levels):
            g = dataclasses.replace(grid, ckpt_format=fmt, store_levels=lv)
            res[fmt, lv] = misfit_gradient(*args, g, want_wavelet=True)
    for k in (1, 2):
        assert rel_l2(res["fp32", levels][k].cpu().numpy(), res["fp32", 0][k].cpu().numpy()) < tol
    e_rec = rel_l2(res["bf16", 0][1].cpu().numpy(), gr)
    e_kept = rel_l2(res["bf16", levels][1].cpu().numpy(), gr)
    print(f"bf16 checkpoints: gradient rel L2 {e_rec:.2e} recomputed, {e_kept:.2e} with kept levels")
    assert e_kept <= 1.05 * e_rec
    assert rel_l2(res["bf16", levels][2].cpu().numpy(), gwr) < 5e-3


def test_autograd_matches_fused_call(cuda, orc):
    from neuralmech_gb300 import misfit_gradient, wave_forward
    grid, v, wav, src, rec = small_problem(shape=(50, 140), nshot=2, nt=70, seed=11)
    obs = torch.from_numpy(_observed(orc, grid, v, wav, src, rec)).to(cuda)
    vel = torch.from_numpy(v).to(cuda).requires_grad_(True)
    traces = wave_forward(vel, torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                          torch.from_numpy(rec), grid)
    loss = 0.5 * ((traces - obs) ** 2).sum()
    loss.backward()
    J, g = misfit_gradient(vel.detach(), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
                           torch.from_numpy(rec), obs, grid)
    assert abs(loss.item() - J.item()) / J.item() < 1e-5
    assert rel_l2(vel.grad.cpu().numpy(), g.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("update,tol", [("leapfrog", 1e-5), ("auto", 5e-5)])
def test_adjoint_dot_product(cuda, update, tol):
    """<S w, y> = <w, S^T y> for the linear map S: wavelets -> traces. With the
    leapfrog forward, forward and adjoint are transposes in the same FP32
    arithmetic (1e-5); the summed forward (the default of a gradient) rounds
    differently from the leapfrog adjoint (5e-5 on white-noise wavelets)."""
    import dataclasses
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(64, 180), nshot=3, nsrc=2, nrec=23, nt=110, seed=2)
    grid = dataclasses.replace(grid, update=update)
    rng = np.random.default_rng(0)
    w = torch.from_numpy(rng.standard_normal(wav.shape).astype(np.float32)).to(cuda).requires_grad_(True)
    y = torch.from_numpy(rng.standard_normal((3, 110, 23)).astype(np.float32)).to(cuda)
    traces = wave_forward(torch.from_numpy(v).to(cuda), w, torch.from_numpy(src),
                          torch.from_numpy(rec), grid)
    traces.backward(y)
    lhs = float((traces.detach().double() * y.double()).sum())
    rhs = float((w.detach().double() * w.grad.double()).sum())
    assert abs(lhs - rhs) / max(abs(lhs), abs(rhs)) < tol


def test_gradient_finite_differences(cuda, orc):
    """Directional derivative <grad, d> vs central differences of the FP64
    oracle misfit along 8 seeded directions."""
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(48, 130), nshot=2, nt=90, seed=9)
    obs = _observed(orc, grid, v, wav, src, rec)
    J, g = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                           torch.from_numpy(src), torch.from_numpy(rec),
                           torch.from_numpy(obs).to(cuda), grid)
    g = g.cpu().numpy().astype(np.float64)
    rng = np.random.default_rng(1)
    geo = oracle_geometry(orc, grid, v, wav, src, rec)
    from scipy.ndimage import gaussian_filter
    for _ in range(8):
        d = gaussian_filter(rng.standard_normal(v.shape), 3.0)
        d *= 1e-3 * np.abs(v).mean() / np.abs(d).max()
        eps = 1.0
        Js = []
        for sgn in (1, -1):
            geo.vel = v.astype(np.float64) + sgn * eps * d
            Js.append(0.5 * ((orc.forward(geo) - obs) ** 2).sum())
        fd = (Js[0] - Js[1]) / (2 * eps)
        an = float((g * d).sum())
        # relative to |fd|, and to |g||d| for directions nearly orthogonal to g
        bound = 1e-3 * abs(fd) + 1e-4 * np.linalg.norm(g) * np.linalg.norm(d)
        assert abs(fd - an) < bound, (fd, an)


@pytest.mark.parametrize("order,fmt,form,tol", [(8, "fp32", "auto", 2e-4), (4, "fp32", "auto", 2e-4),
                                                (8, "fp32", "leapfrog", 2e-4), (8, "bf16", "auto", 2e-3),
                                                (8, "bf16", "leapfrog", 5e-3)])
def test_gradient_3d_matches_oracle(cuda, orc, order, fmt, form, tol):
    """The 3D gradient against the FP64 oracle. A gradient's forward takes the
    summed (increment) form by default ("auto"); "leapfrog" forces the
    two-level update. With BF16 checkpoints the summed form's (d, u) pair
    keeps the increment to BF16's relative precision, so its bound is tighter."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(68, 22, 70), nshot=2, nt=48, order=order, sponge=5,
                                           ckpt_every=10, ckpt_format=fmt, nrec=30, seed=4)
    grid = dataclasses.replace(grid, update=form)
    obs = _observed(orc, grid, v, wav, src, rec)
    J, g, gw = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                               torch.from_numpy(src), torch.from_numpy(rec),
                               torch.from_numpy(obs).to(cuda), grid, want_wavelet=True)
    Jr, gr, gwr, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    assert abs(J.item() - Jr) / Jr < 2e-4
    err = rel_l2(g.cpu().numpy(), gr)
    print(f"3D order {order} checkpoint {fmt} {form}: gradient rel L2 {err:.3e}")
    assert err < tol
    if fmt == "fp32":
        assert rel_l2(gw.cpu().numpy(), gwr) < 1e-4


def test_3d_unequal_spacings_match_oracle(cuda, orc):
    """Unequal dz, dy, dx: the 3D kernel with separate weights per axis (equal
    spacings take the one-weight-per-k path the other 3D tests cover)."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient, wave_forward
    grid, v, wav, src, rec = small_problem(shape=(60, 24, 70), nshot=2, nt=40, order=8, sponge=5,
                                           ckpt_every=10, nrec=30, seed=9)
    grid = dataclasses.replace(grid, spacing=(12.0, 11.0, 10.0))
    geo = oracle_geometry(orc, grid, v, wav, src, rec)
    traces = wave_forward(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                          torch.from_numpy(src), torch.from_numpy(rec), grid)
    ref = orc.forward(geo)
    assert rel_l2(traces.cpu().numpy(), ref) < 1e-5
    obs = _observed(orc, grid, v, wav, src, rec)
    J, g = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                           torch.from_numpy(src), torch.from_numpy(rec), torch.from_numpy(obs).to(cuda), grid)
    Jr, gr, _, _ = orc.gradient(geo, obs)
    assert abs(J.item() - Jr) / Jr < 2e-4
    assert rel_l2(g.cpu().numpy(), gr) < 2e-4


def test_misfit_gradient_overlap_matches(cuda, orc):
    """observed_ready: the observed traces copied on a second stream while the
    forward runs give the same misfit and gradient as resident data."""
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(60, 150), nshot=3, nt=80, ckpt_every=9, seed=21)
    obs = _observed(orc, grid, v, wav, src, rec)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    J1, g1 = misfit_gradient(*args, torch.from_numpy(obs).to(cuda), grid)
    host = torch.from_numpy(obs).pin_memory()
    side = torch.cuda.Stream()
    ob = torch.empty(host.shape, dtype=torch.float32, device=cuda)
    ready = torch.cuda.Event()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        ob.copy_(host, non_blocking=True)
        ready.record(side)
    J2, g2 = misfit_gradient(*args, ob, grid, observed_ready=ready)
    assert abs(J2.item() - J1.item()) <= 1e-12 * J1.item()  # (FP64 atomic sums: order may differ)
    assert rel_l2(g2.cpu().numpy(), g1.cpu().numpy()) < 1e-6
    # shot groups: the wait comes before the first group's residual
    import dataclasses
    grouped = dataclasses.replace(grid, group_shots=2)
    J3, g3 = misfit_gradient(*args, ob, grouped, observed_ready=ready)
    assert abs(J3.item() - J1.item()) <= 1e-12 * J1.item()
    assert rel_l2(g3.cpu().numpy(), g1.cpu().numpy()) < 1e-6


def test_shot_groups_match_one_batch(cuda, orc):
    """group_shots runs the shots in sequential groups on one workspace; the
    misfit, gradient, traces and wavelet gradient equal the one-batch call."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient, wave_forward
    grid, v, wav, src, rec = small_problem(shape=(50, 150), nshot=5, nt=70, ckpt_every=9, seed=13)
    obs = torch.from_numpy(_observed(orc, grid, v, wav, src, rec)).to(cuda)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    J1, g1, w1, t1 = misfit_gradient(*args, obs, grid, want_wavelet=True, want_traces=True)
    grouped = dataclasses.replace(grid, group_shots=2)
    J2, g2, w2, t2 = misfit_gradient(*args, obs, grouped, want_wavelet=True, want_traces=True)
    assert abs(J1.item() - J2.item()) <= 1e-12 * J1.item()
    assert rel_l2(g2.cpu().numpy(), g1.cpu().numpy()) < 1e-6
    assert rel_l2(w2.cpu().numpy(), w1.cpu().numpy()) < 1e-6
    assert torch.equal(t1, t2)
    f1 = wave_forward(*args, grid)
    f2 = wave_forward(*args, grouped)
    assert torch.equal(f1, f2)


@pytest.mark.parametrize("order,nt,ckpt,fmt", [(8, 101, 15, "fp32"), (4, 80, 0, "fp32"),
                                               (2, 64, 64, "fp32"), (8, 90, 9, "i16")])
def test_gradient_two_step_blocking(cuda, orc, order, nt, ckpt, fmt):
    """Checkpointed gradient with two steps per launch (odd and even segment
    lengths, odd step counts) against the exact FP64 oracle gradient."""
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(70, 250), nshot=3, nt=nt, order=order, ckpt_every=ckpt,
                                           ckpt_format=fmt, step_block=2, seed=17, nrec=24)
    src[0, 0] = [32, 120]  # on a tile seam
    rec[1, 3] = [31, 119]
    obs = _observed(orc, grid, v, wav, src, rec)
    J, g, gw = misfit_gradient(torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda),
                               torch.from_numpy(src), torch.from_numpy(rec),
                               torch.from_numpy(obs).to(cuda), grid, want_wavelet=True)
    Jr, gr, gwr, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    assert abs(J.item() - Jr) / Jr < 2e-4
    assert rel_l2(g.cpu().numpy(), gr) < 2e-4
    assert rel_l2(gw.cpu().numpy(), gwr) < 2e-4


def test_two_step_matches_one_step_autograd(cuda, orc):
    import dataclasses
    from neuralmech_gb300 import wave_forward
    grid, v, wav, src, rec = small_problem(shape=(64, 200), nshot=2, nt=71, ckpt_every=10, seed=23)
    obs = torch.from_numpy(_observed(orc, grid, v, wav, src, rec)).to(cuda)
    grads = []
    for sb in (1, 2):  # (the two-step kernel has the leapfrog form only)
        g = dataclasses.replace(grid, step_block=sb, update="leapfrog")
        vel = torch.from_numpy(v).to(cuda).requires_grad_(True)
        t = wave_forward(vel, torch.from_numpy(wav).to(cuda), torch.from_numpy(src), torch.from_numpy(rec), g)
        (0.5 * ((t - obs) ** 2).sum()).backward()
        grads.append(vel.grad.cpu().numpy())
    assert rel_l2(grads[1], grads[0]) < 1e-5


@pytest.mark.parametrize("nt,ckpt,levels", [(101, 15, 40), (90, 9, 200), (64, 64, 0), (77, 10, 10 ** 6)])
def test_block_float_levels(cuda, orc, nt, ckpt, levels):
    """Kept levels in block floating point (level_format "bfp16": int16
    mantissas, one exponent byte per 4 cells) against FP32 kept levels, with
    some segments kept and the rest recomputed, only the last kept (levels 0,
    here the only one, from u_0), and every one kept (10^6); odd step counts and
    checkpoint intervals; a source on a tile seam (its block encoded again after
    the injection). Only the adjoint's u_k differ, by the 2^-15 block rounding:
    the misfits agree to 1e-12 and the wavelet gradients (which do not see u_k)
    to 1e-6; the velocity gradients within 3e-4 of each other and of the FP64
    oracle."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient
    grid, v, wav, src, rec = small_problem(shape=(70, 250), nshot=3, nt=nt, ckpt_every=ckpt, seed=31, nrec=24,
                                           ckpt_format="fp32")
    src[0, 0] = [32, 120]  # on a tile seam of the two-step kernel
    src[1, 0] = [33, 119]
    grid = dataclasses.replace(grid, step_block=2, store_levels=levels)
    obs = _observed(orc, grid, v, wav, src, rec)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec), torch.from_numpy(obs).to(cuda))
    J32, g32, w32 = misfit_gradient(*args, grid, want_wavelet=True)
    J16, g16, w16 = misfit_gradient(*args, dataclasses.replace(grid, level_format="bfp16"), want_wavelet=True)
    assert abs(J16.item() - J32.item()) <= 1e-12 * J32.item()
    assert rel_l2(w16.cpu().numpy(), w32.cpu().numpy()) < 1e-6
    e16 = rel_l2(g16.cpu().numpy(), g32.cpu().numpy())
    Jr, gr, _, _ = orc.gradient(oracle_geometry(orc, grid, v, wav, src, rec), obs)
    e_or = rel_l2(g16.cpu().numpy(), gr)
    print(f"bfp16 levels: vs FP32 levels {e16:.2e}, vs FP64 oracle {e_or:.2e} "
          f"(FP32 levels {rel_l2(g32.cpu().numpy(), gr):.2e})")
    assert 0 < e16 < 3e-4
    assert e_or < 3e-4


@pytest.mark.parametrize("nt,ckpt,levels", [(101, 15, 0), (90, 9, 40), (64, 64, 0)])
def test_summed_two_step_matches_one_step(cuda, orc, nt, ckpt, levels):
    """The summed forward with two steps per launch (d_{n+1} kept on chip,
    the intermediate level written only for a checkpoint or a kept level)
    against the summed one-step forward: odd step counts (a last single
    step), odd checkpoint intervals (checkpoints at odd steps), kept levels.
    The two kernels form L u differently (centre weight against neighbour
    differences), so they agree to FP32 rounding, not bit for bit: misfits
    within 1e-5, velocity and wavelet gradients within 5e-5 of each other;
    each one's traces within 1e-5 and gradient within 1e-4 of the FP64
    oracle."""
    import dataclasses
    from neuralmech_gb300 import misfit_gradient, wave_forward
    grid, v, wav, src, rec = small_problem(shape=(70, 250), nshot=3, nt=nt, ckpt_every=ckpt, seed=29, nrec=24,
                                           ckpt_format="fp32")
    src[0, 0] = [32, 120]  # on a tile seam of the two-step kernel
    grid = dataclasses.replace(grid, update="summed", store_levels=levels)
    obs = _observed(orc, grid, v, wav, src, rec)
    args = (torch.from_numpy(v).to(cuda), torch.from_numpy(wav).to(cuda), torch.from_numpy(src),
            torch.from_numpy(rec))
    out = {sb: misfit_gradient(*args, torch.from_numpy(obs).to(cuda), dataclasses.replace(grid, step_block=sb),
                               want_wavelet=True) for sb in (1, 2)}
    J1, g1, w1 = out[1]
    J2, g2, w2 = out[2]
    assert abs(J1.item() - J2.item()) <= 1e-5 * J1.item()
    assert rel_l2(g2.cpu().numpy(), g1.cpu().numpy()) < 5e-5
    assert rel_l2(w2.cpu().numpy(), w1.cpu().numpy()) < 5e-5
    geo = oracle_geometry(orc, grid, v, wav, src, rec)
    Jr, gr, _, tr = orc.gradient(geo, obs)
    assert rel_l2(g1.cpu().numpy(), gr) < 1e-4
    assert rel_l2(g2.cpu().numpy(), gr) < 1e-4
    for sb in (1, 2):
        t = wave_forward(*args, dataclasses.replace(grid, step_block=sb))
        assert rel_l2(t.cpu().numpy(), tr) < 1e-5
