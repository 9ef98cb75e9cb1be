"""CPU tests of the Python host layer: argument shaping, sponge profiles, the
synthetic workload generators, the refusal of CPU tensors (there is no CPU
path), the variable-density CFL speed bound, and the JSON line of the
benchmark's CPU reference arm."""
import math

import numpy as np
import pytest
import torch


def test_positions_and_wavelet_broadcast():
    from neuralmech_gb300.wavefd import _positions, _wavelet
    p = _positions(np.array([[3, 7], [4, 9]]), 3, 2, "cpu")
    assert p.shape == (3, 2, 3) and p.dtype == torch.int32
    assert p[2, 1].tolist() == [4, 0, 9]
    p3 = _positions(np.zeros((2, 5, 3)), 2, 3, "cpu")
    assert p3.shape == (2, 5, 3)
    with pytest.raises(ValueError):
        _positions(np.zeros((2, 5, 2)), 3, 2, "cpu")
    w = _wavelet(np.arange(10.0), 4, 10, 2, "cpu")
    assert w.shape == (4, 10, 2) and float(w[3, 7, 1]) == 7.0
    w2 = _wavelet(np.ones((4, 10)), 4, 10, 3, "cpu")
    assert w2.shape == (4, 10, 3)
    with pytest.raises(ValueError):
        _wavelet(np.ones(9), 4, 10, 2, "cpu")


def test_sponge_profile():
    from neuralmech_gb300 import sponge_profile
    g = sponge_profile(100, 20, 10, 0.3)
    assert g.dtype == np.float32
    assert np.all(g[20:90] == 1.0)
    assert np.isclose(g[0], np.exp(-0.09)) and np.isclose(g[99], np.exp(-0.09))
    assert np.all(np.diff(g[:21]) > 0) and np.all(np.diff(g[89:]) < 0)
    assert np.all(sponge_profile(50, 0, 0) == 1.0)


def test_grid_sponge_widths():
    from neuralmech_gb300 import Grid, sponge_profiles
    g = Grid((40, 60), (10.0, 10.0), 1e-3, 10, sponge=[(0, 8), (5, 5)])
    gz, gy, gx = sponge_profiles(g)
    assert gy is None and gz[0] == 1.0 and gz[-1] < 1.0 and gx[0] < 1.0
    g0 = Grid((40, 60), (10.0, 10.0), 1e-3, 10, sponge=0)
    assert all(p is None for p in sponge_profiles(g0))
    with pytest.raises(ValueError):
        Grid((40, 60), (10.0, 10.0), 1e-3, 10, sponge=[(1, 1)]).sponge_widths()


def test_cpu_tensors_refused():
    from neuralmech_gb300 import Grid, wave_forward
    g = Grid((40, 60), (10.0, 10.0), 1e-3, 10)
    with pytest.raises(ValueError, match="CUDA"):
        wave_forward(torch.ones(40, 60), torch.zeros(10), [[10, 10]], [[10, 20]], g)


def test_synthetic_workloads():
    from neuralmech_gb300 import stable_dt
    from neuralmech_gb300.synth import workload
    w = workload("fwd256")
    assert w.vel.shape == (256, 256) and w.src.shape == (1, 1, 2) and w.rec.shape == (1, 256, 2)
    assert w.src[0, 0].tolist() == [5, 128]
    assert set(np.unique(np.round(w.vel[[0, 100, 200], 5], -2))) <= {1400.0, 1500, 1600, 2300, 2400,
                                                                     2500, 2600, 2700, 3200, 3300,
                                                                     3400, 3500, 3600, 3700, 3800}
    assert np.isclose(w.grid.dt * w.vel.max() / 10.0, 0.5)
    assert w.grid.dt < stable_dt((10.0, 10.0), float(w.vel.max()), 8)
    w2 = workload("fwd256")
    assert np.array_equal(w.vel, w2.vel)  # seeded
    f = workload("fwi1024", scale=0.125)
    assert f.vel.shape == (128, 128) and f.vel_true is not None and f.src.shape[0] == 64
    assert not np.array_equal(f.vel, f.vel_true)
    d3 = workload("fwi384_3d", scale=0.1)
    assert d3.vel.ndim == 3 and d3.src.shape[-1] == 3
    assert np.isclose(d3.grid.dt * float(max(d3.vel.max(), d3.vel_true.max())) / 10.0, 0.45)
    b = workload("batch8")
    assert len(b) == 8 and sum(x.nshot for x in b) == 128
    assert all(512 <= x.vel.shape[0] <= 1536 and x.vel.shape[0] % 64 == 0 for x in b)
    assert all(1000 <= x.grid.nt <= 3000 for x in b)


def test_autotune_selection_and_cache(tmp_path):
    from neuralmech_gb300 import Grid, autotune
    g = Grid((256, 512), (10.0, 10.0), 1e-3, 10)
    calls = []

    def fake(cfg):
        calls.append(cfg)
        if cfg["step_block"] == 2:
            return 9.0
        return abs(cfg["shots_per_cta"] - 4) + (0.5 if cfg["tile_rows"] == 32 else 0.0) + 1.0

    path = str(tmp_path / "cache.json")
    best = autotune.tune(g, 12, timer=fake, path=path)
    assert best == {"tile_rows": 16, "shots_per_cta": 4, "step_block": 1}
    n = len(calls)
    assert n == len(autotune.candidates(12))
    assert autotune.tune(g, 12, timer=fake, path=path) == best and len(calls) == n
    assert autotune.tune(g, 12, timer=fake, path=path, refresh=True) == best and len(calls) == 2 * n
    g3 = Grid((32, 32, 32), (10.0,) * 3, 1e-3, 10)
    assert autotune.tune(g3, 4, timer=fake, path=path) == {"tile_rows": 0, "shots_per_cta": 0, "step_block": 0}
    # a faster two-step candidate wins
    best2 = autotune.tune(Grid((64, 512), (10.0, 10.0), 1e-3, 10), 2, path=path,
                          timer=lambda c: 0.5 if c["step_block"] == 2 else 1.0)
    assert best2["step_block"] == 2


@pytest.mark.parametrize("order", [2, 4, 8])
def test_vd_speed_bound_covers_jumps(orc, order):
    """vd_vmax bounds the spectral radius of kappa Lb, in the form of the
    library's CFL check (radius <= vmax^2 S (1/dz^2 + 1/dx^2), S = 4
    (sum|c_k|)^2, here on a unit grid), where 1/rho jumps by three orders of
    magnitude (solid beside air, the two-phase medium's materials; the jump
    along x and along z) and in a random medium, and within a factor 6 of it.
    max sqrt(kappa / rho) is not a bound at the jump; in a smooth medium the
    two agree."""
    from helpers import vd_operator
    from neuralmech_gb300.wavefd import _stag_weights, vd_vmax
    c = orc.stag_coeffs(order)
    assert np.allclose(_stag_weights(order // 2), c, rtol=1e-15, atol=0)
    S = 4.0 * float(np.abs(c).sum()) ** 2
    n = 14 if order < 8 else 20
    kappa = np.full((n, n), 6.87e8)
    rho = np.full((n, n), 2643.0)
    kappa[:, n // 2:] = 1.419e5
    rho[:, n // 2:] = 1.204
    rng = np.random.default_rng(order)
    cases = [(kappa, rho), (kappa.T.copy(), rho.T.copy()),
             (rng.uniform(1.0, 1e3, (n, n)), rng.uniform(0.01, 10.0, (n, n)))]
    for i, (k, r) in enumerate(cases):
        radius = float(np.max(np.abs(np.linalg.eigvals(vd_operator(k, r, c)))))
        bound = vd_vmax(torch.from_numpy(k), torch.from_numpy(r), order) ** 2 * S * 2.0
        assert radius <= bound * (1 + 1e-12) and radius > bound / 6, (i, radius / bound)
        if i < 2:
            assert radius > float((k / r).max()) * S * 2.0
    smooth = vd_vmax(torch.full((n, n), 4.0, dtype=torch.float64), torch.full((n, n), 2.0, dtype=torch.float64), order)
    assert abs(smooth - math.sqrt(2.0)) < 1e-12


def test_bench_reference_arm_contract():
    """`bench.py --impl reference` (the CPU arm, no GPU needed) prints one JSON
    line with the contract's keys: the same metric, unit and config as the GPU
    arm, a cpu_baseline describing the run, and an e2e block with no copies."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r["impl"] == "reference" and r["n_gpus"] == 1 and r["steps"] == 1 and r["warmup"] == 0
    assert r["value"] > 0 and r["ms_per_step"] > 0 and r["higher_is_better"] is True
    metric = unit = None
    for ln in open(os.path.join(root, "bench.py")):  # the GPU arm's constants
        if ln.startswith("METRIC = "):
            metric = json.loads(ln.split("=", 1)[1])
        elif ln.startswith("UNIT = "):
            unit = json.loads(ln.split("=", 1)[1])
    assert r["metric"] == metric and r["unit"] == unit
    assert r["scaling"] == "weak" and r["vs_baseline"] is None
    assert r["data"].startswith("synthetic") and r["config"]["workload"].startswith("fwi1024")
    cb = r["cpu_baseline"]
    assert cb["value"] == r["value"] and cb["unit"] == r["unit"] and cb["cores"] >= 1
    assert cb["kind"] in ("reference", "port") and cb["sample"]
    e2e = r["e2e"]
    assert e2e["value"] == r["value"] and e2e["unit"] == r["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def _bfp16_decode(q16, t):
    """The kept-level format of WFD_LEVEL_BFP16 as include/wavefd.h states it:
    per 4 cells along x one exponent byte t and four stored 16-bit values
    u = q + 32768, v = q 2^(t - 141) (t = 0: the block is 0)."""
    q = q16.astype(np.int64) - 32768
    return np.where(t[..., None] > 0, np.ldexp(q.astype(np.float64), t[..., None].astype(np.int64) - 141), 0.0)


def _bfp16_encode(v):
    """An encoder of that format, from the statement alone: t the FP32 exponent
    field of the block's largest magnitude M (0 when it is below 15),
    q = rint(v 2^(141 - t)) (ties to even) clamped to +-32767."""
    v = v.astype(np.float32).reshape(-1, 4)
    M = np.abs(v).max(axis=1)
    t = ((M.view(np.uint32) >> 23) & 0xFF).astype(np.int64)
    t = np.where(t >= 15, t, 0)
    q = np.rint(np.ldexp(v.astype(np.float64), (141 - t)[:, None])).clip(-32767, 32767)
    q = np.where(t[:, None] > 0, q, 0)
    return (q + 32768).astype(np.uint16), t.astype(np.uint8)


def test_block_float_level_format():
    """The documented kept-level format: 2.25 bytes per cell, decoding exact in
    FP32 (every decoded value is an FP32 number), each value within one step
    2^(t - 141) of the original (half a step unless clamped at the block's
    top), and blocks below 2^-112 stored as 0."""
    rng = np.random.default_rng(5)
    v = (rng.standard_normal((4096, 4)) * np.exp(rng.uniform(-40, 40, (4096, 1)))).astype(np.float32)
    v[::9] *= np.float32(1e-35)  # blocks below the format's range
    q16, t = _bfp16_encode(v)
    assert q16.dtype.itemsize * 4 + t.dtype.itemsize == 9  # 2.25 bytes per cell
    d = _bfp16_decode(q16.reshape(-1, 4), t)
    assert np.array_equal(d, d.astype(np.float32).astype(np.float64))
    live = t > 0
    step = np.ldexp(1.0, t[live].astype(np.int64) - 141)[:, None]
    err = np.abs(d[live] - v[live].astype(np.float64))
    assert np.all(err <= step)
    top = np.abs(v[live]).astype(np.float64) >= 32767.5 * step  # the clamped values
    assert np.all((err <= 0.5 * step) | top)
    M = np.abs(v).max(axis=1)
    assert np.all((M[~live] < 2.0 ** -112)) and np.all(d[~live] == 0)
    # relative to the block's largest value M: within 2^-15 M (M >= 2^(t - 127))
    assert np.all(err <= 2.0 ** -15 * np.abs(v[live]).astype(np.float64).max(axis=1, keepdims=True))
