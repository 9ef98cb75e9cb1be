"""Uneven multi-model batch in one CUDA graph, and the autotuner on the GPU.
Tolerances: batch vs per-model calls with the batch's own per-model
configuration 1e-6 relative L2 (the same kernels; only the atomic order of the
gradient sums differs); misfits 1e-9 relative."""
import dataclasses

import numpy as np
import pytest
import torch

from conftest import rel_l2
from helpers import oracle_geometry, small_problem

pytestmark = pytest.mark.gpu


def _models(orc, cuda):
    specs = [dict(shape=(64, 200), nshot=3, nt=90, seed=1, ckpt_every=10),
             dict(shape=(48, 140), nshot=2, nt=60, seed=2, ckpt_every=8, order=4),
             dict(shape=(90, 260), nshot=4, nt=110, seed=3, ckpt_every=11)]
    out = []
    for sp in specs:
        grid, v, wav, src, rec = small_problem(**sp)
        rng = np.random.default_rng(sp["seed"])
        vt = (v * (1 + 0.04 * rng.standard_normal(v.shape).clip(-2, 2))).astype(np.float32)
        obs = orc.forward(oracle_geometry(orc, grid, vt, wav, src, rec)).astype(np.float32)
        out.append(dict(vel=torch.from_numpy(v).to(cuda), wavelet=torch.from_numpy(wav).to(cuda),
                        src=torch.from_numpy(src), rec=torch.from_numpy(rec),
                        observed=torch.from_numpy(obs).to(cuda), grid=grid))
    return out


def test_batch_graph_matches_single_calls(cuda, orc, tmp_path, monkeypatch):
    from neuralmech_gb300 import misfit_gradient
    from neuralmech_gb300.batch import BatchFWI
    monkeypatch.setenv("WAVEFD_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    models = _models(orc, cuda)
    batch = BatchFWI(models, autotune=True)
    tuned = [x.call.grid for x in batch.models]  # the configuration the tuner picked per model
    for _ in range(2):  # two replays give the same answer
        J, grads = batch.run()
        torch.cuda.synchronize()
        for i, m in enumerate(models):
            Jr, gr = misfit_gradient(m["vel"], m["wavelet"], m["src"], m["rec"], m["observed"], tuned[i])
            assert abs(J[i].item() - Jr.item()) <= 1e-9 * Jr.item()
            assert rel_l2(grads[i].cpu().numpy(), gr.cpu().numpy()) < 1e-6
    # updated inputs are seen by the next replay
    v2 = models[1]["vel"] * 1.01
    batch.set_velocity(1, v2)
    J, grads = batch.run()
    Jr, gr = misfit_gradient(v2, models[1]["wavelet"], models[1]["src"], models[1]["rec"],
                             models[1]["observed"], tuned[1])
    assert abs(J[1].item() - Jr.item()) <= 1e-9 * Jr.item()
    assert rel_l2(grads[1].cpu().numpy(), gr.cpu().numpy()) < 1e-6
    assert batch.cell_updates > 0


def test_batch_level_budget_keeps_levels(cuda, orc, tmp_path, monkeypatch):
    """A shared budget of kept forward levels: every model keeps some levels
    (fewer recomputed segments) and the gradients equal the per-model calls
    that recompute (FP32 checkpoints: the recomputed levels are the kept ones)."""
    from neuralmech_gb300 import misfit_gradient
    from neuralmech_gb300.batch import BatchFWI
    monkeypatch.setenv("WAVEFD_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    models = _models(orc, cuda)
    level_bytes = [4 * m["grid"].shape[0] * ((m["grid"].shape[1] + 7) // 8 * 8) * m["observed"].shape[0]
                   for m in models]
    budget = 0.5 * sum(b * (m["grid"].nt + 1) for b, m in zip(level_bytes, models))
    batch = BatchFWI(models, autotune=False, level_budget=budget)
    for x, m in zip(batch.models, models):
        K = m["grid"].ckpt_every
        assert x.call.grid.store_levels >= 2 * K + 2  # at least one segment beyond the last
    J, grads = batch.run()
    torch.cuda.synchronize()
    for i, m in enumerate(models):
        Jr, gr = misfit_gradient(m["vel"], m["wavelet"], m["src"], m["rec"], m["observed"], m["grid"])
        assert abs(J[i].item() - Jr.item()) <= 1e-9 * Jr.item()
        assert rel_l2(grads[i].cpu().numpy(), gr.cpu().numpy()) < 1e-6


def test_autotune_on_gpu_picks_a_valid_config(cuda, tmp_path, monkeypatch):
    from neuralmech_gb300 import Grid, autotune
    g = Grid((128, 256), (10.0, 10.0), 1e-3, 8)
    best = autotune.tune(g, 8, steps=4, path=str(tmp_path / "t.json"))
    assert (best["step_block"] == 2 or
            (best["tile_rows"] in (16, 32) and 1 <= best["shots_per_cta"] <= 8))

    def no_timing(*a, **k):
        raise AssertionError("the cached choice should be used")

    monkeypatch.setattr(autotune, "_gpu_timer", no_timing)
    assert autotune.tune(g, 8, steps=4, path=str(tmp_path / "t.json")) == best
