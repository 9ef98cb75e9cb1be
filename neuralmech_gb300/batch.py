"""Uneven multi-model batches in one CUDA graph.

A batch holds several velocity models of different grid sizes and step
counts, each with its own shots, wavelets, receivers and observed traces.
This is the fwi workload family of many surveys at once (e.g. 8 models
512^2..1536^2, 1000..3000 steps, 128 shots in total).

``BatchFWI`` works in four steps:
  * it chooses each model's kernel configuration with the autotuner (for
    the forward of a gradient: the summed update form where the grid asks
    for it);
  * it allocates every workspace and output once;
  * the library plans the batch (``wfd_batch_plan``): it runs each model's
    checkpointed forward + adjoint (``wfd_misfit_gradient``) once on a stream
    of its own and records the same calls as one CUDA graph with the models
    on parallel branches, so the GPU overlaps the models' step kernels;
  * ``run()`` replays that graph (``wfd_batch_run``): one host call per batch
    gradient.

Inputs live in tensors owned by the batch. ``set_velocity`` / ``set_observed``
update them in place, so the next replay sees the new values.
"""
from __future__ import annotations

import ctypes
import dataclasses

import torch

from . import _lib
from . import autotune as _autotune
from .wavefd import Grid, _misfit_gradient_into, _prepare, _ptr, _stream, _workspace, levels_for_budget


def _level_shares(models, budget: float) -> list:
    """Bytes of kept forward levels per model (see BatchFWI)."""
    if budget <= 0:
        return [0.0] * len(models)
    want = []
    for m in models:
        g = m["grid"]
        nx = g.shape[-1]
        cells = 1
        for n in g.shape[:-1]:
            cells *= n
        cells *= (nx + 7) // 8 * 8
        want.append(4.0 * cells * m["observed"].shape[0] * (g.nt + 1))
    total = sum(want)
    return [min(w, budget * w / total) for w in want]


@dataclasses.dataclass
class _Model:
    call: object
    observed: torch.Tensor
    ws: torch.Tensor
    grad: torch.Tensor
    misfit: torch.Tensor
    stream: torch.cuda.Stream


class BatchFWI:
    """Misfit gradients of many models (uneven sizes) from one graph replay.

    models: sequence of dicts with keys vel (nz, nx) CUDA tensor, wavelet,
    src, rec (as for ``wave_forward``), observed (nshot, nt, nrec) CUDA tensor
    and grid (``Grid``). ``autotune`` picks tile_rows / shots_per_cta per
    model; ``graph=False`` runs the same calls eagerly on the streams.
    ``level_budget`` (bytes) is shared among the models' adjoints for the
    forward levels they keep instead of recomputing (``Grid.store_levels``),
    in proportion to the levels each would keep with unlimited memory (a
    kept level saves one recomputed step of its model, whatever its size, so
    any split that no model can use up saves the same work); 0 keeps each
    model's own ``store_levels``.
    """

    def __init__(self, models, *, autotune: bool = True, graph: bool = True, tune_kw=None,
                 level_budget: float = 0.0):
        if not models:
            raise ValueError("empty batch")
        self.device = models[0]["vel"].device
        self.models = []
        shares = _level_shares(models, level_budget)
        for m, share in zip(models, shares):
            grid: Grid = m["grid"]
            obs = m["observed"].to(torch.float32).contiguous()
            nshot = obs.shape[0]
            if autotune:
                grid = _autotune.tuned(grid, nshot, vel=m["vel"], for_gradient=True, **(tune_kw or {}))
            if share > 0:
                grid = dataclasses.replace(grid, store_levels=levels_for_budget(grid, nshot, share))
            call = _prepare(m["vel"], torch.as_tensor(m["wavelet"], device=self.device), m["src"], m["rec"],
                            grid, nshot)
            call.vel = call.vel.clone()  # the batch owns its inputs (set_velocity updates them)
            self.models.append(_Model(call, obs, _workspace(call, True), torch.empty_like(call.vel),
                                      torch.zeros((), dtype=torch.float64, device=self.device),
                                      torch.cuda.Stream(device=self.device)))
        self.configs = [(x.call.grid.tile_rows, x.call.grid.shots_per_cta, x.call.grid.step_block)
                        for x in self.models]
        self.graph = None  # the library's batch plan (its graph), when graph=True
        self.graph_kernels = 0  # kernels of one replay
        if not graph:
            self._launch()  # eager run: validates arguments
            torch.cuda.synchronize(self.device)
            return
        self._items = (_lib.BatchItem * len(self.models))()
        for it, m in zip(self._items, self.models):
            gz, gy, gx = m.call.sponges
            it.problem = ctypes.pointer(m.call.problem)
            for name, t in (("vel", m.call.vel), ("sponge_z", gz), ("sponge_y", gy), ("sponge_x", gx),
                            ("wavelet", m.call.wavelet), ("src", m.call.src), ("rec", m.call.rec),
                            ("observed", m.observed), ("grad_vel", m.grad), ("misfit", m.misfit),
                            ("workspace", m.ws)):
                setattr(it, name, _ptr(t))
            it.workspace_bytes = m.ws.numel()
        lib = _lib.load()
        plan = ctypes.c_void_p()
        _lib.check(lib.wfd_batch_plan(self._items, len(self.models), _stream(), ctypes.byref(plan)),
                   "wfd_batch_plan")
        self.graph = plan
        self.graph_kernels = int(lib.wfd_batch_launches(plan))
        torch.cuda.synchronize(self.device)

    def __del__(self):
        if getattr(self, "graph", None) is not None and _lib is not None:
            _lib.load().wfd_batch_free(self.graph)
            self.graph = None

    def _launch(self):
        main = torch.cuda.current_stream(self.device)
        for m in self.models:
            m.stream.wait_stream(main)
            with torch.cuda.stream(m.stream):
                _misfit_gradient_into(m.call, m.observed, m.ws, m.grad, m.misfit)
        for m in self.models:
            main.wait_stream(m.stream)

    def set_velocity(self, i: int, vel: torch.Tensor):
        self.models[i].call.vel.copy_(vel)

    def set_observed(self, i: int, observed: torch.Tensor):
        self.models[i].observed.copy_(observed)

    def run(self):
        """(misfits float64 [n_models], [grad_vel per model]) of the current inputs."""
        if self.graph is not None:
            _lib.check(_lib.load().wfd_batch_run(self.graph, _stream()), "wfd_batch_run")
        else:
            self._launch()
        return torch.stack([m.misfit for m in self.models]), [m.grad for m in self.models]

    @property
    def cell_updates(self) -> float:
        """Counted cell-updates (forward + adjoint) of one batch gradient."""
        tot = 0.0
        for m in self.models:
            g = m.call.grid
            R = g.order // 2
            inner = 1
            for n in g.shape:
                inner *= n - 2 * R
            tot += 2.0 * m.call.problem.nshot * inner * g.nt
        return tot
