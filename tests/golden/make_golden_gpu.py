"""Generates the golden vectors of the reference kernels whose block barriers
and warp shuffles do not run in the CPU build, from the reference's own source
compiled for the GPU (oracle/Makefile.ref: step2D_wave_ieee.cubin, IEEE
division, no fused multiply-adds; loaded by oracle/ref_gpu.cpp). Runs on a
machine with a GPU and the module files (built where the reference sources
are), never at test time:

    python tests/golden/make_golden_gpu.py [out_dir]

Outputs (default: this folder):
  scaled_step.npz    scaled_step (step2D_wave.cu:128-183, int16 + FP32 scale
                     per 32 values, warp-shuffle block maxima) on the inputs
                     and in the layout of make_golden.py: the levels after
                     the first, second and last step, in-place rotation as in
                     2D_wave_cuda_scaled.py
  ref_gpu_digests.json  SHA-256 digests of what temporal_step
                     (step2D_wave.cu:244-304, block barriers) itself returns
                     after one and two launches from the two levels of each
                     case of temporal_step.npz (the levels make_golden.py made
                     by 8 and 16 padded_step updates): the CPU tests check the
                     committed levels against them without a second copy
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import torch  # noqa: E402

from make_golden import CASES, initial  # noqa: E402
from oracle import numpy_ref as nr  # noqa: E402
from oracle import ref  # noqa: E402


def scaled(out_dir):
    dev = torch.device("cuda", 0)
    ref.MODE["build"] = "ieee"
    out = {}
    for ci, (N, M, L, steps, seed) in enumerate(CASES):
        MP = (M + 63) // 64 * 64
        dx, dy = L[0] / (N - 1), L[1] / (M - 1)
        c = 1.0
        dt = 0.95 * min(dx, dy) / c / math.sqrt(2)
        u = initial(N, MP, MP, L, seed)
        u[:, M:] = 0
        q, s = nr.scaled_encode(u)
        out[f"c{ci}_q0"], out[f"c{ci}_s0"] = q.copy(), s.copy()
        out[f"c{ci}_params"] = np.array([N, M, MP, steps, c, dt, dx, dy], dtype=np.float64)
        t = lambda x: torch.from_numpy(x.copy()).to(dev)
        a, b = (t(q), t(s)), (t(q), t(s))
        f = lambda x: float(np.float32(x))
        for k in range(steps):  # u0 = step(u0, u1, u0); swap
            ref.scaled_step_gpu(a[0], a[1], b[0], b[1], a[0], a[1], f(c), f(dt), f(dx), f(dy), N, M)
            a, b = b, a
            if k in (0, 1, steps - 1):
                torch.cuda.synchronize()
                out[f"c{ci}_step{k}_q"], out[f"c{ci}_step{k}_s"] = b[0].cpu().numpy(), b[1].cpu().numpy()
    np.savez_compressed(os.path.join(out_dir, "scaled_step.npz"), **out)


def temporal(out_dir):
    """temporal_step itself on the inputs of the committed temporal golden
    file (whose levels come from 8 and 16 padded_step updates)."""
    dev = torch.device("cuda", 0)
    ref.MODE["build"] = "ieee"
    g = dict(np.load(os.path.join(HERE, "temporal_step.npz")))
    out = {}
    ci = 0
    while f"c{ci}_params" in g:
        N, M, MP, c, dt, dx, dy = g[f"c{ci}_params"][:7]
        N, M = int(N), int(M)
        u0, u1 = torch.from_numpy(g[f"c{ci}_u0"]).to(dev), torch.from_numpy(g[f"c{ci}_u1"]).to(dev)
        v0, v1 = torch.zeros_like(u0), torch.zeros_like(u0)
        w0, w1 = torch.zeros_like(u0), torch.zeros_like(u0)
        args = tuple(float(np.float32(x)) for x in (c, dt, dx, dy))
        ref.temporal_step_gpu(u0, u1, v0, v1, *args, N, M)
        ref.temporal_step_gpu(v0, v1, w0, w1, *args, N, M)
        torch.cuda.synchronize()
        out[f"c{ci}_after8_v0"], out[f"c{ci}_after8_v1"] = v0.cpu().numpy(), v1.cpu().numpy()
        out[f"c{ci}_after16_v0"], out[f"c{ci}_after16_v1"] = w0.cpu().numpy(), w1.cpu().numpy()
        ci += 1
    digests = {k: digest(v) for k, v in sorted(out.items())}
    with open(os.path.join(out_dir, "ref_gpu_digests.json"), "w") as f:
        json.dump({"temporal_step": digests}, f, indent=1, sort_keys=True)


def digest(a: np.ndarray) -> str:
    """SHA-256 of a C-contiguous array's dtype, shape and bytes."""
    h = hashlib.sha256()
    a = np.ascontiguousarray(a)
    h.update(str(a.dtype).encode())
    h.update(str(a.shape).encode())
    h.update(a.tobytes())
    return h.hexdigest()


if __name__ == "__main__":
    if not ref.gpu_available():
        raise SystemExit("the reference's GPU module files are not built")
    od = sys.argv[1] if len(sys.argv) > 1 else HERE
    os.makedirs(od, exist_ok=True)
    scaled(od)
    temporal(od)
