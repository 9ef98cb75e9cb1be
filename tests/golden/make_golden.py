"""Generates the golden vectors in this folder from the reference's own step
kernels, compiled for the CPU from projects/18_simple_wave_fd/step2D_wave.cu and
step1D_wave.cu by oracle/Makefile.ref (oracle.ref). Needs the reference
sources, so it runs where they are mounted, never at test time:

    python tests/golden/make_golden.py

Outputs (small .npz files, committed):
  padded_step.npz  seeded FP32 inputs (u0, u1) and the fields after the first,
                   second and last of a few steps of padded_step, in-place rotation as in
                   2D_wave_cuda_padding.py:83-85, on two grids (odd M, M_padded
                   a multiple of 32 as in the driver)
  mixed_step.npz   the same for mixed_step (FP16 storage)
  step1d.npz       the same for step1D
  scaled_step.npz  written by make_golden_gpu.py from the reference's own
                   scaled_step built for the GPU (its warp shuffles do not run
                   in the CPU build); scaled_golden() below gives the same
                   arrays from the NumPy restatement oracle.numpy_ref.scaled_step
                   (a CPU test checks that they are equal)
  temporal_step.npz  two distinct levels (u0, u1) and the level pairs after 8
                   and 16 padded_step updates: what one and two temporal_step
                   launches return (step2D_wave.cu:244-304; the reference states
                   the two kernels are bit-identical, README.md:38-40, and its
                   block barriers do not run in the CPU build)
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import ref  # noqa: E402

CASES = [
    # N, M, lengths, steps, seed
    (67, 150, (1.0, 2.0), 12, 1),
    (40, 33, (1.0, 1.0), 9, 2),
]


def initial(N, M, MP, lengths, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, lengths[0], N)[:, None]
    y = np.linspace(0, lengths[1], M)[None, :]
    g = np.exp(-((x - 0.4 * lengths[0]) ** 2 + (y - 0.55 * lengths[1]) ** 2) / (2 * 0.08**2))
    u = np.zeros((N, MP), dtype=dtype)
    u[:, :M] = g + 0.01 * rng.standard_normal((N, M))
    return u


def main():
    if not ref.build():
        raise SystemExit("reference sources not found; cannot generate golden vectors")
    out = {}
    for ci, (N, M, L, steps, seed) in enumerate(CASES):
        MP = (M + 31) // 32 * 32
        dx, dy = L[0] / (N - 1), L[1] / (M - 1)
        c = 1.0
        dt = 0.95 * min(dx, dy) / c / math.sqrt(2)  # 2D_wave_cuda_padding.py:39-40
        u0 = initial(N, MP, MP, L, seed)[:, :MP]
        u0[:, M:] = 0
        u1 = u0.copy()
        out[f"c{ci}_u0"] = u0.copy()
        out[f"c{ci}_u1"] = u1.copy()
        out[f"c{ci}_params"] = np.array([N, M, MP, steps, c, dt, dx, dy], dtype=np.float64)
        a, b = u0.copy(), u1.copy()
        for t in range(steps):
            a = ref.padded_step(a, b, a, np.float32(c), np.float32(dt), np.float32(dx), np.float32(dy), N, M)
            a, b = b, a
            if t in (0, 1, steps - 1):
                out[f"c{ci}_step{t}"] = b.copy()  # the newest level
    np.savez_compressed(os.path.join(HERE, "padded_step.npz"), **out)

    out = {}
    for ci, (N, M, L, steps, seed) in enumerate(CASES):
        MP = (M + 31) // 32 * 32
        dx, dy = L[0] / (N - 1), L[1] / (M - 1)
        c = 1.0
        dt = 0.95 * min(dx, dy) / c / math.sqrt(2)
        u0 = initial(N, MP, MP, L, seed).astype(np.float16)
        u0[:, M:] = 0
        a, b = u0.copy(), u0.copy()
        out[f"c{ci}_u0"] = a.copy()
        out[f"c{ci}_params"] = np.array([N, M, MP, steps, c, dt, dx, dy], dtype=np.float64)
        for t in range(steps):
            a = ref.mixed_step(a, b, a, np.float32(c), np.float32(dt), np.float32(dx), np.float32(dy), N, M)
            a, b = b, a
            if t in (0, 1, steps - 1):
                out[f"c{ci}_step{t}"] = b.copy()
    np.savez_compressed(os.path.join(HERE, "mixed_step.npz"), **out)

    N = 301
    dx = 1.0 / (N - 1)
    dt = 0.95 * dx
    x = np.linspace(0, 1, N)
    u = np.exp(-((x - 0.3) ** 2) / (2 * 0.03**2)).astype(np.float32)
    a, b = u.copy(), u.copy()
    out = {"u0": u.copy(), "params": np.array([N, 1.0, dt, dx])}
    for t in range(25):
        a = ref.step1d(a, b, a, np.float32(1.0), np.float32(dt), np.float32(dx))
        a, b = b, a
        if t in (0, 1, 24):
            out[f"step{t}"] = b.copy()
    np.savez_compressed(os.path.join(HERE, "step1d.npz"), **out)
    temporal_golden()
    basic_golden()
    print("golden vectors written to", HERE)


def basic_golden():
    """basic_step and coalesced_step (unpadded rows, M_padded = M) from the
    reference's host build: a few steps with the driver's in-place rotation."""
    out = {}
    for ci, (N, M, L, steps, seed) in enumerate(CASES):
        dx, dy = L[0] / (N - 1), L[1] / (M - 1)
        c = 1.0
        dt = 0.95 * min(dx, dy) / c / math.sqrt(2)
        u = initial(N, M, M, L, seed)
        out[f"c{ci}_u0"] = u.copy()
        out[f"c{ci}_params"] = np.array([N, M, steps, c, dt, dx, dy], dtype=np.float64)
        for name, fn in (("basic", ref.basic_step), ("coalesced", ref.coalesced_step)):
            a, b = u.copy(), u.copy()
            for t in range(steps):
                a = fn(a, b, a, np.float32(c), np.float32(dt), np.float32(dx), np.float32(dy))
                a, b = b, a
            out[f"c{ci}_{name}_last"] = b.copy()
    np.savez_compressed(os.path.join(HERE, "basic_step.npz"), **out)


def temporal_golden():
    out = {}
    cases = [(67, 150, (1.0, 2.0), 1), (40, 33, (1.0, 1.0), 2), (36, 300, (1.0, 3.0), 3)]
    for ci, (N, M, L, seed) in enumerate(cases):
        MP = (M + 31) // 32 * 32
        dx, dy = L[0] / (N - 1), L[1] / (M - 1)
        c = 1.0
        dt = 0.95 * min(dx, dy) / c / math.sqrt(2)
        u = initial(N, MP, MP, L, seed)
        u[:, M:] = 0
        a, b = u.copy(), u.copy()
        step = lambda a, b: ref.padded_step(a, b, a, np.float32(c), np.float32(dt), np.float32(dx),
                                            np.float32(dy), N, M)
        for _ in range(3):  # two distinct levels to start from
            a = step(a, b)
            a, b = b, a
        out[f"c{ci}_u0"], out[f"c{ci}_u1"] = a.copy(), b.copy()
        out[f"c{ci}_params"] = np.array([N, M, MP, c, dt, dx, dy], dtype=np.float64)
        for t in range(16):
            a = step(a, b)
            a, b = b, a
            if t == 15 or (t == 7 and ci < 2):
                out[f"c{ci}_after{t + 1}_v0"], out[f"c{ci}_after{t + 1}_v1"] = a.copy(), b.copy()
    np.savez_compressed(os.path.join(HERE, "temporal_step.npz"), **out)


def scaled_golden(write: bool = True):
    """scaled_step vectors from the NumPy restatement (oracle.numpy_ref), in
    the layout of scaled_step.npz (which make_golden_gpu.py writes from the
    reference's own kernel). Returns them; writes them only when asked."""
    from oracle import numpy_ref as nr
    out = {}
    for ci, (N, M, L, steps, seed) in enumerate(CASES):
        MP = (M + 63) // 64 * 64
        dx, dy = L[0] / (N - 1), L[1] / (M - 1)
        c = 1.0
        dt = 0.95 * min(dx, dy) / c / math.sqrt(2)
        u = initial(N, MP, MP, L, seed)
        u[:, M:] = 0
        q, s = nr.scaled_encode(u)
        a, b = (q.copy(), s.copy()), (q.copy(), s.copy())
        out[f"c{ci}_q0"], out[f"c{ci}_s0"] = q.copy(), s.copy()
        out[f"c{ci}_params"] = np.array([N, M, MP, steps, c, dt, dx, dy], dtype=np.float64)
        for t in range(steps):
            a = nr.scaled_step(a[0], a[1], b[0], b[1], np.float32(c), np.float32(dt), np.float32(dx),
                               np.float32(dy), N, M)
            a, b = b, a
            if t in (0, 1, steps - 1):
                out[f"c{ci}_step{t}_q"], out[f"c{ci}_step{t}_s"] = b[0].copy(), b[1].copy()
    if write:
        np.savez_compressed(os.path.join(HERE, "scaled_step.npz"), **out)
    return out


if __name__ == "__main__":
    main()
