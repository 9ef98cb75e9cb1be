"""Multi-rank shot sharding on CPU ranks (gloo, world size 2): the host logic
of the multi-GPU path, with the FP64 oracle standing in for each rank's GPU
gradient. Also the failure path: a rank that raises before the collective
makes the other rank's all-reduce end with an error after a short timeout
(no GPU is involved, nothing hangs past the timeout). And the benchmark's CPU
reference arm launched under torchrun: one line from rank 0."""
import datetime
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from neuralmech_gb300.shard import shard_range


def test_shard_range_partitions():
    for nshot in (1, 5, 64, 129):
        for world in (1, 2, 3, 8):
            parts = [shard_range(nshot, r, world) for r in range(world)]
            assert parts[0].start == 0 and parts[-1].stop == nshot
            assert all(a.stop == b.start for a, b in zip(parts, parts[1:]))
            sizes = [p.stop - p.start for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _problem():
    import oracle
    from helpers import oracle_geometry, small_problem
    grid, v, wav, src, rec = small_problem(shape=(36, 60), nshot=5, nt=40, sponge=6, nrec=7, seed=21)
    rng = np.random.default_rng(3)
    vt = v * (1 + 0.03 * rng.standard_normal(v.shape))
    obs = oracle.forward(oracle_geometry(oracle, grid, vt, wav, src, rec))
    return grid, v, wav, src, rec, obs


def _oracle_compute(vel, wav, src, rec, obs, grid):
    import oracle
    from helpers import oracle_geometry
    J, g, _, _ = oracle.gradient(oracle_geometry(oracle, grid, vel.numpy(), wav.numpy(), src.numpy(),
                                                 rec.numpy()), obs.numpy())
    return torch.tensor(J, dtype=torch.float64), torch.from_numpy(g)


def _worker(rank, world, port, mode, result_dir):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=5))
    from neuralmech_gb300.shard import distributed_misfit_gradient
    grid, v, wav, src, rec, obs = _problem()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    try:
        if mode == "fail" and rank == 1:
            raise RuntimeError("rank 1 fails before its collective")
        if mode == "bench":  # the benchmark's weak-scaling survey: the shots once per rank
            import bench
            survey = bench.weak_survey(t(wav), t(src), t(rec), t(obs), world, rank)
            J, g = distributed_misfit_gradient(t(v.astype(np.float64)), *survey, grid, compute=_oracle_compute)
        else:
            J, g = distributed_misfit_gradient(t(v.astype(np.float64)), t(wav), t(src), t(rec), t(obs), grid,
                                               compute=_oracle_compute)
        np.save(os.path.join(result_dir, f"g{rank}.npy"), g.numpy())
        np.save(os.path.join(result_dir, f"J{rank}.npy"), J.numpy())
        status = "ok"
    except Exception as e:  # noqa: BLE001 - the test inspects the failure kind
        status = type(e).__name__ + ": " + str(e)[:200]
    with open(os.path.join(result_dir, f"status{rank}.txt"), "w") as f:
        f.write(status)
    try:
        dist.destroy_process_group()
    except Exception:  # noqa: BLE001
        pass


def _spawn(mode, tmp_path):
    ctx = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, mode, str(tmp_path))) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        if p.is_alive():
            p.kill()
            pytest.fail("a rank did not finish")
    return [open(os.path.join(tmp_path, f"status{r}.txt")).read() for r in range(2)]


def test_two_ranks_match_one_process(tmp_path):
    status = _spawn("ok", tmp_path)
    assert status == ["ok", "ok"], status
    grid, v, wav, src, rec, obs = _problem()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    J, g = _oracle_compute(t(v.astype(np.float64)), t(wav), t(src), t(rec), t(obs), grid)
    for r in range(2):
        gr = np.load(tmp_path / f"g{r}.npy")
        Jr = float(np.load(tmp_path / f"J{r}.npy"))
        assert np.linalg.norm(gr - g.numpy()) <= 1e-12 * np.linalg.norm(g.numpy())
        assert abs(Jr - float(J)) <= 1e-12 * float(J)


def test_bench_weak_survey_two_ranks(tmp_path):
    """The multi-GPU benchmark's path (bench.weak_survey + the shard module)
    on two gloo ranks: each rank computes its own block of the doubled survey,
    and the all-reduced misfit and gradient are twice those of one block."""
    status = _spawn("bench", tmp_path)
    assert status == ["ok", "ok"], status
    grid, v, wav, src, rec, obs = _problem()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    J, g = _oracle_compute(t(v.astype(np.float64)), t(wav), t(src), t(rec), t(obs), grid)
    for r in range(2):
        gr = np.load(tmp_path / f"g{r}.npy")
        Jr = float(np.load(tmp_path / f"J{r}.npy"))
        assert np.linalg.norm(gr - 2 * g.numpy()) <= 1e-12 * np.linalg.norm(g.numpy())
        assert abs(Jr - 2 * float(J)) <= 1e-12 * float(J)


def test_failed_rank_surfaces_as_collective_error(tmp_path):
    status = _spawn("fail", tmp_path)
    assert status[1].startswith("RuntimeError: rank 1 fails")
    assert status[0] != "ok"  # rank 0's all-reduce ended with an error, not a hang


def test_bench_reference_arm_under_torchrun():
    """`bench.py --impl reference` launched as the multi-GPU bench is (torchrun,
    two ranks on 127.0.0.1): rank 0 alone times the CPU reference and prints
    one JSON line for the whole job; the other rank exits 0 without work."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
           "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    out = subprocess.run(cmd, cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.lstrip().startswith("{")]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r["impl"] == "reference" and r["n_gpus"] == 2 and r["value"] > 0
