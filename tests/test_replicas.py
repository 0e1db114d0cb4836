"""Multi-rank host logic on CPU (gloo, world size 2): replicas with no data-path
collective, the max-over-ranks timing and the whole-job rate, and the
reference arm's rank > 0 exit.  Each rank's "job" is the CPU oracle's FX path
on its own seeded input, standing in for the per-GPU job."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
S, N, K = 4, 1024, 8


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    sys.path[:0] = [str(ROOT / "cellspe-tasklib_gb300"), str(ROOT)]
    import time

    import torch.distributed as dist

    import oracle
    import replicas
    import synth

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    raw = synth.stations_offset_binary(S, N * K, rho=0.1, seed=replicas.job_seed(rank))
    dist.barrier()
    t0 = time.perf_counter()
    vis = oracle.fx_fp32(raw, S, N, K)
    ms = (time.perf_counter() - t0) * 1e3 + 10.0 * rank      # rank 1 made the slowest
    ms_max = replicas.max_over_ranks(ms, dist)
    rate = replicas.aggregate_gsamples(world, S * N * K, ms_max)
    np.savez(Path(out_dir) / f"rank{rank}.npz", vis=vis, ms=ms, ms_max=ms_max, rate=rate)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_run_independent_replicas(tmp_path, orc):
    import torch.multiprocessing as mp

    import replicas
    import synth

    mp.spawn(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    r = [np.load(tmp_path / f"rank{i}.npz") for i in range(2)]
    # every rank correlated its own input, exactly as a single process would
    for i in range(2):
        raw = synth.stations_offset_binary(S, N * K, rho=0.1, seed=replicas.job_seed(i))
        assert np.array_equal(r[i]["vis"], orc.fx_fp32(raw, S, N, K))
    assert not np.array_equal(r[0]["vis"], r[1]["vis"])
    # the step time is the slowest rank's, and the rate counts both ranks' samples
    slowest = max(float(r[0]["ms"]), float(r[1]["ms"]))
    for i in range(2):
        assert float(r[i]["ms_max"]) == pytest.approx(slowest)
        assert float(r[i]["rate"]) == pytest.approx(2 * S * N * K / (slowest * 1e-3) / 1e9)


def test_single_process_reduction_is_identity():
    import replicas

    assert replicas.max_over_ranks(3.5, None) == 3.5
    assert replicas.aggregate_gsamples(1, 2_000_000_000, 1000.0) == pytest.approx(2.0)
    assert replicas.job_seed(0) != replicas.job_seed(1)


def test_reference_arm_other_ranks_exit_without_output():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
