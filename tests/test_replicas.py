"""CPU: the N > 1 path of bench.py (independent replicas, one per GPU) with
two gloo ranks: the job's time is the slowest rank's, the whole-job rate
sums the ranks' work, the replicas solve different sun directions, and the
CPU reference arm runs on rank 0 only."""
import os
import socket

import numpy as np
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench
from fluxpy_gb300 import terrain


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms_local = [120.0, 150.0][rank]
        ms = bench.job_time_ms(ms_local, dist, torch.device("cpu"))
        dirs = bench.replica_directions(terrain, 16, rank)
        gathered = [torch.zeros(16, 3, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(gathered, torch.as_tensor(dirs))
        out[rank] = (ms, bench.job_rate(1024, world, 5, ms),
                     not torch.equal(gathered[0], gathered[1]))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_replicas():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        ms, rate, distinct = res[rank]
        assert ms == 150.0                       # slowest rank
        assert np.isclose(rate, 2 * 1024 * 5 / 0.150)
        assert distinct
    # rank 0 keeps the workload's own directions (seed 2)
    assert np.array_equal(bench.replica_directions(terrain, 16, 0),
                          terrain.random_sun_directions(16, seed=2))


def test_reference_arm_runs_on_rank_zero_only(capsys, monkeypatch):
    import argparse
    monkeypatch.setenv("RANK", "1")
    ns = argparse.Namespace(gpus=2, steps=1, warmup=0, grid=512, rhs=1024, tol=1e-5)
    bench.run_reference(ns)
    assert capsys.readouterr().out == ""


def test_cpu_baseline_uses_every_requested_process():
    r = bench.cpu_baseline(None, seconds=1.0, workers=2)
    assert r["cores"] == 2 and r["kind"] == "port"
    assert r["value"] > 0 and r["value"] == r["measured_solves_per_s_at_sample"]


def test_workload_cpu_baselines_run():
    sizes = np.array([2000, 5000, 60000])
    r = bench.craters_cpu_baseline(sizes, seconds=0.5)
    assert r["cores"] == 1 and 0 < r["value"] < r["sample_facet_steps_per_s"]
    r = bench.adjoint_cpu_baseline(seconds=0.1)
    assert r["cores"] == 1 and r["value"] > 0
