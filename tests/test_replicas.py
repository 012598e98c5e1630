"""The multi-GPU path of bench.py: query-sharded replicas. Every rank holds the whole index and
searches the queries of its own id range; the job's time is the slowest rank's, the job's
throughput counts every query once, and the ranks' results are gathered in query-id order; the
reference arm runs on rank 0 alone. Checked with world-size-2 gloo process groups on the CPU (the
same all_reduce / all_gather the NCCL run makes), with a deterministic stand-in for the search."""
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        step_ms, e2e_ms = times[rank]
        out.put((rank, bench.replica_aggregate(step_ms, e2e_ms, 1000, world, device="cpu")))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_replica_aggregate_takes_the_slowest_rank():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    times = [(10.0, 30.0), (12.5, 20.0)]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank in (0, 1):
        step_ms, e2e_ms, value, e2e_value = got[rank]
        assert step_ms == 12.5 and e2e_ms == 30.0  # max over ranks, each column on its own
        # 1000 distinct queries in the job, each counted once, at the slowest rank's time
        assert value == pytest.approx(1000 / 0.0125) and e2e_value == pytest.approx(1000 / 0.030)


def test_single_rank_is_its_own_job():
    sys.path.insert(0, ROOT)
    import bench

    step_ms, e2e_ms, value, e2e_value = bench.replica_aggregate(8.0, 10.0, 500, 1, device="cpu")
    assert (step_ms, e2e_ms) == (8.0, 10.0)
    assert value == pytest.approx(500 / 0.008) and e2e_value == pytest.approx(500 / 0.010)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun the other ranks of --impl reference exit 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""


def _fake_search(torch, qids):
    """A deterministic stand-in for the search of queries `qids`: [len, 10] ids."""
    return (qids[:, None] * 7919 + torch.arange(10)[None, :] * 31) % 100_003


def _shard_worker(rank, world, port, nq, out):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = bench.shard_range(nq, world, rank)
        local = _fake_search(torch, torch.arange(lo, hi))
        gathered = bench.gather_shards(local, nq, world)
        out.put((rank, (lo, hi), gathered.numpy()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("nq", [1000, 1001])
def test_sharded_queries_gather_to_the_single_rank_result(nq):
    import numpy as np
    import torch
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, nq, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = {}
    for _ in procs:
        rank, rng, arr = out.get(timeout=120)
        got[rank] = (rng, arr)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    single = _fake_search(torch, torch.arange(nq)).numpy()
    (lo0, hi0), (lo1, hi1) = got[0][0], got[1][0]
    assert lo0 == 0 and hi0 == lo1 and hi1 == nq  # disjoint id ranges that cover every query once
    for rank in (0, 1):
        np.testing.assert_array_equal(got[rank][1], single)
