"""The multi-GPU path of bench.py, which is replicas only (the search does not shard): every rank
times its own copy, the job's time is the slowest rank's and the job's throughput counts every
rank's queries; the reference arm runs on rank 0 alone. Checked with world-size-2 gloo process
groups on the CPU (the same all_reduce the NCCL run makes)."""
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
        assert value == pytest.approx(2 * 1000 / 0.0125) and e2e_value == pytest.approx(2 * 1000 / 0.030)


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
