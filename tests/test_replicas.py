"""Replica runs across ranks (fmf.replicas) on host cores: two gloo ranks, each with
its own timing; the reported time is the slowest rank's and the throughput counts
every replica's cells.  The time step exchanges nothing between ranks, so the
reduction of the timing is the only collective."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "fel-multi-phase-flow_gb300"))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    from fmf import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w = replicas.world()
        replicas.barrier()
        my_ms = 10.0 + 5.0 * rank  # rank 1 is the slow replica
        ms = replicas.max_over_ranks(my_ms)
        v = replicas.throughput(1000, 4, ms * 1e-3)
        replicas.barrier()
        q.put((r, w, ms, v))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_whole_job_throughput_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    codes = [p.exitcode for p in procs]
    for p in procs:
        if p.is_alive():
            p.kill()
    assert codes == [0, 0], codes
    out = sorted(q.get(timeout=5) for _ in range(2))
    for r, (rank, world, ms, v) in enumerate(out):
        assert rank == r and world == 2
        assert ms == 15.0  # every rank reports the slowest replica's time
        assert v == pytest.approx(2 * 1000 * 4 / 15e-3)


def test_single_process_without_group():
    pytest.importorskip("torch")
    from fmf import replicas

    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.throughput(10, 2, 0.5) == 40.0
    with pytest.raises(ValueError):
        replicas.throughput(10, 2, 0.0)


def test_reference_arm_other_ranks_exit_without_work():
    """Under a multi-rank launch only rank 0 times the CPU reference; the other
    ranks print nothing and exit 0."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
