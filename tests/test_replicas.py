"""Replicas (several GPUs, no data-path exchange) on the CPU: the max-over-ranks timing and
the per-rank streams with world size 2 on the gloo backend, and the reference arm's rank
behaviour under torchrun."""

import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from pyalbsim_gb300.replicas import aggregate_rate, max_over_ranks, replica_seed

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = max_over_ranks(100.0 + 50.0 * rank)  # rank 1 is the slow one
        seeds = [replica_seed(1, rank, s) for s in range(3)]
        out.put((rank, ms, seeds, aggregate_rate(1000.0, world, ms)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_distinct_streams_with_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, s0, v0), (r1, ms1, s1, v1) = res
    assert ms0 == ms1 == 150.0  # every rank reports the slowest rank's time
    assert v0 == v1 == 2 * 1000.0 / 0.150
    assert not set(s0) & set(s1) and len(set(s0)) == 3  # no two ranks or steps share a stream


def test_max_over_ranks_without_a_process_group():
    from pyalbsim_gb300.replicas import max_over_ranks

    assert max_over_ranks(3.5) == 3.5


def test_reference_arm_only_runs_on_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_replica_seeds_do_not_collide_across_base_rank_and_step():
    """Adjacent base seeds, ranks and steps give distinct Philox keys (a sum of the three
    would give (base 0, rank 1) and (base 1, rank 0) the same key)."""
    from pyalbsim_gb300.replicas import replica_seed

    keys = {replica_seed(b, r, s) for b in range(4) for r in range(4) for s in range(4)}
    assert len(keys) == 64
    assert replica_seed(0, 1) != replica_seed(1, 0)
    with pytest.raises(ValueError):
        replica_seed(1, 1 << 12)
