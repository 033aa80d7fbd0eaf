"""bench.py's N>1 path on CPU: two gloo ranks on 127.0.0.1 (replicas: no data-path collective).
Checks the rendezvous, the barrier, the max-over-ranks timing and the whole-job value, and that
only rank 0 runs and prints the reference arm."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local = bench.dist_setup(world)
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(w)
    # each rank "timed" a different duration; every rank must see the slowest
    slowest = bench.max_over_ranks(1.0 + rank, w)

    class Args:
        workload = "icosphere256"
    ref = bench.run_reference(Args(), w, r) if r != 0 else "rank0"
    import torch.distributed as dist
    dist.destroy_process_group()
    out.put((rank, slowest, ref))


def test_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [2.0, 2.0]
    assert got[1][2] is None  # rank 1 does no reference work and prints nothing
    # whole-job throughput with the slowest rank's time: world x units / time
    units_per_rank, slowest_s = 20480, 2.0
    assert world * units_per_rank / slowest_s == 20480.0
