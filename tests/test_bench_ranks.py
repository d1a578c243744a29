"""bench.py's multi-rank path on CPU: two gloo ranks, as torchrun would start
them (127.0.0.1 rendezvous).  Each rank builds its own replica of the job
(seeded by rank, no collective on the data path); the job's step time is the
slowest rank's and its lines are the sum over ranks; the reference arm runs on
rank 0 alone and the other ranks exit at once."""
import os
import socket
import sys
import time
from types import SimpleNamespace

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    args = SimpleNamespace(workload="c2v_small", jmax=None, seed=1, gpus=world, steps=1,
                           warmup=0)
    prob = bench.make_problem(args, rank)
    e0 = float(prob.blocks[(1, 0)].energies[0])
    dt, pre, post = bench.across_ranks(0.1 * (rank + 1), 100 + rank, 50 + rank, "cpu")
    t0 = time.perf_counter()
    ref_rc = bench.main_reference(args) if rank == 1 else None
    ref_s = time.perf_counter() - t0
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, dt, pre, post, e0, ref_rc, ref_s))


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, dt0, pre0, post0, e00, _, _), (r1, dt1, pre1, post1, e01, rc1, s1) = out
    assert dt0 == dt1 == pytest.approx(0.2)          # the slowest rank's time
    assert pre0 == pre1 == 201 and post0 == post1 == 101  # lines summed over ranks
    assert e00 != e01                                 # independent replicas (seed + rank)
    assert rc1 == 0 and s1 < 5.0                      # reference arm: rank 1 does no work
