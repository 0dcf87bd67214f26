"""The N>1 path of bench.py on CPU: world_size-2 gloo ranks (replicas only — no data exchange on the
path; ranks meet only for the barrier and the max-over-ranks timing)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    ws, r = bench.init_dist("gloo")
    bench.barrier()
    elapsed = 1.0 + rank            # rank 1 is the slower replica
    m = bench.max_over_ranks(elapsed)
    out.put((rank, ws, m))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_barrier_and_max():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2, 2]
    assert all(r[2] == 2.0 for r in res)      # every rank sees the slowest replica's time


def test_reference_arm_other_ranks_exit(monkeypatch):
    """Under torchrun only rank 0 runs the CPU reference; the other ranks return 0 without work."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class A:
        steps, warmup = 1, 3
    assert bench.run_reference(A()) == 0
