"""bench.py's multi-rank bookkeeping (replicas only: no data-path
collective) on CPU with gloo, world_size 2: the timed value is the max over
ranks and the work is summed over ranks."""
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


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MRF_BENCH_BACKEND="gloo")
    import bench
    r, w = bench.dist_setup()
    t = bench.max_over_ranks(10.0 + rank, w)
    s = bench.sum_over_ranks(100.0 * (rank + 1), w)
    bench.barrier(w)
    q.put((r, w, t, s))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[:2] for o in out] == [(0, 2), (1, 2)]
    assert all(o[2] == 11.0 for o in out)
    assert all(o[3] == 300.0 for o in out)
