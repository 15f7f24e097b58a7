"""The multi-process path of bench.py (replicas, one process per GPU) with two
gloo ranks on the CPU: reductions of the timing and sample counts, barrier,
and the row split."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from mcrt_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    r, w, _ = replicas.init("gloo")
    step_ms = 10.0 + 5.0 * r                     # rank 1 is the slower replica
    replicas.barrier()
    mx = replicas.max_over_ranks(step_ms)
    total = replicas.sum_over_ranks(1000 * (r + 1))
    q.put((r, mx, total, replicas.split_rows(1080, r, w)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    assert [o[2] for o in out] == [3000.0, 3000.0]
    assert out[0][3] == (0, 540) and out[1][3] == (540, 1080)


@pytest.mark.parametrize("h,world", [(1080, 3), (7, 4), (1, 2), (1000, 8)])
def test_split_rows_covers_image(h, world):
    rows = [replicas.split_rows(h, r, world) for r in range(world)]
    assert rows[0][0] == 0 and rows[-1][1] == h
    assert all(a[1] == b[0] for a, b in zip(rows, rows[1:]))
    assert max(b - a for a, b in rows) - min(b - a for a, b in rows) <= 1
