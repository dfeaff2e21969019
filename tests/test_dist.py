"""CPU, world size 2 over gloo: the replica path of bench.py (barrier,
max-over-ranks timing, whole-job aggregation).  The solve itself has no
exchange step, so no collective touches the data path."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    d.barrier()
    per_rank_ms = 100.0 * (rank + 1)           # rank 1 is the slow one
    value, ms = bench.aggregate(d, 1000, per_rank_ms)
    q.put((rank, value, ms, d.max(rank)))
    d.close()


def test_two_rank_replicas():
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
    for rank, value, ms, mx in out:
        assert ms == 200.0                      # max over ranks
        assert value == pytest.approx(2 * 1000 / 0.2)
        assert mx == 1.0
