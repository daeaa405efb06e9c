"""The N>1 path on CPU: replicas on world_size-2 gloo ranks.

A single simulation does not shard (no domain decomposition in the reference),
so bench.py runs one replica per GPU and aggregates with the slowest rank's
time and the summed work.  Here two gloo ranks each run an oracle replica and
aggregate through bench.aggregate_replicas.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from hydro_rs_gb300 import ics
    from oracle import oracle as O

    p = ics.sod_1d(64 * (rank + 1))
    s = O.OracleSim(p, n_threads=1)
    s.run(max_steps=5)
    my_ms = 10.0 * (rank + 1)

    def red(op):
        def f(vals):
            t = torch.tensor(vals, dtype=torch.float64)
            dist.all_reduce(t, op=op)
            return t.tolist()
        return f

    (ms,), (faces,) = bench.aggregate_replicas([my_ms], [float(s.active_faces)], red(dist.ReduceOp.MAX),
                                               red(dist.ReduceOp.SUM))
    q.put((rank, ms, faces, s.active_faces))
    dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    out.sort()
    total = out[0][3] + out[1][3]
    for rank, ms, faces, own in out:
        assert ms == 20.0
        assert faces == total
    assert out[0][3] == 5 * 65 and out[1][3] == 5 * 129
