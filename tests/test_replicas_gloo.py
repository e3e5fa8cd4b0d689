"""Multi-GPU runs are independent replicas (one problem per GPU, no data-path
collective); bench.py only needs a barrier and max / sum reductions of its
timings across ranks.  This checks that host logic with two gloo ranks on
the CPU, rendezvous on 127.0.0.1."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    q.put((rank, d.max(10.0 * (rank + 1)), d.sum(float(rank + 1))))
    d.close()


def test_two_replicas_reduce_timings():
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
    assert out == [(0, 20.0, 3.0), (1, 20.0, 3.0)]
