"""bench.py's N-GPU path is N independent replicas (the solve path has no
collective): under torchrun each rank solves its own copy of the workload and
the ranks only agree on timings -- a barrier around the timed region, the
maximum time over ranks and the sum of the work.  Those host-side steps run
here as two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    ws, r, local, pg = bench.dist_setup(world)
    assert (ws, r, local) == (world, rank, rank) and pg is not None
    bench.barrier(pg)
    t_max = bench.allmax(pg, 1.0 + rank)         # the slowest rank's time
    work = bench.allsum(pg, 100.0 * (rank + 1))  # every rank's units
    bench.barrier(pg)
    out.put((rank, t_max, work))
    pg.destroy_process_group()


def test_two_replicas_agree_on_time_and_work():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert res == [(0, 2.0, 300.0), (1, 2.0, 300.0)]
