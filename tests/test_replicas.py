"""Multi-GPU form of the benchmark: independent replicas (the path has no
exchange step), one process per GPU, max-over-ranks timing.  The host logic
(rank setup from the torchrun environment, barrier, max over ranks, whole-job
throughput = units of all ranks / max time) runs here as two gloo processes
on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local, pg = bench.dist_setup(world)
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(pg)
    ms = 10.0 * (rank + 1)                 # rank 1 is the slower replica
    ms_step = bench.allmax(pg, ms)
    units_per_rank = 1000
    value = units_per_rank * w / (ms_step / 1e3)
    out.put((rank, ms_step, value))
    pg.destroy_process_group()


def test_replicas_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slower replica's time; throughput counts both ranks' units
    assert [r[1] for r in res] == [20.0, 20.0]
    assert res[0][2] == res[1][2] == pytest.approx(2 * 1000 / 0.020)
