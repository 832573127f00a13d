"""Multi-GPU is replicas only: each rank runs its own domain and the ranks
meet once, for the max-over-ranks time of the benchmark.  The host side of
that path (process group set-up, the reduction, rank-0-only output) runs here
as two gloo ranks on the CPU."""
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
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    r, ws, dist = bench.dist_setup(world)
    t = bench.reduce_max(dist, 10.0 * (rank + 1))          # per-rank elapsed ms
    out[rank] = (r, ws, t, os.environ["CUDA_VISIBLE_DEVICES"])
    dist.destroy_process_group()


def test_replica_ranks_take_the_max_time_over_gloo():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    world, port = 2, _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for rank in range(world):
        r, ws, t, dev = res[rank]
        assert (r, ws) == (rank, world)
        assert t == 10.0 * world                              # the slowest rank's time
        assert dev == str(rank)                               # one GPU per replica
