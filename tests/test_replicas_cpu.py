"""The multi-GPU path of bench.py is replicas: every rank runs its own
system, the job's time is the slowest rank's, its throughput every rank's
units over that time. These host-side pieces run here as two gloo ranks on
the CPU (one process per rank, rendezvous on 127.0.0.1)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    from cosmosim_gb300 import lib

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_env()
    times = bench.max_over_ranks(torch, [1.0 + rank, 5.0 - rank, 0.5], "cpu")
    rate = bench.job_rate(1000, w, times[0])
    # each rank's ensemble is its own (rank-dependent seeds)
    bodies, parts = bench.ensemble_bodies(lib.generate_ics, r)
    out.put((rank, r, w, local, times, rate, float(bodies["x"][:100].sum()), len(bodies)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_bench():
    world, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=240) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, r, w, local, times, rate, xsum, n in res:
        assert (r, w, local) == (rank, 2, rank)
        assert times == [2.0, 5.0, 0.5]          # max over ranks
        assert rate == pytest.approx(1000 * 2 / 2.0)
    assert res[0][7] == res[1][7]  # the same galaxy sizes on every rank
    assert res[0][6] != res[1][6]  # but each rank's galaxies are its own
