"""The multi-process side of bench.py without a GPU: two gloo ranks (one
process per GPU in a real run) each time a region, the job's time is the
slowest rank's, the whole-job throughput counts every rank's frames, and
only rank 0 of the reference arm does any work."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import sys

    import torch.distributed as dist

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    w, r, local = bench.dist_env()
    assert (w, r, local) == (world, rank, rank)
    my_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    job_ms = bench.max_over_ranks(my_ms, world)
    out[rank] = (job_ms, bench.job_throughput(world, 10, job_ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world, port = 2, _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank_main, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 150.0
    assert abs(res[0][1] - 2 * 10 / 0.150) < 1e-9


def test_reference_arm_works_on_rank_0_only(monkeypatch):
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    called = []
    monkeypatch.setattr(bench, "workload", lambda *a, **k: called.append(1))

    class A:
        steps, warmup = 1, 1
    bench.run_reference(A)
    assert not called
