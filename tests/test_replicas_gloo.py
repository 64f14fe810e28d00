"""The N > 1 path of bench.py on CPU: two gloo ranks, each timing its own
replica; the job time is the slower rank's and the throughput counts both
ranks' suffixes (no GPU, no collective on the data path)."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # rank r "took" 10 * (r + 1) ms for its replica
    t = bench.max_over_ranks(0.010 * (rank + 1), dist, "cpu")
    v = bench.job_throughput(1000, world, 2, t)
    out[rank] = (t, v)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_over_ranks_and_job_throughput():
    port = 29500 + (os.getpid() % 2000)
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        t, v = res[r]
        assert abs(t - 0.020) < 1e-12
        assert abs(v - 1000 * 2 * 2 / 0.020 / 1e6) < 1e-9


def test_single_process_helpers():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert abs(bench.job_throughput(2 ** 20, 1, 4, 0.5) - 2 ** 20 * 4 / 0.5 / 1e6) < 1e-9
