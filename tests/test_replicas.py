"""bench.py's multi-GPU path is replicas only: every rank runs its own join,
ranks meet at barriers, and the timing is the maximum over ranks.  Here two
gloo ranks on the CPU check that host logic (the GPU work itself is not
sharded and needs no collective)."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w, "gloo")
    d.barrier()
    t_max = d.max(10.0 + 5.0 * r)  # a slower rank decides the time
    d.barrier()
    d.close()
    out[rank] = (r, w, local, t_max)


def test_two_gloo_replicas_take_the_slowest_time():
    torch = pytest.importorskip("torch")
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed unavailable")
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        ctx = mp.get_context("spawn")
        ps = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in ps:
            p.start()
        for p in ps:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0][:3] == (0, 2, 0) and res[1][:3] == (1, 2, 1)
    assert res[0][3] == res[1][3] == 15.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup, cpu_sample = 1, 0, 10

    assert bench.run_reference(Args()) == 0  # returns at once, no work, no output
