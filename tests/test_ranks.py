"""The N-GPU bench path's host logic with two processes over gloo on the CPU (no GPU): the
process group from torchrun's environment, the barriers, the maximum of the ranks' times that
the whole-job number divides by, and the reference arm, which only rank 0 runs."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port),
                       "RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world)})
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks("gloo")
    r.barrier()
    # each rank "took" a different time; every rank gets the slowest
    t = r.max(1.5 + rank)
    rate = bench.whole_job_rate(r.world, 1e7, t)
    r.barrier()
    r.close()
    # the reference arm: ranks other than 0 leave at once, without work or output
    class A:
        steps, warmup, gpus = 1, 0, world
    ref_rc = bench.run_reference(A()) if rank != 0 else None
    out.put((rank, r.world, r.rank, t, rate, ref_rc))


@pytest.mark.parametrize("world", [2])
def test_two_ranks_over_gloo(world):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    slowest = 1.5 + (world - 1)
    for rank, (r, w, rr, t, rate, ref_rc) in enumerate(res):
        assert (r, w, rr) == (rank, world, rank)
        assert t == slowest
        assert rate == pytest.approx(world * 1e7 / slowest / 1e6)
        assert ref_rc == (None if rank == 0 else 0)


def test_one_rank_needs_no_process_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    sys.path.insert(0, ROOT)
    import bench
    r = bench.Ranks("gloo")
    assert (r.world, r.rank, r.local) == (1, 0, 0)
    r.barrier()
    assert r.max(2.25) == 2.25
    r.close()
