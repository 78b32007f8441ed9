"""bench.py's multi-rank plumbing on CPU: two gloo ranks, as torchrun runs
them (RANK / WORLD_SIZE / MASTER_* from the environment). Replicas only: the
sole collectives are a barrier and a max / sum of per-rank scalars."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist()
    d.barrier()
    mx = d.reduce(float(rank + 1) * 10.0, "max")
    sm = d.reduce(float(rank + 1), "sum")
    d.barrier()
    out.put((rank, d.world, mx, sm))
    d.close()


def test_two_gloo_ranks_reduce_like_the_bench():
    pytest.importorskip("torch")
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2, 20.0, 3.0), (1, 2, 20.0, 3.0)]


def test_reference_arm_prints_only_on_rank_zero(capsys):
    """Under torchrun only rank 0 runs the CPU reference arm and prints."""
    sys.path.insert(0, ROOT)
    import bench

    class FakeDist:
        rank = 1

    class Args:
        pass

    bench.run_reference_arm(Args(), FakeDist())
    bench.run_reference_arm_pbf(Args(), FakeDist())
    bench.run_reference_arm_batched(Args(), FakeDist())
    assert capsys.readouterr().out == ""
