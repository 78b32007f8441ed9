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


def test_batched_instances_partition_over_ranks():
    """Every instance goes to exactly one rank, longest first, loads balanced."""
    sys.path.insert(0, ROOT)
    from amca3d_gb300 import decks, shard

    cases = decks.config_batched_64()
    for world in (1, 2, 4, 8):
        parts = shard.partition(cases, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(cases)))
        loads = [sum(shard.instance_work(cases[i]) for i in p) for p in parts]
        assert max(loads) <= 1.1 * (sum(loads) / world) + max(shard.instance_work(c) for c in cases)
        # the heaviest instance goes to rank 0 first
        heaviest = max(range(len(cases)), key=lambda i: shard.instance_work(cases[i]))
        assert parts[0][0] == heaviest


def _instance_rank(rank: int, world: int, port: int, names, out):
    """One gloo rank: runs its share of the given instances on the C oracle
    (standing in for its GPU) and gathers the field digests like the bench."""
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import amca_oracle

    import bench
    from amca3d_gb300 import decks, shard

    cases = [c for c in decks.config_batched_64() if c.name in names]
    d = bench.Dist()
    mine = shard.partition(cases, d.world)[d.rank]
    local = {}
    for i in mine:
        r = amca_oracle.run_plain(cases[i])
        local[cases[i].name] = (shard.field_digest(r["orient"]), int(r["steps"]))
    gathered = {}
    for part in d.gather(local):
        gathered.update(part)
    out.put((rank, len(mine), gathered))
    d.close()


def test_two_ranks_gather_instance_digests_that_match_the_reference(oracle):
    """The N-GPU batched leg's plumbing on two gloo ranks: the smallest four
    instances of batched_64 split over the ranks, each rank's digests
    gathered on every rank and equal to the instances' reference runs."""
    pytest.importorskip("torch")
    import json
    import multiprocessing as mp

    from amca3d_gb300 import decks

    golden = json.load(open(os.path.join(ROOT, "tests", "golden", "batched_64_golden.json")))
    names = [c.name for c in sorted(decks.config_batched_64(), key=lambda c: c.n_interior)[:4]]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_instance_rank, args=(r, 2, port, names, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0][1] + res[1][1] == 4 and res[0][1] > 0 and res[1][1] > 0
    for _rank, _n, gathered in res:
        assert sorted(gathered) == sorted(names)
        for name in names:
            assert gathered[name] == (golden[name]["orient_sha256"], golden[name]["steps"]), name
