"""Batched plain realms (amca_batch_*) against the unmodified reference.

A batch runs many independent realms in one cooperative launch, teams of
blocks taking realms from a queue. Every realm's fields must be bit-exact to
its own np=1 reference run, whatever the team size and queue order:
  * the small golden decks of cases.py (digests in plain_golden.json), as
    one batch, at several team sizes, and again after the autotuner;
  * the 64 instances of the batched workload at full size (edges 32..128),
    against batched_64_golden.json made by make_golden.py --batched.
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, GOLD)
import cases  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(GOLD, "plain_golden.json")))


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def amca():
    import amca3d_gb300

    amca3d_gb300.load_library()
    return amca3d_gb300


def open_realms(amca, decks_):
    realms = []
    for c in decks_:
        r = amca.CellularAutomataRealm(c.to_yaml(), seed=c.seed)
        r.initialize()
        realms.append(r)
    return realms


def check_golden(realms, decks_, golden):
    bad = []
    for r, c in zip(realms, decks_):
        g = golden[c.name]
        st = r.stats()
        if st["step"] != g["steps"] or sha(r.field("orientation_id")) != g["orient_sha256"] \
                or sha(r.field("grain_id")) != g["grain_sha256"]:
            bad.append(c.name)
    return bad


@pytest.fixture(scope="module")
def small_batch(amca):
    decks_ = cases.small_cases()
    realms = open_realms(amca, decks_)
    yield decks_, realms
    for r in realms:
        r.close()


@pytest.mark.parametrize("team", [1, 3, 8, 32])
def test_batch_of_small_decks_matches_reference(amca, small_batch, team):
    decks_, realms = small_batch
    with amca.Batch(realms, team_size=team) as b:
        b.run()
        assert check_golden(realms, decks_, GOLDEN) == []
        st = b.stats()
        assert st["team_size"] == team and st["realms"] == len(realms) and st["runs"] == 1
        assert st["cell_updates"] == sum(r.stats()["step"] * c.n_interior for r, c in zip(realms, decks_))
        # a second run starts again from the initial state
        b.run()
        assert check_golden(realms, decks_, GOLDEN) == []


def test_batch_reads_like_single_runs(amca, small_batch):
    """After a batch run each handle's stats and fields are those of
    amca_reset + amca_run on that handle alone."""
    decks_, realms = small_batch
    with amca.Batch(realms, team_size=4) as b:
        b.run()
        got = [(r.stats(), r.field("orientation_id"), r.field("site_undercooling")) for r in realms]
    keys = ("step", "time", "dt", "liquid_cells", "grains", "orientations", "done", "captures", "nucleations")
    for r, (st, o, s) in zip(realms, got):
        r.reset()
        r.run()
        ref = r.stats()
        assert {k: st[k] for k in keys} == {k: ref[k] for k in keys}
        assert np.array_equal(o, r.field("orientation_id"))
        assert np.array_equal(s, r.field("site_undercooling"))


@pytest.mark.parametrize("layout", [((1, 4, 16), (5, 3, 2)), ((2, 64), (4, 1)), ((3,), (1,))])
def test_batch_mixed_layouts_match_reference(amca, small_batch, layout):
    """Teams of several sizes in one launch (realm r in class r mod k), and a
    single team that runs every realm in turn."""
    decks_, realms = small_batch
    sizes, teams = layout
    with amca.Batch(realms) as b:
        b.set_layout(sizes, teams, [r % len(sizes) for r in range(len(realms))])
        st = b.stats()
        assert st["grid_blocks"] == sum(s * t for s, t in zip(sizes, teams)) and st["n_classes"] == len(sizes)
        b.run()
        assert check_golden(realms, decks_, GOLDEN) == []


def test_batch_autotune_keeps_results(amca, small_batch):
    decks_, realms = small_batch
    with amca.Batch(realms) as b:
        t = b.tune(repeats=1)
        st = b.stats()
        assert t == st["team_size"] and len(st["tuned"]) >= 5 and (t == 0 or t in st["tuned"])
        assert st["mixed_ms"] > 0 or t != 0
        assert st["graph"] == 1, "the batched run is not replayed as a CUDA graph"
        b.run()
        assert check_golden(realms, decks_, GOLDEN) == []
        ts, tn, rc, qo = b.layout()
        assert sorted(qo) == list(range(len(realms))) and int((ts * tn).sum()) == b.stats()["grid_blocks"]
    # the tuned layout set on another batch of the same realms
    with amca.Batch(realms) as b2:
        b2.set_layout(ts, tn, rc, qo)
        assert [list(x) for x in b2.layout()] == [list(x) for x in (ts, tn, rc, qo)]
        b2.run()
        assert check_golden(realms, decks_, GOLDEN) == []


def test_batch_rejects_bad_handles(amca, small_batch):
    decks_, realms = small_batch
    with pytest.raises(amca.AmcaError, match="appears twice"):
        amca.Batch([realms[0], realms[1], realms[0]])
    with pytest.raises(amca.AmcaError, match="team size"):
        amca.Batch(realms[:2], team_size=100000)
    with amca.Batch(realms[:2]) as b:
        with pytest.raises(amca.AmcaError, match="more blocks"):
            b.set_layout([64], [100], [0, 0])
        with pytest.raises(amca.AmcaError, match="out of range"):
            b.set_layout([4], [2], [0, 1])
        with pytest.raises(amca.AmcaError, match="permutation"):
            b.set_layout([4], [2], [0, 0], [1, 1])


def test_batched_64_full_size_matches_reference(amca):
    """The batched workload as measured: 64 instances, edges 32..128 (about
    44M cells), one tuned, graph-replayed launch; every instance bit-exact to
    its own reference run."""
    from amca3d_gb300 import decks

    golden = json.load(open(os.path.join(GOLD, "batched_64_golden.json")))
    decks_ = decks.config_batched_64()
    realms = open_realms(amca, decks_)
    try:
        with amca.Batch(realms) as b:
            b.tune(repeats=1)
            b.run()
            assert check_golden(realms, decks_, golden) == []
            # a mixed layout: the 8 largest realms on teams of 32, the rest on 2
            big = set(np.argsort([-c.n_interior for c in decks_])[:8])
            b.set_layout([32, 2], [8, 100], [0 if r in big else 1 for r in range(len(decks_))])
            b.run()
            assert check_golden(realms, decks_, golden) == []
    finally:
        for r in realms:
            r.close()
