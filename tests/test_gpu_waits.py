"""Failure detection on the GPU without a fault: the grid barrier of the step
kernels bounds every wait and reports through an error word.

A barrier that expects one more arrival than the launch has blocks never
completes; with a 50 ms limit every block's wait runs out, the error word
reads 1 (barrier wait timed out), every block's barrier returns failure, and
the context stays usable (a complete barrier and a plain realm run after it).
An error word set before a barrier that does complete is reported by every
block (thread 0 samples the word as it arrives).
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
KERR_BARRIER = 1


@pytest.fixture(scope="module")
def amca():
    import amca3d_gb300

    amca3d_gb300.load_library()
    return amca3d_gb300


@pytest.mark.parametrize("blocks", [1, 4, 16])
def test_barrier_with_a_missing_arrival_times_out_and_reports(amca, blocks):
    err, verdicts = amca.selftest_barrier(blocks, blocks + 1, wait_ns=50_000_000)
    assert err == KERR_BARRIER
    assert verdicts.tolist() == [0] * blocks


def test_barrier_completes_and_reports_an_error_raised_before_it(amca):
    err, verdicts = amca.selftest_barrier(8, 8, wait_ns=50_000_000)
    assert err == 0 and verdicts.tolist() == [1] * 8
    err, verdicts = amca.selftest_barrier(8, 8, wait_ns=50_000_000, preset_error=7)
    assert err == 7 and verdicts.tolist() == [0] * 8


def test_context_usable_after_a_timed_out_barrier(amca):
    err, _ = amca.selftest_barrier(4, 5, wait_ns=10_000_000)
    assert err == KERR_BARRIER
    golden = json.load(open(os.path.join(GOLD, "plain_golden.json")))
    c = cases.small_cases()[0]
    r = amca.CellularAutomataRealm(c.to_yaml(), seed=c.seed)
    try:
        r.initialize()
        r.run()
        o = np.ascontiguousarray(r.field("orientation_id"), dtype="<i4")
        assert hashlib.sha256(o.tobytes()).hexdigest() == golden[c.name]["orient_sha256"]
    finally:
        r.close()


def test_selftest_rejects_bad_arguments(amca):
    with pytest.raises(amca.AmcaError, match="bad argument"):
        amca.selftest_barrier(0, 1, wait_ns=1_000_000)
    with pytest.raises(amca.AmcaError, match="bad argument"):
        amca.selftest_barrier(4, 5, wait_ns=10_000_000_000)

