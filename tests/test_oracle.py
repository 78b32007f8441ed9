"""The C oracle against the reference's golden vectors (CPU only).

tests/golden/*.npz and plain_golden.json come from the unmodified reference
(make_golden.py); kat_*.json/npz from the reference's own Octahedron class
and the glibc / libstdc++ streams it draws from (make_kats.py).
"""
import ctypes
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

import sys  # noqa: E402

sys.path.insert(0, GOLD)
import cases  # noqa: E402


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


GOLDEN = json.load(open(os.path.join(GOLD, "plain_golden.json")))


@pytest.mark.parametrize("case", cases.small_cases(), ids=lambda c: c.name)
def test_oracle_matches_reference_run(oracle, case):
    g = GOLDEN[case.name]
    r = oracle.run_plain(case)
    assert r["steps"] == g["steps"]
    assert sha(r["orient"]) == g["orient_sha256"]
    assert sha(r["grain"]) == g["grain_sha256"]
    npz = np.load(os.path.join(GOLD, f"{case.name}.npz"))
    assert np.array_equal(r["orient"], npz["orient"])
    if "grain" in npz:
        assert np.array_equal(r["grain"], npz["grain"])
    # consumed sites print as 0, live sites as their dTc (reference prints 6 digits; stored as float32)
    assert np.allclose(r["site_dtc"].astype(np.float32), npz["site_dtc"], rtol=1e-5, atol=1e-6)


def test_oracle_partial_run_is_a_prefix(oracle):
    """Stopping at termination_time 0.5 equals the golden mid-run state."""
    c = [c for c in cases.small_cases() if c.name == "nucleation_60_t0.5"][0]
    r = oracle.run_plain(c)
    assert r["liquid_cells"] > 0 and r["steps"] == GOLDEN[c.name]["steps"]


def test_glibc_rand_stream_kat():
    kat = json.load(open(os.path.join(GOLD, "kat_streams.json")))
    libc = ctypes.CDLL(None)
    for seed, vals in kat["rand"].items():
        libc.srand(int(seed))
        assert [libc.rand() for _ in vals] == vals


def test_normal_distribution_kat(oracle):
    kat = json.load(open(os.path.join(GOLD, "kat_streams.json")))
    for row in kat["normal"]:
        mean, sd = float.fromhex(row["mean"]), float.fromhex(row["sd"])
        want = [float.fromhex(x) for x in row["draws"]]
        got = oracle.normal_draws(mean, sd, len(want))
        assert got.tolist() == want


def test_octahedron_kat(oracle):
    k = np.load(os.path.join(GOLD, "kat_octahedron.npz"))
    inp, l2g, cap, info, trunc = k["inputs"], k["l2g"], k["captured"], k["info"], k["trunc"]
    assert 0.2 < cap.mean() < 0.9
    for i in range(len(inp)):
        e, g, cc, L, h = inp[i, 0:3], inp[i, 3:6], inp[i, 6:9], inp[i, 9], inp[i, 10]
        m = oracle.rotation(e)
        assert m.tobytes() == l2g[i].tobytes()
        gc = cc - g
        c = oracle.is_captured(m, gc, L)
        assert int(c) == int(cap[i])
        if c:
            out = oracle.capture(m, gc, L, h, trunc[i])
            assert out.tobytes() == info[i].tobytes(), i
