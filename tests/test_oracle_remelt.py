"""The remelting oracle against the unmodified reference (CPU only).

Every FE-coupled fixture in tests/golden/remelt_cases.py was run through the
reference with a per-step state probe (tests/golden/make_remelt_golden.py);
the oracle must reproduce, at every CA step, the orientation, grain,
temperature, cooling, melted and liquid-neighbour fields, the grain table,
the Euler angles, time, dt and the CA's maximum time step bit for bit, and
the voxel tags / parametric coordinates of the FE-to-CA map.
"""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_remelt_golden as M  # noqa: E402
import remelt_cases  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "remelt_golden.json")))
FIXTURES = {fx.case.name: fx for fx in remelt_cases.fixtures()}


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_remelt_oracle_matches_reference_every_step(oracle, tmp_path, name):
    fx = FIXTURES[name]
    M.prepare(fx, str(tmp_path))
    dump = str(tmp_path / "oracle.bin")
    res = oracle.run_remelt(fx.case, str(tmp_path), dump=dump, fields=False)
    tags, pc, steps = M.read_dump(dump)
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    assert M.sha(tags) == GOLDEN[name]["tags"]
    assert M.sha(pc) == GOLDEN[name]["parcoords"]
    assert len(steps) == len(g["digests"]) == res["steps"]
    fields = [str(f) for f in g["fields"]]
    for i, d in enumerate(steps):
        assert d["time"] == g["time"][i] and d["dt"] == g["dt"][i] and d["maxdt"] == g["maxdt"][i], i
        dg = M.step_digests(d)
        bad = [f for f, a, b in zip(fields, dg, g["digests"][i]) if a != b]
        assert not bad, f"step {i + 1}: {bad}"
    last = steps[-1]
    for k in ("orient", "grain", "melted", "cooling", "flag"):
        assert np.array_equal(last[k], g[k]), k
    assert last["ngrains"] == GOLDEN[name]["final"]["ngrains"]
    assert last["norient"] == GOLDEN[name]["final"]["norient"]


def test_is_in_element_axis_aligned_box(oracle):
    """Newton-Raphson on a box: the parametric coordinates are the affine map."""
    lo = np.array([1.0e-5, -2.0e-5, 3.0e-5])
    d = np.array([1.0e-5, 2.0e-5, 0.5e-5])
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    nodes = np.array([lo + d * np.array(c) for c in corners]).reshape(24)
    rng = np.random.default_rng(0)
    for _ in range(50):
        u = rng.random(3)
        ok, para = oracle.is_in_element(nodes, lo + d * u)
        assert ok
        np.testing.assert_allclose(para, 2 * u - 1, atol=1e-9)
    ok, _ = oracle.is_in_element(nodes, lo + d * np.array([1.5, 0.5, 0.5]))
    assert not ok


def test_remelt_oracle_rejects_bad_frame_file(oracle, tmp_path):
    fx = FIXTURES["remelt_random"]
    M.prepare(fx, str(tmp_path))
    path = tmp_path / "frames.txt"
    text = path.read_text().split("\n")
    # the first subtitle line of every frame after the first must be blank
    fourth = [i for i, line in enumerate(text) if line == "Subtitle"][3]
    text[fourth - 1] = "not blank"
    path.write_text("\n".join(text))
    with pytest.raises(RuntimeError, match="check title of line"):
        oracle.run_remelt(fx.case, str(tmp_path), fields=False)


def test_pbf_500_oracle_equals_reference_at_full_size():
    """The full-size pbf_500 record (tests/golden/make_pbf_golden.py): the
    unmodified reference's run and the C restatement's run of the same deck,
    frames and baseplate end at the same step, time and dt with the same
    orientation / grain-id / melted field digests and counts, and the
    reference's record carries its checkpoints."""
    g = json.load(open(os.path.join(HERE, "golden", "pbf_500_golden.json")))
    assert g["cells"] == [500, 250, 100] and g["frames"] == 1550
    ref, ora = g["reference"], g["oracle"]
    assert "unmodified reference" in ref["source"]
    # the restatement's record has no grain-table or Euler digest
    assert set(ora["final"]) >= {"step", "time", "dt", "orient", "grain", "melted", "ngrains", "norient"}
    assert all(ref["final"][k] == v for k, v in ora["final"].items())
    assert ref["final"]["step"] == 7659 and ref["final"]["norient"] == 2036
    steps = [c["step"] for c in ref["checkpoints"]]
    assert steps == sorted(steps) and steps[-1] < ref["final"]["step"] and len(steps) >= 5
