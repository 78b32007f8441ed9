"""FE-coupled remelting realm on the GPU against the unmodified reference.

Every fixture of tests/golden/remelt_cases.py is stepped through the C ABI
and compared, after every CA step, with the reference's per-step state
(tests/golden/<name>.npz, made by make_remelt_golden.py): time and dt, and
64-bit digests of the orientation, grain, temperature, cooling, melted and
liquid-neighbour fields — bit for bit. The synthetic-frame generator on the
GPU and frames passed from memory must give the same run as the text file.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_remelt_golden as M  # noqa: E402
import remelt_cases  # noqa: E402

pytestmark = pytest.mark.gpu

FIX = {fx.case.name: fx for fx in remelt_cases.fixtures()}
STATE = ("orient", "grain", "T", "cooling", "melted", "flag")
FIELD_OF = {"orient": "orientation_id", "grain": "grain_id", "T": "temperature", "cooling": "cooling",
            "melted": "melted", "flag": "liquid_neighbour"}


@pytest.fixture(scope="module")
def amca():
    import amca3d_gb300 as A

    A.load_library()
    return A


def make_realm(A, fx, wd, frames="file"):
    M.prepare(fx, wd)
    r = A.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=wd)
    fs = fx.frames
    if frames == "rosenthal":
        r.set_rosenthal_frames(**fs.rosenthal_kwargs())
    elif frames == "arrays":
        x, y, z = fs.node_coords()
        coords = np.stack([x, y, z], axis=1)
        times = np.array([fs.time_offset + f * fs.frame_dt for f in range(fs.frames)])
        theta = np.stack([fs.frame_values(f) for f in range(fs.frames)])
        r.set_fe_frames(fs.nodes, coords, times, theta)
    r.initialize()
    return r


def digests(r) -> dict:
    return {k: M.d64(r.field(FIELD_OF[k])) for k in STATE}


@pytest.mark.parametrize("name", sorted(FIX))
def test_remelt_gpu_matches_reference_every_step(amca, tmp_path, name):
    fx = FIX[name]
    r = make_realm(amca, fx, str(tmp_path))
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    fields = [str(f) for f in g["fields"]]
    n = len(g["digests"])
    for i in range(n):
        dt = r.single_integration_step()
        st = r.stats()
        assert st["step"] == i + 1
        assert st["time"] == g["time"][i] and dt == g["dt"][i], f"step {i + 1}: time/dt"
        d = digests(r)
        bad = [k for k in STATE if d[k] != g["digests"][i][fields.index(k)]]
        assert not bad, f"step {i + 1}: {bad}"
        assert st["grains"] == g["ngrains"][i] and st["orientations"] == g["norient"][i]
    r.single_integration_step()  # the reference stopped at the end of its frames
    assert r.stats()["step"] == n and r.stats()["done"] == 1
    r.close()


@pytest.mark.parametrize("name", ["remelt_random", "remelt_scaled", "remelt_new_grains"])
def test_remelt_gpu_host_velocities_in_chunks(amca, tmp_path, monkeypatch, name):
    """The hard glibc-pow velocities of a step normally go to the host in one
    request that overlaps the growth of the other cells. With room for 3
    entries a step with 3 or more of them sends them in chunks of 3, one
    request each, before the growth: the run still matches the reference
    step by step, with more host requests than the normal run."""
    fx = FIX[name]
    for sub in ("a", "b"):
        (tmp_path / sub).mkdir()
    r = make_realm(amca, fx, str(tmp_path / "a"))
    r.run()
    calls = r.stats()["reserved"]
    r.close()
    monkeypatch.setenv("AMCA_HOST_VEL_CAP", "3")
    r = make_realm(amca, fx, str(tmp_path / "b"))
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    fields = [str(f) for f in g["fields"]]
    for i in range(len(g["digests"])):
        dt = r.single_integration_step()
        assert r.stats()["time"] == g["time"][i] and dt == g["dt"][i], f"step {i + 1}: time/dt"
        d = digests(r)
        assert not [k for k in STATE if d[k] != g["digests"][i][fields.index(k)]], f"step {i + 1}"
    assert r.stats()["reserved"] > calls > 0
    r.close()


@pytest.mark.parametrize("frames", ["file", "rosenthal", "arrays"])
@pytest.mark.parametrize("name", ["remelt_nucleation", "remelt_scaled", "remelt_new_grains"])
def test_remelt_gpu_full_run(amca, tmp_path, name, frames):
    fx = FIX[name]
    r = make_realm(amca, fx, str(tmp_path), frames)
    r.run()
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    st = r.stats()
    assert st["step"] == len(g["digests"]) and st["time"] == g["time"][-1]
    for k in ("orient", "grain", "melted", "cooling", "flag"):
        assert np.array_equal(r.field(FIELD_OF[k]).astype(g[k].dtype), g[k]), k
    # reset replays the same run
    r.reset()
    r.run()
    assert np.array_equal(r.field("orientation_id"), g["orient"])
    r.close()


def test_remelt_gpu_bad_frame_stops_like_the_reference(amca, tmp_path):
    fx = FIX["remelt_random"]
    r = make_realm(amca, fx, str(tmp_path))
    r.close()
    path = tmp_path / "frames.txt"
    text = path.read_text().split("\n")
    fourth = [i for i, line in enumerate(text) if line == "Subtitle"][3]
    text[fourth - 1] = "not blank"
    path.write_text("\n".join(text))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    r.initialize()
    with pytest.raises(amca.AmcaError, match="check title of line"):
        r.run()
    r.close()


@pytest.mark.parametrize("name", ["remelt_columnar", "remelt_new_grains"])
def test_remelt_gpu_microstructure_from_memory(amca, tmp_path, name):
    """amca_set_microstructure with the restart file's content gives the
    file's run."""
    from amca3d_gb300 import decks

    fx = FIX[name]
    M.prepare(fx, str(tmp_path))
    m = decks.columnar_microstructure(fx.case.cells, fx.case.cell_size, fx.case.origin, fx.columnar_grains,
                                      fx.columnar_seed, fx.grainless_mod)
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    r.set_microstructure(m["grain"], m["orient"], m["euler"], m["grain_cell"], m["grain_orient"],
                         expected=m["expected"])
    r.set_rosenthal_frames(**fx.frames.rosenthal_kwargs())
    r.initialize()
    r.run()
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    for k in ("orient", "grain", "melted"):
        assert np.array_equal(r.field(FIELD_OF[k]).astype(g[k].dtype), g[k]), k
    r.close()


def test_remelt_gpu_output_files_match_reference(amca, tmp_path):
    """VTR snapshots (temperature, grain id, orientation, melted flag), PVTR/PVD,
    the restart file, finalGrains.vtk and finalResult.txt: byte for byte the
    reference's (SHA-256 of each file)."""
    import json

    fx = remelt_cases.output_fixture()
    M.prepare(fx, str(tmp_path))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path), write_outputs=True)
    r.initialize()
    r.run()
    r.write_outputs()
    golden = json.load(open(os.path.join(HERE, "golden", "remelt_outputs.json")))
    assert r.stats()["step"] == golden["steps"]
    r.close()
    got = M.output_digests(str(tmp_path))
    assert sorted(got) == sorted(golden["files"])
    bad = [f for f in golden["files"] if got[f] != golden["files"][f]]
    assert not bad, bad


def test_remelt_gpu_appended_vtr_equals_ascii(amca, tmp_path):
    """Binary VTR pieces of the coupled realm carry the values of its ASCII
    pieces (which equal the reference's byte for byte): grain ids, melted
    flags and the int-rounded temperatures exactly, Euler angles to the
    text's six digits."""
    import dataclasses

    from amca3d_gb300.vtr import read_vtr

    fx = remelt_cases.output_fixture()
    got = {}
    for fmt in ("ascii", "appended"):
        wd = tmp_path / fmt
        wd.mkdir()
        fx2 = dataclasses.replace(fx, case=dataclasses.replace(fx.case, output_format=fmt))
        M.prepare(fx2, str(wd))
        r = amca.CellularAutomataRealm(fx2.case.to_yaml(), seed=fx.case.seed, workdir=str(wd), write_outputs=True)
        r.initialize()
        r.run()
        r.write_outputs()
        r.close()
        got[fmt] = {os.path.relpath(os.path.join(d, f), str(wd)): read_vtr(os.path.join(d, f))
                    for d, _, fs in os.walk(str(wd)) for f in fs if f.endswith(".vtr")}
    assert sorted(got["ascii"]) == sorted(got["appended"]) and len(got["ascii"]) >= 1
    for rel, a in got["ascii"].items():
        b = got["appended"][rel]
        assert list(a) == list(b) and "cell_temperature" in b and "melted_flag" in b
        for k in ("grain_id", "melted_flag", "cell_temperature"):
            assert np.array_equal(a[k], b[k]), (rel, k)
        assert np.allclose(a["grain_orientation"], b["grain_orientation"], rtol=5e-6, atol=1e-12), rel


def test_cli_runs_the_deck_like_the_reference(amca, tmp_path):
    """amca3d -i Inputfile.i -o run.log in the deck's directory writes the
    reference's output files."""
    import json
    import subprocess

    fx = remelt_cases.output_fixture()
    M.prepare(fx, str(tmp_path))
    cli = os.path.join(os.path.dirname(HERE), "amca3d_gb300", "amca3d")
    r = subprocess.run([cli, "-i", "Inputfile.i", "-o", "cli.log", "--seed", str(fx.case.seed)], cwd=str(tmp_path),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    golden = json.load(open(os.path.join(HERE, "golden", "remelt_outputs.json")))
    got = M.output_digests(str(tmp_path))
    got.pop("cli.log", None)
    assert got == golden["files"]
    assert f"Time Step Count: {golden['steps']}" in (tmp_path / "cli.log").read_text()


def scan_kwargs_of(fs):
    """amca_scan fields of a one-track FrameSpec (the Rosenthal frames' source)."""
    r = fs.rosenthal_kwargs()
    assert not r.pop("void_above_set")
    for k in ("void_above", "t_void"):
        r.pop(k)
    r.update(x_turn=0.0, hatch=0.0, track_time=0.0, ntracks=1)
    return r


@pytest.mark.parametrize("window", ["2", "5"])
@pytest.mark.parametrize("name", ["remelt_nucleation", "remelt_new_grains"])
def test_remelt_gpu_frames_streamed_through_a_ring(amca, tmp_path, monkeypatch, name, window):
    """Frames produced on the GPU a few at a time into a ring of window + 4
    slots (the kernel stops when it needs a frame not yet produced) give the
    reference's run bit for bit, after a reset too."""
    monkeypatch.setenv("AMCA_FRAME_WINDOW", window)
    fx = FIX[name]
    M.prepare(fx, str(tmp_path))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    r.set_scan_frames(**scan_kwargs_of(fx.frames))
    r.initialize()
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    fields = [str(f) for f in g["fields"]]
    for i in range(40):  # step by step through the first refills
        dt = r.single_integration_step()
        assert r.stats()["time"] == g["time"][i] and dt == g["dt"][i], f"step {i + 1}"
        d = digests(r)
        assert all(d[k] == g["digests"][i][fields.index(k)] for k in STATE), f"step {i + 1}"
    r.run()
    st = r.stats()
    assert st["step"] == len(g["digests"]) and st["time"] == g["time"][-1]
    for k in ("orient", "grain", "melted", "cooling", "flag"):
        assert np.array_equal(r.field(FIELD_OF[k]).astype(g[k].dtype), g[k]), k
    fs = r.frame_stats()
    assert fs["fills"] > 3 and fs["frames"] <= fx.frames.frames
    r.reset()
    r.run()
    assert np.array_equal(r.field("orientation_id"), g["orient"])
    r.close()


@pytest.mark.parametrize("name", sorted(FIX))
def test_remelt_gpu_text_frames_streamed(amca, tmp_path, monkeypatch, name):
    """Text frames read a window at a time while the run goes on (the
    reader of load_next_step_nodal_data, 3 frames per window) give the
    reference's run at every step, and again after a reset (the file is read
    again from its start)."""
    monkeypatch.setenv("AMCA_FRAME_STREAM", "1")
    monkeypatch.setenv("AMCA_FRAME_WINDOW", "3")
    fx = FIX[name]
    r = make_realm(amca, fx, str(tmp_path))
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    fields = [str(f) for f in g["fields"]]
    n = len(g["digests"])
    for i in range(n):
        dt = r.single_integration_step()
        st = r.stats()
        assert st["time"] == g["time"][i] and dt == g["dt"][i], f"step {i + 1}: time/dt"
        d = digests(r)
        bad = [k for k in STATE if d[k] != g["digests"][i][fields.index(k)]]
        assert not bad, f"step {i + 1}: {bad}"
    r.single_integration_step()  # the reference stopped at the end of its frames
    assert r.stats()["step"] == n and r.stats()["done"] == 1
    fs = r.frame_stats()
    assert fs["fills"] > 3
    r.reset()
    r.run()
    assert np.array_equal(r.field("orientation_id"), g["orient"])
    r.close()


def test_remelt_gpu_streamed_bad_frame_stops_like_the_reference(amca, tmp_path, monkeypatch):
    monkeypatch.setenv("AMCA_FRAME_STREAM", "1")
    monkeypatch.setenv("AMCA_FRAME_WINDOW", "2")
    fx = FIX["remelt_random"]
    r = make_realm(amca, fx, str(tmp_path))
    r.close()
    path = tmp_path / "frames.txt"
    text = path.read_text().split("\n")
    fourth = [i for i, line in enumerate(text) if line == "Subtitle"][3]
    text[fourth - 1] = "not blank"
    path.write_text("\n".join(text))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    r.initialize()
    with pytest.raises(amca.AmcaError, match="check title of line"):
        r.run()
    r.close()


def test_remelt_gpu_pbf_500_full_size(amca):
    """pbf_500, the benchmarked FE-coupled workload (500 x 250 x 100 cells,
    1,550 Rosenthal frames, 2,000-grain baseplate), at full size against the
    unmodified reference's run of the same deck (tests/golden/make_pbf_golden.py):
    the step count, time and dt, the orientation / grain-id / melted field
    digests, grain and orientation counts and the Euler angles at every
    checkpoint the reference recorded and at the end."""
    import hashlib
    import json

    from amca3d_gb300 import decks

    path = os.path.join(HERE, "golden", "pbf_500_golden.json")
    if not os.path.exists(path):
        pytest.skip("no reference run recorded for pbf_500")
    golden = json.load(open(path))
    ref = golden.get("reference") or golden.get("oracle")
    case, frames, m = decks.config_pbf_500()
    r = amca.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    r.set_microstructure(m["grain"], m["orient"], m["euler"], m["grain_cell"], m["grain_orient"],
                         expected=m["expected"])
    r.set_rosenthal_frames(**frames.rosenthal_kwargs())
    r.initialize()

    def sha(a, dt):
        return hashlib.sha256(np.ascontiguousarray(a, dt).tobytes()).hexdigest()

    def check(rec, where):
        st = r.stats()
        assert st["step"] == rec["step"], where
        assert st["time"] == float.fromhex(rec["time"]) and st["dt"] == float.fromhex(rec["dt"]), where
        assert sha(r.field("orientation_id"), "<i4") == rec["orient"], where
        assert sha(r.field("grain_id"), "<i4") == rec["grain"], where
        assert sha(r.field("melted"), "u1") == rec["melted"], where
        assert st["grains"] == rec["ngrains"] and st["orientations"] == rec["norient"], where
        if "euler" in rec:
            assert sha(r.orientations(), "<f8") == rec["euler"], where

    for cp in sorted(ref.get("checkpoints", []), key=lambda c: c["step"]):
        r.run(cp["step"] - r.stats()["step"])
        check(cp, f"step {cp['step']}")
    r.run()
    assert r.stats()["done"] == 1
    check(ref["final"], "end of the frames")
    r.close()
