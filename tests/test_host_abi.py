"""Host logic of the library and its C ABI, without a GPU.

Checks that libamca3d.so loads and exports every entry point declared in
include/amca3d.h, that decks parse as the reference reads them (keys,
defaults, yaml-cpp 0.3 number rules, errors), and that the host half of
initialize (sites, orientation stream) equals the oracle's.
"""
import dataclasses
import os
import re
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import cases  # noqa: E402


@pytest.fixture(scope="session")
def amca():
    import amca3d_gb300

    if not os.path.exists(amca3d_gb300.LIB_PATH):
        from amca3d_gb300 import build

        build.build()
    amca3d_gb300.load_library()
    return amca3d_gb300


def declared_functions():
    text = open(os.path.join(ROOT, "include", "amca3d.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(amca_[a-z_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(amca):
    lib = amca.load_library()
    names = declared_functions()
    assert len(names) >= 14
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(amca.EXPORTS) == names


def test_release_cached_memory_without_a_cached_arena(amca):
    """Nothing is kept before a realm was destroyed: releasing is a no-op."""
    amca.release_cached_memory(-1)
    amca.release_cached_memory(0)


@pytest.mark.parametrize("case", cases.small_cases() + cases.large_cases(), ids=lambda c: c.name)
def test_deck_grid(amca, case):
    r = amca.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    assert r.cells == tuple(case.cells)
    assert r.origin == tuple(case.origin)
    assert r.cell_size == case.cell_size
    r.close()


def test_reference_example_deck_parses(amca):
    deck = """
simulations:
  - name: test
    time_integrator: ti_1
solvers:
   - cellular_automata
realms:
  - name: realm1
    type: cellular_automata
    dimension: 3
    domain:
      type: cubic
      original_point: [0,0,0]
      lateral_sizes: [0.03, 0.03, 0.03]
    discretization:
      cell_size: 0.0005
      number_cells: [800, 720, 252]
    nucleation_rules:
      - surface:
          type: Gaussian
          site_density: 0.0
          mean: 2
          standard_deviation: 0.5
      - bulk:
          type: Gaussian
          site_density: 10e6     # yaml-cpp 0.3 reads this as 1e7
          mean: 3
          standard_deviation: 1
    problem_physics:
        type: RappazGandin
        initial_temperature: -0.2
        melting_temperature: 0.0
        t_dot: -20
        a1: -0.544e-4
        a2: 2.03e-4
        a3: 0.0
    solution_options:
       name: my_options
       options:
         - random_type:
             rejection_sampling: no
         - cell_grain_length_cutoff_factor:
             factor_value: 4.0
         - output_microstructure_information:
             file_name: grainInfo.txt
         - parallel_specification:
             direction_with_all_processes: y
    output:
      output_data_base_name: ./Results/Grains
      output_frequency: 100
      output_variables:
        - grain_ID
time_integrators:
  - standard_time_integrator:
      name: ti_1
      termination_time: 17.81
      termination_step_count: 10000
      time_step: 0.001
      realms:
        - realm1
"""
    r = amca.CellularAutomataRealm(deck)
    # lateral_sizes wins over number_cells: n = int(0.03 / 0.0005) = 60
    assert r.cells == (60, 60, 60)
    r.prepare()
    cells, dtc = r.sites()
    assert len(cells) == 269  # 270 draws at 1e7 m^-3, one duplicate


@pytest.mark.parametrize("bad,code", [
    ("solvers: [cellular_automata]\n", -2),                                  # no realms
    ("realms:\n  - type: cellular_automata\n", -2),                          # no solvers
    ("solvers: [cellular_automata]\nrealms: [\n", -2),                       # YAML syntax
])
def test_bad_decks_fail_with_parse_error(amca, bad, code):
    with pytest.raises(amca.AmcaError) as e:
        amca.CellularAutomataRealm(bad)
    assert e.value.code == code


def _strip_key(deck, key):
    return "\n".join(l for l in deck.splitlines() if not l.strip().startswith(key + ":"))


@pytest.mark.parametrize("key", ["cell_size", "original_point", "termination_time", "time_step", "site_density"])
def test_missing_required_key_is_named(amca, key):
    deck = _strip_key(cases.small_cases()[2].to_yaml(), key)
    with pytest.raises(amca.AmcaError) as e:
        amca.CellularAutomataRealm(deck)
    assert e.value.code == -2 and key in str(e.value)


def test_output_format_key(amca):
    """output_format (a key of this library) accepts ascii / appended and
    names itself on anything else; decks without it read as before."""
    base = dataclasses.replace(cases.small_cases()[2], output_frequency=5)
    for fmt in ("ascii", "appended"):
        amca.CellularAutomataRealm(dataclasses.replace(base, output_format=fmt).to_yaml()).close()
    with pytest.raises(amca.AmcaError) as e:
        amca.CellularAutomataRealm(dataclasses.replace(base, output_format="hdf5").to_yaml())
    assert e.value.code == -2 and "output_format" in str(e.value)


def test_vtr_reader_on_reference_ascii_pieces(tmp_path):
    """amca3d_gb300.vtr.read_vtr reads the reference's ASCII pieces and an
    appended piece built here byte by byte."""
    from amca3d_gb300.vtr import read_vtr

    c = cases.output_case()
    n = c.cells[0] * c.cells[1] * c.cells[2]
    d = os.path.join(ROOT, "tests", "golden", "outputs_tiny", "Results", "grainsTimeStates", "timeStep_00007",
                     "Grains00000.vtr")
    a = read_vtr(d)
    assert list(a) == ["grain_id", "grain_orientation", "X_Coordinates", "Y_Coordinates", "Z_Coordinates"]
    assert a["grain_id"].shape == (n,) and a["grain_orientation"].shape == (n, 3)
    assert np.allclose(a["X_Coordinates"], c.origin[0] + np.arange(c.cells[0] + 1) * c.cell_size, rtol=1e-5)
    ids = np.array([3, -1, 7], np.int64)
    xs = np.array([0.0, 0.5], np.float64)
    head = ('<?xml version="1.0"?>\n<VTKFile type="RectilinearGrid" version="0.1" byte_order="LittleEndian" '
            'header_type="UInt64">\n<CellData>\n<DataArray type="Int64" Name="grain_id" format="appended" '
            'offset="0"/>\n</CellData>\n<Coordinates>\n<DataArray type="Float64" Name="X_Coordinates" '
            'format="appended" offset="32"/>\n</Coordinates>\n<AppendedData encoding="raw">\n   _')
    blob = np.uint64(24).tobytes() + ids.tobytes() + np.uint64(16).tobytes() + xs.tobytes()
    p = tmp_path / "piece.vtr"
    p.write_bytes(head.encode() + blob + b"\n</AppendedData>\n</VTKFile>\n")
    b = read_vtr(str(p))
    assert np.array_equal(b["grain_id"], ids) and np.array_equal(b["X_Coordinates"], xs)


def test_problem_physics_type_checked(amca):
    deck = cases.small_cases()[2].to_yaml().replace("type: RappazGandin", "type: Other")
    with pytest.raises(amca.AmcaError):
        amca.CellularAutomataRealm(deck)


@pytest.mark.parametrize("case", [c for c in cases.small_cases() if c.n_ghost < 60000], ids=lambda c: c.name)
def test_host_sites_and_orientations_equal_oracle(amca, oracle, case):
    r = amca.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    r.prepare()
    cells, dtc = r.sites()
    o = oracle.run_plain(case, max_steps=0)
    site_cells = np.nonzero(o["site_dtc"] >= 0)[0]
    assert np.array_equal(cells, site_cells)
    assert np.array_equal(dtc, o["site_dtc"][site_cells])
    full = oracle.run_plain(case, euler_cap=max(1, len(cells)))
    e = r.orientations(all=True)
    assert e.shape == (len(cells), 3)
    n = full["num_orient"]
    assert np.array_equal(e[:n], full["euler"])
    r.close()


def test_gpu_calls_fail_loudly_without_initialize(amca):
    r = amca.CellularAutomataRealm(cases.small_cases()[2].to_yaml())
    with pytest.raises(amca.AmcaError) as e:
        r.run(1)
    assert e.value.code == -4
    r.close()


def test_batch_checks_handles_before_touching_the_gpu(amca):
    """amca_batch_create: uninitialized realms are a state error, remelting
    realms and empty lists an argument error; no GPU call is made."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import remelt_cases

    r = amca.CellularAutomataRealm(cases.small_cases()[2].to_yaml())
    with pytest.raises(amca.AmcaError) as e:
        amca.Batch([r])
    assert e.value.code == -4 and "not initialized" in str(e.value)
    rm = amca.CellularAutomataRealm(remelt_cases.fixtures()[0].case.to_yaml())
    with pytest.raises(amca.AmcaError) as e:
        amca.Batch([rm])
    assert e.value.code == -1 and "plain realms" in str(e.value)
    with pytest.raises(amca.AmcaError) as e:
        amca.Batch([])
    assert e.value.code == -1
    lib = amca.load_library()
    assert lib.amca_batch_run(None, None) == -1
    assert lib.amca_batch_get_stats(None, None) == -1
    assert lib.amca_batch_last_error(None)
    lib.amca_batch_destroy(None)
    r.close()
    rm.close()


# ---------------------------------------------------------------------------
# FE-coupled remelting decks (host half only)
# ---------------------------------------------------------------------------
def _remelt_fixtures():
    import remelt_cases

    return {fx.case.name: fx for fx in remelt_cases.fixtures()}


@pytest.mark.parametrize("name", sorted(_remelt_fixtures()))
def test_remelt_prepare_matches_reference_orientation_stream(amca, tmp_path, name):
    """Random / restart microstructure, sites and the nucleation orientation
    stream are drawn on the host exactly as the reference draws them: the
    Euler angles equal the reference's orientation list after the first and
    the last CA step."""
    import make_remelt_golden as M

    fx = _remelt_fixtures()[name]
    M.prepare(fx, str(tmp_path))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    assert r.cells == tuple(fx.case.cells)
    r.prepare()
    g = np.load(os.path.join(ROOT, "tests", "golden", f"{name}.npz"))
    ie = [str(f) for f in g["fields"]].index("euler")
    e = r.orientations(all=True)
    for i in (0, len(g["norient"]) - 1):
        n = int(g["norient"][i])
        assert M.d64(np.ascontiguousarray(e[:n]).reshape(-1)) == g["digests"][i][ie]
    cells, dtc = r.sites()
    assert (len(cells) > 0) == fx.case.nucleation
    assert np.all(np.diff(cells) > 0)
    r.close()


def test_remelt_deck_errors(amca):
    import remelt_cases

    deck = remelt_cases.fixtures()[0].case.to_yaml()
    with pytest.raises(amca.AmcaError, match="lines_for_title"):
        amca.CellularAutomataRealm(deck.replace("lines_for_title: 4", "lines_for_titl: 4"))
    with pytest.raises(amca.AmcaError, match="for_whole_time"):
        amca.CellularAutomataRealm(deck.replace("for_whole_time: yes", "for_whole_time: no"))
    with pytest.raises(amca.AmcaError, match="b1..b3"):
        amca.CellularAutomataRealm(deck.replace("a1: 0.0", "a1: 0.0\n        b2: 2.5"))
    with pytest.raises(amca.AmcaError, match="time_step_factor"):
        amca.CellularAutomataRealm(deck.replace("time_step_factor: 0.4", "time_step_facto: 0.4"))
    r = amca.CellularAutomataRealm(deck)
    with pytest.raises(amca.AmcaError, match="before amca_initialize|out of order"):
        r.field("temperature")
    r.close()


def test_remelt_frames_from_arrays_need_two_frames(amca):
    import remelt_cases

    fx = remelt_cases.fixtures()[0]
    r = amca.CellularAutomataRealm(fx.case.to_yaml())
    x, y, z = fx.frames.node_coords()
    coords = np.stack([x, y, z], axis=1)
    with pytest.raises(amca.AmcaError, match="two frames"):
        r.set_fe_frames(fx.frames.nodes, coords, np.zeros(1), fx.frames.frame_values(0)[None, :])
    with pytest.raises(amca.AmcaError, match="two frames"):
        r.set_rosenthal_frames(nodes=(3, 3, 3), frames=1, spacing=1.0)
    r.close()


def test_cli_help_and_missing_deck(amca, tmp_path):
    import subprocess

    cli = os.path.join(ROOT, "amca3d_gb300", "amca3d")
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    r = subprocess.run([cli, "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--input-deck" in r.stderr
    r = subprocess.run([cli, "-i", str(tmp_path / "none.i")], capture_output=True, text=True)
    assert r.returncode == 0 and "does not exist" in r.stderr
    (tmp_path / "bad.i").write_text("solvers: [nothing]\n")
    r = subprocess.run([cli, "-i", str(tmp_path / "bad.i")], capture_output=True, text=True)
    assert r.returncode == 1 and "parsing the deck" in r.stderr


def test_batched_workload_decks_match_their_golden_runs():
    """The 64 batched instances come from Python's Mersenne Twister random()
    (fixed across versions); their grids, cooling rates and site densities
    equal those the reference ran for batched_64_golden.json."""
    import json

    from amca3d_gb300 import decks

    golden = json.load(open(os.path.join(ROOT, "tests", "golden", "batched_64_golden.json")))
    b = decks.config_batched_64()
    assert len(b) == 64 and sorted(c.name for c in b) == sorted(golden)
    for c in b:
        g = golden[c.name]
        assert list(c.cells) == g["cells"] and c.t_dot == g["t_dot"] and c.bulk[0] == g["bulk_density"]
        assert 32 <= c.cells[0] <= 128 and -200.0 <= c.t_dot <= -5.0 and c.seed == 0
    assert 43e6 < sum(c.n_interior for c in b) < 45e6
