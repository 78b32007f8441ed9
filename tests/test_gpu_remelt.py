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


def rosenthal_kwargs(fs: remelt_cases.FrameSpec) -> dict:
    s = fs.source
    return dict(origin=fs.origin, spacing=fs.spacing, nodes=fs.nodes, frames=fs.frames, length_scale=fs.length_scale,
                frame_dt=fs.frame_dt, time_scale=fs.time_scale, time_offset=fs.time_offset, power=s.power,
                absorptivity=s.absorptivity, speed=s.speed, conductivity=s.conductivity, diffusivity=s.diffusivity,
                t0=s.t0, t_cap=s.t_cap, x_start=s.x_start, y_line=s.y_line, z_top=s.z_top,
                void_above_set=0 if s.void_above is None else 1,
                void_above=0.0 if s.void_above is None else s.void_above, t_void=s.t_void)


def make_realm(A, fx, wd, frames="file"):
    M.prepare(fx, wd)
    r = A.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=wd)
    fs = fx.frames
    if frames == "rosenthal":
        r.set_rosenthal_frames(**rosenthal_kwargs(fs))
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
