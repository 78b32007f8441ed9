"""The coupling calls of the boundary, through the C ABI:

* amca_set_nodal_temperatures + amca_step_coupled: a remelting deck driven
  step by step by a solver outside the realm. The driver here replays the
  deck's own frames the way the FE realm does (LoadDataFromFile.cpp:207-313:
  frame pair, time ratio, node interpolation with the void rule) and hands in
  each step's node temperatures with dT_FE as the dt bound; the run must
  equal the reference's at every step (time, dt, field digests).
* amca_run_until: stopping at a time and going on gives the same run.
* the plain realm's dt bound.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import cases  # noqa: E402
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


class FrameReplay:
    """The FE realm's frame replay, restated for the driver
    (FiniteElementManager::pseudo_single_integration_step,
    CA/src/LoadDataFromFile.cpp:207-313): times scaled like the reader's."""

    def __init__(self, fs, void_t=-1.0e8):
        self.theta = np.stack([fs.frame_values(f) for f in range(fs.frames)])
        t0 = fs.time_offset
        self.times = [((fs.time_offset + f * fs.frame_dt) - t0) * fs.time_scale for f in range(fs.frames)]
        self.times[0] = 0.0
        self.void_t = void_t
        self.ts1, self.ts0 = self.times[0], self.times[1]
        self.f_new, self.f_next = 1, 2
        self.fe_time = 0.0
        self.current = self.theta[0].copy()
        self.dT_FE = self.ts0 - self.ts1

    def advance(self, dt: float) -> bool:
        """False when the frames are used up (the reference stops there)."""
        if self.fe_time == 0:
            self.fe_time = self.ts1
        self.fe_time += dt
        while self.fe_time >= self.ts0:
            if self.f_next >= len(self.times):
                return False
            self.ts1 = self.ts0
            self.ts0 = self.times[self.f_next]
            self.f_new = self.f_next
            self.f_next += 1
        ratio = (self.fe_time - self.ts1) / (self.ts0 - self.ts1)
        th0, th1 = self.theta[self.f_new], self.theta[self.f_new - 1]
        v = np.where(th0 <= self.void_t, self.void_t, np.where(th1 <= self.void_t, th0, ratio * (th0 - th1) + th1))
        self.current = v
        self.dT_FE = self.ts0 - self.fe_time
        return True


def digests(r) -> dict:
    return {k: M.d64(r.field(FIELD_OF[k])) for k in STATE}


@pytest.mark.parametrize("name", ["remelt_nucleation", "remelt_new_grains", "remelt_scaled"])
def test_external_node_temperatures_reproduce_the_reference(amca, tmp_path, name):
    fx = FIX[name]
    M.prepare(fx, str(tmp_path))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    r.initialize()
    g = np.load(os.path.join(HERE, "golden", f"{name}.npz"))
    fields = [str(f) for f in g["fields"]]
    rep = FrameReplay(fx.frames)
    n = len(g["digests"])
    for i in range(n):
        r.set_nodal_temperatures(rep.current)
        dt = r.step_coupled(rep.dT_FE)
        st = r.stats()
        assert st["step"] == i + 1
        assert st["time"] == g["time"][i] and dt == g["dt"][i], f"step {i + 1}: time/dt"
        d = digests(r)
        bad = [k for k in STATE if d[k] != g["digests"][i][fields.index(k)]]
        assert not bad, f"step {i + 1}: {bad}"
        more = rep.advance(dt)
        assert more == (i + 1 < n), f"step {i + 1}: the frames end where the reference's did"
    # a step without fresh node temperatures is refused
    with pytest.raises(amca.AmcaError):
        r.step_coupled(1e-6)
    # reset returns to the frames: the replayed run again
    r.reset()
    r.run()
    assert np.array_equal(r.field("orientation_id"), g["orient"])
    r.close()


def test_remelt_run_until_then_on_equals_one_run(amca, tmp_path):
    fx = FIX["remelt_nucleation"]
    M.prepare(fx, str(tmp_path))
    r = amca.CellularAutomataRealm(fx.case.to_yaml(), seed=fx.case.seed, workdir=str(tmp_path))
    r.initialize()
    g = np.load(os.path.join(HERE, "golden", "remelt_nucleation.npz"))
    t_mid = float(g["time"][len(g["time"]) // 2])
    r.run_until(t_mid)
    st = r.stats()
    k = int(np.searchsorted(g["time"], t_mid))  # first step whose end time reaches t_mid
    assert st["time"] >= t_mid and st["step"] == k + 1 and st["time"] == g["time"][k]
    r.run_until(t_mid)  # nothing more to do
    assert r.stats()["step"] == k + 1
    r.run()
    assert r.stats()["step"] == len(g["time"])
    assert np.array_equal(r.field("orientation_id"), g["orient"])
    r.close()


def test_plain_run_until_and_dt_cap(amca):
    case = [c for c in cases.small_cases() if c.name == "mixed_24_s1"][0]
    golden = np.load(os.path.join(HERE, "golden", "mixed_24_s1.npz"))
    r = amca.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    r.initialize()
    r.run()
    t_total, n_total = r.stats()["time"], r.stats()["step"]
    r.reset()
    r.run_until(0.5 * t_total)
    st = r.stats()
    assert 0.5 * t_total <= st["time"] < t_total and 0 < st["step"] < n_total
    r.run()
    assert np.array_equal(r.field("orientation_id"), golden["orient"]) and r.stats()["step"] == int(golden["steps"])
    # a dt bound below the realm's own dt sets the step's dt; an unbounded step is amca_step
    r2 = amca.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    r2.initialize()
    dt0 = r2.single_integration_step()
    dt1 = r2.step_coupled(0.25 * dt0)
    assert dt1 == 0.25 * dt0 and r2.stats()["time"] == dt0 + 0.25 * dt0
    dt2 = r2.step_coupled(float("inf"))
    r3 = amca.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
    r3.initialize()
    r3.single_integration_step()
    r3.step_coupled(0.25 * dt0)
    assert r3.single_integration_step() == dt2
    for x in (r, r2, r3):
        x.close()
