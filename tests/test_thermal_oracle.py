"""CPU checks of the thermal model's restatement (oracle/thermal_oracle.py)
that the GPU's gradients are compared with: its analytic gradients against
central finite differences in FP64, and its FE field against the frame
writer's (amca3d_gb300.decks.Rosenthal.field) for one track."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import thermal_oracle as TO  # noqa: E402

from amca3d_gb300 import decks  # noqa: E402
from amca3d_gb300.grainstats import grain_stats  # noqa: E402


def small_model(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(TO.param_total())
    for _k, (o, s) in TO.layout().items():
        fan = s[-1]
        p[o:o + int(np.prod(s))] = rng.uniform(-1, 1, int(np.prod(s))) * np.sqrt(3.0 / fan)
    enc = dict(fourier=rng.normal(0, 2.0, (64, 5)).astype(np.float32), in_shift=np.zeros(5, np.float32),
               in_scale=np.ones(5, np.float32), t_shift=300.0, t_scale=1000.0)
    return p, enc


def test_oracle_gradients_match_finite_differences():
    p, enc = small_model(1)
    rng = np.random.default_rng(2)
    raw = rng.uniform(-1, 1, (16, 5)).astype(np.float32)
    y = rng.uniform(-0.5, 1.5, 16)
    g, mu, s, _ = TO.forward_backward(p, raw, y, enc, bf16_points=False)
    assert np.all((s > TO.S_MIN) & (s < TO.S_MAX))
    # a few coordinates of every parameter block
    for k, (o, shp) in TO.layout().items():
        size = int(np.prod(shp))
        for idx in rng.choice(size, size=min(3, size), replace=False):
            i = o + int(idx)
            eps = 1e-6 * max(1.0, abs(p[i]))
            pp, pm = p.copy(), p.copy()
            pp[i] += eps
            pm[i] -= eps
            fd = (TO.loss_total(pp, raw, y, enc, mu) - TO.loss_total(pm, raw, y, enc, mu)) / (2 * eps)
            assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (k, idx, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.00390625, 1.0078125, 1.005859375, 1.001953125, -3.14159, 0.0], np.float64)
    r = TO.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # halfway: ties to even
    assert r[2] == 1.0078125
    assert r[3] == 1.0078125
    assert r[4] == 1.0
    assert abs(r[5] + 3.140625) < 1e-12
    assert r[6] == 0.0


def test_scan_field_equals_the_frame_writer_on_one_track():
    src = decks.Rosenthal(power=200.0, absorptivity=0.4, speed=1.0, conductivity=20.0, diffusivity=5e-6, t0=300.0,
                          t_cap=3000.0, x_start=-5e-5, y_line=2.5e-4, z_top=2e-4)
    scan = dict(power=200.0, absorptivity=0.4, speed=1.0, conductivity=20.0, diffusivity=5e-6, t0=300.0,
                t_cap=3000.0, x_start=-5e-5, x_turn=1e-3, y_line=2.5e-4, z_top=2e-4, hatch=1e-4, track_time=1e-3,
                ntracks=1)
    rng = np.random.default_rng(3)
    x, y, z = rng.uniform(0, 1e-3, 2000), rng.uniform(0, 5e-4, 2000), rng.uniform(0, 2e-4, 2000)
    for t in (0.0, 3.7e-4, 9.9e-4):
        assert np.array_equal(TO.scan_field(scan, x, y, z, t), src.field(x, y, z, t))


def test_scan_alternates_direction_and_steps_the_hatch():
    scan = dict(speed=1.0, x_start=-5e-5, x_turn=1.05e-3, y_line=1e-4, hatch=1e-4, track_time=1.1e-3, ntracks=3)
    x0, y0, d0 = TO.scan_position(scan, 1e-4)
    x1, y1, d1 = TO.scan_position(scan, 1.1e-3 + 1e-4)
    x2, y2, d2 = TO.scan_position(scan, 10.0)  # past the end: the last track
    assert d0 == 1.0 and d1 == -1.0 and d2 == 1.0
    assert abs(x0 - 5e-5) < 1e-15 and abs(x1 - 9.5e-4) < 1e-15
    assert y0 == 1e-4 and abs(y1 - 2e-4) < 1e-18 and abs(y2 - 3e-4) < 1e-18


def test_grain_stats_of_a_known_field():
    cells = (4, 3, 2)
    o = np.full((4, 5, 6), -1, np.int32)
    o[1:-1, 1:-1, 1:-1] = 0
    o[1, 1, 1:3] = 1
    euler = np.array([[0.0, 0.0, 0.0], [0.3, 0.9, 0.2]])  # grain 0: <100> on z; grain 1: tilted by 0.9 rad
    st = grain_stats(o.ravel(), euler, cells)
    assert st["grains"] == 2 and st["cells"] == 24
    assert st["mean_size_cells"] == 12.0
    assert abs(st["frac_100z"] - 22 / 24) < 1e-12
