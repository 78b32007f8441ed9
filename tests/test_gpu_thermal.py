"""The thermal model's tensor-core kernels against the FP64 restatement
(oracle/thermal_oracle.py), through the C ABI.

* gradients of one batch (the layer GEMMs, their epilogues, split-K
  weight gradients, head and bias reductions) against the restatement with
  the same bf16 rounding points;
* the fused inference kernel against the restatement and against the
  training forward pass;
* training lowers the loss and the trained model beats the untrained one on
  the FE field near the liquidus;
* model frames: fallback to the FE field exactly where the rule says;
* a remelting realm runs on model frames.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import thermal_oracle as TO  # noqa: E402

from amca3d_gb300 import decks  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def A():
    import amca3d_gb300 as A

    A.load_library()
    return A


def window_inputs(spec, n, seed):
    rng = np.random.default_rng(seed)
    lo, hi = np.array(spec["window_lo"]), np.array(spec["window_hi"])
    raw = np.empty((n, 5), np.float32)
    raw[:, :3] = lo + (hi - lo) * rng.random((n, 3))
    raw[:, 3] = rng.uniform(spec["power_lo"], spec["power_hi"], n)
    raw[:, 4] = rng.uniform(spec["speed_lo"], spec["speed_hi"], n)
    return raw


def fe_temperature(spec, raw):
    """FE temperature (K) of raw inputs: the source at the origin on the
    surface, each sample with its own power and speed (vectorised
    thermal_oracle.scan_field)."""
    r = raw.astype(np.float64)
    xi, dy, dz, p, v = r[:, 0], r[:, 1], -r[:, 2], r[:, 3], r[:, 4]
    rad = np.maximum(np.sqrt((xi * xi + dy * dy) + dz * dz), 1e-9)
    q = (spec["absorptivity"] * p) / ((2.0 * np.pi * spec["conductivity"]) * rad)
    T = spec["t0"] + q * TO.field_exp(-(v * (rad + xi)) / (2.0 * spec["diffusivity"]))
    return np.minimum(T, spec["t_cap"])


def fe_target(spec, raw):
    return TO.target_of(fe_temperature(spec, raw), spec)


def enc_of(m):
    e = m.encoding()
    return dict(fourier=e["fourier"], in_shift=e["in_shift"], in_scale=e["in_scale"], t_shift=e["t_shift"],
                t_scale=e["t_scale"], log_output=e["log_output"])


@pytest.mark.parametrize("n", [256, 8192])
def test_gradients_match_the_fp64_restatement(A, n):
    spec = decks.thermal_spec()
    m = A.ThermalModel(**spec)
    p = m.params().astype(np.float64)
    raw = window_inputs(spec, n, seed=n)
    y = fe_target(spec, raw).astype(np.float32)
    g, pred = m.gradients(raw, y)
    g_ref, mu, s, _ = TO.forward_backward(p, raw, y.astype(np.float64), enc_of(m), bf16_points=True)
    assert np.max(np.abs(pred[:, 0] - mu)) < 2e-2 * max(1.0, np.max(np.abs(mu)))
    assert np.max(np.abs(pred[:, 1] - s)) < 2e-2 * max(1.0, np.max(np.abs(s)))
    for k, (o, shp) in TO.layout().items():
        sz = int(np.prod(shp))
        a, b = g[o:o + sz].astype(np.float64), g_ref[o:o + sz]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        cos = float(a @ b) / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
        assert rel < 3e-2 and cos > 0.999, (k, rel, cos)
    m.close()


def test_fused_inference_matches_restatement_and_training_forward(A):
    spec = decks.thermal_spec()
    m = A.ThermalModel(**spec)
    raw = window_inputs(spec, 1000, seed=5)  # not a multiple of 128: a partial tile
    T, e = m.eval(raw)
    T_ref, e_ref = TO.predict(m.params().astype(np.float64), raw, enc_of(m))
    dT = np.abs(T - T_ref)
    assert np.max(dT) < 10.0 and np.mean(dT) < 1.0, (np.max(dT), np.mean(dT))
    assert np.all(np.abs(e / e_ref - 1) < 0.05)
    # the training forward on the same inputs (first 896 rows: a multiple of 128)
    _, pred = m.gradients(raw[:896], np.zeros(896, np.float32))
    mu = pred[:, 0].astype(np.float64)
    T_train = spec["t_shift"] + spec["t_scale"] * (np.exp(mu) if spec["log_output"] else mu)
    assert np.max(np.abs(T_train - T[:896])) < 2.0
    m.close()


@pytest.fixture(scope="module")
def trained(A):
    spec = decks.thermal_spec()
    m = A.ThermalModel(**spec)
    st = m.train(samples=8_000_000, steps=3000, batch=16384, lr_max=1e-3, lr_min=1e-5)
    yield spec, m, st
    m.close()


def test_training_lowers_the_loss(trained):
    _spec, _m, st = trained
    assert st["steps"] == 3000 and st["samples_seen"] == 3000 * 16384
    assert st["last_loss"] < st["first_loss"] / 10, st


def test_trained_model_beats_the_untrained_one_near_the_liquidus(A, trained):
    spec, m, _ = trained
    raw = window_inputs(spec, 200_000, seed=9)
    T_fe = fe_temperature(spec, raw)
    mushy = (T_fe > 1600.0) & (T_fe < 1800.0)
    assert mushy.sum() > 50
    T, e = m.eval(raw)
    untrained = A.ThermalModel(**spec)
    T0, e0 = untrained.eval(raw)
    err_t = np.abs(T[mushy] - T_fe[mushy])
    err_u = np.abs(T0[mushy] - T_fe[mushy])
    assert np.median(err_t) < np.median(err_u) / 10, (np.median(err_t), np.median(err_u))
    # with a 60 K error threshold the trained model keeps a good share of the mushy-zone points, the
    # untrained none
    keep_t, keep_u = np.mean(e[mushy] <= 60.0), np.mean(e0[mushy] <= 60.0)
    assert keep_t > 0.2 and keep_u == 0.0, (keep_t, keep_u)
    # and the points it keeps are accurate to its estimate more often than not
    assert np.mean(err_t[e[mushy] <= 60.0] <= 60.0) > 0.8
    untrained.close()


def test_model_frames_fall_back_to_the_fe_field_by_the_rule(A, trained):
    spec, m, _ = trained
    sc = decks.scan_of((100, 60, 40), 2.0e-6, tracks=2, hatch=4.0e-5)
    scan = A.Scan.of(**sc)
    f0, nf = 80, 6
    always, fe, c_always = m.frames(scan, f0, nf, 1700.0, 150.0, 0.0, with_fe=True)
    never, _, c_never = m.frames(scan, f0, nf, 1700.0, 150.0, 1e30)
    assert c_always[0] == c_never[0] > 0 and c_always[1] == c_never[1] and c_never[2] == 0
    assert c_always[2] == c_always[1]
    # with threshold 0 every node near the liquidus holds the FE value exactly
    near = np.abs(never - 1700.0) < 150.0
    assert np.array_equal(always[near], fe[near])
    assert np.array_equal(always[~near], never[~near])
    # FE frames equal the restatement of the field
    nx, ny, nz = sc["nodes"]
    K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x, y, z = ((sc["origin"][0] + sc["spacing"] * I).ravel(), (sc["origin"][1] + sc["spacing"] * J).ravel(),
               (sc["origin"][2] + sc["spacing"] * K).ravel())
    for k in range(nf):
        t = (f0 + k) * sc["frame_dt"]
        assert np.array_equal(fe[k], TO.scan_field(sc, x, y, z, t))


def test_realm_runs_on_model_frames(A, trained):
    """A remelting realm on a 2-track raster with frames from the model
    (fallback to the FE field near the liquidus) runs to the end of its
    frames, and its grain statistics stay close to the run on the FE field's
    frames."""
    from amca3d_gb300.grainstats import grain_stats

    _spec, m, _ = trained
    case, sc, micro = decks.config_thermal_block("thermal_block", (120, 60, 40), tracks=2, hatch=4.0e-5, grains=60)
    out = {}
    for kind in ("fe", "model"):
        r = A.CellularAutomataRealm(case.to_yaml(), seed=case.seed)
        r.set_microstructure(micro["grain"], micro["orient"], micro["euler"], micro["grain_cell"],
                             micro["grain_orient"], expected=micro["expected"])
        if kind == "fe":
            r.set_scan_frames(**sc)
        else:
            r.set_thermal_frames(m, 1700.0, 100.0, 5.0, **sc)
        r.initialize()
        r.run()
        st, fs = r.stats(), r.frame_stats()
        assert st["done"] == 1 and fs["frames"] == sc["frames"]
        out[kind] = grain_stats(r.field("orientation_id"), r.orientations(), case.cells)
        if kind == "model":
            assert fs["model_nodes"] > 0 and 0 < fs["fallbacks"] <= fs["near_liquidus"]
        r.close()
    a, b = out["model"], out["fe"]
    assert abs(a["grains"] - b["grains"]) <= max(3, 0.25 * b["grains"]), out
    assert abs(a["mean_size_cells"] - b["mean_size_cells"]) <= 0.25 * b["mean_size_cells"], out
