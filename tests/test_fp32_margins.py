"""Adversarial checks of the FP32 shortcuts that stand in for FP64
comparisons, with the kernels' own arithmetic (amca3d_gb300/csrc/ca_math.h,
compiled for the host without contraction; tests/fp32_margins.cpp):

* the plain kernel's FP32 containment pre-test (captured_f32) against the FP64
  test of Octahedron::cell_is_captured on (envelope, neighbour) pairs with
  |c'|_1 within a few ulps of L, and at 2^-30..2^-6 relative distances: tiny,
  unit and huge half-diagonals, grids far from the origin, every neighbour;
  and the lower bound of |c'|_1 behind the wake keys (never above the FP64
  |c'|_1);
* the remelting kernel's FP32 interpolation bound against the FP64
  interpolation (MapVoxelManager::evaluate_temperature) at the liquidus,
  nullMatTemp_ and nullMatTemp_ + 0.01;
* the decentring rewrite (capture_f64) against the C restatement of the
  reference's Octahedron::capture_cell, bit for bit.

An FP32 verdict may be "undecided" (the kernel then evaluates in FP64) but
never wrong. 1M cases per check, fixed seed (the full differential ran
20M)."""
import os
import shutil
import subprocess
import tempfile

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.mark.skipif(shutil.which("g++") is None or shutil.which("gcc") is None, reason="needs gcc and g++")
def test_fp32_shortcuts_never_decide_wrongly():
    with tempfile.TemporaryDirectory() as wd:
        obj = os.path.join(wd, "oracle.o")
        exe = os.path.join(wd, "fp32_margins")
        subprocess.run(["gcc", "-std=c99", "-O2", "-ffp-contract=off", "-c", os.path.join(ROOT, "oracle", "amca_oracle.c"),
                        "-o", obj], check=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(HERE, "fp32_margins.cpp"), obj,
                        "-o", exe, "-lm"], check=True)
        out = subprocess.run([exe, "1000000", "7"], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.strip().splitlines():
        name, n, und, wrong = line.split()
        res[name] = (int(n), int(und), int(wrong))
    assert set(res) == {"containment0", "containment1", "containment2", "lower0", "lower1", "lower2", "interp0",
                        "interp1", "interp2", "capture"}
    for name, (n, und, wrong) in res.items():
        assert wrong == 0, (name, res[name])
        assert n > 0
    # the shortcuts decide most pairs that are not within rounding of the threshold
    assert res["interp2"][1] < 0.1 * res["interp2"][0], res["interp2"]
    assert res["containment2"][1] < 0.6 * res["containment2"][0], res["containment2"]
    assert res["capture"][0] > 100000
