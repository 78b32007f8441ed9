"""The envelope arithmetic of the CUDA kernels (amca3d_gb300/csrc/ca_math.h),
compiled for the host with the same no-contraction rule, against the
reference Octahedron known answers (tests/golden/kat_octahedron.npz)."""
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_ca_math_matches_reference_octahedron():
    k = np.load(os.path.join(HERE, "golden", "kat_octahedron.npz"))
    inp = k["inputs"]
    n = len(inp)
    gc = inp[:, 6:9] - inp[:, 3:6]
    rows = np.concatenate([k["l2g"], gc, inp[:, 9:11], k["trunc"][:, None],
                           k["captured"][:, None].astype(np.float64), k["info"]], axis=1)
    assert rows.shape == (n, 20)
    with tempfile.TemporaryDirectory() as wd:
        exe = os.path.join(wd, "kat")
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", os.path.join(HERE, "ca_math_kat.cpp"),
                        "-o", exe], check=True)
        data = os.path.join(wd, "kat.bin")
        with open(data, "wb") as f:
            f.write(struct.pack("<i", n))
            f.write(rows.astype("<f8").tobytes())
        out = subprocess.run([exe, data], check=True, capture_output=True, text=True).stdout.split()
    total, caps, bad = map(int, out)
    assert total == n and caps == int(k["captured"].sum()) and bad == 0
