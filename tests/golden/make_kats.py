"""Known-answer vectors from the reference's own code and libraries.

Compiles a small driver against the UNMODIFIED reference sources
CA/src/Octahedron.cpp, Envelope.cpp, Grain.cpp and Orientation.cpp (with the
oracle shims on the include path) and records:
  kat_octahedron.npz  Octahedron::set_coordinate_transformation_matrix,
                      cell_is_captured and capture_cell on seeded random
                      envelopes / cells (default and custom truncation);
  kat_streams.json    the first glibc rand() values for seeds 0..3 and the
                      first std::normal_distribution draws of a default-seeded
                      std::default_random_engine (hex floats, exact).
Usage: python tests/golden/make_kats.py [REFERENCE_CHECKOUT]
"""
from __future__ import annotations

import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
SHIM = os.path.join(ROOT, "oracle", "shim")

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>
#include "Octahedron.h"
#include "Grain.h"
#include "Orientation.h"
int main(int argc, char** argv) {
  // envelope vectors: stdin gives n, then per case: 3 euler, 3 grain centre, 3 cell centre, length, h, trunc_f (<0: default)
  int n; if (scanf("%d", &n) != 1) return 1;
  FILE* out = fopen(argv[1], "wb");
  for (int c = 0; c < n; ++c) {
    double e[3], g[3], cc[3], L, h, tf;
    for (int i = 0; i < 3; ++i) scanf("%la", &e[i]);
    for (int i = 0; i < 3; ++i) scanf("%la", &g[i]);
    for (int i = 0; i < 3; ++i) scanf("%la", &cc[i]);
    scanf("%la %la %la", &L, &h, &tf);
    Octahedron oct;
    if (tf > 0) oct.set_truncation_coefficient(tf);
    Orientation o(0, 3, e);
    Grain gr(nullptr, false);
    gr.xc_ = g[0]; gr.yc_ = g[1]; gr.zc_ = g[2]; gr.length_ = L; gr.orientation_ = &o;
    bool cap = oct.cell_is_captured(&gr, cc);
    double info[4] = {0, 0, 0, 0};
    if (cap) {
      double gc[3] = {cc[0] - g[0], cc[1] - g[1], cc[2] - g[2]};
      oct.capture_cell(gc, L, h, info);
    }
    double capd = cap ? 1.0 : 0.0;
    fwrite(oct.transMatrixLocal2Global, sizeof(double), 9, out);
    fwrite(&capd, sizeof(double), 1, out);
    fwrite(info, sizeof(double), 4, out);
    fwrite(&oct.truncationCoefficient_, sizeof(double), 1, out);
  }
  fclose(out);
  // streams
  FILE* s = fopen(argv[2], "w");
  for (int seed = 0; seed < 4; ++seed) {
    srand(seed);
    fprintf(s, "rand %d", seed);
    for (int i = 0; i < 16; ++i) fprintf(s, " %d", rand());
    fprintf(s, "\n");
  }
  double mu[2] = {3.0, 2.0}, sd[2] = {1.0, 0.5};
  for (int k = 0; k < 2; ++k) {
    std::default_random_engine gen;
    std::normal_distribution<double> d(mu[k], sd[k]);
    fprintf(s, "normal %a %a", mu[k], sd[k]);
    for (int i = 0; i < 32; ++i) fprintf(s, " %a", d(gen));
    fprintf(s, "\n");
  }
  fclose(s);
  return 0;
}
"""


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src = os.path.join(ref, "CA", "src")
    rng = np.random.default_rng(20261203)
    n = 2500
    h = 2e-6
    rows = []
    for c in range(n):
        e = (rng.uniform(0, 2 * np.pi), np.arccos(rng.uniform(-1, 1)), rng.uniform(0, 0.5 * np.pi))
        I, J, K = rng.integers(1, 300, size=3)
        cc = (h * (I - 0.5), h * (J - 0.5), h * (K - 0.5))
        L = rng.uniform(0.05, 3.0) * h
        # grain centre offset: mostly near the octahedron surface so both outcomes occur
        d = rng.normal(size=3)
        d = d / np.abs(d).sum() * L * rng.uniform(0.3, 1.3)
        g = (cc[0] - d[0], cc[1] - d[1], cc[2] - d[2])
        tf = -1.0 if c % 4 else rng.uniform(0.5, 3.0)
        rows.append((e, g, cc, L, h, tf))
    with tempfile.TemporaryDirectory() as wd:
        drv = os.path.join(wd, "kat.cpp")
        open(drv, "w").write(DRIVER)
        exe = os.path.join(wd, "kat")
        cmd = ["g++", "-std=c++11", "-O2", "-ffp-contract=off", "-w", "-I", SHIM, "-I", os.path.join(ref, "CA", "include"),
               drv] + [os.path.join(src, f) for f in ("Octahedron.cpp", "Envelope.cpp", "Grain.cpp", "Orientation.cpp")]
        subprocess.run(cmd + ["-o", exe], check=True)
        text = [str(n)]
        for e, g, cc, L, hh, tf in rows:
            vals = list(e) + list(g) + list(cc) + [L, hh, tf]
            text.append(" ".join(float(v).hex() for v in vals))
        binp, strp = os.path.join(wd, "env.bin"), os.path.join(wd, "streams.txt")
        subprocess.run([exe, binp, strp], input="\n".join(text), text=True, check=True)
        raw = np.fromfile(binp, np.float64).reshape(n, 15)
        inputs = np.array([list(e) + list(g) + list(cc) + [L, hh, tf] for e, g, cc, L, hh, tf in rows])
        np.savez_compressed(os.path.join(HERE, "kat_octahedron.npz"), inputs=inputs, l2g=raw[:, :9],
                            captured=raw[:, 9].astype(np.int8), info=raw[:, 10:14], trunc=raw[:, 14])
        streams = {"rand": {}, "normal": []}
        for line in open(strp):
            t = line.split()
            if t[0] == "rand":
                streams["rand"][t[1]] = [int(x) for x in t[2:]]
            else:
                streams["normal"].append({"mean": t[1], "sd": t[2], "draws": t[3:]})
    with open(os.path.join(HERE, "kat_streams.json"), "w") as f:
        json.dump(streams, f, indent=1)
    print("captured fraction", raw[:, 9].mean())


if __name__ == "__main__":
    main()
