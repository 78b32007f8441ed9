"""Grain statistics of a final orientation field, the "matched grain stats"
the thermal-model workload compares between runs: grain count, mean grain
size and the <100> || z texture fraction.

* grains: distinct orientation ids among the interior cells (cells without an
  orientation, id < 0, are left out);
* mean_size_cells: interior cells with an orientation per grain;
* frac_100z: share of those cells whose crystal has a <100> axis within
  15 degrees of z. A crystal axis e_i maps to column i of the local->global
  matrix (Bunge angles, the reference's order, CA/src/Octahedron.cpp:282-310),
  so its angle with z is acos(|L[2][i]|).
"""
from __future__ import annotations

import numpy as np


def z_row(euler: np.ndarray) -> np.ndarray:
    """Third row of the local->global matrix of each orientation: the z
    components of the three crystal axes, [n x 3]."""
    e = np.asarray(euler, np.float64).reshape(-1, 3)
    b, g = e[:, 1], e[:, 2]
    return np.stack([np.sin(b) * np.sin(g), np.sin(b) * np.cos(g), np.cos(b)], axis=1)


def grain_stats(orient: np.ndarray, euler: np.ndarray, cells, max_angle_deg: float = 15.0) -> dict:
    nx, ny, nz = cells
    o = np.asarray(orient).reshape(nz + 2, ny + 2, nx + 2)[1:-1, 1:-1, 1:-1].ravel()
    o = o[o >= 0]
    ids, counts = np.unique(o, return_counts=True)
    if len(ids) == 0:
        return dict(grains=0, mean_size_cells=0.0, frac_100z=0.0, cells=0)
    zr = np.abs(z_row(np.asarray(euler).reshape(-1, 3)[ids]))
    aligned = zr.max(axis=1) >= np.cos(np.radians(max_angle_deg))
    return dict(grains=int(len(ids)), mean_size_cells=float(o.size / len(ids)),
                frac_100z=float(counts[aligned].sum() / o.size), cells=int(o.size))


def relative_difference(a: dict, b: dict) -> dict:
    """|a - b| / b for grains and mean size; absolute difference of the texture fraction."""
    return dict(grains=abs(a["grains"] - b["grains"]) / max(b["grains"], 1),
                mean_size_cells=abs(a["mean_size_cells"] - b["mean_size_cells"]) / max(b["mean_size_cells"], 1e-30),
                frac_100z=abs(a["frac_100z"] - b["frac_100z"]))
