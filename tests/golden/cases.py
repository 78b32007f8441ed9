"""The decks the golden fixtures were made from (see make_golden.py).

Each case is a uniform-cooling deck in the reference's YAML surface. Small
cases keep their full ghost-inclusive fields in <name>.npz; the 320^3 case
keeps SHA-256 digests of its fields in plain_golden.json.
"""
from __future__ import annotations

import dataclasses
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from amca3d_gb300.decks import (PlainCase, bulk_density_for_sites, config_nucleation_60,  # noqa: E402
                                config_uniform_320, surface_density_for_sites)


def _mixed(name, cells, seed, surf_sites, bulk_sites, h=1e-5, **kw) -> PlainCase:
    return PlainCase(name=name, cells=cells, cell_size=h,
                     surface=(surface_density_for_sites(surf_sites, cells, h), 2.0, 0.5),
                     bulk=(bulk_density_for_sites(bulk_sites, cells, h), 3.0, 1.0),
                     seed=seed, t_dot=kw.pop("t_dot", -50.0), **kw)


def small_cases() -> list:
    c0 = config_nucleation_60()
    mid = dataclasses.replace(c0, name="nucleation_60_t0.5", termination_time=0.5)
    return [
        c0,
        mid,
        _mixed("mixed_24_s1", (24, 24, 24), 1, 60, 80),
        _mixed("ragged_30x20x16_s2", (30, 20, 16), 2, 50, 40, origin=(-1e-4, 2e-4, 5e-5)),
        _mixed("tall_16x28x20_s3", (16, 28, 20), 3, 70, 30),  # ny > nx: the surface-cell scan quirk
        _mixed("envelope_32_s4", (32, 32, 32), 4, 30, 120, max_half_diagonal_length=1.5, time_step_factor_ca=0.35,
               a=(1.0e-5, 2.03e-4, 1.0e-5)),
        _mixed("dense_20_s5", (20, 20, 20), 5, 400, 2000),  # many duplicate site draws
        _mixed("fastcool_18_s6", (18, 18, 18), 6, 20, 25, t_dot=-400.0, time_step=0.0005),
        dataclasses.replace(_mixed("nosite_6x5x4", (6, 5, 4), 0, 0, 0), termination_time=0.0105),
        _mixed("single_cell", (1, 1, 1), 0, 0, 1),
        _mixed("shuffle_16_s8", (16, 16, 16), 8, 30, 40, shuffle_vtr=True),
        # one cell thick: every cell is a surface cell, listed once per face
        # it lies on, and the x-end rule of the surface list meets nx == 1
        _mixed("slab_1x20x24_s9", (1, 20, 24), 9, 40, 20),
        _mixed("plate_24x20x1_s10", (24, 20, 1), 10, 40, 20),
        # one cell thick in two directions: a line of cells along x, and along z
        _mixed("line_40x1x1_s11", (40, 1, 1), 11, 12, 6),
        _mixed("column_1x1x30_s12", (1, 1, 30), 12, 10, 5),
    ]


def output_case() -> PlainCase:
    """A tiny deck whose every output file is kept verbatim under outputs_tiny/."""
    c = _mixed("tiny_outputs", (12, 10, 8), 9, 12, 10, shuffle_vtr=False)
    return dataclasses.replace(c, output_frequency=7, output_variables=("grain_ID", "grain_orientation"),
                               microstructure_file="grainInfo.txt")


def large_cases() -> list:
    return [config_uniform_320()]
