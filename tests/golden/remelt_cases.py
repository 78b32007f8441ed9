"""FE-coupled remelting cases for the golden fixtures and the parity tests.

The reference's PBF examples ship without their temperature histories, so
every case here replays a synthetic thermal history: the quasi-steady
Rosenthal solution for a point source moving along x on the top surface of a
semi-infinite body,

    T = T0 + (A P) / (2 pi k R) * exp(-v (R + xi) / (2 alpha)),
    xi = x - (x_start + v t),  R = |(xi, y - y_l, z - z_top)|,

capped at ``t_cap`` near the source, evaluated with IEEE add/mul/div/sqrt
only (``det_exp`` below, no libm) so that every platform, and the device
generator in the library, produce the same doubles; sampled on a structured
node grid and
written in the reference's text frame format (title lines, then per frame a
subtitle whose 4th line holds "step step time time x0 x1 y0 y1 z0 z1", then
"x y z T" per node with x fastest; CA/src/LoadDataFromFile.cpp:21-191). Values
are written with 17 significant digits, so the reference's istream and this
library's reader see identical doubles.

Loaded microstructures use the reference's restart format
(CA/src/CellularAutomataManager_3DRemelting.cpp:166-307): columnar grains,
one Voronoi region per seed point in the x-y plane, one grain per interior
cell.
"""
from __future__ import annotations

import dataclasses
import math
import os
import sys
from typing import Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
from amca3d_gb300 import decks  # noqa: E402
from amca3d_gb300.decks import FrameSpec, RemeltCase, Rosenthal, det_exp  # noqa: E402,F401


def columnar_microstructure(case: RemeltCase, grains: int, seed: int, path: str, grainless_mod: int = 0) -> None:
    """Write a restart file (``<stem>0.txt``) of ``grains`` columnar grains
    (amca3d_gb300.decks.columnar_microstructure) for the case's grid."""
    m = decks.columnar_microstructure(case.cells, case.cell_size, case.origin, grains, seed, grainless_mod)
    decks.write_restart(path, m, case.origin, case.cells, case.cell_size)


@dataclasses.dataclass
class RemeltFixture:
    case: RemeltCase
    frames: FrameSpec
    columnar_grains: int = 0      # >0: write a restart file with that many grains
    columnar_seed: int = 0
    grainless_mod: int = 0


def _small_frames(**kw) -> FrameSpec:
    src = Rosenthal(**kw.pop("src", {}))
    d = dict(origin=(-1.0e-5, -1.0e-5, -1.0e-5), spacing=1.0e-5, nodes=(11, 7, 5), frame_dt=1.0e-6,
             frames=190, source=src)
    d.update(kw)
    return FrameSpec(**d)


def fixtures() -> list:
    """Small decks the reference finishes in seconds."""
    base = dict(cells=(40, 20, 12), cell_size=2.0e-6, termination_time=1.0, time_step=1.0e-6)
    out = []
    out.append(RemeltFixture(RemeltCase(name="remelt_random", **base), _small_frames()))
    out.append(RemeltFixture(
        RemeltCase(name="remelt_nucleation", seed=3, nucleation=True,
                   surface=(2.0e9, 15.0, 3.0), bulk=(4.0e14, 20.0, 5.0), **base),
        _small_frames(src=dict(power=34.0))))
    out.append(RemeltFixture(
        RemeltCase(name="remelt_columnar", seed=2, nucleation=True, microstructure="grainInfoIn.txt",
                   bulk=(4.0e14, 20.0, 5.0), **base),
        _small_frames(), columnar_grains=12, columnar_seed=2))
    out.append(RemeltFixture(
        RemeltCase(name="remelt_new_grains", seed=5, nucleation=True, microstructure="grainInfoIn.txt",
                   bulk=(4.0e14, 20.0, 5.0), surface=(2.0e9, 15.0, 3.0), **base),
        _small_frames(src=dict(power=33.0, y_line=1.8e-5)), columnar_grains=9, columnar_seed=7, grainless_mod=3))
    out.append(RemeltFixture(
        RemeltCase(name="remelt_void", void_temperature=293.0001, has_been_melted=True,
                   cutoff_factor=None, time_step_factor_ca=0.3, **base),
        _small_frames(src=dict(void_above=-0.3e-5, power=36.0))))
    # two cells thick, the source on its top surface: the pool melts through
    thin = dict(base)
    thin["cells"] = (40, 20, 2)
    out.append(RemeltFixture(
        RemeltCase(name="remelt_thin", seed=6, nucleation=True, bulk=(4.0e14, 20.0, 5.0), **thin),
        _small_frames(src=dict(z_top=4.0e-6))))
    # the track along the domain's y = 0 face: half the pool lies over the ghost layer
    out.append(RemeltFixture(
        RemeltCase(name="remelt_edge", seed=8, nucleation=True, bulk=(4.0e14, 20.0, 5.0), **base),
        _small_frames(src=dict(y_line=0.0))))
    mm = dict(base)
    mm["origin"] = (1.0e-3, 2.0e-3, 0.0)
    out.append(RemeltFixture(
        RemeltCase(name="remelt_scaled", length_scale=1.0e-3, time_scale=1.0e-3, offset=(0.0, 0.0, 0.0),
                   a=(1.0e-5, 2.5e-4, 0.0), bin_size=(3, 4, 5), **mm),
        _small_frames(origin=(0.99, 1.99, -0.01), spacing=0.01, length_scale=1.0e-3, frame_dt=1.0e-3,
                      time_scale=1.0e-3, time_offset=5.0,
                      src=dict(x_start=0.99e-3, y_line=2.02e-3, z_top=2.4e-5))))
    return out


def output_fixture() -> RemeltFixture:
    """A tiny deck whose every output file is compared byte for byte: VTR
    snapshots of temperature, grain id, orientation and melted flag, the
    restart file, finalGrains.vtk and finalResult.txt."""
    cells = (12, 8, 6)
    case = RemeltCase(name="remelt_outputs", cells=cells, cell_size=2.0e-6, nucleation=True, seed=4,
                      bulk=(2.0e15, 15.0, 4.0), termination_time=1.0, time_step=1.0e-6, output_frequency=150,
                      output_base="./Results/Grains", output_microstructure_file="grainOut.txt",
                      output_variables=("temperature", "grain_ID", "grain_orientation", "melted_flag"))
    frames = FrameSpec(origin=(-1.0e-5, -1.0e-5, -1.0e-5), spacing=1.0e-5, nodes=(6, 5, 5), frame_dt=1.0e-6,
                       frames=110, source=Rosenthal(power=14.0, x_start=-1.0e-5, y_line=8.0e-6, z_top=1.2e-5))
    return RemeltFixture(case, frames)
