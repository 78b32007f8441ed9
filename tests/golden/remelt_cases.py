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
from amca3d_gb300.decks import RemeltCase  # noqa: E402


@dataclasses.dataclass
class Rosenthal:
    """Moving point source (SI units)."""

    power: float = 30.0          # W
    absorptivity: float = 0.4
    speed: float = 1.0           # m/s along +x
    conductivity: float = 20.0   # W/(m K)
    diffusivity: float = 5e-6    # m^2/s
    t0: float = 300.0            # K
    t_cap: float = 3000.0        # K, cap near the source
    x_start: float = -1.0e-5     # source x at t = 0
    y_line: float = 2.0e-5       # track y
    z_top: float = 2.4e-5        # surface z
    void_above: Optional[float] = None  # nodes with z > z_top + void_above get t_void
    t_void: float = 293.0

    def field(self, x, y, z, t):
        xi = x - (self.x_start + self.speed * t)
        dy = y - self.y_line
        dz = z - self.z_top
        r = np.sqrt((xi * xi + dy * dy) + dz * dz)
        r = np.maximum(r, 1e-9)
        q = (self.absorptivity * self.power) / ((2.0 * math.pi * self.conductivity) * r)
        T = self.t0 + q * det_exp(-(self.speed * (r + xi)) / (2.0 * self.diffusivity))
        T = np.minimum(T, self.t_cap)
        if self.void_above is not None:
            T = np.where(z > self.z_top + self.void_above, self.t_void, T)
        return T


LN2 = 0.6931471805599453
INV_LN2 = 1.4426950408889634
EXP_TAYLOR = [1.0 / math.factorial(n) for n in range(14)]


def det_exp(a):
    """exp(a) for a <= 0 from IEEE add/mul and ldexp only: k = rint(a/ln2),
    r = a - k ln2, a degree-13 Taylor polynomial in Horner form, times 2^k.
    Relative error below 1e-13; the point is that it is the same double on
    every IEEE platform (no libm, no contraction), host or device."""
    a = np.asarray(a, dtype=np.float64)
    a = np.maximum(a, -700.0)
    k = np.rint(a * INV_LN2)
    r = a - k * LN2
    p = np.full_like(r, EXP_TAYLOR[13])
    for n in range(12, -1, -1):
        p = p * r + EXP_TAYLOR[n]
    return np.ldexp(p, k.astype(np.int64))


@dataclasses.dataclass
class FrameSpec:
    """Structured FE node grid and frame times (file units, before length_scale)."""

    origin: Tuple[float, float, float]
    spacing: float
    nodes: Tuple[int, int, int]
    frame_dt: float
    frames: int
    source: Rosenthal
    length_scale: float = 1.0     # file coordinate * length_scale = metres
    time_scale: float = 1.0       # file time * time_scale = seconds
    time_offset: float = 0.0      # time written for frame 0

    def node_coords(self):
        nx, ny, nz = self.nodes
        i = np.arange(nx)
        j = np.arange(ny)
        k = np.arange(nz)
        K, J, I = np.meshgrid(k, j, i, indexing="ij")
        x = self.origin[0] + self.spacing * I
        y = self.origin[1] + self.spacing * J
        z = self.origin[2] + self.spacing * K
        return x.ravel(), y.ravel(), z.ravel()

    def frame_values(self, f: int) -> np.ndarray:
        x, y, z = self.node_coords()
        s = self.length_scale
        return self.source.field(x * s, y * s, z * s, (f * self.frame_dt) * self.time_scale)

    def write(self, path: str, title_lines: int = 4) -> None:
        nx, ny, nz = self.nodes
        x, y, z = self.node_coords()
        xyz = [f"{a!r} {b!r} {c!r}" for a, b, c in zip(x.tolist(), y.tolist(), z.tolist())]
        with open(path, "w") as f:
            for t in range(title_lines):
                f.write("Title\n" if t == 0 else ("End of title\n" if t == title_lines - 1 else "synthetic Rosenthal frames\n"))
            for fr in range(self.frames):
                T = self.frame_values(fr)
                tt = self.time_offset + fr * self.frame_dt
                f.write("\n")
                f.write("Subtitle\n")
                f.write("No. step   No. step    time   time   x0    x1   y0   y1    z0   z1\n")
                f.write(f"{fr + 1} {fr + 1} {tt!r} {tt!r} 0 {nx - 1} 0 {ny - 1} 0 {nz - 1}\n")
                f.write("x  y  z  tn\n")
                f.write("".join(f"{p} {v!r}\n" for p, v in zip(xyz, T.tolist())))


def columnar_microstructure(case: RemeltCase, grains: int, seed: int, path: str, grainless_mod: int = 0) -> None:
    """Write a restart file (``<stem>0.txt``) holding ``grains`` columnar
    grains: Voronoi regions of seed points in the x-y plane, extruded in z.
    Every interior cell is its own grain object carrying its region's
    orientation; ghost cells carry grain and orientation -1. With
    grainless_mod > 0, interior cells with (i + 2j + 3k) % grainless_mod == 0
    keep their orientation but get no grain object (grain id -1), so that
    captures and nucleations there create new grains."""
    rng = np.random.default_rng(seed)
    nx, ny, nz = case.cells
    h = case.cell_size
    gx, gy, gz = nx + 2, ny + 2, nz + 2
    pts = rng.random((grains, 2)) * np.array([nx * h, ny * h]) + np.array(case.origin[:2])
    # products of uniform draws and constants only: the same doubles on every platform
    euler = np.stack([rng.random(grains) * (2 * math.pi), rng.random(grains) * math.pi,
                      rng.random(grains) * (0.5 * math.pi)], axis=1)
    I = np.arange(1, nx + 1)
    J = np.arange(1, ny + 1)
    cx = case.origin[0] + h * (I - 0.5)
    cy = case.origin[1] + h * (J - 0.5)
    CY, CX = np.meshgrid(cy, cx, indexing="ij")
    d2 = (CX[..., None] - pts[:, 0]) ** 2 + (CY[..., None] - pts[:, 1]) ** 2
    region = np.argmin(d2, axis=2)  # [ny, nx]
    ncell = gx * gy * gz
    grain = np.full(ncell, -1, np.int64)
    orient = np.full(ncell, -1, np.int64)
    glist = []
    for k in range(1, nz + 1):
        for j in range(1, ny + 1):
            for i in range(1, nx + 1):
                c = k * gx * gy + j * gx + i
                orient[c] = region[j - 1, i - 1]
                if grainless_mod and (i + 2 * j + 3 * k) % grainless_mod == 0:
                    continue
                grain[c] = len(glist)
                glist.append((c, case.origin[0] + h * (i - 0.5), case.origin[1] + h * (j - 0.5),
                              case.origin[2] + h * (k - 0.5), int(orient[c])))
    stem = path[: path.rfind(".")] if "." in os.path.basename(path) else path
    with open(stem + "0.txt", "w") as f:
        f.write("numCell; numOrientation; numLocalGrain; numGlobalExpectedGrain; start Point X; Y; Z; number Point nx; ny; nz; dCell\n")
        f.write(f"{ncell}  {grains}  {len(glist)}  {grains}  {case.origin[0]!r}  {case.origin[1]!r}  {case.origin[2]!r}  "
                f"{gx}  {gy}  {gz}  {h!r}\n")
        f.write("Cell informatin: ID; grainID; orientationID; hasBeenMelted; undercooling of seed\n")
        f.write("".join(f"{c}  {grain[c]}  {orient[c]}  0  -1\n" for c in range(ncell)))
        f.write("Orientation informatin: ID; EularAngle\n")
        f.write("".join(f"{o}  {float(euler[o, 0])!r}  {float(euler[o, 1])!r}  {float(euler[o, 2])!r}  \n"
                        for o in range(grains)))
        f.write("Grain information: ID; cellID; grainCenter; orientationID\n")
        f.write("".join(f"{g}  {c}  {x!r}  {y!r}  {z!r}  {o}   \n" for g, (c, x, y, z, o) in enumerate(glist)))


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
    mm = dict(base)
    mm["origin"] = (1.0e-3, 2.0e-3, 0.0)
    out.append(RemeltFixture(
        RemeltCase(name="remelt_scaled", length_scale=1.0e-3, time_scale=1.0e-3, offset=(0.0, 0.0, 0.0),
                   a=(1.0e-5, 2.5e-4, 0.0), bin_size=(3, 4, 5), **mm),
        _small_frames(origin=(0.99, 1.99, -0.01), spacing=0.01, length_scale=1.0e-3, frame_dt=1.0e-3,
                      time_scale=1.0e-3, time_offset=5.0,
                      src=dict(x_start=0.99e-3, y_line=2.02e-3, z_top=2.4e-5))))
    return out
