"""Input decks in AMCA3D's YAML surface, built from plain parameters.

A deck written here is read unchanged by the AMCA3D reference program and by
this library's C-ABI (``amca_create``). Keys, nesting and defaults follow the
reference's loaders: ``CellularAutomataManager_3D::load``
(CA/src/CellularAutomataManager_3D.cpp:71-361), ``ProblemPhysics_RappazGandin1993::load``
(CA/src/ProblemPhysics.cpp:58-102), ``VtrManager::load`` (CA/src/VtrManager.cpp:60-103)
and the time-integrator block read in ``CellularAutomataSolver::load``
(CA/src/CellularAutomataSolver.cpp:99-128).
"""
from __future__ import annotations

import dataclasses
import math
import os
from typing import Optional, Sequence, Tuple


def _num(x: float) -> str:
    """Shortest text that reads back (via istream >> double) as exactly ``x``."""
    r = repr(float(x))
    return r


@dataclasses.dataclass
class PlainCase:
    """One uniform-cooling CA run (realm type ``cellular_automata``)."""

    name: str
    cells: Tuple[int, int, int]
    cell_size: float
    origin: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    # surface / bulk nucleation: (site density, mean dTc, std dTc)
    surface: Tuple[float, float, float] = (0.0, 2.0, 0.5)
    bulk: Tuple[float, float, float] = (0.0, 3.0, 1.0)
    seed: int = 0
    initial_temperature: float = -0.2
    melting_temperature: float = 0.0
    t_dot: float = -20.0
    a: Tuple[float, float, float] = (-0.544e-4, 2.03e-4, 0.0)
    time_step: float = 0.001
    termination_time: float = 1.0e4
    time_step_factor_ca: Optional[float] = None
    max_half_diagonal_length: Optional[float] = None
    output_frequency: int = 0
    output_base: str = "./Results/Grains"
    output_variables: Sequence[str] = ("grain_ID",)
    output_format: Optional[str] = None  # "appended": binary VTR pieces (a key the reference ignores)
    microstructure_file: Optional[str] = None
    shuffle_vtr: bool = False
    shuffle_vtk: Optional[bool] = None

    @property
    def n_interior(self) -> int:
        return self.cells[0] * self.cells[1] * self.cells[2]

    @property
    def n_ghost(self) -> int:
        return (self.cells[0] + 2) * (self.cells[1] + 2) * (self.cells[2] + 2)

    def trunc_coeff(self) -> float:
        """Octahedron truncation coefficient as the reference stores it:
        ``sqrtf(3.0)`` by default (CA/src/Octahedron.cpp:25), else
        ``sqrtf(2)*f*0.5`` (CA/src/Octahedron.cpp:316-320), float sqrt promoted."""
        import numpy as np

        if self.max_half_diagonal_length is not None and self.max_half_diagonal_length > 0:
            return float(np.float32(np.sqrt(np.float32(2.0)))) * self.max_half_diagonal_length * 0.5
        return float(np.float32(np.sqrt(np.float32(3.0))))

    def to_yaml(self) -> str:
        nx, ny, nz = self.cells
        ns, mus, sgs = self.surface
        nv, muv, sgv = self.bulk
        a1, a2, a3 = self.a
        opts = ["         - random_type:", "             rejection_sampling: no"]
        if self.shuffle_vtr:
            opts.append("             shuffer_vtr_grain_ID: yes")
        if self.shuffle_vtk is not None:
            opts.append(f"             shuffer_vtk_grain_ID: {'yes' if self.shuffle_vtk else 'no'}")
        if self.microstructure_file:
            opts += ["         - output_microstructure_information:",
                     f"             file_name: {self.microstructure_file}"]
        if self.max_half_diagonal_length is not None:
            opts += ["         - envelope:",
                     f"             max_half_diagonal_length: {_num(self.max_half_diagonal_length)}"]
        ti = [f"      termination_time: {_num(self.termination_time)}",
              f"      time_step: {_num(self.time_step)}"]
        if self.time_step_factor_ca is not None:
            ti.append(f"      time_step_factor_ca: {_num(self.time_step_factor_ca)}")
        outv = "\n".join(f"        - {v}" for v in self.output_variables)
        fmt = f"\n      output_format: {self.output_format}" if self.output_format else ""
        return f"""# {self.name} (seed {self.seed})
simulations:
  - name: {self.name}
    time_integrator: ti_1

solvers:
   - cellular_automata

realms:
  - name: realm1
    type: cellular_automata
    dimension: 3

    domain:
      type: cubic
      original_point: [{_num(self.origin[0])}, {_num(self.origin[1])}, {_num(self.origin[2])}]

    discretization:
      cell_size: {_num(self.cell_size)}
      number_cells: [{nx}, {ny}, {nz}]

    nucleation_rules:
      - surface:
          type: Gaussian
          site_density: {_num(ns)}
          mean: {_num(mus)}
          standard_deviation: {_num(sgs)}

      - bulk:
          type: Gaussian
          site_density: {_num(nv)}
          mean: {_num(muv)}
          standard_deviation: {_num(sgv)}

    problem_physics:
        type: RappazGandin
        initial_temperature: {_num(self.initial_temperature)}
        melting_temperature: {_num(self.melting_temperature)}
        t_dot: {_num(self.t_dot)}
        a1: {_num(a1)}
        a2: {_num(a2)}
        a3: {_num(a3)}

    solution_options:
       name: my_options
       options:
{chr(10).join(opts)}

    output:
      output_data_base_name: {self.output_base}
      output_frequency: {self.output_frequency}{fmt}
      output_variables:
{outv}

time_integrators:
  - standard_time_integrator:
      name: ti_1
{chr(10).join(ti)}
      realms:
        - realm1
"""


def bulk_density_for_sites(sites: float, cells: Tuple[int, int, int], h: float) -> float:
    """Bulk site density giving ``sites`` draws by the reference's count
    ``int(round(h^3 * n_v * N) + 0.5)`` (CA/src/CellularAutomataManager.cpp:171)."""
    n = cells[0] * cells[1] * cells[2]
    return sites / (h * h * h * n)


def surface_density_for_sites(sites: float, cells: Tuple[int, int, int], h: float) -> float:
    """Surface site density giving ``sites`` draws. The reference's surface
    list holds each face cell once per face it lies on
    (CA/src/CellularAutomataManager_3D.cpp:958-1000), i.e. 2(nx ny + nx nz + ny nz)
    entries for nx >= ny."""
    nx, ny, nz = cells
    n = 2 * (nx * ny + nx * nz + ny * nz)
    return sites / (h * h * n)


# ---------------------------------------------------------------------------
# The workloads this library is measured on.
# ---------------------------------------------------------------------------

def config_nucleation_60() -> PlainCase:
    """The reference's own nucleation example (example/nucleation/Inputfile.i):
    60^3 cells of 0.5 mm, bulk Gaussian sites 1e7 m^-3 (mean 3 K, std 1 K),
    T0 = -0.2, t_dot = -20 K/s, seed 0."""
    return PlainCase(name="nucleation_60", cells=(60, 60, 60), cell_size=0.0005,
                     surface=(0.0, 2.0, 0.5), bulk=(10e6, 3.0, 1.0), seed=0,
                     t_dot=-20.0, time_step=0.001, termination_time=17.81)


def config_uniform_320() -> PlainCase:
    """Uniform cooling at scale: 320^3 cells of 2 um, t_dot = -50 K/s, about
    20,000 bulk sites (mean 3 K, std 1 K) and about 4,000 surface sites on all
    six faces (mean 2 K, std 0.5 K), seed 1."""
    cells = (320, 320, 320)
    h = 2e-6
    return PlainCase(name="uniform_320", cells=cells, cell_size=h,
                     surface=(surface_density_for_sites(4000, cells, h), 2.0, 0.5),
                     bulk=(bulk_density_for_sites(20000, cells, h), 3.0, 1.0),
                     seed=1, t_dot=-50.0, time_step=0.001, termination_time=1.0e4)


def batched_instances(count: int, seed: int, edges=(32, 128), t_dot=(-200.0, -5.0), sites=(50, 2000),
                      cell_size: float = 2e-6, prefix: str = "batched") -> list:
    """Independent uniform-cooling instances: cube edges uniform on the
    integers edges[0]..edges[1], t_dot log-uniform on t_dot, bulk Gaussian
    sites (mean 3 K, std 1 K) with a density that draws a uniform integer
    count in sites[0]..sites[1], no surface sites, the KGT coefficients and
    temperatures of nucleation_60, and seed 0 (the reference's srand at np=1).
    Draws come from Python's Mersenne Twister ``random()`` alone, whose
    sequence for a seed is fixed across Python versions."""
    import random

    rng = random.Random(seed)
    out = []
    lo_t, hi_t = math.log(-t_dot[1]), math.log(-t_dot[0])
    for i in range(count):
        e = edges[0] + int(rng.random() * (edges[1] - edges[0] + 1))
        td = -math.exp(lo_t + rng.random() * (hi_t - lo_t))
        ns = sites[0] + int(rng.random() * (sites[1] - sites[0] + 1))
        cells = (e, e, e)
        out.append(PlainCase(name=f"{prefix}_{i:02d}", cells=cells, cell_size=cell_size,
                             surface=(0.0, 2.0, 0.5), bulk=(bulk_density_for_sites(ns, cells, cell_size), 3.0, 1.0),
                             seed=0, t_dot=td, time_step=0.001, termination_time=1.0e4))
    return out


def config_batched_64() -> list:
    """64 independent uniform-cooling instances: edges 32..128 cells of 2 um
    (seed 3), t_dot log-uniform on [-200, -5] K/s, 50..2,000 bulk sites each;
    about 44M interior cells in all."""
    return batched_instances(64, 3)


@dataclasses.dataclass
class RemeltCase:
    """One FE-coupled remelting run: a ``finite_element`` realm that replays
    nodal temperature frames from a text file and a
    ``cellular_automata_remelting`` realm, coupled by ``transfers``
    (CA/src/CafeSolver.cpp:40-137, CA/src/FiniteElementManager.cpp:66-142,
    CA/src/MapVoxelManager.cpp:62-89,
    CA/src/CellularAutomataManager_3DRemelting.cpp:51-76)."""

    name: str
    cells: Tuple[int, int, int]
    cell_size: float
    origin: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    frames_file: str = "./frames.txt"
    length_scale: float = 1.0
    time_scale: float = 1.0
    lines_for_title: int = 4
    lines_for_subtitle: int = 5
    offset: Tuple[float, float, float] = (0.0, 0.0, 0.0)
    bin_size: Tuple[int, int, int] = (5, 5, 5)
    tolerance: float = 1.0e-16
    max_iterations: int = 20
    void_temperature: Optional[float] = None
    surface: Tuple[float, float, float] = (0.0, 0.5, 0.1)
    bulk: Tuple[float, float, float] = (0.0, 10.0, 1.0)
    nucleation: bool = False
    seed: int = 0
    melting_temperature: float = 1700.0
    solidus_temperature: float = 1600.0
    min_nucleation_temperature: Optional[float] = None
    a: Tuple[float, float, float] = (0.0, 2.03e-4, 0.0)
    has_been_melted: bool = False
    cutoff_factor: Optional[float] = 4.0
    microstructure: str = "random"
    load_seeds: bool = False
    output_microstructure_file: Optional[str] = None
    shuffle_vtr: bool = False
    termination_time: float = 1.0
    time_step: float = 1.0e-6
    time_step_factor: float = 0.4
    time_step_factor_ca: Optional[float] = None
    output_base: str = "./Results/Grains"
    output_frequency: int = 100000
    output_variables: Sequence[str] = ("grain_orientation",)
    output_format: Optional[str] = None  # "appended": binary VTR pieces (a key the reference ignores)

    @property
    def n_interior(self) -> int:
        return self.cells[0] * self.cells[1] * self.cells[2]

    @property
    def n_ghost(self) -> int:
        return (self.cells[0] + 2) * (self.cells[1] + 2) * (self.cells[2] + 2)

    def to_yaml(self) -> str:
        nx, ny, nz = self.cells
        ns, mus, sgs = self.surface
        nv, muv, sgv = self.bulk
        a1, a2, a3 = self.a
        tr = [f"     bin_size: [{self.bin_size[0]}, {self.bin_size[1]}, {self.bin_size[2]}]",
              f"     tolerance: {_num(self.tolerance)}",
              f"     max_iterations: {self.max_iterations}"]
        if self.void_temperature is not None:
            tr.append(f"     void_temperature: {_num(self.void_temperature)}")
        phys = [f"        melting_temperature: {_num(self.melting_temperature)}",
                f"        solidus_temperature: {_num(self.solidus_temperature)}"]
        if self.min_nucleation_temperature is not None:
            phys.append(f"        minimum_temperature_for_nucleation: {_num(self.min_nucleation_temperature)}")
        phys += [f"        a1: {_num(a1)}", f"        a2: {_num(a2)}", f"        a3: {_num(a3)}"]
        opts = ["         - random_type:", "             rejection_sampling: no"]
        if self.shuffle_vtr:
            opts.append("             shuffer_vtr_grain_ID: yes")
        opts += ["         - phase_state:",
                 f"             has_been_melted: {'yes' if self.has_been_melted else 'no'}"]
        if self.cutoff_factor is not None:
            opts += ["         - cell_grain_length_cutoff_factor:",
                     f"             factor_value: {_num(self.cutoff_factor)}"]
        if self.output_microstructure_file:
            opts += ["         - output_microstructure_information:",
                     f"             file_name: {self.output_microstructure_file}"]
        opts += ["         - load_microstructure_information:",
                 f"             file_name: {self.microstructure}"]
        if self.load_seeds:
            opts.append("             load_seeds: yes")
        opts += ["         - criterion_to_activate_grain:",
                 f"             using_nucleation_seed: {'yes' if self.nucleation else 'no'}"]
        ti = [f"      termination_time: {_num(self.termination_time)}",
              f"      time_step: {_num(self.time_step)}",
              f"      time_step_factor: {_num(self.time_step_factor)}"]
        if self.time_step_factor_ca is not None:
            ti.append(f"      time_step_factor_ca: {_num(self.time_step_factor_ca)}")
        outv = "\n".join(f"        - {v}" for v in self.output_variables)
        fmt = f"\n      output_format: {self.output_format}" if self.output_format else ""
        return f"""# {self.name} (seed {self.seed})
simulations:
  - name: {self.name}
    time_integrator: ti_1

solvers:
   - cellular_automata
   - finite_element_method

transfers:
   - name: fe_ca
{chr(10).join(tr)}

realms:

  - name: realm0
    type: finite_element
    dimension: 3
    mesh: {self.frames_file}

    solution_options:
       name: my_options
       options:
         - load_data_from_file:
             theta: theta
             for_whole_time: yes
             length_scale: {_num(self.length_scale)}
             time_scale: {_num(self.time_scale)}
             lines_for_title: {self.lines_for_title}
             lines_for_subtitle: {self.lines_for_subtitle}
             x_offset: {_num(self.offset[0])}
             y_offset: {_num(self.offset[1])}
             z_offset: {_num(self.offset[2])}

    output:
      output_data_base_name: ./Results/FEM
      output_frequency: 100000000
      output_variables:
        - temperature

  - name: realm1
    type: cellular_automata_remelting
    dimension: 3

    domain:
      type: cubic
      original_point: [{_num(self.origin[0])}, {_num(self.origin[1])}, {_num(self.origin[2])}]

    discretization:
      cell_size: {_num(self.cell_size)}
      number_cells: [{nx}, {ny}, {nz}]

    nucleation_rules:
      - surface:
          type: Gaussian
          site_density: {_num(ns)}
          mean: {_num(mus)}
          standard_deviation: {_num(sgs)}

      - bulk:
          type: Gaussian
          site_density: {_num(nv)}
          mean: {_num(muv)}
          standard_deviation: {_num(sgv)}

    problem_physics:
        type: RappazGandin
{chr(10).join(phys)}

    solution_options:
       name: my_options
       options:
{chr(10).join(opts)}

    output:
      output_data_base_name: {self.output_base}
      output_frequency: {self.output_frequency}{fmt}
      output_variables:
{outv}

time_integrators:
  - standard_time_integrator:
      name: ti_1
{chr(10).join(ti)}
      realms:
        - realm0
        - realm1
"""


# ---------------------------------------------------------------------------
# Synthetic FE inputs: Rosenthal frames and columnar restart microstructures.
# The reference's PBF examples ship without their temperature histories;
# these stand in for them in the reference's own file formats.
# ---------------------------------------------------------------------------
LN2 = 0.6931471805599453
INV_LN2 = 1.4426950408889634
EXP_TAYLOR = [1.0 / math.factorial(n) for n in range(14)]


def det_exp(a):
    """exp(a) for a <= 0 from IEEE add/mul and ldexp only: k = rint(a/ln2),
    r = a - k ln2, a degree-13 Taylor polynomial in Horner form, times 2^k.
    Relative error below 1e-13; the point is that it is the same double on
    every IEEE platform (no libm, no contraction), host or device
    (amca_set_rosenthal_frames evaluates the same operations on the GPU)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    a = np.maximum(a, -700.0)
    k = np.rint(a * INV_LN2)
    r = a - k * LN2
    p = np.full_like(r, EXP_TAYLOR[13])
    for n in range(12, -1, -1):
        p = p * r + EXP_TAYLOR[n]
    return np.ldexp(p, k.astype(np.int64))


@dataclasses.dataclass
class Rosenthal:
    """Quasi-steady field of a point source moving along +x on the top surface
    of a semi-infinite body (SI units):
    T = t0 + (A P)/(2 pi k R) exp(-v (R + xi)/(2 alpha)), xi = x - (x_start + v t),
    capped at t_cap near the source."""

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
        import numpy as np

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


@dataclasses.dataclass
class FrameSpec:
    """Structured FE node grid and frame times in file units; the text format
    is the reference's (CA/src/LoadDataFromFile.cpp:21-191): title lines, then
    per frame a subtitle whose 4th line holds "step step time time x0 x1 y0 y1
    z0 z1" and one "x y z T" line per node, x fastest. Values are written with
    17 significant digits, so every reader sees the same doubles."""

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
        import numpy as np

        nx, ny, nz = self.nodes
        K, J, I = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        x = self.origin[0] + self.spacing * I
        y = self.origin[1] + self.spacing * J
        z = self.origin[2] + self.spacing * K
        return x.ravel(), y.ravel(), z.ravel()

    def frame_values(self, f: int):
        x, y, z = self.node_coords()
        s = self.length_scale
        return self.source.field(x * s, y * s, z * s, (f * self.frame_dt) * self.time_scale)

    def write(self, path: str, title_lines: int = 4) -> None:
        nx, ny, nz = self.nodes
        x, y, z = self.node_coords()
        xyz = [f"{a!r} {b!r} {c!r}" for a, b, c in zip(x.tolist(), y.tolist(), z.tolist())]
        with open(path, "w") as f:
            for t in range(title_lines):
                f.write("Title\n" if t == 0 else ("End of title\n" if t == title_lines - 1
                                                   else "synthetic Rosenthal frames\n"))
            for fr in range(self.frames):
                T = self.frame_values(fr)
                tt = self.time_offset + fr * self.frame_dt
                f.write("\n")
                f.write("Subtitle\n")
                f.write("No. step   No. step    time   time   x0    x1   y0   y1    z0   z1\n")
                f.write(f"{fr + 1} {fr + 1} {tt!r} {tt!r} 0 {nx - 1} 0 {ny - 1} 0 {nz - 1}\n")
                f.write("x  y  z  tn\n")
                f.write("".join(f"{p} {v!r}\n" for p, v in zip(xyz, T.tolist())))

    def rosenthal_kwargs(self) -> dict:
        """Arguments of CellularAutomataRealm.set_rosenthal_frames for these frames."""
        s = self.source
        return dict(origin=self.origin, spacing=self.spacing, nodes=self.nodes, frames=self.frames,
                    length_scale=self.length_scale, frame_dt=self.frame_dt, time_scale=self.time_scale,
                    time_offset=self.time_offset, power=s.power, absorptivity=s.absorptivity, speed=s.speed,
                    conductivity=s.conductivity, diffusivity=s.diffusivity, t0=s.t0, t_cap=s.t_cap,
                    x_start=s.x_start, y_line=s.y_line, z_top=s.z_top,
                    void_above_set=0 if s.void_above is None else 1,
                    void_above=0.0 if s.void_above is None else s.void_above, t_void=s.t_void)


def columnar_microstructure(cells, cell_size: float, origin, grains: int, seed: int, grainless_mod: int = 0) -> dict:
    """Restart microstructure (the content of grainInfo<rank>.txt) of
    `grains` columnar grains: Voronoi regions of seed points in the x-y plane,
    extruded in z. Every interior cell is its own grain object with its
    region's orientation; ghost cells hold grain and orientation -1. With
    grainless_mod > 0, interior cells with (i + 2j + 3k) % grainless_mod == 0
    keep the orientation but get no grain object. Returns the arrays of
    CellularAutomataRealm.set_microstructure."""
    import numpy as np

    rng = np.random.default_rng(seed)
    nx, ny, nz = cells
    h = cell_size
    gx, gy, gz = nx + 2, ny + 2, nz + 2
    pts = rng.random((grains, 2)) * np.array([nx * h, ny * h]) + np.array(origin[:2])
    # products of uniform draws and constants only: the same doubles on every platform
    euler = np.stack([rng.random(grains) * (2 * math.pi), rng.random(grains) * math.pi,
                      rng.random(grains) * (0.5 * math.pi)], axis=1)
    cx = origin[0] + h * (np.arange(1, nx + 1) - 0.5)
    cy = origin[1] + h * (np.arange(1, ny + 1) - 0.5)
    CY, CX = np.meshgrid(cy, cx, indexing="ij")
    CX, CY = CX.ravel(), CY.ravel()
    region = np.empty(CX.size, np.int64)
    for lo in range(0, CX.size, 8192):  # nearest seed, lowest index on ties
        hi = min(CX.size, lo + 8192)
        d2 = (CX[lo:hi, None] - pts[:, 0]) ** 2 + (CY[lo:hi, None] - pts[:, 1]) ** 2
        region[lo:hi] = np.argmin(d2, axis=1)
    region = region.reshape(ny, nx)
    K, J, I = np.meshgrid(np.arange(1, nz + 1), np.arange(1, ny + 1), np.arange(1, nx + 1), indexing="ij")
    K, J, I = K.ravel(), J.ravel(), I.ravel()
    cell = K * gx * gy + J * gx + I
    orient = np.full(gx * gy * gz, -1, np.int32)
    grain = np.full(gx * gy * gz, -1, np.int32)
    orient[cell] = region[J - 1, I - 1]
    has = np.ones(cell.size, bool) if not grainless_mod else (I + 2 * J + 3 * K) % grainless_mod != 0
    gcell = cell[has]
    grain[gcell] = np.arange(gcell.size, dtype=np.int32)
    return dict(grain=grain, orient=orient, euler=euler, grain_cell=gcell.astype(np.int32),
                grain_orient=orient[gcell].astype(np.int32), expected=grains,
                grain_centre=np.stack([origin[0] + h * (I[has] - 0.5), origin[1] + h * (J[has] - 0.5),
                                       origin[2] + h * (K[has] - 0.5)], axis=1))


def write_restart(path: str, m: dict, origin, cells, cell_size: float) -> str:
    """Write a columnar_microstructure() as the reference's restart file
    ("<stem>0.txt" for the stem of `path`); returns the file written."""
    import numpy as np

    nx, ny, nz = cells
    gx, gy, gz = nx + 2, ny + 2, nz + 2
    ncell = gx * gy * gz
    stem = path[: path.rfind(".")] if "." in os.path.basename(path) else path
    out = stem + "0.txt"
    grain, orient, euler = m["grain"], m["orient"], m["euler"]
    with open(out, "w") as f:
        f.write("numCell; numOrientation; numLocalGrain; numGlobalExpectedGrain; start Point X; Y; Z; "
                "number Point nx; ny; nz; dCell\n")
        f.write(f"{ncell}  {len(euler)}  {len(m['grain_cell'])}  {m['expected']}  {float(origin[0])!r}  "
                f"{float(origin[1])!r}  {float(origin[2])!r}  {gx}  {gy}  {gz}  {float(cell_size)!r}\n")
        f.write("Cell informatin: ID; grainID; orientationID; hasBeenMelted; undercooling of seed\n")
        f.write("".join(f"{c}  {g}  {o}  0  -1\n" for c, (g, o) in enumerate(zip(grain.tolist(), orient.tolist()))))
        f.write("Orientation informatin: ID; EularAngle\n")
        f.write("".join(f"{o}  {a!r}  {b!r}  {c!r}  \n" for o, (a, b, c) in enumerate(euler.tolist())))
        f.write("Grain information: ID; cellID; grainCenter; orientationID\n")
        cen = m["grain_centre"].tolist()
        f.write("".join(f"{g}  {c}  {x!r}  {y!r}  {z!r}  {o}   \n"
                        for g, (c, (x, y, z), o) in enumerate(zip(m["grain_cell"].tolist(), cen,
                                                                   m["grain_orient"].tolist()))))
    return out


def config_pbf_500():
    """A laser powder-bed-fusion track, the FE-coupled workload: 500 x 250 x
    100 cells of 2 um (12.5M) on a columnar baseplate of 2,000 grains (seed 2),
    one laser pass along x at mid-width on the top surface. Frames every 1 us
    on 10 um FE nodes from the Rosenthal field (P = 200 W, A = 0.4, v = 1 m/s,
    k = 20 W/(m K), alpha = 5e-6 m^2/s, T0 = 300 K), 1,550 frames (the source
    runs from x = -50 um to 1.5 mm, past the melt-pool tail). Liquidus 1700 K,
    solidus 1600 K, bulk sites 1e13 m^-3 (mean 8 K, std 2 K), KGT a2 = 2.03e-4.
    Returns (deck, frames, microstructure arrays)."""
    case = RemeltCase(name="pbf_500", cells=(500, 250, 100), cell_size=2.0e-6, nucleation=True, seed=2,
                      bulk=(1.0e13, 8.0, 2.0), surface=(0.0, 0.5, 0.1), melting_temperature=1700.0,
                      solidus_temperature=1600.0, a=(0.0, 2.03e-4, 0.0), microstructure="baseplate.txt",
                      termination_time=1.0, time_step=1.0e-6, time_step_factor=0.4)
    frames = pbf_frames(case.cells, case.cell_size, 1550)
    micro = columnar_microstructure(case.cells, case.cell_size, case.origin, 2000, 2)
    return case, frames, micro


def pbf_frames(cells, cell_size: float, nframes: int) -> FrameSpec:
    """Rosenthal frames of the PBF workload for a block of `cells`: 10 um
    nodes from -10 um to one node past the block, the track at mid-width on
    the top surface."""
    nx, ny, nz = cells
    sp = 1.0e-5
    nodes = tuple(int(math.ceil(n * cell_size / sp)) + 3 for n in (nx, ny, nz))
    src = Rosenthal(power=200.0, absorptivity=0.4, speed=1.0, conductivity=20.0, diffusivity=5.0e-6, t0=300.0,
                    t_cap=3000.0, x_start=-5.0e-5, y_line=0.5 * ny * cell_size, z_top=nz * cell_size)
    return FrameSpec(origin=(-sp, -sp, -sp), spacing=sp, nodes=nodes, frame_dt=1.0e-6, frames=nframes, source=src)


# ---------------------------------------------------------------------------
# Thermal model workload: a multi-track raster scan over a large block, with
# the FE field or the learned model as the frame source.
# ---------------------------------------------------------------------------
def thermal_spec(seed: int = 4, fourier_sigma: float = 0.5, fourier_sigma_pv: float = 0.1, log_output: int = 0,
                 near_fraction: float = 0.3, shell_fraction: float = 0.4) -> dict:
    """amca_thermal_spec of the learned thermal model: laser power 150-350 W,
    scan speed 0.5-1.5 m/s, the PBF physics (A = 0.4, k = 20 W/(m K),
    alpha = 5e-6 m^2/s, T0 = 300 K, cap 3000 K), a window from 1.2 mm behind
    to 0.15 mm ahead of the source, +-0.25 mm across and 0.3 mm deep; of the
    samples, near_fraction from the melt-pool box (the region where the field
    exceeds 1450 K anywhere in the power and speed ranges) and shell_fraction
    from that box until the field lies between 1450 and 1950 K (around the
    1600-1700 K mushy zone); T = 300 K + 1000 K * output, or
    299 K + 100 K * exp(output) with log_output."""
    return dict(power_lo=150.0, power_hi=350.0, speed_lo=0.5, speed_hi=1.5, absorptivity=0.4, conductivity=20.0,
                diffusivity=5.0e-6, t0=300.0, t_cap=3000.0,
                window_lo=(-1.2e-3, -0.25e-3, -0.02e-3), window_hi=(0.15e-3, 0.25e-3, 0.3e-3),
                near_lo=(-1.05e-3, -0.14e-3, -0.01e-3), near_hi=(0.06e-3, 0.14e-3, 0.14e-3),
                near_fraction=near_fraction, shell_lo=1450.0, shell_hi=1950.0, shell_fraction=shell_fraction,
                fourier_sigma=fourier_sigma, fourier_sigma_pv=fourier_sigma_pv, log_output=log_output,
                t_shift=299.0 if log_output else 300.0, t_scale=100.0 if log_output else 1000.0, seed=seed)


# Training schedule of the learned thermal model: 50M samples (seed 4), Adam
# 1e-3 -> 1e-5 on a cosine schedule, 20,000 steps of 32,768.
THERMAL_TRAIN = dict(samples=50_000_000, steps=20_000, batch=32_768, lr_max=1.0e-3, lr_min=1.0e-5)


def scan_of(cells, cell_size: float, tracks: int, hatch: float, power: float = 200.0, speed: float = 1.0,
            margin_start: float = 5.0e-5, margin_end: float = 5.0e-4, frame_dt: float = 1.0e-6) -> dict:
    """amca_scan fields of a raster of `tracks` passes along x over a block of
    `cells`: 10 um FE nodes from -10 um to one node past the block, tracks
    centred across y with `hatch` spacing on the top surface, alternating
    direction; each pass runs from margin_start before the block to margin_end
    past it (the melt-pool tail leaves the block) at `speed`, frames every
    frame_dt for the whole scan."""
    nx, ny, nz = cells
    sp = 1.0e-5
    nodes = tuple(int(math.ceil(n * cell_size / sp)) + 3 for n in (nx, ny, nz))
    length = nx * cell_size
    track_time = (margin_start + length + margin_end) / speed
    y0 = 0.5 * ny * cell_size - 0.5 * (tracks - 1) * hatch
    frames = int(math.ceil(tracks * track_time / frame_dt)) + 2
    return dict(origin=(-sp, -sp, -sp), spacing=sp, nodes=nodes, frames=frames, length_scale=1.0,
                frame_dt=frame_dt, time_scale=1.0, time_offset=0.0, power=power, absorptivity=0.4, speed=speed,
                conductivity=20.0, diffusivity=5.0e-6, t0=300.0, t_cap=3000.0, x_start=-margin_start,
                x_turn=length + margin_start, y_line=y0, z_top=nz * cell_size, hatch=hatch, track_time=track_time,
                ntracks=tracks)


def config_thermal_block(name: str, cells, tracks: int, hatch: float, grains: int, seed: int = 4):
    """A raster-scan workload on a columnar baseplate with the PBF physics:
    liquidus 1700 K, solidus 1600 K, bulk sites 1e13 m^-3 (8 K, 2 K), KGT
    a2 = 2.03e-4, 2 um cells, 200 W at 1 m/s. Returns (deck, scan fields,
    microstructure arrays)."""
    case = RemeltCase(name=name, cells=tuple(cells), cell_size=2.0e-6, nucleation=True, seed=seed,
                      bulk=(1.0e13, 8.0, 2.0), surface=(0.0, 0.5, 0.1), melting_temperature=1700.0,
                      solidus_temperature=1600.0, a=(0.0, 2.03e-4, 0.0), microstructure="baseplate.txt",
                      termination_time=1.0, time_step=1.0e-6, time_step_factor=0.4)
    scan = scan_of(cells, case.cell_size, tracks=tracks, hatch=hatch)
    micro = columnar_microstructure(cells, case.cell_size, case.origin, grains, seed)
    return case, scan, micro


def config_thermal_1024():
    """The learned-model workload: a 5-track raster (100 um hatch, alternating
    direction, 200 W, 1 m/s) over 1024 x 512 x 256 cells of 2 um (134M) on a
    columnar baseplate of 8,000 grains (seed 4)."""
    return config_thermal_block("thermal_1024", (1024, 512, 256), tracks=5, hatch=1.0e-4, grains=8000)
