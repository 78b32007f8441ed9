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
      output_frequency: {self.output_frequency}
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
      output_frequency: {self.output_frequency}
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
