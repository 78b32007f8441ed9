// deck.h — the realm configuration read from an AMCA3D YAML deck.
//
// Keys, defaults and required/optional status follow the reference loaders:
//   Simulation::load                      CA/src/Simulation.cpp:36-74
//   CellularAutomataSolver::load          CA/src/CellularAutomataSolver.cpp:40-130
//   CellularAutomataManager_3D::load      CA/src/CellularAutomataManager_3D.cpp:71-361
//   CellularAutomataManager ctor defaults CA/src/CellularAutomataManager.cpp:32-68
//   ProblemPhysics_RappazGandin1993::load CA/src/ProblemPhysics.cpp:33-102
//   VtrManager::load                      CA/src/VtrManager.cpp:60-103
#pragma once

#include <string>
#include <vector>

namespace amca {

struct OutputConfig {
  int frequency = 0;                       // output_frequency (< 1: time based)
  std::string base = "./Results/Grains";   // output_data_base_name
  double time_interval = 0.0;              // output_time_interval
  bool time_interval_set = false;
  std::vector<int> variables;              // ids into the reference's variable-name table
  // output_format: "ascii" (the reference's text pieces, default) or
  // "appended" (the same arrays as raw little-endian binary in one appended
  // block; a key of this library, which the reference does not read)
  bool appended = false;
};

struct PlainConfig {
  std::string realm_type;  // "cellular_automata"
  int dimension = 3;
  // domain / discretization
  double x0 = 0, y0 = 0, z0 = 0, h = 0;
  int nx = 0, ny = 0, nz = 0;
  // nucleation_rules (CellularAutomataManager.cpp:48-53 defaults)
  double ns = 0.0, mu_s = 0.5, sigma_s = 0.1;
  double nv = 0.0, mu_v = 6.0, sigma_v = 0.1;
  // solution_options
  bool shuffle_vtr = false, shuffle_vtk = false;
  bool micro_out = false;
  std::string micro_out_file;
  bool micro_out_seeds = false;
  double trunc_coeff = 0.0;           // Octahedron truncation (default (double)sqrtf(3.0f))
  double length_cutoff_factor = 1e8;  // cell_grain_length_cutoff_factor (times h)
  // problem_physics (RappazGandin)
  double T0 = 300.0, Tm = 0.0, Ts = -1.0e8, Tmin_nuc = -1.0e8, Tdot = -2.3;
  double a1 = 0.0, a2 = 0.0, a3 = 0.0, b1 = 1.0, b2 = 2.0, b3 = 3.0;
  // time integrator
  double final_time = 0.0, max_dt = 0.0;
  int max_steps = 1000;
  double time_step_factor = 0.2;
  OutputConfig output;
};

// Parse a deck for the plain CA solver (solvers: [cellular_automata], realm
// type cellular_automata, dimension 3). Throws std::runtime_error with a
// message naming the key (and line) on a missing key or unsupported content.
PlainConfig parse_plain_deck(const std::string &yaml_text);

// finite_element realm replaying temperature frames from a text file
// (FiniteElementManager::load, CA/src/FiniteElementManager.cpp:66-142).
struct FeConfig {
  std::string mesh;               // frame file (realm key "mesh")
  int title_lines = -1;           // load_data_from_file.lines_for_title (no default in the reference)
  int subtitle_lines = -1;        // lines_for_subtitle (>= 4; the 4th holds step and time)
  double length_scale = 1.0, time_scale = 1.0;
  double offset[3] = {0.0, 0.0, 0.0};
  bool whole_time = false;        // for_whole_time: replay frames instead of solving
  int output_frequency = 0;       // VtuManager output_frequency
};

// transfers (MapVoxelManager::load, CA/src/MapVoxelManager.cpp:26-89)
struct TransferConfig {
  int bin[3] = {10, 10, 10};
  double tolerance = 1.0e-16;
  int max_iter = 20;
  double void_temperature = -1.0e8;
};

// FE-coupled remelting deck: solvers [cellular_automata, finite_element_method],
// a finite_element realm and a cellular_automata_remelting realm
// (CafeSolver::load, CA/src/CafeSolver.cpp:40-137;
// CellularAutomataManager_3DRemelting::load, CA/src/CellularAutomataManager_3DRemelting.cpp:51-76).
struct RemeltConfig {
  PlainConfig ca;                 // grid, nucleation rules, physics, CA options, VTR output
  FeConfig fe;
  TransferConfig tr;
  bool nucleation = false;        // criterion_to_activate_grain.using_nucleation_seed (setNucleationSite_)
  bool initial_melted = true;     // phase_state.has_been_melted (setInitialStatedAsMelted_)
  bool random_micro = true;       // load_microstructure_information.file_name: random (or no option)
  std::string micro_file;         // restart file stem (rank suffix "0.txt" appended)
  bool load_seeds = false;        // load_microstructure_information.load_seeds
  double time_step_factor_fe = 0; // time_step_factor (read by CafeSolver, unused when replaying frames)
};

// true when the deck selects both the CA and the FE solver (CafeSolver)
bool deck_is_coupled(const std::string &yaml_text);

// Parse an FE-coupled remelting deck (throws like parse_plain_deck).
RemeltConfig parse_remelt_deck(const std::string &yaml_text);

// The reference's output variable names (CA/include/CafeMacro.h:16-24).
int output_variable_id(const std::string &name);

}  // namespace amca
