// deck.cpp — see deck.h.
#include "deck.h"

#include <cmath>
#include <stdexcept>

#include "yaml_lite.h"

namespace amca {

namespace {

using yaml::Node;

[[noreturn]] void fail(const std::string &what, const Node *at = nullptr) {
  throw std::runtime_error(at ? what + " (line " + std::to_string(at->line()) + ")" : what);
}

const Node &required(const Node &map, const std::string &key) {
  const Node *v = map.find(key);
  if (!v) fail("parsing missing required key: " + key, &map);
  return *v;
}

void opt_double(const Node &map, const std::string &key, double &out) {
  if (const Node *v = map.find(key)) out = v->as_double();
}
void opt_int(const Node &map, const std::string &key, int &out) {
  if (const Node *v = map.find(key)) out = v->as_int();
}
void opt_bool(const Node &map, const std::string &key, bool &out) {
  if (const Node *v = map.find(key)) out = v->as_bool();
}

// operator>>(node, double*) / (node, int*): two or three components
// (CA/src/CafeParsing.cpp:67-83).
void read3(const Node &seq, double out[3]) {
  if (!seq.is_seq()) fail("expected a sequence", &seq);
  out[0] = seq.at(0).as_double();
  out[1] = seq.at(1).as_double();
  if (seq.size() > 2) out[2] = seq.at(2).as_double();
}
void read3(const Node &seq, int out[3]) {
  if (!seq.is_seq()) fail("expected a sequence", &seq);
  out[0] = seq.at(0).as_int();
  out[1] = seq.at(1).as_int();
  if (seq.size() > 2) out[2] = seq.at(2).as_int();
}

// expect_map(node, key, optional=true): present but not a map is an error
// (CA/src/CafeParsing.cpp:86-121).
const Node *expect_map(const Node &node, const std::string &key) {
  const Node *v = node.find(key);
  if (v && !v->is_map()) fail("parsing expected type Map for key " + key + " - check indentation", v);
  return v;
}
const Node *expect_seq(const Node &node, const std::string &key) {
  const Node *v = node.find(key);
  if (v && !v->is_seq()) fail("parsing expected type Sequence for key " + key + " - check indentation", v);
  return v;
}

float sqrtf_ref(float x) { return std::sqrt(x); }

}  // namespace

int output_variable_id(const std::string &name) {
  static const char *names[] = {"temperature", "temperature_rate", "grain_ID",   "grain_orientation", "grain_velocity",
                                "element_birth", "melted_flag",    "phase_ID",   "alpha_phase",       "phase_orientation",
                                "velocity",      "debug",          "debugMC"};
  for (int i = 0; i < 13; ++i)
    if (name == names[i]) return i;
  return -1;
}

namespace {

std::unique_ptr<Node> parse_doc(const std::string &text) {
  std::unique_ptr<Node> doc;
  try {
    doc = yaml::parse(text);
  } catch (const yaml::ParseError &e) {
    throw std::runtime_error(std::string("YAML: ") + e.what());
  }
  if (!doc->is_map()) fail("the deck is not a YAML mapping");
  return doc;
}

// Simulation::load solver selection (CA/src/Simulation.cpp:36-74)
void solvers_of(const Node &doc, bool &ca, bool &fem) {
  const Node *solvers = doc.find("solvers");
  if (!solvers) fail("parser error: at least one solver should be specified!");
  ca = fem = false;
  for (size_t i = 0; i < solvers->size(); ++i) {
    const std::string n = solvers->at(i).as_string();
    if (n == "cellular_automata") ca = true;
    if (n == "finite_element_method") fem = true;
  }
}

// CellularAutomataManager_3D::load (+ the remelting additions when rm is set),
// ProblemPhysics_RappazGandin1993::load and VtrManager::load for one CA realm.
void parse_ca_realm(const Node &realm, PlainConfig &c, RemeltConfig *rm) {
  c.realm_type = required(realm, "type").as_string();
  opt_int(realm, "dimension", c.dimension);
  if (c.dimension != 3) fail("only 3-D CA realms are supported (dimension: 3)", &realm);

  const Node *domain = realm.find("domain");
  if (!domain) fail("parser error: realm-domain", &realm);
  if (domain->find("load_microstructure_information"))
    fail("domain.load_microstructure_information is not supported; use the solution option "
         "load_microstructure_information.file_name",
         domain);
  double origin[3] = {-1 - 1 - 1};
  double lateral[3] = {-1 - 1 - 1};
  int ncell[3] = {-1 - 1 - 1};
  read3(required(*domain, "original_point"), origin);
  if (const Node *ls = domain->find("lateral_sizes")) read3(*ls, lateral);
  const Node *disc = realm.find("discretization");
  if (!disc) fail("parser error: realm-discretization", &realm);
  const double dcell = required(*disc, "cell_size").as_double();
  if (lateral[0] < 0) {
    read3(required(*disc, "number_cells"), ncell);
  } else {
    for (int i = 0; i < 3; ++i) {
      ncell[i] = (int)(lateral[i] / dcell);  // implicit double -> int (truncation)
      lateral[i] = ncell[i] * dcell;
    }
  }
  c.x0 = origin[0];
  c.y0 = origin[1];
  c.z0 = origin[2];
  c.h = dcell;
  c.nx = ncell[0];
  c.ny = ncell[1];
  c.nz = ncell[2];
  if (c.nx < 1 || c.ny < 1 || c.nz < 1) fail("number of cells must be positive on every axis", disc);
  if (!(c.h > 0)) fail("cell_size must be positive", disc);
  if ((double)(c.nx + 2) * (c.ny + 2) * (c.nz + 2) > 2147483647.0)
    fail("grid too large: (nx+2)(ny+2)(nz+2) must fit a 32-bit cell index", disc);

  if (const Node *rules = realm.find("nucleation_rules")) {
    for (size_t i = 0; i < rules->size(); ++i) {
      const Node &r = rules->at(i);
      if (const Node *s = r.find("surface")) {
        required(*s, "type").as_string();
        c.ns = required(*s, "site_density").as_double();
        c.mu_s = required(*s, "mean").as_double();
        c.sigma_s = required(*s, "standard_deviation").as_double();
      }
      if (const Node *b = r.find("bulk")) {
        if (const Node *t = b->find("type")) t->as_string();
        c.nv = required(*b, "site_density").as_double();
        c.mu_v = required(*b, "mean").as_double();
        c.sigma_v = required(*b, "standard_deviation").as_double();
      }
    }
  }

  c.trunc_coeff = (double)sqrtf_ref(3.0f);  // Octahedron::Octahedron (CA/src/Octahedron.cpp:25)
  bool random_micro = false, load_micro = false;
  int criterion = -1;
  if (const Node *so = realm.find("solution_options")) {
    required(*so, "name").as_string();
    if (const Node *opts = expect_seq(*so, "options")) {
      for (size_t i = 0; i < opts->size(); ++i) {
        const Node &o = opts->at(i);
        if (const Node *m = expect_map(o, "output_microstructure_information")) {
          c.micro_out_file = required(*m, "file_name").as_string();
          c.micro_out = true;
          opt_bool(*m, "output_seeds", c.micro_out_seeds);
        } else if (const Node *m2 = expect_map(o, "random_type")) {
          opt_bool(*m2, "shuffer_vtr_grain_ID", c.shuffle_vtr);
          c.shuffle_vtk = c.shuffle_vtr;  // get_if_present(..., shafferVtkID_, shafferVtrID_)
          opt_bool(*m2, "shuffer_vtk_grain_ID", c.shuffle_vtk);
          opt_bool(*m2, "random_microstructure_information", random_micro);
        } else if (const Node *m3 = expect_map(o, "phase_state")) {
          bool melted = true;
          opt_bool(*m3, "has_been_melted", melted);
          if (rm) rm->initial_melted = melted;
        } else if (const Node *m4 = expect_map(o, "cell_grain_length_cutoff_factor")) {
          opt_double(*m4, "factor_value", c.length_cutoff_factor);
        } else if (expect_map(o, "parallel_specification")) {
          // decomposition hint of the MPI build; one GPU holds the whole domain
        } else if (const Node *m5 = expect_map(o, "envelope")) {
          double f = -1;
          opt_double(*m5, "max_half_diagonal_length", f);
          if (f > 0) c.trunc_coeff = (double)sqrtf_ref(2.0f) * f * 0.5;  // CA/src/Octahedron.cpp:316-320
        } else if (const Node *m6 = expect_map(o, "load_microstructure_information")) {
          if (!rm) fail("load_microstructure_information (restart) is not supported by the plain realm", &o);
          // CellularAutomataManager_3D.cpp:318-338: skipped once random is set
          if (random_micro) continue;
          const std::string name = required(*m6, "file_name").as_string();
          if (name == "random") {
            load_micro = false;
            random_micro = true;
          } else {
            load_micro = true;
            rm->micro_file = name;
            opt_bool(*m6, "load_seeds", rm->load_seeds);
            if (rm->load_seeds) rm->nucleation = false;
          }
        } else if (const Node *m7 = expect_map(o, "criterion_to_activate_grain")) {
          // read after the 3-D options (CellularAutomataManager_3DRemelting.cpp:51-76)
          if (rm) criterion = required(*m7, "using_nucleation_seed").as_bool() ? 1 : 0;
        }
      }
    }
  }
  if (rm) {
    // CellularAutomataManager_3D.cpp:343-358: neither or both -> random
    if (!(random_micro ^ load_micro)) {
      if (!random_micro) random_micro = true;
      load_micro = false;
    }
    rm->random_micro = random_micro;
    if (rm->random_micro) rm->micro_file.clear();
    if (criterion >= 0) rm->nucleation = criterion == 1;
  }

  // VtrManager::load
  const Node *out = realm.find("output");
  if (!out) fail("parser error: realm-output", &realm);
  opt_int(*out, "output_frequency", c.output.frequency);
  if (const Node *b = out->find("output_data_base_name")) c.output.base = b->as_string();
  if (const Node *t = out->find("output_time_interval")) {
    c.output.time_interval = t->as_double();
    c.output.time_interval_set = true;
  }
  if (const Node *vars = out->find("output_variables")) {
    for (size_t i = 0; i < vars->size(); ++i) {
      int id = output_variable_id(vars->at(i).as_string());
      if (id >= 0) c.output.variables.push_back(id);
    }
  }
  if (c.output.variables.empty()) c.output.variables.push_back(output_variable_id("grain_ID"));
  if (const Node *fmt = out->find("output_format")) {
    const std::string f = fmt->as_string();
    if (f == "appended" || f == "binary")
      c.output.appended = true;
    else if (f != "ascii")
      fail("output_format must be ascii or appended", fmt);
  }

  // ProblemPhysics_RappazGandin1993::load
  const Node *pp = realm.find("problem_physics");
  if (!pp) fail("parsing error: realm-problem_physics-RappazGandin", &realm);
  if (required(*pp, "type").as_string() != "RappazGandin") fail("parsing error: realm-problem_physics-RappazGandin", pp);
  opt_double(*pp, "initial_temperature", c.T0);
  opt_double(*pp, "liquidus_temperature", c.Tm);
  opt_double(*pp, "melting_temperature", c.Tm);
  opt_double(*pp, "solidus_temperature", c.Ts);
  c.Tmin_nuc = c.Ts;
  opt_double(*pp, "minimum_temperature_for_nucleation", c.Tmin_nuc);
  opt_double(*pp, "t_dot", c.Tdot);
  opt_double(*pp, "a1", c.a1);
  opt_double(*pp, "a2", c.a2);
  opt_double(*pp, "a3", c.a3);
  opt_double(*pp, "b1", c.b1);
  opt_double(*pp, "b2", c.b2);
  opt_double(*pp, "b3", c.b3);
}

}  // namespace

bool deck_is_coupled(const std::string &text) {
  std::unique_ptr<Node> doc = parse_doc(text);
  bool ca = false, fem = false;
  solvers_of(*doc, ca, fem);
  return ca && fem;
}

PlainConfig parse_plain_deck(const std::string &text) {
  std::unique_ptr<Node> doc = parse_doc(text);
  PlainConfig c;
  bool ca = false, fem = false;
  solvers_of(*doc, ca, fem);
  if (fem) fail("finite_element_method decks use the FE-coupled realm, not the plain CA solver");
  if (!ca) fail("parser error: the plain CA solver needs solvers: [cellular_automata]");

  // CellularAutomataSolver::load: realms
  const Node *realms = doc->find("realms");
  if (!realms || !realms->is_seq() || realms->size() == 0) fail("parser error: realms");
  if (realms->size() != 1) fail("only one CA realm per deck is supported");
  const Node &realm = realms->at(0);
  const std::string type = required(realm, "type").as_string();
  if (type != "cellular_automata")
    fail("realm type '" + type + "' is not the plain CA realm (cellular_automata)", &realm);
  parse_ca_realm(realm, c, nullptr);

  // time_integrators (CellularAutomataSolver.cpp:99-128)
  const Node *ti = doc->find("time_integrators");
  if (!ti) fail("parser error: tiem_integrations");
  for (size_t i = 0; i < ti->size(); ++i) {
    const Node *sti = ti->at(i).find("standard_time_integrator");
    if (!sti) continue;
    c.final_time = required(*sti, "termination_time").as_double();
    c.max_dt = required(*sti, "time_step").as_double();
    opt_int(*sti, "termination_step_count", c.max_steps);
    opt_double(*sti, "time_step_factor_ca", c.time_step_factor);
  }
  return c;
}

RemeltConfig parse_remelt_deck(const std::string &text) {
  std::unique_ptr<Node> doc = parse_doc(text);
  RemeltConfig r;
  bool ca = false, fem = false;
  solvers_of(*doc, ca, fem);
  if (!(ca && fem)) fail("the FE-coupled realm needs solvers: [cellular_automata, finite_element_method]");

  // CafeSolver::load (CA/src/CafeSolver.cpp:40-137)
  const Node *realms = doc->find("realms");
  if (!realms || !realms->is_seq() || realms->size() == 0) fail("parser error: realms");
  bool have_ca = false, have_fe = false;
  for (size_t i = 0; i < realms->size(); ++i) {
    const Node &realm = realms->at(i);
    const std::string type = required(realm, "type").as_string();
    if (type == "cellular_automata_remelting") {
      if (have_ca) fail("only one CA realm per deck is supported", &realm);
      parse_ca_realm(realm, r.ca, &r);
      have_ca = true;
    } else if (type == "cellular_automata") {
      fail("the FE-coupled path supports the cellular_automata_remelting realm only", &realm);
    } else if (type == "finite_element") {
      if (have_fe) fail("only one finite_element realm per deck is supported", &realm);
      int dim = 3;
      opt_int(realm, "dimension", dim);
      if (dim != 3) fail("only 3-D finite_element realms are supported", &realm);
      if (const Node *so = realm.find("solution_options")) {
        required(*so, "name").as_string();
        if (const Node *opts = expect_seq(*so, "options")) {
          for (size_t k = 0; k < opts->size(); ++k) {
            if (const Node *ld = expect_map(opts->at(k), "load_data_from_file")) {
              opt_bool(*ld, "for_whole_time", r.fe.whole_time);
              opt_int(*ld, "lines_for_title", r.fe.title_lines);
              opt_int(*ld, "lines_for_subtitle", r.fe.subtitle_lines);
              opt_double(*ld, "length_scale", r.fe.length_scale);
              opt_double(*ld, "time_scale", r.fe.time_scale);
              opt_double(*ld, "x_offset", r.fe.offset[0]);
              opt_double(*ld, "y_offset", r.fe.offset[1]);
              opt_double(*ld, "z_offset", r.fe.offset[2]);
            }
          }
        }
      }
      r.fe.mesh = required(realm, "mesh").as_string();
      if (const Node *out = realm.find("output")) opt_int(*out, "output_frequency", r.fe.output_frequency);
      have_fe = true;
    } else {
      fail("parser error: realm-type", &realm);
    }
  }
  if (!have_ca) fail("the FE-coupled deck has no cellular_automata_remelting realm");
  if (!have_fe) fail("the FE-coupled deck has no finite_element realm");
  if (!r.fe.whole_time)
    fail("the finite_element realm must replay frames (load_data_from_file.for_whole_time: yes); "
         "solving the heat equation is not part of this library");
  if (r.fe.title_lines < 0) fail("parsing missing required key: lines_for_title");
  if (r.fe.subtitle_lines < 4) fail("lines_for_subtitle must be at least 4 (the 4th line holds step and time)");

  const Node *ti = doc->find("time_integrators");
  if (!ti) fail("parser error: tiem_integrations");
  for (size_t i = 0; i < ti->size(); ++i) {
    const Node *sti = ti->at(i).find("standard_time_integrator");
    if (!sti) continue;
    r.ca.final_time = required(*sti, "termination_time").as_double();
    r.ca.max_dt = required(*sti, "time_step").as_double();
    r.time_step_factor_fe = required(*sti, "time_step_factor").as_double();
    opt_int(*sti, "termination_step_count", r.ca.max_steps);
    opt_double(*sti, "time_step_factor_ca", r.ca.time_step_factor);
  }

  // MapVoxelManager::load (CA/src/MapVoxelManager.cpp:62-89)
  if (const Node *tr = doc->find("transfers")) {
    for (size_t i = 0; i < tr->size(); ++i) {
      const Node &t = tr->at(i);
      if (const Node *b = t.find("bin_size")) read3(*b, r.tr.bin);
      opt_double(t, "tolerance", r.tr.tolerance);
      opt_int(t, "max_iterations", r.tr.max_iter);
      opt_double(t, "void_temperature", r.tr.void_temperature);
    }
  }
  for (int a = 0; a < 3; ++a)
    if (r.tr.bin[a] < 1) fail("transfers.bin_size must be positive");
  for (double b : {r.ca.b1, r.ca.b2, r.ca.b3})
    if (b != 1.0 && b != 2.0 && b != 3.0)
      fail("problem_physics b1..b3 must be 1, 2 or 3 (integer powers are evaluated exactly)");
  return r;
}

}  // namespace amca
