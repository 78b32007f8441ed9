/*
 * amca_oracle — plain-C restatement of AMCA3D's 3-D cellular-automaton
 * timestep, used ONLY as the test oracle (and the timed CPU baseline of the
 * benchmark). It is never linked into, or called by, the product library.
 *
 * It follows the reference's sequential algorithm step for step, in the same
 * floating-point operation order (build with -ffp-contract=off), and draws
 * from the same random streams (glibc rand() for sites and orientations, a
 * restated libstdc++ minstd_rand0 + normal_distribution for critical
 * undercoolings). Every function cites the reference file:line it follows.
 */
#ifndef AMCA_ORACLE_H
#define AMCA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters of the plain (uniform-cooling) CA realm, as the reference reads
 * them from its YAML deck (CellularAutomataManager_3D.cpp:71-361,
 * ProblemPhysics.cpp:58-102, CellularAutomataSolver.cpp:99-128). */
typedef struct {
  int nx, ny, nz;            /* interior cells per axis */
  double x0, y0, z0;         /* domain origin */
  double h;                  /* cell size */
  double ns, mu_s, sigma_s;  /* surface sites: density (per area), mean, std of dTc */
  double nv, mu_v, sigma_v;  /* bulk sites: density (per volume), mean, std of dTc */
  unsigned seed;             /* glibc srand() seed (reference: procID*10000 at np=1 -> 0) */
  double T0, Tm, Tdot;       /* uniform temperature T(t) = T0 + Tdot*t; melting temperature */
  double a1, a2, a3;         /* KGT polynomial v = a1*dT + a2*dT^2 + a3*dT^3 */
  double max_dt;             /* time_step */
  double final_time;         /* termination_time */
  double time_step_factor;   /* time_step_factor_ca (default 0.2) */
  double trunc_coeff;        /* Octahedron truncation coefficient (default (double)sqrtf(3.0f)) */
  int shuffle_vtr;           /* random_type.shuffer_vtr_grain_ID: std::random_shuffle draws rand() before nucleation */
} amca_oracle_plain_params;

typedef struct {
  int steps;             /* CA steps taken */
  double time;           /* simulation time reached */
  double last_dt;        /* dt of the last step */
  int64_t num_grains;    /* envelopes created (grainVector_ size) */
  int64_t num_orient;    /* orientations created */
  int64_t liquid_cells;  /* interior liquid cells left */
  int64_t active_grains; /* active envelopes left */
  int64_t tests;         /* octahedron containment tests performed */
  int64_t num_sites;     /* distinct nucleation sites */
} amca_oracle_result;

/* Run the plain CA until solid / final_time / max_steps (max_steps < 0: no
 * limit). Outputs are over the ghost-inclusive grid (nx+2)(ny+2)(nz+2) in the
 * reference's index order k*(nx+2)(ny+2) + j*(nx+2) + i:
 *   orient_out: cellOrientationID_ (-1 liquid, 0 on the ghost layer)
 *   grain_out:  cellGrainID_       (envelope index owning the cell)
 *   site_dtc_out: cellNucleationDT_ (-1 no site, 0 consumed site, else dTc)
 * Any output pointer may be NULL. euler_out (3 doubles per orientation, up to
 * euler_cap orientations) receives the orientation Euler angles.
 * Returns 0 on success, <0 on allocation failure / bad parameters. */
int amca_oracle_run_plain(const amca_oracle_plain_params *p, int max_steps, int32_t *orient_out, int32_t *grain_out,
                          double *site_dtc_out, double *euler_out, int64_t euler_cap, amca_oracle_result *res);

/* Building blocks exposed for known-answer tests. */
/* libstdc++ std::normal_distribution<double>(mean, sigma) driven by a
 * default-constructed std::default_random_engine (minstd_rand0, seed 1):
 * writes the first n draws. */
void amca_oracle_normal_draws(double mean, double sigma, int n, double *out);
/* Orientation angles + local->global rotation matrix, from three glibc
 * rand() values (CellularAutomataManager_3D.cpp:839-850, Octahedron.cpp:282-310). */
void amca_oracle_orientation(int r0, int r1, int r2, double euler[3], double l2g[9]);
/* Octahedron::set_coordinate_transformation_matrix (Octahedron.cpp:282-310) */
void amca_oracle_rotation(const double euler[3], double l2g[9]);
/* Octahedron containment test and decentred capture for one (envelope, cell)
 * pair (Octahedron.cpp:99-128, 134-275). l2g is the local->global matrix. */
int amca_oracle_is_captured(const double l2g[9], const double gc[3], double length);
void amca_oracle_capture(const double l2g[9], const double gc[3], double length, double h, double trunc_coeff,
                         double new_info[4]);

/* ---------------------------------------------------------------------
 * FE-coupled remelting realm (CafeSolver weak coupling at np=1):
 * FiniteElementManager replaying text frames (LoadDataFromFile.cpp),
 * MapVoxelManager voxel tagging and trilinear interpolation
 * (MapVoxelManager.cpp), CellularAutomataManager_3DRemelting.
 * --------------------------------------------------------------------- */
typedef struct {
  /* CA grid */
  int nx, ny, nz;
  double x0, y0, z0, h;
  /* problem_physics (ProblemPhysics.cpp:58-102) */
  double Tm, Ts, Tnuc_min;
  double a1, a2, a3, b1, b2, b3;
  /* CA options */
  double time_step_factor_ca; /* time_step_factor_ca, default 0.2 */
  double trunc_coeff;         /* Octahedron truncation coefficient */
  double cutoff_factor;       /* cell_grain_length_cutoff_factor (default 1e8), times h */
  int initial_melted;         /* phase_state.has_been_melted (default yes) */
  int nucleation;             /* criterion_to_activate_grain.using_nucleation_seed */
  double ns, mu_s, sigma_s, nv, mu_v, sigma_v;
  unsigned seed;
  int shuffle_vtr;
  const char *microstructure; /* NULL: random (one grain per interior cell); else restart file path */
  int load_seeds;
  /* transfers (MapVoxelManager.cpp:62-89) */
  int bin[3];
  double tolerance;
  int max_iter;
  double void_temperature;
  /* finite_element realm (FiniteElementManager.cpp:66-142) */
  const char *frames;         /* frame file path */
  int title_lines, subtitle_lines;
  double length_scale, time_scale;
  double offset[3];
  /* time integrator (CafeSolver.cpp:102-131) */
  double final_time;
} amca_oracle_remelt_params;

typedef struct {
  int steps;
  double time;
  double last_dt;
  int64_t num_grains, num_orient, num_sites, tests;
  int64_t nodes, elements, frames_read;
  int frames_exhausted;       /* 1 if the run ended on the end of the frame file */
  double loop_seconds;        /* wall time of the coupled time loop (set-up excluded) */
} amca_oracle_remelt_result;

/* Run the coupled loop to final_time or the end of the frames (max_steps < 0:
 * no limit). Ghost-inclusive outputs (any may be NULL): orientation, grain,
 * temperature, melted, cooling, liquid-neighbour flags. When dump_path is
 * non-NULL, appends the state after every CA step in the record layout of
 * oracle/ref_probe/state_dump.cpp. Returns 0, or <0 with a message in err. */
int amca_oracle_run_remelt(const amca_oracle_remelt_params *p, int max_steps, const char *dump_path,
                           int32_t *orient_out, int32_t *grain_out, double *temp_out, uint8_t *melted_out,
                           uint8_t *cooling_out, uint8_t *flag_out, amca_oracle_remelt_result *res, char *err,
                           int errlen);

/* MapVoxelManager::is_in_element (MapVoxelManager.cpp:487-699) for one hex
 * (8 node coordinates, reference node order) and point. */
int amca_oracle_is_in_element(const double node_xyz[24], const double point[3], double tolerance, int max_iter,
                              double para[3]);

#ifdef __cplusplus
}
#endif
#endif
