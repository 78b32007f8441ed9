/*
 * amca3d.h — C ABI of the GB300 CA-timestep library (libamca3d.so).
 *
 * One handle runs one AMCA3D cellular-automaton realm on one GPU, read from
 * the reference's own YAML input deck. Every call returns an int status
 * (AMCA_OK == 0) and never throws; amca_last_error() gives the message of the
 * last failure on a handle. The library owns all device memory; callers own
 * host buffers. A handle is used by one host thread at a time and has its own
 * CUDA stream.
 *
 * Each entry point cites the reference interface it replaces.
 */
#ifndef AMCA3D_H
#define AMCA3D_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  AMCA_OK = 0,
  AMCA_ERR_ARG = -1,      /* bad argument / unsupported deck content */
  AMCA_ERR_PARSE = -2,    /* YAML syntax or a missing required key */
  AMCA_ERR_CUDA = -3,     /* a CUDA call failed (no GPU, no memory, ...) */
  AMCA_ERR_STATE = -4,    /* call out of order (e.g. step before initialize) */
  AMCA_ERR_DEVICE = -5,   /* a kernel reported an internal error (bounded wait ran out) */
  AMCA_ERR_IO = -6        /* output file could not be written */
};

typedef struct amca_t amca_t;

/* Options the reference takes from its environment rather than the deck. */
typedef struct {
  int device;           /* CUDA device ordinal */
  unsigned seed;        /* glibc srand() seed offset: the reference seeds srand(procID*10000), i.e. 0 at np=1 */
  int write_outputs;    /* 1: write VTR/PVTR/PVD snapshots every output_frequency steps, like VtrManager::execute */
  const char *workdir;  /* directory that relative output paths in the deck are resolved against (NULL: cwd) */
} amca_opts;

/* Parse a deck and select the realm.
 * Replaces Simulation::load -> CellularAutomataSolver::load ->
 * CellularAutomataManager_3D::load / ProblemPhysics_RappazGandin1993::load
 * (CA/src/CellularAutomataSolver.cpp:40-130, CA/src/CellularAutomataManager_3D.cpp:71-361,
 * CA/src/ProblemPhysics.cpp:58-102). opts may be NULL (device 0, seed 0, no outputs). */
int amca_create(const char *yaml_text, const amca_opts *opts, amca_t **out);

/* Grid of the realm: interior cells per axis, origin and cell size (the
 * values CellularAutomataManager_3D::load derives, CA/src/CellularAutomataManager_3D.cpp:155-190).
 * Needs no GPU. Any pointer may be NULL. */
int amca_get_grid(const amca_t *h, int32_t cells[3], double origin[3], double *cell_size);

/* Host half of initialize: draw the nucleation sites and the orientation
 * stream (glibc rand(), libstdc++ normal_distribution, glibc libm), as
 * CellularAutomataManager_3D::initialize does (CA/src/CellularAutomataManager_3D.cpp:366-379,
 * CA/src/CellularAutomataManager.cpp:153-213,471-518). Needs no GPU;
 * amca_initialize calls it when it has not run yet. */
int amca_prepare(amca_t *h);

/* Nucleation sites after amca_prepare: ghost-inclusive cell ids in ascending
 * order and their critical undercoolings (nucleationCellIDList_ /
 * cellNucleationDT_, CA/src/CellularAutomataManager.cpp:153-213). Either
 * array may be NULL; *n_out receives the site count. */
int amca_get_sites(const amca_t *h, int32_t *cells, double *dtc, size_t cap, size_t *n_out);

/* Move the prepared tables to the GPU and build the cell field.
 * Replaces CellularAutomataManager_3D::initialize (CA/src/CellularAutomataManager_3D.cpp:366-379). */
int amca_initialize(amca_t *h);

/* One CA step: nucleation, dt, growth and the capture sweep.
 * Replaces CellularAutomataManager_3D::calculate_time_step + single_integration_step
 * (CA/src/CellularAutomataManager_3D.cpp:441-669). dt_out may be NULL. */
int amca_step(amca_t *h, double *dt_out);

/* Steps until the domain is solid, the deck's termination_time is reached,
 * or max_steps steps were taken (max_steps < 0: no step limit).
 * Replaces CellularAutomataManager::time_integration (CA/src/CellularAutomataManager.cpp:134-147). */
int amca_run(amca_t *h, int max_steps);

/* ---- Coupling with a solver that advances beside the realm ----
 * One step whose dt is also bounded by dt_cap (the coupled solver's time
 * step; dt_cap <= 0 or +inf: no bound): dt = min(dt of amca_step, dt_cap).
 * Replaces CellularAutomataManager::setup_time_step_for_coupling
 * (CA/include/CellularAutomataManager.h:42) as CafeSolver applies it,
 * dT = min(dT_FE, dT_CA) (CA/src/CafeSolver.cpp:190-206). For an FE-coupled
 * realm whose node temperatures come from amca_set_nodal_temperatures, dt_cap
 * is the FE time step itself (the reference's dT_FE and the CA's
 * maxTimestep_, CA/src/CafeSolver.cpp:183-184,213-216). dt_out may be NULL. */
int amca_step_coupled(amca_t *h, double dt_cap, double *dt_out);

/* Steps while time < t_end (and the realm's own end conditions allow):
 * the loop of CafeSolver::time_integration_weak_coupling and
 * CellularAutomataManager::time_integration with the final time t_end
 * (CA/src/CafeSolver.cpp:188, CA/src/CellularAutomataManager.cpp:134-147).
 * The last step may end past t_end, as in the reference. */
int amca_run_until(amca_t *h, double t_end);

/* FE-coupled realms: the node temperatures (n = node count, in the node order
 * of the frames, x fastest) that the next step interpolates, handed in by an
 * FE solver that advances beside the realm: the FE realm's thetaArray_ after
 * its own solve (CA/src/CafeSolver.cpp:207-216 with solveProblemMyself_),
 * which MapVoxelManager::evaluate_temperature reads
 * (CA/src/MapVoxelManager.cpp:746-799). From the first call on, the realm
 * stops replaying its frames: before every step the caller hands in that
 * step's node temperatures and advances it with amca_step_coupled (its dt_cap
 * the FE time step). After amca_initialize; amca_reset returns to the frames. */
int amca_set_nodal_temperatures(amca_t *h, const double *theta, int64_t n);

enum {
  AMCA_FIELD_ORIENTATION_ID = 0, /* int32, ghost-inclusive grid: cellOrientationID_ (the output "grain_id") */
  AMCA_FIELD_GRAIN_ID = 1,       /* int32, ghost-inclusive grid: cellGrainID_ (envelope index per cell) */
  AMCA_FIELD_SITE_UNDERCOOLING = 2, /* float64, ghost-inclusive grid: cellNucleationDT_ */
  /* FE-coupled remelting realm only (CA/include/CellularAutomataManager.h:104-109): */
  AMCA_FIELD_TEMPERATURE = 3,       /* float64: cellTemperature_ of the last step (-1: no material) */
  AMCA_FIELD_MELTED = 4,            /* uint8: hasBeenMelted_ */
  AMCA_FIELD_COOLING = 5,           /* uint8: cooling_ */
  AMCA_FIELD_LIQUID_NEIGHBOUR = 6   /* uint8: cellLiquidNeigh */
};
/* Copy a whole field to host memory. bytes must equal cells * element size,
 * cells = (nx+2)(ny+2)(nz+2), in the reference's index order
 * k*(nx+2)(ny+2) + j*(nx+2) + i.
 * Replaces reading cellOrientationID_ / cellGrainID_ / cellNucleationDT_
 * (CA/include/CellularAutomataManager.h:20-246). */
int amca_get_field(amca_t *h, int field, void *host_dst, size_t bytes);

/* Euler angles (3 doubles per orientation, in orientation-id order) of the
 * orientations created so far; with all=1, of the whole pre-drawn stream
 * (one per site, available after amca_prepare).
 * Replaces orientationVector_ (CA/src/CellularAutomataManager_3D.cpp:1130-1215). */
int amca_get_orientations(amca_t *h, double *euler, size_t cap, size_t *n_out, int all);

/* ---- FE-coupled remelting realm (solvers [cellular_automata, finite_element_method],
 * realm types finite_element + cellular_automata_remelting) ----
 * amca_create selects it from the deck; amca_prepare / amca_initialize /
 * amca_step / amca_run / amca_get_field / amca_get_stats / amca_reset then
 * drive CafeSolver::time_integration_weak_coupling (CA/src/CafeSolver.cpp:178-219).
 * By default the frames are read from the finite_element realm's mesh file
 * (FiniteElementManager::load_mesh_and_first_two_steps_results_from_txt_file,
 * CA/src/LoadDataFromFile.cpp:21-191). The two calls below replace that file;
 * both must come before amca_initialize. */

/* Frames from host memory, in the file's units: node coordinates (3 per node,
 * x fastest over nodes[0] x nodes[1] x nodes[2]), the time of each frame and
 * frame-major node temperatures. The deck's offsets and length/time scales are
 * applied exactly as the reader applies them. */
int amca_set_fe_frames(amca_t *h, const int32_t nodes[3], const double *coords, int32_t nframes,
                       const double *times, const double *theta);

/* Synthetic frames generated on the GPU: the Rosenthal quasi-steady field of a
 * point source moving along +x over a structured node grid,
 *   T = t0 + (A P) / (2 pi k R) exp(-v (R + xi) / (2 alpha)),  xi = x - (x_start + v t),
 * capped at t_cap, evaluated with IEEE add/mul/div/sqrt only (exp by a fixed
 * degree-13 polynomial after ln 2 range reduction), so the frames equal those
 * a host writer produces with the same arithmetic. Node file coordinates are
 * origin + spacing * index; the field is evaluated at file coordinate *
 * length_scale; frame f has file time time_offset + f * frame_dt and the field
 * time (f * frame_dt) * time_scale. Nodes with z > z_top + void_above (when
 * void_above_set) hold t_void. */
typedef struct {
  double origin[3];
  double spacing;
  int32_t nodes[3];
  int32_t frames;
  double length_scale, frame_dt, time_scale, time_offset;
  double power, absorptivity, speed, conductivity, diffusivity;
  double t0, t_cap, x_start, y_line, z_top;
  int32_t void_above_set;
  double void_above, t_void;
} amca_rosenthal;
int amca_set_rosenthal_frames(amca_t *h, const amca_rosenthal *p);

/* Synthetic FE frames of a raster scan, generated on the GPU: ntracks
 * passes along x with alternating direction (even tracks from x_start in +x,
 * odd tracks from x_turn in -x), track k on y = y_line + k * hatch, each
 * track_time seconds long; every frame holds the Rosenthal field of the
 * current pass (the amca_rosenthal formula with xi measured along the
 * direction of travel). Node grid, units and frame times as in
 * amca_rosenthal. With ntracks = 1 the frames are amca_set_rosenthal_frames'
 * bit for bit. The frames are produced a window at a time into a ring of
 * device slots as the run reaches them, so device memory does not grow with
 * the frame count. Before amca_initialize. Stands in for the frame file of
 * FiniteElementManager (CA/src/LoadDataFromFile.cpp:21-191). */
typedef struct amca_scan_s {
  double origin[3];
  double spacing;
  int32_t nodes[3];
  int32_t frames;
  double length_scale, frame_dt, time_scale, time_offset;
  double power, absorptivity, speed, conductivity, diffusivity, t0, t_cap;
  double x_start, x_turn, y_line, z_top, hatch, track_time;
  int32_t ntracks;
} amca_scan;
int amca_set_scan_frames(amca_t *h, const amca_scan *p);

/* ---- Thermal model: a learned stand-in for the FE nodal temperatures ----
 * No counterpart in the reference, which reads FE frames from text files
 * (CA/src/LoadDataFromFile.cpp:21-191) and interpolates them at every CA
 * step (CA/src/MapVoxelManager.cpp:746-799). The model maps (along-track
 * offset from the laser, lateral offset, depth below the top surface, power,
 * speed) to a temperature and an error estimate: 64 Fourier features, four
 * hidden layers of 256 with SiLU (bf16 tensor-core GEMMs, FP32 accumulation),
 * an FP32 head. It is trained on the GPU by this library's own forward and
 * backward kernels on samples of the FE field of a scanning source
 * (amca_scan's formula) and can then produce a realm's frames, falling back
 * to the FE field at nodes near the liquidus whose error estimate is above a
 * threshold. One model per handle; calls on a handle are not thread-safe. */
typedef struct amca_thermal amca_thermal;

typedef struct {
  double power_lo, power_hi;                 /* training range of the laser power (W) */
  double speed_lo, speed_hi;                 /* training range of the scan speed (m/s) */
  double absorptivity, conductivity, diffusivity, t0, t_cap;  /* FE field physics */
  double window_lo[3], window_hi[3];         /* offsets from the source the model covers (m):
                                                along-track, lateral, depth */
  double near_lo[3], near_hi[3];             /* melt-pool box sampled more densely (m) */
  double near_fraction;                      /* share of the training samples from that box */
  double shell_lo, shell_hi;                 /* temperature band (K) sampled more densely ... */
  double shell_fraction;                     /* ... this share of the samples: points of the melt-pool
                                                box redrawn (up to 64 times) until their FE temperature
                                                lies in the band */
  double fourier_sigma;                      /* spread of the Fourier frequencies along the three offsets
                                                (turns per window half-width) */
  double fourier_sigma_pv;                   /* the same along power and speed (turns per range half-width) */
  int32_t log_output;                        /* 0: T = t_shift + t_scale * mu;
                                                1: T = t_shift + t_scale * exp(mu) (t_shift below t0) */
  double t_shift, t_scale;                   /* output map (K) */
  uint64_t seed;
} amca_thermal_spec;

typedef struct {
  int64_t steps, samples_seen;
  double first_loss, last_loss; /* mean 0.5 (mu - y)^2 (normalised units) over the first and last 5% of steps */
  double ms;                    /* wall time of the training loop */
} amca_thermal_train_stats;

int amca_thermal_create(int device, const amca_thermal_spec *spec, amca_thermal **out);
/* Adam on `samples` training samples generated on the GPU from the spec's
 * seed: `steps` steps of `batch` samples (a multiple of 128), learning rate
 * from lr_max to lr_min on a cosine schedule after a short warm-up. */
int amca_thermal_train(amca_thermal *m, int64_t samples, int steps, int batch, double lr_max, double lr_min,
                       amca_thermal_train_stats *st);
/* Temperatures and error estimates (K) of n points given as raw inputs
 * (5 floats each: along-track offset, lateral offset, depth (m), power (W),
 * speed (m/s)); host buffers. Runs the fused inference kernel. */
int amca_thermal_eval(amca_thermal *m, const float *raw, int64_t n, float *T, float *err);
/* Gradients of the training loss of one batch (n a multiple of 128; raw
 * inputs and normalised targets in host memory) with respect to every
 * parameter, without updating them, and the network outputs (mu, s per
 * sample). For checking the training kernels. */
int amca_thermal_gradients(amca_thermal *m, const float *raw, const float *target, int64_t n, float *grad,
                           float *pred);
/* Parameter vector (FP32 masters): per hidden layer l its weights [256][in]
 * (in = 128 for l = 0, else 256) then its 256 biases, then the head weights
 * [2][256] and its 2 biases. */
int64_t amca_thermal_param_count(void);
int amca_thermal_get_params(amca_thermal *m, float *params);
int amca_thermal_set_params(amca_thermal *m, const float *params);
/* The fixed encoding: Fourier matrix [64][5], u = (raw - shift) * scale, and
 * the output map (t_shift, t_scale, log_output of the spec). */
int amca_thermal_get_encoding(amca_thermal *m, float *fourier, float *in_shift, float *in_scale, float *t_shift,
                              float *t_scale, int32_t *log_output);
/* Frames f0 .. f0 + nf - 1 of a scan from the model into host memory
 * (nf x nodes): nodes inside the model's window around the source take the
 * model's temperature, the others t0; a node whose model temperature lies
 * within band (K) of t_liq and whose error estimate exceeds thresh (K) takes
 * the FE field instead. counts[0..2] (may be NULL) = nodes evaluated, near the
 * liquidus, fallbacks. fe = NULL, or nf x nodes doubles receiving the FE
 * field of the same frames (amca_set_scan_frames' values) for comparison. */
int amca_thermal_frames(amca_thermal *m, const amca_scan *scan, int32_t f0, int32_t nf, double t_liq, double band,
                        double thresh, double *frames, double *fe, int64_t *counts);
const char *amca_thermal_last_error(const amca_thermal *m);
void amca_thermal_destroy(amca_thermal *m);

/* Frames of a scan from a trained model instead of the FE field (the realm
 * keeps a reference to the model, which must outlive it): as
 * amca_thermal_frames, produced a window at a time into a ring of device
 * slots while the run reaches them. Before amca_initialize. */
int amca_set_thermal_frames(amca_t *h, amca_thermal *m, const amca_scan *p, double t_liq, double band,
                            double thresh);

/* Frame production of a realm whose frames come from amca_set_scan_frames or
 * amca_set_thermal_frames: out[0] frames produced, out[1] window fills,
 * out[2..4] (model frames) nodes the model evaluated, nodes near the
 * liquidus, fallbacks to the FE field. No counterpart in the reference. */
int amca_get_frame_stats(amca_t *h, int64_t out[5]);

/* Restart microstructure from memory instead of the deck's
 * load_microstructure_information file (same content as grainInfo<rank>.txt,
 * CellularAutomataManager_3DRemelting::load_microstructure_information,
 * CA/src/CellularAutomataManager_3DRemelting.cpp:164-307): per ghost-inclusive
 * cell its grain id, orientation id (-1: take the grain's), melted flag and
 * seed undercooling (dtc may be NULL: no seeds; melted may be NULL: 0); the
 * Euler angles of norient orientations; per grain its cell and orientation;
 * expected = the header's numGlobalExpectedGrains. Before amca_prepare. */
int amca_set_microstructure(amca_t *h, const int32_t *grain, const int32_t *orient, const uint8_t *melted,
                            const double *dtc, int64_t norient, const double *euler, int64_t ngrains,
                            const int32_t *grain_cell, const int32_t *grain_orient, int64_t expected);

/* Final outputs of a finished run: finalGrains.vtk, <pvd dir>/finalResult.txt,
 * the last VTR/PVTR/PVD snapshot and, when the deck asks for it,
 * grainInfo<rank>.txt. Replaces CellularAutomataSolver::finalize +
 * CellularAutomataManager_3D::output_microstructure_information
 * (CA/src/CellularAutomataSolver.cpp:166-201, CA/src/CellularAutomataManager_3D.cpp:1221-1639,1836-1913). */
int amca_write_outputs(amca_t *h);

typedef struct {
  int64_t step;          /* iStep_ */
  double time;           /* time_ */
  double dt;             /* dT_ of the last step */
  int64_t liquid_cells;  /* interior cells still liquid */
  int64_t grains;        /* envelopes created (grainVector_.size()) */
  int64_t orientations;  /* orientations created */
  int64_t active;        /* active envelopes */
  int64_t sites;         /* distinct nucleation sites */
  int64_t cells;         /* interior cells */
  int64_t tests;         /* octahedron containment tests evaluated (by the envelopes woken or created) */
  int64_t tests_fp64;    /* ... of which needed the exact FP64 evaluation */
  int64_t generations;   /* capture generations processed */
  int32_t done;          /* 1 when no liquid cell is left */
  int32_t reserved;
  double kernel_ms;    /* device time of the CA kernels (CUDA events), accumulated */
  int64_t launches;      /* CA kernel launches issued, accumulated */
  /* work counters, summed over steps since the last reset */
  int64_t sites_scanned;    /* live nucleation sites read */
  int64_t nucleations;      /* envelopes created by nucleation */
  int64_t captures;         /* envelopes created by capture */
  int64_t active_grown;     /* generation-0 entries processed: woken envelopes and nuclei */
  int64_t grains_processed; /* envelopes processed over all generations */
  double algorithmic_bytes; /* HBM bytes the step must move by the counting rule of the design notes */
  int64_t h2d_bytes;        /* host->device bytes copied by this handle */
  int64_t d2h_bytes;        /* device->host bytes copied by this handle */
  /* device wall time per phase of the step kernel, ms: [0] nucleation,
   * [1] claim, [2] resolve, [3] step end (each up to the grid barrier that
   * closes it), [4] the generation-0 part of [1]; per-block busy time before
   * the barrier: [5] claim mean over blocks, [6] claim slowest block,
   * [7] resolve mean, [8] resolve slowest block (summed over phases); [6]
   * and [8] are gathered only when the environment variable
   * AMCA_PHASE_DETAIL is set to a nonzero value when the handle is
   * initialized (zero otherwise: it adds a global load per block and phase) */
  double phase_ms[9];
  /* Remelting realm only (zeros otherwise), ms summed over steps: per-block
   * busy time between grid barriers, mean over blocks [0..5] and slowest
   * block [6..11], for the work closed by the barrier after phase A, B, C,
   * D, E and after the host velocity answers; block 0's new-grain ids [12]
   * and nucleation [13]; the slowest block's liquid-neighbour flag pass in
   * phase B [14]. Plain realm: per-block busy time, mean over blocks, of
   * nucleation [0], the wake scan [1] and list compactions [2]; the slowest
   * block's busy time in nucleation and wake scan [3] (AMCA_PHASE_DETAIL
   * only); block 0's time inside grid barriers [4]. */
  double detail_ms[16];
  /* Plain realm only (zeros otherwise), summed since the last reset: list
   * positions read by the wake scans, liquid-count decrements, counts that
   * reached zero in a capture generation, compactions of the envelope list. */
  int64_t keys_scanned;
  int64_t decrements;
  int64_t zero_events;
  int64_t compactions;
  /* Plain realm only: envelopes the reference's walk visits (its active
   * envelopes after nucleation, summed over steps; algorithmic_bytes counts
   * these), and the bytes this implementation moves by its own accounting
   * (it processes only the envelopes that may change). */
  int64_t reference_walked;
  double step_bytes;
} amca_stats;
/* For the FE-coupled remelting realm the fields mean: liquid_cells -1 (not
 * tracked), grains = grain objects, active = flagged (liquid-neighbour) cells
 * summed over steps, generations = exact FP64 cell temperatures evaluated,
 * done = the run reached termination_time or the end of the frames,
 * reserved = host velocity round trips, sites_scanned = active elements
 * visited, active_grown = cells visited by the phase update, grains_processed =
 * liquid cells that flagged neighbours, phase_ms[0..4] = phase update,
 * liquid-neighbour flags + site conditions, nucleation + minimum temperature,
 * velocities + growth + claims, captures + frame replay; phase_ms[5] = block 0's
 * wait for host velocity answers, phase_ms[6] = block 0's time in grid barriers. */
int amca_get_stats(amca_t *h, amca_stats *out);

/* Number of distinct orientation ids present in the field, the ghost layer
 * (id 0) included, as the reference reports "Final Number of Grains".
 * Replaces get_amount_of_final_orientations (CA/src/CellularAutomataManager_3D.cpp:2000-2034). */
int amca_final_grain_count(amca_t *h, int32_t *count);

/* Restore the state right after amca_initialize (all cells liquid, sites
 * live, time 0) without re-reading the deck or re-uploading tables: the
 * same realm can be run again. Counters in amca_stats restart too. */
int amca_reset(amca_t *h);

/* Page-locked host memory for fast field copies (cudaMallocHost); free
 * with amca_host_free. */
int amca_host_alloc(size_t bytes, void **out);
int amca_host_free(void *p);

/* Evaluate the envelope arithmetic on the GPU for n independent
 * (envelope, cell) pairs given in host memory: l2g = local->global matrix
 * (9 per pair), gc = cell centre minus envelope centre (3 per pair),
 * length = half-diagonal, trunc = truncation coefficient per pair, h = cell
 * size. Outputs: captured (FP64 test), captured_fast (the FP32 pre-test with
 * FP64 fallback that the step kernel uses), info = decentred new envelope
 * (centre offset xyz, half-diagonal; zeros when not captured).
 * Replaces Octahedron::cell_is_captured / capture_cell (CA/src/Octahedron.cpp:99-275). */
int amca_envelope_eval(int device, size_t n, const double *l2g, const double *gc, const double *length, double h,
                       const double *trunc, int32_t *captured, int32_t *captured_fast, double *info);

/* A destroyed realm's device buffers (the plain realm's one arena, the
 * remelting realm's arrays) are kept for the realms created after it on the
 * same device (up to 32 GiB per device, the larger ones kept first; a buffer
 * is reused when it is at most twice the size asked for). This frees the
 * kept buffers of `device` (every device when device < 0). */
int amca_release_cached_memory(int device);

/* Self-test of the device-side failure detection: one cooperative launch of
 * `blocks` blocks (1..64) through the grid barrier the step kernels use,
 * which here expects `parties` arrivals and bounds every wait by wait_ns
 * (1 us..2 s), with the error word preset to preset_error. With parties >
 * blocks one arrival never comes: every wait runs out, the error word reads
 * 1 (barrier wait timed out) and every verdict 0, and the context stays
 * usable; with parties == blocks and preset_error != 0 the barrier completes
 * and every block reports the error it saw. *error_out = the error word
 * afterwards, verdicts[b] = 1 when block b's barrier returned success. No
 * counterpart in the reference, whose errors abort the run. */
int amca_selftest_barrier(int device, int blocks, int parties, int64_t wait_ns, int32_t preset_error,
                          int32_t *error_out, int32_t *verdicts);

/* Plain-realm parameters as plain numbers (what amca_create reads from a deck). */
typedef struct {
  int32_t nx, ny, nz;                 /* interior cells per axis */
  double x0, y0, z0, h;               /* origin, cell size */
  double T0, Tm, Tdot;                /* uniform T(t) = T0 + Tdot*t; melting temperature */
  double a1, a2, a3;                  /* KGT coefficients */
  double max_dt, final_time;          /* time_step, termination_time */
  double time_step_factor;            /* time_step_factor_ca (0.2 by default) */
  double trunc_coeff;                 /* envelope truncation coefficient ((double)sqrtf(3.0f) by default) */
} amca_plain_params;

typedef struct {
  int64_t steps;
  double time;
  int64_t grains, orientations, liquid_cells;
  int32_t done;
} amca_plain_result;

/* Whole plain-realm run that allocates no memory. This entry point has no
 * counterpart in the reference.
 *
 * Who needs it: callers that cannot let a library call cudaMalloc -- a
 * coupled solver that has already reserved the GPU's memory for its own pool,
 * or a host loop that must not take cudaMalloc/cudaFree's implicit device
 * synchronisation. The caller passes every input and output in device
 * memory it owns: site cells (ascending ghost-inclusive ids) and their
 * critical undercoolings, the local->global orientation matrices (9 doubles
 * per site, as amca_get_orientations' angles give through the reference's
 * Bunge formula with the host's libm), and the int32 orientation field
 * ((nx+2)(ny+2)(nz+2) cells, filled by this call). The run's other state
 * lives in one static device array of 32 MiB, which every GPU that loads the
 * library holds until the process exits; grids that need more (about
 * 148 bytes per interior cell plus 37 per site and 300 KB, i.e. roughly
 * 225,000 interior cells, a 61^3 cube) are rejected with AMCA_ERR_ARG and a
 * message.
 *
 * The site list is checked on the GPU before the run (every site cell an
 * interior cell, ids strictly ascending, at most one site per interior cell);
 * a bad list is rejected with AMCA_ERR_ARG naming the first bad site. The
 * caller's current device is the same after the call as before it.
 *
 * The first call on a device looks up the array's device address (the host
 * name of the array is not a device address) and keeps it for later calls;
 * make that first call before any stream capture, and do not reset the
 * device (cudaDeviceReset) between calls: the kept address would then be
 * stale. Every call shares the one array and clears what must
 * start at zero; calls that overlap on the GPU (two host threads, or two
 * streams) race and corrupt each other. Runs until solid, final_time or
 * max_steps (< 0: no limit) on `stream` (NULL: default stream) and waits for
 * it. Errors go to err (errlen bytes, may be NULL). */
int amca_plain_run_noalloc(int device, const amca_plain_params *p, const int32_t *site_cell, const double *site_dtc,
                           int64_t nsites, const double *l2g, int32_t *orient, int max_steps, void *stream,
                           amca_plain_result *res, char *err, size_t errlen);

/* ---- Batches: many independent plain realms in one launch -------------
 * No counterpart in the reference, which runs one deck per process: a batch
 * stands in for n separate np=1 runs of the reference program (CA/src/Cafe.cpp:39-120),
 * each CellularAutomataSolver::execute -> CellularAutomataManager_3D::time_integration
 * (CA/src/CellularAutomataSolver.cpp:148-160). Every realm's result is the one
 * it gives when run alone. */
typedef struct amca_batch amca_batch;

/* A batch over n distinct, initialized plain-realm handles on one device
 * (1 <= n <= 65535). The handles stay the caller's and must outlive the
 * batch; while it exists they are run only through it. team_size = blocks
 * that run one realm (0: 8, until amca_batch_tune picks one). */
int amca_batch_create(amca_t *const *realms, int n, int team_size, amca_batch **out);

/* Run every realm of the batch from its initial state (what amca_reset
 * gives) to its end (solid, or termination_time), all in one cooperative
 * launch: teams of team_size blocks take realms from a queue, longest first
 * once amca_batch_tune has measured them. Each run replays one CUDA graph
 * (reset of every realm, the launch, a gather of the realms' control
 * blocks) on the batch's own stream and waits for it. Afterwards each handle
 * reads as after amca_reset + amca_run(h, -1) (amca_get_field,
 * amca_get_stats, amca_write_outputs, ...), except that no VTR snapshot is
 * written during the run. device_ms (may be NULL): CUDA-event time of the
 * graph on that stream. AMCA_ERR_DEVICE names the realm whose bounded wait
 * ran out. */
int amca_batch_run(amca_batch *b, double *device_ms);

/* Autotuning: runs the batch once to measure each realm and orders the
 * queue longest realm first; times every realm at uniform team sizes 1, 2,
 * 4, ... (up to 128 and the largest that fits), `repeats` times each (at
 * least 1); then builds a mixed layout from those per-realm times (each
 * realm on the team size that spends the fewest block-milliseconds while
 * finishing within the smallest makespan whose teams fit; teams of one size
 * share a queue, longest realm first) and times it too. The fastest layout
 * is kept. *team_size_out (may be NULL) = the uniform size kept, or 0 when
 * the mixed layout was kept. */
int amca_batch_tune(amca_batch *b, int repeats, int *team_size_out);

/* Set the launch layout by hand: nclasses classes, class c made of
 * teams[c] teams of team_size[c] blocks; realm r is run by a team of class
 * realm_class[r]. Within a class realms are queued in the order they appear
 * in queue_order (a permutation of the realm indices), or, when it is NULL,
 * longest first once amca_batch_tune has measured them, else in handle
 * order. The blocks of all teams must fit on the device
 * (amca_batch_stats.max_blocks). */
int amca_batch_set_layout(amca_batch *b, int nclasses, const int32_t *team_size, const int32_t *teams,
                          const int32_t *realm_class, const int32_t *queue_order);

/* The current layout, in amca_batch_set_layout's terms: *nclasses classes
 * (team_size and teams filled for the first `cap` of them), realm_class and
 * queue_order (one entry per realm each; any array may be NULL). Setting it
 * on another batch of the same decks reproduces the launch. */
int amca_batch_get_layout(const amca_batch *b, int cap, int32_t *team_size, int32_t *teams, int32_t *realm_class,
                          int32_t *queue_order, int *nclasses);

typedef struct {
  int32_t realms;
  int32_t team_size;     /* blocks per realm of a uniform layout; 0 for a mixed layout */
  int32_t teams;         /* teams in the launch */
  int32_t max_blocks;    /* co-resident blocks of the batched kernel on this device */
  int32_t graph;         /* 1: runs replay a CUDA graph; 0: plain launches (capture unavailable) */
  int32_t n_tuned;       /* entries of tuned_* filled by the last amca_batch_tune */
  int64_t runs;
  double last_ms;        /* device time of the last run */
  double total_ms;
  int64_t cell_updates;  /* sum over realms of interior cells x CA steps, last run */
  int32_t tuned_team[8];
  double tuned_ms[8];    /* best time of each uniform team size tried */
  double mixed_ms;       /* best time of the mixed layout tried (0: none) */
  int32_t grid_blocks;   /* blocks of the launch */
  int32_t n_classes;     /* team classes of the layout (at most 8 reported) */
  int32_t class_team[8];    /* team size of each class */
  int32_t class_teams[8];   /* teams of each class */
  int32_t class_realms[8];  /* realms of each class */
} amca_batch_stats;

int amca_batch_get_stats(const amca_batch *b, amca_batch_stats *out);

/* Message of the last failing call on b (or of the last failing
 * amca_batch_create when b is NULL). Never NULL. */
const char *amca_batch_last_error(const amca_batch *b);

void amca_batch_destroy(amca_batch *b);

/* Message of the last failing call on h (or of the last failing
 * amca_create / amca_envelope_eval when h is NULL). Never NULL. */
const char *amca_last_error(const amca_t *h);

void amca_destroy(amca_t *h);

#ifdef __cplusplus
}
#endif
#endif
