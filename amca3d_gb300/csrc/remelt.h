// remelt.h — device state and launch API of the FE-coupled remelting realm.
//
// Reference: CafeSolver::time_integration_weak_coupling (CA/src/CafeSolver.cpp:178-219)
// driving CellularAutomataManager_3DRemelting (CA/src/CellularAutomataManager_3DRemelting.cpp)
// with temperatures interpolated by MapVoxelManager::evaluate_temperature
// (CA/src/MapVoxelManager.cpp:746-799) from frames replayed by
// FiniteElementManager::pseudo_single_integration_step (CA/src/LoadDataFromFile.cpp:207-313).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "ca_math.h"

namespace amca {

constexpr int32_t kPendingGrain = 0x7fffffff;  // grain created this step, id assigned after the step
constexpr int kNewGrainCap = 16384;            // new grain objects one step may create
constexpr int kRemeltErrBarrier = 1, kRemeltErrFrame = 2, kRemeltErrNewGrains = 3, kRemeltErrRatio = 4,
              kRemeltErrList = 5, kRemeltErrHost = 6, kRemeltErrRing = 7;
// why a launch returned
constexpr int kRemeltRunning = 0, kRemeltFinalTime = 1, kRemeltFramesEnd = 2, kRemeltNeedOrient = 3,
              kRemeltStepLimit = 4, kRemeltNeedFrames = 5, kRemeltTimeStop = 6;

// Growth velocities whose glibc pow() rounding cannot be decided on the GPU
// (an integer power within 0.02 ulp of a rounding midpoint; glibc's pow errs
// by at most 0.52 ulp) are evaluated by the host's libm: the kernel posts the
// temperatures in this mapped, page-locked buffer and waits (bounded) for
// the host service thread to answer.
constexpr int kHostVelCap = 1 << 16;
struct HostVelocity {
  unsigned int seq_req, seq_done, n, pad;
  double T[kHostVelCap];
  double v[kHostVelCap];
};

// Temperature classes of a liquid cell (the comparisons the capture sweep and
// the liquid-neighbour pass make with it): T < Tm, T <= Tm, T > nullMatTemp_,
// T >= nullMatTemp_ + 0.01.
constexpr uint8_t kTlt = 1, kTle = 2, kTgtNull = 4, kTgeNullPlus = 8;

struct RemeltCtrl {
  unsigned int bar_count, bar_gen;  // one 64-bit arrival counter of the grid barrier, zero at every launch
  int error;
  int status;
  // coupling scalars, published by block 0 at the end of every step
  long long step;      // completed CA steps (iStep_)
  double time;         // CafeSolver time == CA time_
  double dt;           // dT_ of the last step
  double dt_prev;      // dT_ of the step before it
  double dT_FE;        // FiniteElementManager::get_max_time_step()
  double max_ts;       // CA maxTimestep_
  double fe_time, ts0, ts1, ratio;  // FiniteElementManager time_, inTimeSeries_[0], [1], last ratio
  int f_new;           // frame held in theta_[0] (theta_[1] is f_new - 1)
  int f_next;          // next frame to load
  int theta_init;      // thetaArray_ still equals frame 0 (no pseudo step yet)
  int pad0;
  long long n_orient, n_grains;
  // work lists of the current step (parity-indexed where a list outlives a step)
  unsigned int n_liq, n_claim, n_new, n_hard;
  unsigned int host_seq;  // requests posted to the host so far
  int vmin_hard;          // the velocity at the minimum temperature came from the host
  double vmin;
  unsigned int n_flag[2];
  unsigned int n_eact[2];
  unsigned long long minT_key;
  // counters
  unsigned long long tests, tests64, captures, nucleations, flagged, liquid, exact_T, melts, host_vel, host_calls,
      cells_visited, elements_active;
  unsigned long long ns_phase[5];
  unsigned long long ns_host;  // block 0's wait for host velocity answers
  unsigned long long ns_barrier;  // block 0's time inside grid barriers
  // per-block busy time between barriers, by the barrier that closes it
  // (0 A, 1 B, 2 C, 3 D, 4 E, 5 host velocities): sum over blocks and the
  // sum over steps of the slowest block; scratch holds the current step's max
  unsigned long long ns_work_sum[6], ns_work_max[6], work_scratch[6];
  unsigned long long ns_newgrain, ns_nucleation;  // block 0's new-grain ids (phase A) and nucleation (phase C)
  unsigned long long ns_flags_max, flags_scratch;  // slowest block's liquid-neighbour flag pass (phase B)
  int fstat_frame[2];          // frame whose per-element extrema each slot holds (-1: none)
  int any_near;                // some element met a frame near the void threshold: rebuild every step
  unsigned int n_nuc_sites[2];  // sites that nucleate in the step, by step parity (phase B counts, C reads)
};

static_assert(offsetof(RemeltCtrl, bar_count) == 0 && offsetof(RemeltCtrl, bar_gen) == 4,
              "barrier words must form one aligned 64-bit word");

struct RemeltDevice {
  Grid g;
  int64_t ncells;
  // physics (ProblemPhysics.cpp:58-158)
  double Tm, Ts, Tnuc, a1, a2, a3;
  int b1, b2, b3;
  double tsf_ca, h, trunc, cutoff, final_time, void_t;
  float h32, coord_err;
  // the liquidus and nullMatTemp_ + 0.01 rounded down and up to float: the
  // FP32 temperature bounds are compared with these (float_bounds)
  float tm_lo, tm_hi, np_lo, np_hi;
  // cells (ghost-inclusive)
  int32_t *orient;     // cellOrientationID_ (claims during a step: INT_MIN + sweep position)
  int32_t *grain;      // cellGrainID_
  uint8_t *melted;     // hasBeenMelted_
  uint32_t *flagbits;  // cellLiquidNeigh as a bitmap
  uint8_t *tcls;       // liquid cells, this step: temperature classes (kTlt.. bits below)
  const float *pc32;   // parCoordsList_ rounded to float, for the FP32 classification
  const int32_t *tag;  // MapVoxelManager elementTagList_
  const double *pc;    // parCoordsList_
  // grain records, one per cell (the grain its cell owns)
  double *gx, *gy, *gz, *glen;
  int32_t *gori;
  float *gdx, *gdy, *gdz;  // grain centre - own cell centre, FP32, for the pre-test
  // orientations
  const double *omat;
  const float *omat32;
  long long orient_cap;
  // nucleation sites (ascending cell id)
  const int32_t *site_cell;
  const double *site_dtc;
  int nsites;
  // FE replay
  int nn[3];
  int64_t nnodes, nelem;
  const double *frames;      // ring of frame_slots frames (frame f in slot f % frame_slots), nnodes each
  const double *frame_time;  // per frame, scaled (every frame)
  int nframes;               // frames in all
  int frame_slots;           // slots of the ring (nframes when every frame is resident)
  int frames_avail;          // frames 0 .. frames_avail - 1 have been loaded (the last frame_slots of them are held)
  int bad_frame;             // index of a malformed frame, or -1
  // coupling with an external solver (amca_step_coupled, amca_run_until, amca_set_nodal_temperatures)
  double dt_cap;             // extra upper bound on dt (+inf: none)
  double t_stop;             // the launch stops before a step that starts at time >= t_stop (+inf: none)
  int external;              // node temperatures come from the host between steps: no frame replay
  double *theta[3];          // node temperatures by CA step (mod 3)
  float *theta32[3];         // the same, rounded to float
  double *emax, *emin;       // per element bounds on the interpolated temperature (current step)
  int force_exact;           // some parametric coordinate is not finite: no bound shortcuts
  int detail;                // nonzero: also gather the slowest block's busy time per barrier
  uint8_t *evoid;            // per element: some node below void_temperature + 1e-5
  int32_t *eliq;             // per element: interior liquid cells it holds
  double *fmax[2], *fmin[2]; // per element: node extrema of a frame (slot = frame index & 1)
  uint8_t *fnear[2];         // per element: some node of that frame near void_temperature + 1e-5 (or NaN)
  const int64_t *ecell_start;  // element -> its interior cells (CSR)
  const int32_t *ecell;
  int32_t *eact[2];          // elements whose cells the next phase update visits, by step parity
  uint8_t *snuc;             // per site: nucleates this step (1), and creates a grain object (2)
  // lists
  int32_t *liq;              // liquid cells whose neighbours may be flagged
  int32_t *flagged[2];       // flagged cells, by step parity
  int32_t *claimed;          // cells claimed in the sweep
  unsigned long long *newkey;  // new-grain events: (sweep position << 5 | neighbour index)
  int32_t *newcell;
  double *fvel;              // growth velocity per flagged-list entry
  int32_t *hard_idx;         // flagged-list entries whose velocity the host evaluates
  double *hard_T;
  HostVelocity *host;        // device view of the mapped host buffer
  int host_cap;              // entries of `host` one request may use (kHostVelCap; smaller in tests)
  int64_t list_cap;
  RemeltCtrl *ctrl;
};

// Per-voxel search of MapVoxelManager::tag_voxels / is_in_element
// (CA/src/MapVoxelManager.cpp:357-699), one thread per ghost-inclusive voxel.
struct TagPlan {
  double mm[6], dbin[3];
  int nbin[3];
  const int64_t *bin_start;
  const int32_t *bin_elems;
  const double *erange;  // 6 per element
  const double *coord;   // 3 per node
  int nn[3];
  double tolerance;
  int max_iter;
  unsigned long long *counts;  // [0] voxels with an element, [1] voxels with a non-finite parametric coordinate
};
cudaError_t remelt_tag_voxels(const Grid &g, const TagPlan &p, int32_t *tag, double *pc, cudaStream_t s);

// Synthetic frames: the Rosenthal moving-source field on a structured node
// grid, evaluated with IEEE add/mul/div/sqrt and a fixed exp polynomial.
struct RosenthalParams {
  double origin[3], spacing;  // node coordinates in file units: origin + spacing * index
  int nodes[3];
  double length_scale;        // file unit -> m for the field evaluation
  double frame_dt, time_scale;  // frame f at file time f * frame_dt (plus an offset)
  double power, absorptivity, speed, conductivity, diffusivity, t0, t_cap, x_start, y_line, z_top;
  int void_above_set;
  double void_above, t_void;
};
cudaError_t remelt_rosenthal_frames(const RosenthalParams &p, int nframes, double *frames, cudaStream_t s);

// pc32[i] = (float)pc[i]
cudaError_t remelt_round_coords(const double *pc, float *pc32, int64_t n, cudaStream_t s);

// Frame-0 node temperatures and element bounds before the first step.
cudaError_t remelt_init_theta(const RemeltDevice &d, cudaStream_t s);

// Grain records (centre, half-diagonal) of the initial microstructure from
// the grain field already on the device: cell centre and length 0 for every
// interior cell that holds a grain, zeros elsewhere.
cudaError_t remelt_init_records(const RemeltDevice &d, cudaStream_t s);

// Grid size for the persistent kernel: per_sm co-resident blocks per SM (at
// most what fits).
int remelt_persistent_grid(int device, int per_sm);

// Run CA steps until `limit` steps in total, the final time, the end of the
// frames, or an orientation stream shorter than a step may need.
cudaError_t remelt_run_steps(const RemeltDevice &d, long long limit, int blocks, cudaStream_t s);

// Node temperatures of the next step (`step` = steps completed so far) from
// the host's theta (device copy, nnodes doubles): the node arrays of that
// step, each element's bounds and void flag, and the list of elements whose
// cells the step's phase update visits (an external solver's frame).
cudaError_t remelt_external_theta(const RemeltDevice &d, long long step, const double *theta, cudaStream_t s);

// Every cell's temperature and cooling flag of the last completed step (the
// values the reference holds in cellTemperature_ / cooling_), plus the
// liquid-neighbour flags as bytes.
cudaError_t remelt_state_fields(const RemeltDevice &d, long long step, double dt_prev, double *T, uint8_t *cooling,
                                uint8_t *flag, cudaStream_t s);

}  // namespace amca
