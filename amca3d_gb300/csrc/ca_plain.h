// ca_plain.h — device state and launch API of the plain (uniform-cooling)
// CA step on one GPU.
//
// HBM layout (one realm):
//   orient      u32[(nx+2)(ny+2)(nz+2)]  cellOrientationID_, ghost-inclusive, reference index order
//   solid       1 bit per cell (+2 words): solid before the current generation; the
//               claim phase's liquidity test reads this (L2-resident) instead of orient
//   claimed     1 bit per cell (+2 words): set with every claim. A claimed cell is
//               captured in that generation and never liquid again, so stale bits
//               are never looked at and the map is never cleared during a run
//   site_*      nucleation sites sorted by cell id: cell i32, dTc f64, live u8
//   omat/omat32 per orientation: local->global matrix, 9 x f64 and 9 x f32
//   g*          envelope table by id (capacity = interior cells), written once per
//               envelope: centre f64 x3, orientation i32, cell i32
//   act[2]      the envelope list: 32-byte records in walk order, appended to by
//               nucleation and captures, dead entries left in place (tombstones)
//               until a compaction into the other buffer; per entry beside it:
//               key[2]   f32 wake key (cumulative growth at which the entry may
//                        contain a liquid neighbour; NaN = dead)
//               lstep[2] i32 step up to which the record's half-diagonal is grown
//   late        i32 per entry: step of the last capture next to it by a later rank
//   cellw       u32 per ghost-inclusive cell: list position of the live envelope
//               on the cell << 5 | its liquid neighbours now; kNoEntry (all
//               ones) for none, which the at most 26 decrements a cell sees
//               while it has no envelope never bring to a zero count
//   wlist       i32 per entry: positions woken this step, in walk order
//   zlist[2]    i32 per entry: entries whose liquid count reached zero in a
//               generation, by generation parity
//   dvh         f64 ring of the growth increment of each step
//   liq/con     per-rank neighbour masks of the generation being processed
//   cellr       per-rank cell of the generation being processed
//   child       per new envelope: parent's list position << 5 | neighbour index
//   scanA..D    decoupled look-back status words, one per block: nucleation and
//               wake scan (two sets each, by step parity), capture, compaction
//               (two sets, by compaction parity)
//   ctrl        control block: counters, time, barrier words, error flag
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "ca_math.h"

namespace amca {

// Look-back status words per phase: an upper bound on the persistent grid.
constexpr long long kStatusWords = 4096;
// Child records and cell words pack a list position into 27 bits: a realm
// has fewer than kMaxCells interior cells.
constexpr long long kMaxCells = 1ll << 27;
// Steps of the growth-increment ring; every live entry is woken (its record
// brought up to date) at least every kWakeAll steps, well inside the ring.
constexpr long long kDvRing = 4096;
constexpr long long kWakeAll = 2048;
// The wake scan reads keys in tiles of this many positions; key arrays hold
// that many more entries than the list can (the tail of the last tile).
constexpr long long kKeyTile = 128;
// Cell word of a cell without an envelope; its position field (all ones)
// is never a list position (the list holds fewer than kMaxCells entries).
constexpr uint32_t kNoEntry = 0xFFFFFFFFu;
AMCA_HD bool has_entry(uint32_t w) { return (w >> 5) != (kNoEntry >> 5); }
// Defaults of PlainDevice::warp_sched and PlainDevice::mark_split.
constexpr int kWarpSched = 32;
constexpr int kMarkSplit = 1024;
constexpr int kDecWarps = 2;
constexpr int kCompactSlack = 4096;
constexpr int kMarkBatch = 4;  // ranks per thread whose marks are computed before any is stored
// Warps per block that start a claim phase with the decrements on teams of
// at most 64 blocks (the batched launch).
constexpr int kDecWarpsTeam = 4;

// Control block. Between launches it holds the realm's state (step, time,
// active count, ...). Inside a launch every block keeps the per-step values
// in shared memory (identical in every block); the fields written by one
// block in a phase are read by all only after the barrier that closes that
// phase.
struct PlainCtrl {
  unsigned bar_count;  // with bar_gen: one 64-bit arrival counter of the grid barrier, zero at every launch
  unsigned bar_gen;
  int error;        // 0, or where a bounded wait ran out (see kErr*)
  int cur_list;     // which act[] holds the envelope list
  long long n_orient;
  long long next_grain;
  long long n_active;          // active envelopes between launches
  long long a_len;             // entries of the envelope list (live and dead) between launches
  long long n_active_nuc[2];   // list length after the step's nucleation, by step parity
  long long n_woken[2];        // entries of the list the wake scan picked, by step parity
  long long compact_len;       // live entries after the last compaction
  long long deaths[3];         // entries leaving the active list in step s, in slot s % 3
  long long gen_surv;          // survivors of the last resolved generation
  unsigned long long zn[2];    // zero-count events of a generation, by generation parity
  double grown;                // growth of the envelopes since the start of the run (sum of dv)
  long long liquid;
  long long gen_n;  // captures of the last resolved generation
  long long step;
  double time;
  double dt;
  int done;
  int pad;
  unsigned long long tests;
  unsigned long long tests64;
  unsigned long long gens;
  unsigned long long captures;
  // work counters behind the algorithmic-bytes figure
  unsigned long long sites_scanned;    // live sites read by nucleation, summed over steps
  unsigned long long nucleations;      // envelopes created by nucleation
  unsigned long long ref_walked;       // the reference walk's generation 0 (active envelopes after nucleation), summed over steps
  unsigned long long active_grown;     // generation-0 entries processed (woken and nuclei), summed over steps
  unsigned long long grains_processed; // entries processed in every generation, summed
  unsigned long long keys_scanned;     // list positions the wake scan read, summed over steps
  unsigned long long decrements;       // liquid-count decrements that reached an envelope's cell word
  unsigned long long zero_events;      // liquid counts that reached zero in a capture generation
  unsigned long long compactions;      // compactions of the envelope list
  unsigned long long compacted;        // entries moved by them
  // wall time of each phase as block 0 sees it (phase start to barrier exit), ns
  unsigned long long ns_nucleation, ns_claim, ns_resolve, ns_step_end;
  unsigned long long ns_claim_gen0;                    // part of ns_claim spent on generation 0
  unsigned long long ns_claim_work_sum, ns_claim_work_max;  // per-block busy time in claim phases
  unsigned long long ns_resolve_work_sum, ns_resolve_work_max;
  unsigned long long ns_nuc_work_sum, ns_wake_work_sum, ns_compact_work_sum;  // per-block busy time, summed
  unsigned long long ns_barrier_block0;  // block 0's time inside grid barriers (arrival to release)
  unsigned long long ns_nuc_work_max;                  // slowest block's busy time in nucleation + wake scan (detail)
  unsigned long long phase_max_scratch[3];             // running max of the current phase
  unsigned long long claim_next;                       // next unclaimed rank batch of the claim phase
  unsigned long long mark_next;                        // next rank batch of a separate marking pass
};

// The barrier reads (bar_count, bar_gen) as one 64-bit word, generation in
// the high half.
static_assert(offsetof(PlainCtrl, bar_count) == 0 && offsetof(PlainCtrl, bar_gen) == 4,
              "barrier words must form one aligned 64-bit word");

enum { kErrBarrier = 1, kErrLookback = 2 };

// One envelope as the envelope list carries it: everything the neighbour
// tests need in one 32-byte record.
struct alignas(16) EnvRec {
  double L;            // half-diagonal length
  float dx, dy, dz;    // centre minus own-cell centre, rounded to float
  int32_t cell;        // ghost-inclusive cell index
  int32_t ori;         // orientation id
  int32_t id;          // envelope id (index of the by-id table)
};
static_assert(sizeof(EnvRec) == 32, "EnvRec must stay one 32-byte sector");

struct PlainDevice {
  Grid grid;
  // physics
  double T0, Tm, Tdot, a1, a2, a3;
  double max_dt, final_time, tsf, trunc;
  // coupling with an external solver; 0 (the zero-initialised default) means none
  double dt_cap;  // extra upper bound on dt
  double t_stop;  // no step starts at time >= t_stop
  float h32;
  float coord_err;  // bound on FP64 cell-centre rounding, per component
  int phase_detail; // nonzero: also gather the slowest block's busy time per phase
  int warp_sched;   // ranks per block of the team up to which claims are handed out warp by warp (else block by block)
  int mark_split;   // ranks per block of the team up to which a generation is marked inside the resolve pass
  int dec_warps;    // warps per block that start a claim phase with the liquid-count decrements (1..kWarps)
  int compact_slack;  // the list is compacted when it holds more than 2 x active + this many entries
  // arrays
  uint32_t *orient;
  uint32_t *solid;    // 1 bit per cell: solid at the start of the current generation (ghosts included)
  uint32_t *claimed;  // 1 bit per cell: some envelope claimed it (only ever read on cells still liquid)
  int64_t ncells;
  const int32_t *site_cell;
  const double *site_dtc;
  uint8_t *site_live;
  int64_t nsites;
  const double *omat;
  const float *omat32;
  double *gx, *gy, *gz;
  int32_t *gori, *gcell;
  int64_t gcap;
  EnvRec *act[2];
  float *key[2];
  int32_t *lstep[2];
  int32_t *late;
  uint32_t *cellw;
  int32_t *wlist;
  int32_t *zlist[2];
  double *dvh;
  uint32_t *liq, *con;
  int32_t *cellr;
  uint32_t *child;
  unsigned long long *scanA, *scanB, *scanC, *scanD;
  PlainCtrl *ctrl;
};

// One team of the batched launch: its barrier words and the realm it runs in
// the current round, by round parity (-1: none left).
struct alignas(8) BatchTeam {
  unsigned count;  // with gen: one 64-bit arrival counter of the team barrier, zero at every launch
  unsigned gen;
  int slot[2];
};

// Layout of a batched launch (device arrays): per block its team and rank
// in the team; per team its size and class; per class the (first position,
// count) of its realms in the launch's order array.
struct BatchPlanDev {
  const int2 *blk;
  const int *tsize;
  const int *tclass;
  const int2 *crange;
};

// Self-test of the bounded grid barrier with `blocks` blocks (cooperative)
// expecting `parties` arrivals, every wait limited to wait_ns, the error word
// preset to `preset`: *error_out = the error word afterwards, verdicts[b] =
// 1 when block b's barrier returned true.
cudaError_t plain_barrier_selftest(int blocks, int parties, long long wait_ns, int preset, int *error_out,
                                   int *verdicts);

// Fill the orientation field: -1 interior, 0 on the ghost layer
// (CellularAutomataManager.cpp:316-326, CellularAutomataManager_3D.cpp:736-833),
// the solid bitmap to match, and the cell -> list position map with -1.
cudaError_t plain_init_field(const PlainDevice &d, cudaStream_t s);

// Words of the solid bitmap for `ncells` cells.
AMCA_HD long long solid_words(long long ncells) { return (ncells + 31) / 32 + 2; }

// Blocks of the persistent kernel that fit on the device at once.
int plain_persistent_grid(int device);

// Run CA steps until solid, final_time, or ctrl->step reaches step_limit.
// One cooperative launch; every phase boundary is a bounded grid barrier.
cudaError_t plain_run_steps(const PlainDevice &d, long long step_limit, int grid_blocks, cudaStream_t s);

// Blocks of the batched kernel that fit on the device at once.
int plain_batched_grid(int device);

// Every realm of insts[0..ninst) (a device array) back to its state right
// after initialize; the nclasses queues, the error word and the nteams team
// records to zero.
cudaError_t plain_batch_reset(const PlainDevice *insts, int ninst, unsigned *queues, int nclasses, BatchTeam *teams,
                              int nteams, int *error, cudaStream_t s);

// One cooperative launch of grid_blocks blocks laid out by `plan`: the teams
// of each class take that class's realms, in order, from the class's queue
// and run each to solid, final_time or step_limit, as plain_run_steps would.
// A team barrier that ran out sets *error; a realm's own failures go to its
// control block.
cudaError_t plain_batched_run(const PlainDevice *insts, const int *order, int ninst, const BatchPlanDev &plan,
                              int grid_blocks, unsigned *queues, BatchTeam *teams, int *error, long long step_limit,
                              cudaStream_t s);

// out[r] (device) = realm r's control block.
cudaError_t plain_batch_gather(const PlainDevice *insts, int ninst, PlainCtrl *out, cudaStream_t s);

// cellGrainID_ from the envelope table: -1 liquid, 0 ghost layer, else the
// id of the envelope created for the cell.
cudaError_t plain_grain_field(const PlainDevice &d, int32_t *out, long long ngrains, cudaStream_t s);

// Device evaluation of the envelope arithmetic on n independent pairs (all
// pointers device memory): FP64 containment, the production FP32/FP64
// decision, and the decentred capture (info: offset xyz + new half-diagonal).
cudaError_t plain_envelope_eval(long long n, const double *l2g, const double *gc, const double *len, double h,
                                const double *trunc, int32_t *cap64, int32_t *capfast, double *info, cudaStream_t s);

}  // namespace amca
