// remelt.cu — the FE-coupled remelting realm on one GB300.
//
// Reference (np = 1): CafeSolver::time_integration_weak_coupling
// (CA/src/CafeSolver.cpp:178-219). Per step the reference
//   1. re-interpolates every cell's temperature from the FE nodes, melts
//      cells at or above the liquidus (or without material), updates the
//      cooling and melted flags (CellularAutomataManager_3DRemelting.cpp:339-404);
//   2. flags solid cells next to undercooled liquid (:484-542);
//   3. nucleates at sites, then takes dt from the coldest flagged cell above
//      the solidus (:656-727, :936-999);
//   4. sweeps the interior in i-outer, j, k-inner order: every flagged cell
//      grows its grain and captures liquid neighbours inside its octahedron;
//      a captured cell is not swept again in the same step (:545-652, :807-847);
//   5. advances the FE replay and interpolates nodal temperatures between two
//      frames (LoadDataFromFile.cpp:207-313).
//
// GB300 design: one persistent cooperative kernel runs whole steps, five
// phases per step separated by bounded grid barriers.
//   A  full-grid pass over interior cells. A cell's temperature is a pure
//      function of the node temperatures, so it is computed in FP64 only where
//      a decision depends on it: liquid cells, and solid cells whose element's
//      node maximum (plus a rounding margin) reaches the liquidus. Every other
//      solid cell costs two 4-byte loads and an L2-resident element lookup.
//      (GB300's FP64 rate is ~1/64 of its FP32 rate; this keeps the step
//      bandwidth-bound.) Liquid cells that can flag neighbours go to a list.
//   B  listed liquid cells set the flag bits of their solid neighbours; each
//      newly flagged cell is appended to the flagged list.
//   C  block 0 nucleates (sites in ascending order, block scan for ids);
//      the other blocks apply the grain-length cutoff and take the minimum
//      temperature over flagged cells (atomicMin on an ordered key).
//   D  dt (uniform); every flagged cell grows its grain and tests its liquid
//      neighbours; a containment claims the neighbour with atomicMin of
//      INT_MIN + sweep position, so the smallest claim is the first capturing
//      cell of the reference's sweep (captures do not cascade within a step).
//   E  claimed cells take the winner's orientation and decentred envelope
//      (FP64, reference operation order); the FE replay advances and the next
//      step's node temperatures and element bounds are computed.
// New grain objects (cells without one) get ids in sweep order: events
// (sweep position, neighbour index) are sorted by block 0 after the step.
#include <cooperative_groups.h>
#include <cooperative_groups/scan.h>
#include <math.h>

#include <algorithm>

#include "remelt.h"

namespace amca {

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
constexpr int kCellPre = 4;  // cells per lane whose phase-update loads are issued together
constexpr unsigned long long kWaitNs = 5000000000ull;  // 5 s bound on any spin

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long atom_add_acq_rel64(unsigned long long *p, unsigned long long x) {
  unsigned long long old;
  asm volatile("atom.add.acq_rel.gpu.global.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(x) : "memory");
  return old;
}
template <typename T>
__device__ __forceinline__ T ld_volatile(const T *p) {
  return *(const volatile T *)p;
}

// When this block left its last grid barrier (thread 0), and its busy time
// per barrier kind, added to the control block once per launch
// (same-address atomics from every block at every barrier would serialise).
__shared__ unsigned long long s_left;
__shared__ unsigned long long s_busy[6];
// Block 0's clocks and host round trips (its thread 0), added to the control
// block once per launch: a read-modify-write of the control block after a
// barrier would hold up block 0 by a global round trip.
enum {
  kClkPhase = 0,  // [0..4] phases A..E
  kClkBarrier = 5,
  kClkHost,
  kClkHostCalls,
  kClkHostVel,
  kClkNewgrain,
  kClkNucleation,
  kClkFlagsMax,
  kClkWorkMax,  // [kClkWorkMax + p], p = 0..5
  kClkN = kClkWorkMax + 6
};
__shared__ unsigned long long s_clk[kClkN];
__shared__ unsigned s_host_seq;  // requests posted to the host so far (every block counts them)
__shared__ int s_bar_ok;         // thread 0's verdict on the block's last barrier

// Counting grid barrier bounded in time; false when a wait ran out or
// thread 0 saw the error word set: sampled as it arrives (the load's latency
// hides behind the arrival) and while it waits. An error raised in this
// block before the barrier is always seen; one raised elsewhere at the latest
// at the next barrier, where every block still running waits on those that
// stopped (every list append is bounds-checked, so the phase between is
// safe). The verdict reaches the block through shared memory. `p` names the
// work it closes (see RemeltCtrl::ns_work_sum) for the busy-time counters;
// the slowest block's time is gathered only with d.detail (a global load per
// block and barrier).
__device__ bool grid_barrier(const RemeltDevice &d, int p) {
  RemeltCtrl *c = d.ctrl;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long tb = now_ns();
    const unsigned long long w = tb - s_left;
    s_busy[p] += w;
    if (d.detail && w > ld_volatile(&c->work_scratch[p])) atomicMax(&c->work_scratch[p], w);
    // (bar_count, bar_gen) as one 64-bit arrival counter that only grows:
    // zero when the launch starts (host reset), one acquire-release atomic
    // per arrival (the block's writes, ordered before it by the block
    // barrier, are released with it; the last arrival acquires the others'
    // through it), and barrier k of the launch ends when it reaches k x
    // gridDim.x; the others wait with acquire loads. No arrival has to open
    // the next barrier with a second atomic.
    unsigned long long *bw = (unsigned long long *)&c->bar_count;
    const int seen = ld_volatile(&c->error);
    const unsigned long long old = atom_add_acq_rel64(bw, 1ull);
    const unsigned long long nb = gridDim.x;
    const unsigned long long target = (old / nb + 1ull) * nb;
    bool ok = true;
    if (old + 1ull != target) {
      const unsigned long long t0 = now_ns();
      unsigned it = 0;
      while (ld_acquire64(bw) < target) {
        if ((++it & 7u) == 0u) {
          if (ld_volatile(&c->error) != 0) {
            ok = false;
            break;
          }
          if (now_ns() - t0 > kWaitNs) {
            atomicCAS(&c->error, 0, kRemeltErrBarrier);
            ok = false;
            break;
          }
        }
        __nanosleep(32);
      }
    }
    s_left = now_ns();
    s_bar_ok = ok && seen == 0;
    if (blockIdx.x == 0) {
      s_clk[kClkBarrier] += s_left - tb;
      if (d.detail) {
        // every block's maximum for this work is in; the next one comes at
        // least four barriers later
        s_clk[kClkWorkMax + p] += ld_volatile(&c->work_scratch[p]);
        c->work_scratch[p] = 0ull;
      }
    }
  }
  __syncthreads();
  return s_bar_ok != 0;
}

__device__ unsigned block_exclusive_scan(unsigned v, unsigned *smem, unsigned *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned w = lane < kWarps ? smem[lane] : 0u;
#pragma unroll
    for (int o = 1; o < kWarps; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kWarps) smem[lane] = w;
  }
  __syncthreads();
  const unsigned before = warp > 0 ? smem[warp - 1] : 0u;
  *total = smem[kWarps - 1];
  __syncthreads();
  return before + x - v;
}

// List append from the threads that reach it together: one atomicAdd per
// coalesced group, ranks within the group (order within a list is free).
__device__ __forceinline__ unsigned append_slot(unsigned *counter) {
  namespace cg = cooperative_groups;
  cg::coalesced_group grp = cg::coalesced_threads();
  unsigned base = 0;
  if (grp.thread_rank() == 0) base = atomicAdd(counter, grp.size());
  return grp.shfl(base, 0) + grp.thread_rank();
}

// Block-staged list appends: entries go to a shared-memory buffer (shared
// atomic), and the block moves the buffer to the global list with one
// global atomicAdd when the phase ends (stage_flush, every thread) — one
// same-address global atomic per block instead of one per warp and
// iteration. Entries beyond the buffer go to the global list directly.
constexpr unsigned kStage = 1024;
__shared__ unsigned s_stage_n;
__shared__ int32_t s_stage[kStage];

__device__ __forceinline__ void stage_push(int32_t v, unsigned *count, int32_t *list, unsigned cap) {
  const unsigned k = atomicAdd(&s_stage_n, 1u);
  if (k < kStage) {
    s_stage[k] = v;
  } else {
    const unsigned slot = atomicAdd(count, 1u);
    if (slot < cap) list[slot] = v;
  }
}

__device__ void stage_flush(unsigned *count, int32_t *list, unsigned cap) {
  __shared__ unsigned s_base;
  __syncthreads();
  const unsigned n = min(s_stage_n, kStage);
  if (threadIdx.x == 0) s_base = n ? atomicAdd(count, n) : 0u;
  __syncthreads();
  for (unsigned i = threadIdx.x; i < n; i += blockDim.x)
    if (s_base + i < cap) list[s_base + i] = s_stage[i];
  __syncthreads();
  if (threadIdx.x == 0) s_stage_n = 0u;
  __syncthreads();
}

// `cnt` consecutive list slots for each thread that reaches it together: one
// atomicAdd per coalesced group, the group's counts placed by an inclusive
// scan (order within a list is free).
__device__ __forceinline__ unsigned append_slots(unsigned *counter, unsigned cnt) {
  namespace cg = cooperative_groups;
  cg::coalesced_group grp = cg::coalesced_threads();
  const unsigned incl = cg::inclusive_scan(grp, cnt);
  unsigned base = 0;
  if (grp.thread_rank() == grp.size() - 1) base = atomicAdd(counter, incl);
  return grp.shfl(base, grp.size() - 1) + incl - cnt;
}

// Short lists whose items carry FP64 work or long load chains are dealt
// across blocks first: item q goes to block first_block + q % nb (thread
// q / nb of it), so the work spreads over every SM instead of filling the
// first few. Visit q = spread_begin(...), then q += spread_stride(...).
__device__ __forceinline__ int64_t spread_begin(int first_block) {
  const int64_t nb = gridDim.x - first_block;
  return (int64_t)threadIdx.x * nb + (blockIdx.x - first_block);
}
__device__ __forceinline__ int64_t spread_stride(int first_block) {
  return (int64_t)(gridDim.x - first_block) * blockDim.x;
}
// The same spread over all blocks, last block first: for short lists whose
// items are heavy, so that they meet the blocks with the least other work in
// the phase (those past the ends of the thread-ordered loops).
__device__ __forceinline__ int64_t spread_begin_last() {
  return (int64_t)threadIdx.x * gridDim.x + (gridDim.x - 1 - blockIdx.x);
}

// Order-preserving key of a double (for atomicMin); NaN never reaches it.
__device__ __forceinline__ unsigned long long dkey(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
  const unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)b);
}

__device__ __forceinline__ double ulp_of(double p) {  // |p| normal
  const long long e = (__double_as_longlong(fabs(p)) >> 52) & 0x7ff;
  return e > 52 ? __longlong_as_double((e - 52) << 52) : 4.9406564584124654e-324;
}

// x^b for b in {1, 2, 3}, correctly rounded (square and cube through exact
// two-products). `near` is raised when the exact power lies within 0.02 ulp
// of a rounding midpoint: there glibc's pow, whose error bound is 0.52 ulp,
// may round to the other neighbour. pow(x, 1) == x holds for every double.
__device__ double ipow_checked(double x, int b, bool &near) {
  if (b == 1) return x;
  const double p = x * x;
  const double e = __fma_rn(x, x, -p);
  if (b == 2) {
    const double u = ulp_of(p);
    near = near || fabs(fabs(e) - 0.5 * u) <= 0.02 * u;
    return p;
  }
  const double q1 = p * x;
  const double r1 = __fma_rn(p, x, -q1);
  const double q2 = e * x;
  const double r2 = __fma_rn(e, x, -q2);
  const double t = (r1 + q2) + r2;
  const double c = q1 + t;
  const double rem = (q1 - c) + t;
  const double u = ulp_of(c);
  near = near || fabs(fabs(rem) - 0.5 * u) <= 0.02 * u;
  return c;
}

// compute_growth_velocity_with_temperature_input (ProblemPhysics.cpp:142-158).
// `hard`: a term with a nonzero coefficient could round differently in glibc.
__device__ double velocity(const RemeltDevice &d, double T, bool &hard) {
  const double dT = d.Tm - T;
  double v = 0.0;
  hard = false;
  if (dT > 0) {
    bool n1 = false, n2 = false, n3 = false;
    const double p1 = ipow_checked(dT, d.b1, n1);
    const double p2 = ipow_checked(dT, d.b2, n2);
    const double p3 = ipow_checked(dT, d.b3, n3);
    hard = (d.a1 != 0 && n1) || (d.a2 != 0 && n2) || (d.a3 != 0 && n3);
    v = d.a1 * p1 + d.a2 * p2 + d.a3 * p3;
    if (v < 0.0) v = 0.0;
  }
  return v;
}

__device__ __forceinline__ unsigned ld_acquire_sys(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.sys.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(unsigned *p, unsigned v) {
  asm volatile("st.release.sys.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Block 0: have the host evaluate the velocities flagged `hard` this step
// (and the velocity at the minimum temperature when `min_hard`), in chunks
// of host_cap entries, one request each (the other blocks count them after
// the barrier that follows). Every wait is bounded; false on a timeout.
__device__ bool host_velocities(const RemeltDevice &d, RemeltCtrl *c, unsigned nh, bool min_hard, double minT) {
  __shared__ int s_ok;
  const unsigned total = nh + (min_hard ? 1u : 0u);
  const unsigned cap = (unsigned)d.host_cap;
  if (threadIdx.x == 0) s_ok = d.host != nullptr;
  __syncthreads();
  for (unsigned base = 0; base < total && s_ok; base += cap) {
    const unsigned cnt = min(total - base, cap);
    for (unsigned k = threadIdx.x; k < cnt; k += blockDim.x) {
      const unsigned i = base + k;
      d.host->T[k] = i < nh ? d.hard_T[i] : minT;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned long long h0 = now_ns();
      const unsigned seq = s_host_seq + 1;
      s_host_seq = seq;
      d.host->n = cnt;
      __threadfence_system();
      st_release_sys(&d.host->seq_req, seq);
      const unsigned long long t0 = now_ns();
      while (ld_acquire_sys(&d.host->seq_done) != seq) {
        if (now_ns() - t0 > kWaitNs) {
          atomicCAS(&c->error, 0, kRemeltErrHost);
          s_ok = 0;
          break;
        }
        __nanosleep(64);
      }
      s_clk[kClkHostCalls] += 1;
      s_clk[kClkHostVel] += cnt;
      s_clk[kClkHost] += now_ns() - h0;
    }
    __syncthreads();
    if (!s_ok) break;
    for (unsigned k = threadIdx.x; k < cnt; k += blockDim.x) {
      const unsigned i = base + k;
      const double v = ld_volatile(&d.host->v[k]);
      if (i < nh)
        d.fvel[d.hard_idx[i]] = v;
      else
        c->vmin = v;
    }
    __syncthreads();
  }
  __threadfence();
  return s_ok != 0;
}

// The overlapped form of host_velocities for a request that fits the mapped
// buffer: block 0 writes the temperatures and posts the request without
// waiting; every block counts it (its s_host_seq names the answer it waits
// for). Called by every block, uniformly.
__device__ void host_post(const RemeltDevice &d, unsigned nh, bool min_hard, double minT) {
  const unsigned total = nh + (min_hard ? 1u : 0u);
  if (blockIdx.x == 0 && d.host != nullptr) {
    for (unsigned k = threadIdx.x; k < total; k += blockDim.x) d.host->T[k] = k < nh ? d.hard_T[k] : minT;
    __syncthreads();
    if (threadIdx.x == 0) {
      d.host->n = total;
      __threadfence_system();
      st_release_sys(&d.host->seq_req, s_host_seq + 1);
      s_clk[kClkHostCalls] += 1;
      s_clk[kClkHostVel] += total;
    }
  }
  if (threadIdx.x == 0) s_host_seq += 1;
}

// Thread 0 waits (bounded) for the answer to the block's last request; the
// block proceeds after a barrier. A wait that runs out (or no host buffer)
// sets the error word, which the next grid barrier reports.
__device__ void host_wait_block(const RemeltDevice &d, RemeltCtrl *c) {
  if (threadIdx.x == 0) {
    const unsigned long long t0 = now_ns();
    if (d.host == nullptr) {
      atomicCAS(&c->error, 0, kRemeltErrHost);
    } else {
      while (ld_acquire_sys(&d.host->seq_done) != s_host_seq) {
        if (now_ns() - t0 > kWaitNs) {
          atomicCAS(&c->error, 0, kRemeltErrHost);
          break;
        }
        __nanosleep(64);
      }
    }
    if (blockIdx.x == 0) s_clk[kClkHost] += now_ns() - t0;
  }
  __syncthreads();
}

__device__ __forceinline__ void elem_nodes(const int nn[3], int64_t e, int64_t nid[8]) {
  const int64_t ncx = nn[0] - 1, ncy = nn[1] - 1;
  const int64_t i = e % ncx, j = (e / ncx) % ncy, k = e / (ncx * ncy);
  const int64_t nxy = (int64_t)nn[0] * nn[1];
  nid[0] = nxy * k + (int64_t)nn[0] * j + i;
  nid[1] = nid[0] + 1;
  nid[2] = nid[1] + nn[0];
  nid[3] = nid[2] - 1;
#pragma unroll
  for (int l = 4; l < 8; l++) nid[l] = nid[l - 4] + nxy;
}

// MapVoxelManager::evaluate_temperature (MapVoxelManager.cpp:746-799):
// false (T untouched) without an element or next to a void node.
__device__ bool eval_T(const RemeltDevice &d, const double *th, int64_t c, double &T) {
  const int32_t e = d.tag[c];
  if (e < 0) return false;
  int64_t nid[8];
  elem_nodes(d.nn, e, nid);
  const double nullMat = d.void_t + 0.00001;
  double t[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    t[i] = th[nid[i]];
    if (t[i] < nullMat) return false;
  }
  T = hex8_interp64(t, d.pc[3 * c], d.pc[3 * c + 1], d.pc[3 * c + 2]);
  return true;
}

// FP32 estimate of evaluate_temperature's value for a cell with material,
// with a bound on its error: the shape functions are convex weights
// (parametric coordinates in [-1, 1]), so the FP32 evaluation of the
// weighted sum, with the coordinates and node values rounded to float, errs
// by less than 2e-6 of the largest node magnitude; the bound returned is
// 2^-16 of it (plus 2^-16 absolute).
__device__ float eval_T32(const RemeltDevice &d, const float *th32, int64_t c, int32_t e, float &err) {
  int64_t nid[8];
  elem_nodes(d.nn, e, nid);
  float t[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) t[i] = th32[nid[i]];
  err = hex8_err32(t);
  return hex8_interp32(t, d.pc32[3 * c], d.pc32[3 * c + 1], d.pc32[3 * c + 2]);
}

// thetaArray_ update of pseudo_single_integration_step (LoadDataFromFile.cpp:281-290)
__device__ __forceinline__ double lerp_node(double th0, double th1, double ratio, double null_mat) {
  if (th0 <= null_mat) return null_mat;
  if (th1 <= null_mat) return th0;
  return ratio * (th0 - th1) + th1;
}

__device__ __forceinline__ bool ghost(const Grid &g, int I, int J, int K) {
  return I == 0 || I == g.nxg - 1 || J == 0 || J == g.nyg - 1 || K == 0 || K == g.nzg - 1;
}

// Bounds of one element for the current node temperatures: the interpolated
// temperature is a convex combination of the 8 node values (all parametric
// coordinates lie in [-1, 1]), so it cannot exceed their maximum by more than
// the rounding of the 8 products and sums (< 2^-48 relative); the margin
// used is 2^-44 of the largest magnitude. NaN forces the exact path.
__device__ void element_bounds(const RemeltDevice &d, int64_t e, const double t[8]) {
  const double nullMat = d.void_t + 0.00001;
  bool vo = false, nan = false;
  double mx = -INFINITY, mn = INFINITY, mg = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double v = t[i];
    if (v < nullMat) vo = true;
    if (v != v) nan = true;
    mx = v > mx ? v : mx;
    mn = v < mn ? v : mn;
    const double a = fabs(v);
    mg = a > mg ? a : mg;
  }
  const double margin = ldexp(mg, -44);
  d.evoid[e] = vo ? 1 : 0;
  d.emax[e] = (nan || d.force_exact) ? INFINITY : mx + margin;
  d.emin[e] = (nan || d.force_exact) ? -INFINITY : mn - margin;
}

// Node extrema of frame f over element e, kept per frame slot: with both
// frames of the current pair clear of the void threshold, every interpolated
// node value lies between them (up to rounding), so the element bounds follow
// without interpolating. `near`: a node within 2^-48 relative of the void
// threshold (or NaN), where the exact interpolation decides.
__device__ void frame_extrema(const RemeltDevice &d, const int64_t nid[8], int f, int64_t e, bool stored,
                              double &mx, double &mn, bool &near) {
  const int sl = f & 1;
  if (stored) {
    mx = d.fmax[sl][e];
    mn = d.fmin[sl][e];
    near = d.fnear[sl][e] != 0;
    return;
  }
  const double *fr = d.frames + (int64_t)(f % d.frame_slots) * d.nnodes;
  const double V = d.void_t + 0.00001;
  mx = -INFINITY;
  mn = INFINITY;
  near = false;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const double v = fr[nid[i]];
    if (!(v >= V + ldexp(fmax(fabs(v), fabs(V)), -48))) near = true;
    mx = v > mx ? v : mx;
    mn = v < mn ? v : mn;
  }
  d.fmax[sl][e] = mx;
  d.fmin[sl][e] = mn;
  d.fnear[sl][e] = near ? 1 : 0;
}

// nullMatTemp_ + 0.01: below it a cell counts as without material in the
// liquid-neighbour pass (Remelting.cpp:504-507)
__device__ __forceinline__ double null_plus() { return -1.0 + 0.01; }

}  // namespace

// ---------------------------------------------------------------------------
// FE -> CA map: MapVoxelManager::tag_voxels + is_in_element (MapVoxelManager.cpp:357-699)
// ---------------------------------------------------------------------------
namespace {

__device__ bool in_element(const double X[8], const double Y[8], const double Z[8], double xp, double yp, double zp,
                           double tol, int max_iter, double para[3]) {
  const double *x = X, *y = Y, *z = Z;
  double j[9], f[3], s[8];
  double xinew = 0.5, etanew = 0.5, zetanew = 0.5;
  double xi = 0.5, eta = 0.5, zeta = 0.5;
  double dd[3] = {1.0, 1.0, 1.0};
  int i = 0;
  do {
    j[0] = -(1.0 - eta) * (1.0 - zeta) * x[1] - (1.0 + eta) * (1.0 - zeta) * x[2] +
           (1.0 + eta) * (1.0 - zeta) * x[3] + (1.0 - eta) * (1.0 + zeta) * x[4] -
           (1.0 - eta) * (1.0 + zeta) * x[5] - (1.0 + eta) * (1.0 + zeta) * x[6] +
           (1.0 + eta) * (1.0 + zeta) * x[7];
    j[1] = (1.0 + xi) * (1.0 - zeta) * x[1] - (1.0 + xi) * (1.0 - zeta) * x[2] - (1.0 - xi) * (1.0 - zeta) * x[3] +
           (1.0 - xi) * (1.0 + zeta) * x[4] + (1.0 + xi) * (1.0 + zeta) * x[5] - (1.0 + xi) * (1.0 + zeta) * x[6] -
           (1.0 - xi) * (1.0 + zeta) * x[7];
    j[2] = (1.0 - eta) * (1.0 + xi) * x[1] + (1.0 + eta) * (1.0 + xi) * x[2] + (1.0 + eta) * (1.0 - xi) * x[3] -
           (1.0 - eta) * (1.0 - xi) * x[4] - (1.0 - eta) * (1.0 + xi) * x[5] - (1.0 + eta) * (1.0 + xi) * x[6] -
           (1.0 + eta) * (1.0 - xi) * x[7];
    j[3] = -(1.0 - eta) * (1.0 - zeta) * y[1] - (1.0 + eta) * (1.0 - zeta) * y[2] +
           (1.0 + eta) * (1.0 - zeta) * y[3] + (1.0 - eta) * (1.0 + zeta) * y[4] -
           (1.0 - eta) * (1.0 + zeta) * y[5] - (1.0 + eta) * (1.0 + zeta) * y[6] +
           (1.0 + eta) * (1.0 + zeta) * y[7];
    j[4] = (1.0 + xi) * (1.0 - zeta) * y[1] - (1.0 + xi) * (1.0 - zeta) * y[2] - (1.0 - xi) * (1.0 - zeta) * y[3] +
           (1.0 - xi) * (1.0 + zeta) * y[4] + (1.0 + xi) * (1.0 + zeta) * y[5] - (1.0 + xi) * (1.0 + zeta) * y[6] -
           (1.0 - xi) * (1.0 + zeta) * y[7];
    j[5] = (1.0 - eta) * (1.0 + xi) * y[1] + (1.0 + eta) * (1.0 + xi) * y[2] + (1.0 + eta) * (1.0 - xi) * y[3] -
           (1.0 - eta) * (1.0 - xi) * y[4] - (1.0 - eta) * (1.0 + xi) * y[5] - (1.0 + eta) * (1.0 + xi) * y[6] -
           (1.0 + eta) * (1.0 - xi) * y[7];
    j[6] = -(1.0 - eta) * (1.0 - zeta) * z[1] - (1.0 + eta) * (1.0 - zeta) * z[2] +
           (1.0 + eta) * (1.0 - zeta) * z[3] + (1.0 - eta) * (1.0 + zeta) * z[4] -
           (1.0 - eta) * (1.0 + zeta) * z[5] - (1.0 + eta) * (1.0 + zeta) * z[6] +
           (1.0 + eta) * (1.0 + zeta) * z[7];
    j[7] = (1.0 + xi) * (1.0 - zeta) * z[1] - (1.0 + xi) * (1.0 - zeta) * z[2] - (1.0 - xi) * (1.0 - zeta) * z[3] +
           (1.0 - xi) * (1.0 + zeta) * z[4] + (1.0 + xi) * (1.0 + zeta) * z[5] - (1.0 + xi) * (1.0 + zeta) * z[6] -
           (1.0 - xi) * (1.0 + zeta) * z[7];
    j[8] = (1.0 - eta) * (1.0 + xi) * z[1] + (1.0 + eta) * (1.0 + xi) * z[2] + (1.0 + eta) * (1.0 - xi) * z[3] -
           (1.0 - eta) * (1.0 - xi) * z[4] - (1.0 - eta) * (1.0 + xi) * z[5] - (1.0 + eta) * (1.0 + xi) * z[6] -
           (1.0 + eta) * (1.0 - xi) * z[7];
    const double jdet = -(j[2] * j[4] * j[6]) + j[1] * j[5] * j[6] + j[2] * j[3] * j[7] - j[0] * j[5] * j[7] -
                        j[1] * j[3] * j[8] + j[0] * j[4] * j[8];
    if (!jdet) {
      i = max_iter;
      break;
    }
    s[0] = (1.0 - eta) * (1.0 - xi) * (1.0 - zeta);
    s[1] = (1.0 - eta) * (1.0 + xi) * (1.0 - zeta);
    s[2] = (1.0 + eta) * (1.0 + xi) * (1.0 - zeta);
    s[3] = (1.0 + eta) * (1.0 - xi) * (1.0 - zeta);
    s[4] = (1.0 - eta) * (1.0 - xi) * (1.0 + zeta);
    s[5] = (1.0 - eta) * (1.0 + xi) * (1.0 + zeta);
    s[6] = (1.0 + eta) * (1.0 + xi) * (1.0 + zeta);
    s[7] = (1.0 + eta) * (1.0 - xi) * (1.0 + zeta);
    f[0] = xp - s[1] * x[1] - s[2] * x[2] - s[3] * x[3] - s[4] * x[4] - s[5] * x[5] - s[6] * x[6] - s[7] * x[7];
    f[1] = yp - s[1] * y[1] - s[2] * y[2] - s[3] * y[3] - s[4] * y[4] - s[5] * y[5] - s[6] * y[6] - s[7] * y[7];
    f[2] = zp - s[1] * z[1] - s[2] * z[2] - s[3] * z[3] - s[4] * z[4] - s[5] * z[5] - s[6] * z[6] - s[7] * z[7];
    xinew = (jdet * xi + f[2] * (j[2] * j[4] - j[1] * j[5]) + f[1] * (j[1] * j[8] - j[2] * j[7]) +
             f[0] * (j[5] * j[7] - j[4] * j[8])) /
            jdet;
    etanew = (eta * jdet + f[2] * (j[0] * j[5] - j[2] * j[3]) + f[1] * (j[2] * j[6] - j[0] * j[8]) +
              f[0] * (j[3] * j[8] - j[5] * j[6])) /
             jdet;
    zetanew = (jdet * zeta + f[2] * (j[1] * j[3] - j[0] * j[4]) + f[1] * (j[0] * j[7] - j[1] * j[6]) +
               f[0] * (j[4] * j[6] - j[3] * j[7])) /
              jdet;
    dd[0] = xinew - xi;
    dd[1] = etanew - eta;
    dd[2] = zetanew - zeta;
    xi = xinew;
    eta = etanew;
    zeta = zetanew;
  } while (!(fabs(0.0 + dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) < tol) && ++i < max_iter);
  para[0] = para[1] = para[2] = 1.7976931348623157e308;
  double dist = 1.7976931348623157e308;
  if (i < max_iter) {
    para[0] = xinew;
    para[1] = etanew;
    para[2] = zetanew;
    dist = 0;
    for (int c = 0; c < 3; c++) {
      if (para[c] > 1.0 && para[c] < 1.000001) para[c] = 1.0;
      if (para[c] < -1.0 && para[c] > -1.000001) para[c] = -1.0;
    }
    for (int c = 0; c < 3; c++)
      if (dist < fabs(para[c])) dist = fabs(para[c]);
  }
  return !(dist > 1.0);
}

__global__ void tag_kernel(Grid g, TagPlan p, int32_t *tag, double *pc) {
  const int64_t nvox = (int64_t)g.nxyg * g.nzg;
  const double h = g.h;
  const double origin[3] = {(0 - 0.5) * h + g.x0, (0 - 0.5) * h + g.y0, (0 - 0.5) * h + g.z0};
  for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < nvox; v += (int64_t)gridDim.x * blockDim.x) {
    tag[v] = -1;
    pc[3 * v] = pc[3 * v + 1] = pc[3 * v + 2] = -2;
    int idx[3], mmb[6];
    idx[2] = (int)(v / g.nxyg);
    idx[1] = (int)((v % g.nxyg) / g.nxg);
    idx[0] = (int)((v % g.nxyg) % g.nxg);
    double cv[3];
    bool out = false;
    for (int c = 0; c < 3; c++) {
      cv[c] = origin[c] + idx[c] * h;
      if (cv[c] < p.mm[2 * c] || cv[c] > p.mm[2 * c + 1]) {
        out = true;
        break;
      }
      const double dist = cv[c] - p.mm[2 * c];
      mmb[2 * c] = (int)floor(dist / p.dbin[c]);
      mmb[2 * c + 1] = (int)ceil(dist / p.dbin[c]);
    }
    if (out) continue;
    for (int c = 0; c < 3; c++) {
      int &lo = mmb[2 * c], &hi = mmb[2 * c + 1];
      if (lo == hi && lo > 0 && hi < p.nbin[c]) {
        lo -= 1;
        hi += 1;
      } else if (hi == 0) {
        hi = 1;
      } else if (hi == p.nbin[c]) {
        if (lo > 0) lo -= 1;
      }
    }
    bool got = false;
    for (int kk = mmb[4]; kk < mmb[5] && !got; kk++)
      for (int jj = mmb[2]; jj < mmb[3] && !got; jj++)
        for (int ii = mmb[0]; ii < mmb[1] && !got; ii++) {
          const int64_t ind = ii + (int64_t)jj * p.nbin[0] + (int64_t)kk * p.nbin[0] * p.nbin[1];
          if (ind < 0 || ind >= (int64_t)p.nbin[0] * p.nbin[1] * p.nbin[2]) continue;
          for (int64_t q = p.bin_start[ind]; q < p.bin_start[ind + 1]; ++q) {
            const int32_t e = p.bin_elems[q];
            const double *r = p.erange + 6 * (int64_t)e;
            if (cv[0] < r[0] || cv[0] > r[1] || cv[1] < r[2] || cv[1] > r[3] || cv[2] < r[4] || cv[2] > r[5]) continue;
            int64_t nid[8];
            elem_nodes(p.nn, e, nid);
            double X[8], Y[8], Z[8], para[3];
            const double *o = p.coord + 3 * nid[0];
            X[0] = Y[0] = Z[0] = 0.0;
            for (int n = 1; n < 8; n++) {
              const double *cn = p.coord + 3 * nid[n];
              X[n] = 0.125 * (cn[0] - o[0]);
              Y[n] = 0.125 * (cn[1] - o[1]);
              Z[n] = 0.125 * (cn[2] - o[2]);
            }
            if (in_element(X, Y, Z, cv[0] - o[0], cv[1] - o[1], cv[2] - o[2], p.tolerance, p.max_iter, para)) {
              tag[v] = e;
              pc[3 * v] = para[0];
              pc[3 * v + 1] = para[1];
              pc[3 * v + 2] = para[2];
              got = true;
              atomicAdd(&p.counts[0], 1ull);
              if (!isfinite(para[0]) || !isfinite(para[1]) || !isfinite(para[2])) atomicAdd(&p.counts[1], 1ull);
              break;
            }
          }
        }
  }
}

}  // namespace

cudaError_t remelt_tag_voxels(const Grid &g, const TagPlan &p, int32_t *tag, double *pc, cudaStream_t s) {
  const int64_t nvox = (int64_t)g.nxyg * g.nzg;
  const int blocks = (int)std::min<int64_t>((nvox + 127) / 128, 152 * 64);
  tag_kernel<<<blocks > 0 ? blocks : 1, 128, 0, s>>>(g, p, tag, pc);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Synthetic frames: Rosenthal moving point source (IEEE add/mul/div/sqrt only)
// ---------------------------------------------------------------------------
namespace {

// 1/n!, n = 0..13, as exact doubles
__constant__ double kExpTaylor[14] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1,
                                      0x1.5555555555555p-3, 0x1.5555555555555p-5, 0x1.1111111111111p-7,
                                      0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13, 0x1.a01a01a01a01ap-16,
                                      0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                                      0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};

// exp(a) for a <= 0: k = rint(a / ln 2), r = a - k ln 2, degree-13 Taylor
// polynomial in r (Horner), times 2^k built from the exponent bits.
__device__ double det_exp(double a) {
  const double kLn2 = 0x1.62e42fefa39efp-1, kInvLn2 = 0x1.71547652b82fep+0;
  a = (a < -700.0) ? -700.0 : a;
  const double k = rint(a * kInvLn2);
  const double r = a - k * kLn2;
  double p = kExpTaylor[13];
#pragma unroll
  for (int n = 12; n >= 0; --n) p = p * r + kExpTaylor[n];
  const long long ki = (long long)k;
  return p * __longlong_as_double((ki + 1023) << 52);
}

__global__ void rosenthal_kernel(RosenthalParams p, int nframes, double *frames) {
  const int64_t nnodes = (int64_t)p.nodes[0] * p.nodes[1] * p.nodes[2];
  const int64_t total = nnodes * nframes;
  const double two_pi_k = 2.0 * 3.141592653589793 * p.conductivity;
  const double ap = p.absorptivity * p.power;
  const double two_alpha = 2.0 * p.diffusivity;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t f = q / nnodes, n = q % nnodes;
    const int64_t I = n % p.nodes[0], J = (n / p.nodes[0]) % p.nodes[1], K = n / ((int64_t)p.nodes[0] * p.nodes[1]);
    const double x = (p.origin[0] + p.spacing * (double)I) * p.length_scale;
    const double y = (p.origin[1] + p.spacing * (double)J) * p.length_scale;
    const double z = (p.origin[2] + p.spacing * (double)K) * p.length_scale;
    const double t = ((double)f * p.frame_dt) * p.time_scale;
    const double xi = x - (p.x_start + p.speed * t);
    const double dy = y - p.y_line;
    const double dz = z - p.z_top;
    double r = sqrt((xi * xi + dy * dy) + dz * dz);
    r = (r < 1e-9) ? 1e-9 : r;
    const double qv = ap / (two_pi_k * r);
    double T = p.t0 + qv * det_exp(-(p.speed * (r + xi)) / two_alpha);
    T = (p.t_cap < T) ? p.t_cap : T;
    if (p.void_above_set && z > p.z_top + p.void_above) T = p.t_void;
    frames[q] = T;
  }
}

__global__ void init_theta_kernel(RemeltDevice d) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.nnodes; n += stride) {
    d.theta[0][n] = d.frames[n];
    d.theta32[0][n] = (float)d.frames[n];
  }
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.nelem; e += stride) {
    int64_t nid[8];
    elem_nodes(d.nn, e, nid);
    double t[8];
    for (int i = 0; i < 8; ++i) t[i] = d.frames[nid[i]];
    element_bounds(d, e, t);
  }
}

// Node temperatures of step `step` handed in by the host (external FE
// solver): the step's node arrays, element bounds and void flags, and its
// list of elements to visit (the rebuild of phase E, from these values).
__global__ void external_theta_kernel(RemeltDevice d, long long step, const double *theta) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int par = (int)(step & 1);
  double *tn = d.theta[step % 3];
  float *tn32 = d.theta32[step % 3];
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.nnodes; n += stride) {
    tn[n] = theta[n];
    tn32[n] = (float)theta[n];
  }
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.nelem; e += stride) {
    int64_t nid[8];
    elem_nodes(d.nn, e, nid);
    double t[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) t[i] = theta[nid[i]];
    const uint8_t void_before = d.evoid[e];
    element_bounds(d, e, t);
    const bool v = d.evoid[e] != 0;
    const bool active = (!v && !(d.emax[e] < d.Tm && d.emin[e] >= null_plus())) || (v != (void_before != 0)) ||
                        (!v && d.eliq[e] > 0);
    if (active) {
      const unsigned slot = atomicAdd(&d.ctrl->n_eact[par], 1u);
      if (slot < (unsigned)d.nelem) d.eact[par][slot] = (int32_t)e;
    }
  }
}

}  // namespace

cudaError_t remelt_external_theta(const RemeltDevice &d, long long step, const double *theta, cudaStream_t s) {
  const int64_t n = d.nnodes > d.nelem ? d.nnodes : d.nelem;
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  external_theta_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(d, step, theta);
  return cudaGetLastError();
}

cudaError_t remelt_rosenthal_frames(const RosenthalParams &p, int nframes, double *frames, cudaStream_t s) {
  const int64_t total = (int64_t)p.nodes[0] * p.nodes[1] * p.nodes[2] * nframes;
  const int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
  rosenthal_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(p, nframes, frames);
  return cudaGetLastError();
}

namespace {
__global__ void round_coords_kernel(const double *pc, float *pc32, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    pc32[i] = (float)pc[i];
}
}  // namespace

cudaError_t remelt_round_coords(const double *pc, float *pc32, int64_t n, cudaStream_t s) {
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  round_coords_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(pc, pc32, n);
  return cudaGetLastError();
}

// Initial grain records: an interior cell that holds a grain gets its
// cell's centre and length 0 (the record of a freshly read or random
// microstructure), every other cell zeros.
__global__ void init_records_kernel(RemeltDevice d) {
  const Grid &g = d.g;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < d.ncells;
       c += (int64_t)gridDim.x * blockDim.x) {
    int I, J, K;
    cell_ijk(g, c, I, J, K);
    const bool has = !ghost(g, I, J, K) && d.grain[c] >= 0;
    d.gx[c] = has ? centre_coord(g.x0, g.h, I) : 0.0;
    d.gy[c] = has ? centre_coord(g.y0, g.h, J) : 0.0;
    d.gz[c] = has ? centre_coord(g.z0, g.h, K) : 0.0;
    d.glen[c] = 0.0;
  }
}

cudaError_t remelt_init_records(const RemeltDevice &d, cudaStream_t s) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  init_records_kernel<<<sms > 0 ? 4 * sms : 256, 256, 0, s>>>(d);
  return cudaGetLastError();
}

cudaError_t remelt_init_theta(const RemeltDevice &d, cudaStream_t s) {
  const int64_t n = std::max<int64_t>(d.nnodes, d.nelem);
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
  init_theta_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(d);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The persistent step kernel
// ---------------------------------------------------------------------------
namespace {

struct StepScalars {
  long long step;
  double time, dt, max_ts, dT_FE, fe_time, ts0, ts1;
  int f_new, f_next;
  long long n_orient, n_grains;
};

__device__ StepScalars read_scalars(const RemeltCtrl *c) {
  StepScalars s;
  s.step = ld_volatile(&c->step);
  s.time = ld_volatile(&c->time);
  s.dt = ld_volatile(&c->dt);
  s.max_ts = ld_volatile(&c->max_ts);
  s.dT_FE = ld_volatile(&c->dT_FE);
  s.fe_time = ld_volatile(&c->fe_time);
  s.ts0 = ld_volatile(&c->ts0);
  s.ts1 = ld_volatile(&c->ts1);
  s.f_new = ld_volatile(&c->f_new);
  s.f_next = ld_volatile(&c->f_next);
  s.n_orient = ld_volatile(&c->n_orient);
  s.n_grains = ld_volatile(&c->n_grains);
  return s;
}

// Sweep position of a cell in the reference's i-outer, j, k-inner order.
__device__ __forceinline__ int32_t sweep_pos(const Grid &g, int I, int J, int K) {
  return (int32_t)(((int64_t)I * g.nyg + J) * g.nzg + K);
}

// Block 0: give the new grain objects of the last step their ids in sweep
// order (bitonic sort of the (sweep position, neighbour) keys in place).
__device__ void assign_new_grains(const RemeltDevice &d, RemeltCtrl *c) {
  const unsigned n = ld_volatile(&c->n_new);
  if (n == 0) return;
  unsigned m = 1;
  while (m < n) m <<= 1;
  for (unsigned i = n + threadIdx.x; i < m; i += blockDim.x) {
    d.newkey[i] = ~0ull;
    d.newcell[i] = -1;
  }
  __syncthreads();
  for (unsigned k = 2; k <= m; k <<= 1)
    for (unsigned j = k >> 1; j > 0; j >>= 1) {
      for (unsigned i = threadIdx.x; i < m; i += blockDim.x) {
        const unsigned l = i ^ j;
        if (l > i) {
          const unsigned long long a = d.newkey[i], b = d.newkey[l];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            d.newkey[i] = b;
            d.newkey[l] = a;
            const int32_t t = d.newcell[i];
            d.newcell[i] = d.newcell[l];
            d.newcell[l] = t;
          }
        }
      }
      __syncthreads();
    }
  const long long base = ld_volatile(&c->n_grains);
  for (unsigned i = threadIdx.x; i < n; i += blockDim.x) d.grain[d.newcell[i]] = (int32_t)(base + i);
  __syncthreads();
  if (threadIdx.x == 0) {
    c->n_grains = base + n;
    c->n_new = 0;
  }
  __syncthreads();
}

// checkup_current_temperature_to_update_phase_state (Remelting.cpp:339-404) and
// the per-cell part of checkup_liquid_cell_neigh_to_growth (:484-517) for one
// interior cell. `count_all`: add every liquid cell to its element's count
// (first step); otherwise only cells that melt now.
// What the phase update needs of a cell's element, read once per element by
// the warp that walks its cells: the nodal FP32 temperatures of this step and
// their error bound, the void flag and whether the frame extrema keep every
// solid cell of it unchanged.
struct ElemView {
  int32_t e;
  bool void_;
  bool quiet;
  float t[8];
  float err;
};

// Warp-collective: the view of element e (every lane gets it).
__device__ __forceinline__ ElemView elem_view(const RemeltDevice &d, const float *th32, int32_t e) {
  ElemView v;
  v.e = e;
  const int lane = threadIdx.x & 31;
  int64_t nid[8];
  elem_nodes(d.nn, e, nid);
  int64_t mine = nid[0];
#pragma unroll
  for (int i = 1; i < 8; ++i)
    if (lane == i) mine = nid[i];
  const float tl = lane < 8 ? th32[mine] : 0.0f;
  v.void_ = d.evoid[e] != 0;
  v.quiet = d.emax[e] < d.Tm && d.emin[e] >= null_plus();
#pragma unroll
  for (int i = 0; i < 8; ++i) v.t[i] = __shfl_sync(0xffffffffu, tl, i);
  v.err = hex8_err32(v.t);
  return v;
}

// What the phase update reads of one cell, loaded for several cells of an
// element at once (their load chains overlap instead of running one after
// another): orientation id, melted flag and FP32 parametric coordinates.
struct CellPre {
  int32_t o;
  uint8_t m;
  float xi, eta, zeta;
};

// A flagged cell's growth inputs other than dt and its velocity (phase D).
struct GrowPre {
  int32_t cell;
  int I, J, K;
  double glen;
  int32_t ori;
  float dx, dy, dz;
  float m32[9];
  uint32_t cand;
};

// eval_T32 with the element's nodal values already at hand (same operands,
// same operation order, same result).
__device__ __forceinline__ float eval_T32_view(const RemeltDevice &d, int64_t c, const ElemView &v, float &err,
                                               const CellPre *pre) {
  err = v.err;
  if (pre) return hex8_interp32(v.t, pre->xi, pre->eta, pre->zeta);
  return hex8_interp32(v.t, d.pc32[3 * c], d.pc32[3 * c + 1], d.pc32[3 * c + 2]);
}

// `ev`: the cell's element view when the caller walks an element's cells
// (the cell's tag is then ev->e), or nullptr; `pre`: the cell's values
// loaded by the caller, or nullptr.
__device__ __forceinline__ void phase_update(const RemeltDevice &d, RemeltCtrl *c, int64_t cell, const double *th,
                                             const float *th32, const StepScalars &S, bool count_all,
                                             unsigned long long &exactT, unsigned long long &melts,
                                             const ElemView *ev = nullptr, const CellPre *pre = nullptr) {
  int32_t o = pre ? pre->o : d.orient[cell];
  uint8_t mel = pre ? pre->m : 0;  // the cell's melted flag as this pass leaves it (with pre)
  const int32_t e = ev ? ev->e : d.tag[cell];
  const bool withMat = e >= 0 && !(ev ? ev->void_ : d.evoid[e] != 0);
  const double np = null_plus();
  // the FP32 estimate decides each comparison unless it is within its error
  // bound of the threshold; then the exact FP64 temperature decides them all
  float T32 = -1.0f, err = 0.0f;
  bool have32 = false;
  double T = -1.0;  // nullMatTemp_ (Remelting.cpp:29)
  bool exact = !withMat;
  // In FP32 (the FP64 pipe is narrow): T lies in [T32 - err, T32 + err], so
  // with those ends rounded outwards and the threshold rounded inwards
  // (thr_lo <= thr <= thr_hi, floats) every decided comparison holds for T;
  // within a float ulp of the threshold it stays undecided.
  auto below = [&](double thr, float thr_lo, float thr_hi) -> int {  // 1: T < thr, 0: T >= thr, -1: undecided
    if (exact) return T < thr ? 1 : 0;
    if (__fadd_ru(T32, err) < thr_lo) return 1;
    if (__fsub_rd(T32, err) >= thr_hi) return 0;
    return -1;
  };
  auto make_exact = [&]() {
    if (!exact) {
      ++exactT;
      eval_T(d, th, cell, T);
      exact = true;
    }
  };
  if (o > -1) {
    if (withMat) {
      // certainly below the liquidus and above nullMatTemp_ + 0.01: nothing changes
      if (ev ? ev->quiet : (d.emax[e] < d.Tm && d.emin[e] >= np)) return;
      T32 = ev ? eval_T32_view(d, cell, *ev, err, pre) : eval_T32(d, th32, cell, e, err);
      have32 = true;
      int b = below(d.Tm, d.tm_lo, d.tm_hi);
      if (b < 0) {
        make_exact();
        b = below(d.Tm, d.tm_lo, d.tm_hi);
      }
      if (b == 1) {  // stays solid; the liquid-neighbour pass clears melted below nullMatTemp_ + 0.01
        int bn = below(np, d.np_lo, d.np_hi);
        if (bn < 0) {
          make_exact();
          bn = below(np, d.np_lo, d.np_hi);
        }
        if (bn == 1 && (pre ? mel : d.melted[cell])) d.melted[cell] = 0;
        return;
      }
    }
    d.orient[cell] = -1;  // melt
    d.melted[cell] = withMat ? 1 : 0;
    mel = withMat ? 1 : 0;
    o = -1;
    ++melts;
    if (e >= 0 && !count_all) atomicAdd(&d.eliq[e], 1);
  }
  if (count_all && e >= 0) atomicAdd(&d.eliq[e], 1);
  // the four comparisons made with a liquid cell's temperature, with the
  // reference's expressions: withMat (Remelting.cpp:505-507), the liquidus
  // test of the liquid-neighbour pass (:521), and the capture sweep's
  // overhot / no-material tests (:588-597)
  bool wm2, flags, le, gtn;
  bool decided = false;
  if (!exact) {
    if (!have32) T32 = ev ? eval_T32_view(d, cell, *ev, err, pre) : eval_T32(d, th32, cell, e, err);
    // the bounds of T rounded outwards, the thresholds inwards (see below());
    // -1 is a float
    const float lo = __fsub_rd(T32, err), hi = __fadd_ru(T32, err);
    const bool ok_np = hi < d.np_lo || lo >= d.np_hi, ok_tm = hi < d.tm_lo || lo > d.tm_hi,
               ok_nl = hi <= -1.0f || lo > -1.0f;
    if (ok_np && ok_tm && ok_nl && T32 == T32) {
      wm2 = lo >= d.np_hi;
      flags = hi < d.tm_lo;
      le = flags;
      gtn = lo > -1.0f;
      decided = true;
    } else {
      make_exact();
    }
  }
  if (!decided) {
    wm2 = !(T < np);
    flags = !(T >= d.Tm);
    le = !(T > d.Tm);
    gtn = T > -1.0;
  }
  const uint8_t m0 = pre ? mel : d.melted[cell];
  uint8_t m1 = m0;
  if (wm2 && S.time >= S.max_ts) m1 = 1;
  if (!wm2) m1 = 0;
  if (m1 != m0) d.melted[cell] = m1;
  d.tcls[cell] = (uint8_t)((flags ? kTlt : 0) | (le ? kTle : 0) | (gtn ? kTgtNull : 0) | (wm2 ? kTgeNullPlus : 0));
  if (wm2 && flags) stage_push((int32_t)cell, &c->n_liq, d.liq, d.list_cap);  // the cell flags its solid neighbours
}

// Register budget of two blocks per SM (128 per thread), run with one block
// per SM: on pbf_500 that is faster than the unconstrained 186 registers, two
// blocks per SM, or 512-thread blocks (740 against 768, 793 and 801 ms per run).
__global__ void __launch_bounds__(kBlock, 2) remelt_kernel(RemeltDevice d, long long limit) {
  __shared__ unsigned smem[kWarps + 2];
  RemeltCtrl *c = d.ctrl;
  const Grid &g = d.g;
  const int tid = threadIdx.x;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + tid;
  const int64_t nthr = (int64_t)gridDim.x * blockDim.x;
  const int64_t M = (int64_t)g.nx * g.ny * g.nz;
  const int64_t nyzg = (int64_t)g.nyg * g.nzg;
  unsigned long long tests = 0, tests64 = 0, caps = 0, exactT = 0, melts = 0, visited = 0, eactive = 0;
  bool ok = true;
  if (tid == 0) {
    s_left = now_ns();
    for (int i = 0; i < 6; ++i) s_busy[i] = 0ull;
    s_stage_n = 0u;
    for (int i = 0; i < kClkN; ++i) s_clk[i] = 0ull;
    s_host_seq = ld_volatile(&c->host_seq);
  }
  for (;;) {
    const StepScalars S = read_scalars(c);
    // --- loop condition of time_integration_weak_coupling (CafeSolver.cpp:188) and launch limits ---
    int stop = kRemeltRunning;
    if (!(S.time < d.final_time)) stop = kRemeltFinalTime;
    else if (!(S.time < d.t_stop)) stop = kRemeltTimeStop;
    else if (S.step >= limit) stop = kRemeltStepLimit;
    else if (d.nsites > 0 && S.n_orient + d.nsites > d.orient_cap) stop = kRemeltNeedOrient;
    // the step's frame replay reads frame f_next (and f_next + 1 when two frames share a time): both loaded,
    // unless the frames end before them
    else if (!d.external && S.f_next + 1 >= d.frames_avail && d.frames_avail < d.nframes) stop = kRemeltNeedFrames;
    if (stop != kRemeltRunning) {
      if (gtid == 0) c->status = stop;
      break;
    }
    const int par = (int)(S.step & 1);
    const double *th = d.theta[S.step % 3];
    const float *th32 = d.theta32[S.step % 3];
    const double *thp = d.theta[(S.step + 2) % 3];
    unsigned long long t_phase = 0;
    if (gtid == 0) t_phase = now_ns();

    // ===== A: phase update + melted flags (Remelting.cpp:339-404, :484-517) =====
    if (blockIdx.x == 0) {
      const unsigned long long tg = tid == 0 ? now_ns() : 0ull;
      assign_new_grains(d, c);
      if (tid == 0) s_clk[kClkNewgrain] += now_ns() - tg;
      if (tid == 0) {
        c->n_claim = 0;
        c->n_eact[par ^ 1] = 0;  // built in phase E for the next step; its last reader was the previous phase A
      }
    }
    {  // clear the previous step's liquid-neighbour flags: every bit set in
       // the bitmap is one of them (phase B sets them, this pass clears them
       // all), so each listed cell's word is zeroed with a plain store
      const int64_t nprev = min((int64_t)ld_volatile(&c->n_flag[par ^ 1]), d.list_cap);
      const int32_t *fl = d.flagged[par ^ 1];
      // (from the last thread down: the first blocks' warps walk two active
      // elements in the update below)
      for (int64_t q = nthr - 1 - gtid; q < nprev; q += nthr) d.flagbits[fl[q] >> 5] = 0u;
    }
    if (S.step == 0) {  // every interior cell; the liquid count per element starts here
      for (int64_t q = gtid; q < M; q += nthr) {
        const int I = (int)(q % g.nx) + 1;
        const int J = (int)((q / g.nx) % g.ny) + 1;
        const int K = (int)(q / ((int64_t)g.nx * g.ny)) + 1;
        phase_update(d, c, (int64_t)K * g.nxyg + (int64_t)J * g.nxg + I, th, th32, S, true, exactT, melts);
      }
      visited += (M + nthr - 1 - gtid) / nthr;
    } else {  // the cells of the active elements (a warp per element)
      const unsigned na = ld_volatile(&c->n_eact[par]);
      const int lane = tid & 31;
      const int64_t gw = gtid >> 5, nw = nthr >> 5;
      for (int64_t w = gw; w < na; w += nw) {
        const int32_t e = d.eact[par][w];
        const int64_t b = d.ecell_start[e], en = d.ecell_start[e + 1];
        const ElemView ev = elem_view(d, th32, e);
        // kCellPre cells per lane at a time: their ids, then everything the
        // update reads of them, each set of loads in flight together
        for (int64_t k0 = b + lane; k0 < en; k0 += 32 * kCellPre) {
          int64_t cl[kCellPre];
          CellPre pre[kCellPre];
#pragma unroll
          for (int j = 0; j < kCellPre; ++j) cl[j] = k0 + 32 * j < en ? d.ecell[k0 + 32 * j] : -1;
#pragma unroll
          for (int j = 0; j < kCellPre; ++j) {
            if (cl[j] < 0) continue;
            pre[j].o = d.orient[cl[j]];
            pre[j].m = d.melted[cl[j]];
            pre[j].xi = d.pc32[3 * cl[j]];
            pre[j].eta = d.pc32[3 * cl[j] + 1];
            pre[j].zeta = d.pc32[3 * cl[j] + 2];
          }
#pragma unroll
          for (int j = 0; j < kCellPre; ++j) {
            if (cl[j] < 0) continue;
            phase_update(d, c, cl[j], th, th32, S, false, exactT, melts, &ev, &pre[j]);
            ++visited;
          }
        }
      }
    }
    stage_flush(&c->n_liq, d.liq, d.list_cap);
    if (gtid == 0) {
      const unsigned long long t1 = now_ns();
      s_clk[kClkPhase + 0] += t1 - t_phase;
      t_phase = t1;
    }
    if (!(ok = grid_barrier(d, 0))) break;

    // ===== B: liquid-neighbour flags (Remelting.cpp:518-540) =====
    if (tid == 0 && blockIdx.x == 0 && d.detail) {
      s_clk[kClkFlagsMax] += ld_volatile(&c->flags_scratch);  // last step's maximum: every block added it before the A barrier
      c->flags_scratch = 0ull;
    }
    const unsigned long long tfl = tid == 0 ? now_ns() : 0ull;
    {
      const unsigned nl = ld_volatile(&c->n_liq);
      if (nl > d.list_cap) {
        if (gtid == 0) atomicCAS(&c->error, 0, kRemeltErrList);
      } else {
        // entries are dealt lane-major over the warps (q = lane * warps +
        // warp): the list holds the cells of an element together, and their
        // flag bits share bitmap words, so neighbouring entries go to
        // different warps rather than into one warp's same-word atomics
        const int64_t nw = nthr >> 5, wid = gtid >> 5, lane = tid & 31;
        for (int64_t q = lane * nw + wid; q < nl; q += nthr) {
          const int32_t cell = d.liq[q];
          // all 26 neighbour states, then all flag updates, in flight at once
          uint32_t solid = 0;
#pragma unroll
          for (int n = 0; n < 26; ++n) {
            int di, dj, dk;
            nbr_offset(n, di, dj, dk);
            solid |= (d.orient[cell + dk * g.nxyg + dj * g.nxg + di] > -1 ? 1u : 0u) << n;
          }
          // the three neighbours of a (dj, dk) row are consecutive cells:
          // one atomicOr per flag word the row touches (one, or two where
          // it crosses a word) sets all of its solid ones, so a cell takes
          // 9 to 18 atomics instead of one per solid neighbour, and fewer
          // of them meet on the same words
          uint32_t fresh = 0;
          unsigned lo_old[9], hi_old[9];
#pragma unroll
          for (int r = 0; r < 9; ++r) {
            const int dj = r % 3 - 1, dk = r / 3 - 1;
            // neighbour index of di = -1, 0, +1 in this row (-1: the centre cell)
            const int nm = r <= 4 ? 3 * r : 3 * r - 1;
            const int nc = r <= 3 ? 3 * r + 1 : (r == 4 ? -1 : 3 * r);
            const int np_ = r <= 3 ? 3 * r + 2 : (r == 4 ? 13 : 3 * r + 1);
            const unsigned pat = ((solid >> nm) & 1u) | (nc >= 0 ? ((solid >> nc) & 1u) << 1 : 0u) |
                                 (((solid >> np_) & 1u) << 2);
            const int32_t rb = cell + dk * g.nxyg + dj * g.nxg - 1;
            const unsigned long long m64 = (unsigned long long)pat << (rb & 31);
            const unsigned lo = (unsigned)m64, hi = (unsigned)(m64 >> 32);
            lo_old[r] = lo ? atomicOr(&d.flagbits[rb >> 5], lo) : 0xffffffffu;
            hi_old[r] = hi ? atomicOr(&d.flagbits[(rb >> 5) + 1], hi) : 0xffffffffu;
          }
#pragma unroll
          for (int r = 0; r < 9; ++r) {
            const int dj = r % 3 - 1, dk = r / 3 - 1;
            const int nm = r <= 4 ? 3 * r : 3 * r - 1;
            const int nc = r <= 3 ? 3 * r + 1 : (r == 4 ? -1 : 3 * r);
            const int np_ = r <= 3 ? 3 * r + 2 : (r == 4 ? 13 : 3 * r + 1);
            const int32_t rb = cell + dk * g.nxyg + dj * g.nxg - 1;
            // bits of this row set here for the first time, by di
            const unsigned long long old64 = (unsigned long long)lo_old[r] | ((unsigned long long)hi_old[r] << 32);
            const unsigned newbits = (unsigned)((~old64) >> (rb & 31)) & 7u;
            const unsigned pat = ((solid >> nm) & 1u) | (nc >= 0 ? ((solid >> nc) & 1u) << 1 : 0u) |
                                 (((solid >> np_) & 1u) << 2);
            const unsigned f = newbits & pat;
            fresh |= (f & 1u) << nm;
            if (nc >= 0) fresh |= ((f >> 1) & 1u) << nc;
            fresh |= ((f >> 2) & 1u) << np_;
          }
          unsigned slot = append_slots(&c->n_flag[par], (unsigned)__popc(fresh));
          while (fresh) {
            const int n = __ffs(fresh) - 1;
            fresh &= fresh - 1;
            int di, dj, dk;
            nbr_offset(n, di, dj, dk);
            if (slot < d.list_cap) d.flagged[par][slot] = cell + dk * g.nxyg + dj * g.nxg + di;
            ++slot;
          }
        }
      }
    }
    __syncthreads();
    if (tid == 0) {
      const unsigned long long w = now_ns() - tfl;
      if (d.detail && w > ld_volatile(&c->flags_scratch)) atomicMax(&c->flags_scratch, w);
    }
    // site conditions of nucleate_at_nucleation_sites (Remelting.cpp:946-960), all blocks
    // (only a liquid, melted cell can nucleate: the temperatures are
    // evaluated for those alone)
    for (int64_t sidx = spread_begin(0); sidx < d.nsites; sidx += spread_stride(0)) {
      const int32_t cell = d.site_cell[sidx];
      uint8_t f = 0;
      if (d.orient[cell] == -1 && d.melted[cell]) {
        double T = -1.0, Told = -1.0;
        const bool withMat = eval_T(d, th, cell, T);
        bool cooling = false;
        if (S.step > 0) {  // cooling_ of this step's phase update (Remelting.cpp:362-373)
          eval_T(d, thp, cell, Told);
          double rate = 410;
          if (Told > 0) rate = (T - Told) / S.dt;
          if (T <= 0) rate = 0;
          cooling = withMat ? (rate < 0) : false;
        }
        if (cooling && T > d.Tnuc) {
          const double dT = d.Tm - T;
          if (dT > d.site_dtc[sidx]) f = d.grain[cell] == -1 ? 2 : 1;
        }
      }
      d.snuc[sidx] = f;
      if (f) atomicAdd(&c->n_nuc_sites[par], 1u);
    }
    if (gtid == 0) {
      const unsigned long long t1 = now_ns();
      s_clk[kClkPhase + 1] += t1 - t_phase;
      t_phase = t1;
    }
    if (!(ok = grid_barrier(d, 1))) break;

    // ===== C: nucleation (block 0) | cutoff + minimum temperature (Remelting.cpp:656-705) =====
    const unsigned nf = ld_volatile(&c->n_flag[par]);
    if (nf > d.list_cap) {
      if (gtid == 0) atomicCAS(&c->error, 0, kRemeltErrList);
    }
    if (blockIdx.x == 0 && tid == 0) c->n_nuc_sites[par ^ 1] = 0u;  // counted again in the next step's phase B
    // (in most steps no site nucleates and the scan over the sites is skipped)
    if (blockIdx.x == 0 && d.nsites > 0 && ld_volatile(&c->n_nuc_sites[par]) > 0u) {
      const unsigned long long tn = tid == 0 ? now_ns() : 0ull;
      // nucleate_at_nucleation_sites (Remelting.cpp:936-999): ascending sites,
      // orientation id = count so far, a grain object created where the cell has none
      unsigned done_o = 0, done_g = 0;
      // block 0 itself gave last step's new grain objects their ids in phase A
      const long long n_grains = ld_volatile(&c->n_grains);
      for (int base = 0; base < d.nsites; base += kBlock) {
        const int sidx = base + tid;
        const uint8_t f = sidx < d.nsites ? d.snuc[sidx] : 0;
        const bool nuc = f != 0, newg = f == 2;
        const int32_t cell = sidx < d.nsites ? d.site_cell[sidx] : -1;
        unsigned tot_o, tot_g;
        const unsigned r_o = block_exclusive_scan(nuc ? 1u : 0u, smem, &tot_o);
        const unsigned r_g = block_exclusive_scan(newg ? 1u : 0u, smem, &tot_g);
        if (nuc) {
          const int32_t oid = (int32_t)(S.n_orient + done_o + r_o);
          int I, J, K;
          cell_ijk(g, cell, I, J, K);
          d.gx[cell] = centre_coord(g.x0, g.h, I);
          d.gy[cell] = centre_coord(g.y0, g.h, J);
          d.gz[cell] = centre_coord(g.z0, g.h, K);
          d.glen[cell] = 0.0;
          d.gori[cell] = oid;
          d.gdx[cell] = d.gdy[cell] = d.gdz[cell] = 0.0f;
          if (newg) d.grain[cell] = (int32_t)(n_grains + done_g + r_g);
          d.orient[cell] = oid;
          const int32_t e = d.tag[cell];
          if (e >= 0) atomicSub(&d.eliq[e], 1);
        }
        done_o += tot_o;
        done_g += tot_g;
      }
      if (tid == 0) {
        c->n_orient = S.n_orient + done_o;
        c->n_grains = n_grains + done_g;
        c->nucleations += done_o;
        s_clk[kClkNucleation] += now_ns() - tn;
      }
    }
    {
      const bool solo = gridDim.x == 1;
      const int64_t g0 = spread_begin(solo ? 0 : 1);
      const int64_t gn = spread_stride(solo ? 0 : 1);
      if (nf <= d.list_cap && (solo || blockIdx.x > 0)) {
        const unsigned long long key_tm = dkey(d.Tm);
        unsigned long long best = key_tm;
        for (int64_t q = g0; q < nf; q += gn) {
          const int32_t cell = d.flagged[par][q];
          int I, J, K;
          cell_ijk(g, cell, I, J, K);
          if (ghost(g, I, J, K)) continue;
          if (d.grain[cell] < 0) continue;
          if (!(d.glen[cell] < d.cutoff)) d.glen[cell] = d.h;  // length reset (:688-694)
          double T = -1.0;
          ++exactT;
          eval_T(d, th, cell, T);
          {  // growth velocity of single_integration_step (Remelting.cpp:569-576)
            bool hard = false;
            const double Targ = (T < d.Ts) ? d.Ts + 0.01 : T;
            d.fvel[q] = velocity(d, Targ, hard);
            if (hard) {
              const unsigned slot = append_slot(&c->n_hard);
              if (slot < d.list_cap) {
                d.hard_idx[slot] = (int32_t)q;
                d.hard_T[slot] = Targ;
                // the host's answer, slot `slot`, is taken in phase D
                // (velocities are never negative)
                d.fvel[q] = -1.0 - (double)slot;
              }
            }
          }
          if (T <= d.Ts) continue;
          if (T == T) {
            const unsigned long long k = dkey(T);
            best = k < best ? k : best;
          }
        }
        if (best < key_tm && best < ld_volatile(&c->minT_key)) atomicMin(&c->minT_key, best);
      }
    }
    if (gtid == 0) {
      const unsigned long long t1 = now_ns();
      s_clk[kClkPhase + 2] += t1 - t_phase;
      t_phase = t1;
    }
    if (!(ok = grid_barrier(d, 2))) break;

    // What the growth of a flagged cell reads besides dt and its velocity:
    // its state, orientation matrix and candidate neighbours (non-ghost
    // liquid neighbours with material at or below Tm, from all 26 neighbour
    // states loaded at once). Neither the dt phase nor another cell's growth
    // changes any of it (a claim leaves a candidate a candidate), so this
    // thread's first flagged cell is loaded while dt is found.
    auto grow_load = [&](int32_t cell, int I, int J, int K) {
      GrowPre p;
      p.cell = cell;
      p.I = I;
      p.J = J;
      p.K = K;
      p.glen = d.glen[cell];
      p.ori = d.gori[cell];
      p.dx = d.gdx[cell];
      p.dy = d.gdy[cell];
      p.dz = d.gdz[cell];
#pragma unroll
      for (int qq = 0; qq < 9; ++qq) p.m32[qq] = d.omat32[9 * (int64_t)p.ori + qq];
      uint32_t cand = 0;
#pragma unroll
      for (int n = 0; n < 26; ++n) {
        int di, dj, dk;
        nbr_offset(n, di, dj, dk);
        const int32_t nb = cell + dk * g.nxyg + dj * g.nxg + di;
        const bool in = !ghost(g, I + di, J + dj, K + dk);
        const int32_t o = in ? d.orient[nb] : 0;
        const uint8_t cls = in ? d.tcls[nb] : 0;  // a liquid neighbour's classes are this step's
        cand |= (in && o <= -1 && (cls & kTle) && (cls & kTgtNull) ? 1u : 0u) << n;
      }
      p.cand = cand;
      return p;
    };
    const int64_t q0 = spread_begin(0);
    GrowPre pre0{};
    bool use0 = false;
    if (q0 < nf && nf <= d.list_cap) {
      const int32_t cell = d.flagged[par][q0];
      int I, J, K;
      cell_ijk(g, cell, I, J, K);
      if (!ghost(g, I, J, K) && d.grain[cell] >= 0) {
        pre0 = grow_load(cell, I, J, K);
        use0 = true;
      }
    }

    // ===== dt (Remelting.cpp:706-726, CafeSolver.cpp:195-199) =====
    const double minT = dkey_inv(ld_volatile(&c->minT_key));
    // the same FP64 velocity for every thread: one thread per block computes it
    __shared__ double s_vmin;
    __shared__ int s_min_hard;
    if (tid == 0) {
      bool h = false;
      s_vmin = velocity(d, minT, h);
      s_min_hard = h ? 1 : 0;
    }
    __syncthreads();
    const bool min_hard = s_min_hard != 0;
    double vmin = s_vmin;
    // The host evaluates the hard velocities while the blocks grow and claim
    // with the others: block 0 posts the request, every block counts it, and
    // a block waits for the answer only before its own hard cells (or before
    // dt, when the velocity at the minimum temperature is one of them). A
    // request larger than the mapped buffer goes in chunks, behind a barrier.
    const unsigned nh = ld_volatile(&c->n_hard);  // uniform: every block read the same counter and key
    const bool ask = nh > 0 || min_hard;
    const bool overlap = ask && nh + 1u <= (unsigned)d.host_cap;
    if (ask && !overlap) {
      if (blockIdx.x == 0 && !host_velocities(d, c, nh, min_hard, minT)) atomicCAS(&c->error, 0, kRemeltErrHost);
      if (!(ok = grid_barrier(d, 5))) break;
      // block 0's requests, one per chunk, counted by the others
      if (tid == 0 && blockIdx.x != 0) s_host_seq += (nh + (min_hard ? 1u : 0u) + d.host_cap - 1u) / d.host_cap;
      if (min_hard) vmin = ld_volatile(&c->vmin);
    }
    if (overlap) {
      host_post(d, nh, min_hard, minT);
      if (min_hard) {
        host_wait_block(d, c);
        vmin = ld_volatile(&d.host->v[nh]);
      }
    }
    const double maxV = vmin > 0 ? vmin : 0;
    const double a = d.tsf_ca * d.h / maxV;
    const double dtLoc = (S.max_ts < a) ? S.max_ts : a;
    const double dT_ = (S.dT_FE < dtLoc) ? S.dT_FE : dtLoc;
    const double dT = (d.dt_cap < dT_) ? d.dt_cap : dT_;  // setup_time_step_for_coupling of an external solver

    // ===== D: grow and claim (Remelting.cpp:545-622) =====
    // one flagged cell: growth by dT * vel and its claims (atomicMin of the
    // sweep position: the order cells are taken in does not matter)
    auto grow_finish = [&](const GrowPre &p, double vel) {
      const int32_t cell = p.cell;
      const int I = p.I, J = p.J, K = p.K;
      const double L = p.glen + dT * vel;
      d.glen[cell] = L;
      if (L == 0) return;  // Octahedron::cell_is_captured: a zero half-diagonal captures nothing
      const int32_t ori = p.ori;
      const int32_t mine = INT_MIN + sweep_pos(g, I, J, K);
      const float dxf = p.dx, dyf = p.dy, dzf = p.dz;
      const float errg = 4.76837158203125e-07f * (d.h32 + fabsf(dxf) + fabsf(dyf) + fabsf(dzf)) + d.coord_err;
      const float L32 = (float)L;
      const float *m32 = p.m32;
      uint32_t cand = p.cand;
      while (cand) {
        const int n = __ffs(cand) - 1;
        cand &= cand - 1;
        int di, dj, dk;
        nbr_offset(n, di, dj, dk);
        const int32_t nb = cell + dk * g.nxyg + dj * g.nxg + di;
        ++tests;
        int f = captured_f32(m32, (float)di * d.h32 - dxf, (float)dj * d.h32 - dyf, (float)dk * d.h32 - dzf, errg,
                             L32);
        if (f < 0) {
          ++tests64;
          const double ccx = centre_coord(g.x0, g.h, I + di);
          const double ccy = centre_coord(g.y0, g.h, J + dj);
          const double ccz = centre_coord(g.z0, g.h, K + dk);
          f = is_captured_f64(d.omat + 9 * (int64_t)ori, ccx - d.gx[cell], ccy - d.gy[cell], ccz - d.gz[cell], L) ? 1
                                                                                                                  : 0;
        }
        if (f) {
          const int32_t old = atomicMin(&d.orient[nb], mine);
          if (old == -1) {
            const unsigned slot = append_slot(&c->n_claim);
            if (slot < d.list_cap) d.claimed[slot] = nb;
          }
        }
      }
    };
    auto grow_claim = [&](int32_t cell, int I, int J, int K, double vel) {
      grow_finish(grow_load(cell, I, J, K), vel);
    };
    bool pending = false;  // a hard velocity of this thread waits for the host's answer
    if (use0) {
      const double vel = d.fvel[q0];  // (the chunked host path rewrites it in the dt phase)
      if (vel < 0)
        pending = true;
      else
        grow_finish(pre0, vel);
    }
    for (int64_t q = q0 + spread_stride(0); q < nf && nf <= d.list_cap; q += spread_stride(0)) {
      const int32_t cell = d.flagged[par][q];
      int I, J, K;
      cell_ijk(g, cell, I, J, K);
      if (ghost(g, I, J, K)) continue;
      if (d.grain[cell] < 0) continue;
      const double vel = d.fvel[q];
      if (vel < 0) {
        pending = true;
        continue;
      }
      grow_claim(cell, I, J, K, vel);
    }
    if (overlap && __syncthreads_or(pending)) {  // uniform within the block
      host_wait_block(d, c);
      for (int64_t q = spread_begin(0); q < nf && nf <= d.list_cap; q += spread_stride(0)) {
        const double vel = d.fvel[q];
        if (!(vel < 0)) continue;
        const int32_t cell = d.flagged[par][q];
        int I, J, K;
        cell_ijk(g, cell, I, J, K);
        if (ghost(g, I, J, K) || d.grain[cell] < 0) continue;
        const double v = ld_volatile(&d.host->v[(unsigned)(-1.0 - vel)]);
        if (q == q0 && use0)
          grow_finish(pre0, v);  // loaded ahead, still current (only this thread grows the cell)
        else
          grow_claim(cell, I, J, K, v);
      }
    }
    if (gtid == 0) {
      const unsigned long long t1 = now_ns();
      s_clk[kClkPhase + 3] += t1 - t_phase;
      t_phase = t1;
    }
    if (!(ok = grid_barrier(d, 3))) break;

    // ===== E: captures (Remelting.cpp:807-847) and the FE replay step (LoadDataFromFile.cpp:207-313) =====
    {
      const unsigned nc = ld_volatile(&c->n_claim);
      if (nc > d.list_cap) {
        if (gtid == 0) atomicCAS(&c->error, 0, kRemeltErrList);
      } else {
        for (int64_t q = spread_begin_last(); q < nc; q += spread_stride(0)) {
          const int32_t nb = d.claimed[q];
          const int32_t w = d.orient[nb] - INT_MIN;
          const int wi = (int)(w / nyzg), wj = (int)((w / g.nzg) % g.nyg), wk = (int)(w % g.nzg);
          const int64_t wc = (int64_t)wk * g.nxyg + (int64_t)wj * g.nxg + wi;
          int I, J, K;
          cell_ijk(g, nb, I, J, K);
          const int32_t ori = d.gori[wc];
          const double px = d.gx[wc], py = d.gy[wc], pz = d.gz[wc], L = d.glen[wc];
          const double ccx = centre_coord(g.x0, g.h, I), ccy = centre_coord(g.y0, g.h, J),
                       ccz = centre_coord(g.z0, g.h, K);
          double out[4];
          capture_f64(d.omat + 9 * (int64_t)ori, ccx - px, ccy - py, ccz - pz, L, d.h, d.trunc, out);
          const double nx = out[0] + px, ny = out[1] + py, nz = out[2] + pz;
          d.gx[nb] = nx;
          d.gy[nb] = ny;
          d.gz[nb] = nz;
          d.glen[nb] = out[3];
          d.gori[nb] = ori;
          d.gdx[nb] = (float)(nx - ccx);
          d.gdy[nb] = (float)(ny - ccy);
          d.gdz[nb] = (float)(nz - ccz);
          if (d.grain[nb] < 0) {  // create_new_grain: id in sweep order after the step
            d.grain[nb] = kPendingGrain;
            const int di = I - wi, dj = J - wj, dk = K - wk;
            int m = (dk + 1) * 9 + (dj + 1) * 3 + (di + 1);
            m = m > 13 ? m - 1 : m;
            const unsigned slot = append_slot(&c->n_new);
            if (slot < (unsigned)kNewGrainCap) {
              d.newkey[slot] = ((unsigned long long)(uint32_t)w << 5) | (unsigned)m;
              d.newcell[slot] = nb;
            } else {
              atomicCAS(&c->error, 0, kRemeltErrNewGrains);
            }
          }
          d.orient[nb] = ori;
          const int32_t e = d.tag[nb];
          if (e >= 0) atomicSub(&d.eliq[e], 1);
          ++caps;
        }
      }
    }
    // FE replay (uniform in every thread)
    double fe_time = S.fe_time, ts0 = S.ts0, ts1 = S.ts1;
    int f_new = S.f_new, f_next = S.f_next;
    bool exhausted = false, bad = false, unloaded = false;
    double ratio = 0.0;
    // an external FE solver hands in the next node temperatures and element bounds between
    // steps (amca_set_nodal_temperatures): no replay then
    if (!d.external) {
      if (fe_time == 0) fe_time = ts1;
      fe_time += dT;
      while (fe_time >= ts0) {
        if (f_next >= d.nframes) {
          exhausted = true;
          bad = (d.bad_frame == f_next);
          break;
        }
        if (f_next >= d.frames_avail) {  // cannot happen after the check at the step's start
          unloaded = true;
          exhausted = true;
          break;
        }
        ts1 = ts0;
        ts0 = d.frame_time[f_next % d.frame_slots];
        f_new = f_next;
        f_next++;
      }
      if (!exhausted) {
        ratio = (fe_time - ts1) / (ts0 - ts1);
        if (ratio < 0.0 && gtid == 0) atomicCAS(&c->error, 0, kRemeltErrRatio);
        const double *f0 = d.frames + (int64_t)(f_new % d.frame_slots) * d.nnodes;
        const double *f1 = d.frames + (int64_t)((f_new - 1) % d.frame_slots) * d.nnodes;
        double *tn = d.theta[(S.step + 1) % 3];
        float *tn32 = d.theta32[(S.step + 1) % 3];
        // four nodes per thread at a time: their frame values are loaded
        // before any interpolated value is stored (a store could alias the
        // next node's loads and would keep them one after another)
        for (int64_t n0 = gtid; n0 < d.nnodes; n0 += 4 * nthr) {
          double a[4], b[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int64_t n = n0 + j * nthr;
            a[j] = n < d.nnodes ? f0[n] : 0.0;
            b[j] = n < d.nnodes ? f1[n] : 0.0;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int64_t n = n0 + j * nthr;
            if (n >= d.nnodes) continue;
            const double v = lerp_node(a[j], b[j], ratio, d.void_t);
            tn[n] = v;
            tn32[n] = (float)v;
          }
        }
        // Element bounds depend on the frame pair only (every interpolated node value lies between
        // its two frame values), so the active list is rebuilt when the pair changes; elements near
        // the void threshold need the exact interpolation and force a rebuild every step.
        const bool rebuild = S.step == 0 || f_new != S.f_new || ld_volatile(&c->any_near) || d.force_exact;
        if (!rebuild) {
          const unsigned na = ld_volatile(&c->n_eact[par]);
          for (int64_t q = gtid; q < na; q += nthr) d.eact[par ^ 1][q] = d.eact[par][q];
          if (gtid == 0) {
            c->n_eact[par ^ 1] = na;
            eactive += na;
          }
        }
        const bool st0 = ld_volatile(&c->fstat_frame[f_new & 1]) == f_new;
        const bool st1 = ld_volatile(&c->fstat_frame[(f_new - 1) & 1]) == f_new - 1;
        for (int64_t e = gtid; e < d.nelem && rebuild; e += nthr) {
          int64_t nid[8];
          elem_nodes(d.nn, e, nid);
          const uint8_t void_before = d.evoid[e];
          double mx0, mn0, mx1, mn1;
          bool near0, near1;
          frame_extrema(d, nid, f_new, e, st0, mx0, mn0, near0);
          frame_extrema(d, nid, f_new - 1, e, st1, mx1, mn1, near1);
          if (near0 || near1 || d.force_exact) {
            if (!ld_volatile(&c->any_near)) atomicOr(&c->any_near, 1);
            double t[8];
  #pragma unroll
            for (int i = 0; i < 8; ++i) t[i] = lerp_node(f0[nid[i]], f1[nid[i]], ratio, d.void_t);
            element_bounds(d, e, t);
          } else {
            const double mx = mx0 > mx1 ? mx0 : mx1, mn = mn0 < mn1 ? mn0 : mn1;
            const double mg = fmax(fabs(mx), fabs(mn));
            d.evoid[e] = 0;
            d.emax[e] = mx + ldexp(mg, -44);
            d.emin[e] = mn - ldexp(mg, -44);
          }
          // the next phase update visits this element's cells when some may change: hot enough to
          // melt or below nullMatTemp_ + 0.01, void status changed, or holding liquid with material
          // (cells of a cold element are solid except those counted in eliq; a void element's cells
          // are all liquid without material once it has been visited)
          const bool v = d.evoid[e] != 0;
          const bool active = (!v && !(d.emax[e] < d.Tm && d.emin[e] >= null_plus())) || (v != (void_before != 0)) ||
                              (!v && ld_volatile(&d.eliq[e]) > 0);
          if (active) {
            const unsigned slot = append_slot(&c->n_eact[par ^ 1]);
            if (slot < (unsigned)d.nelem) d.eact[par ^ 1][slot] = (int32_t)e;
            ++eactive;
          }
        }
      }
    }
    if (gtid == 0) {
      if (bad) atomicCAS(&c->error, 0, kRemeltErrFrame);
      if (unloaded) atomicCAS(&c->error, 0, kRemeltErrRing);
      if (!d.external) {
        if (!exhausted) {
          c->fstat_frame[f_new & 1] = f_new;
          c->fstat_frame[(f_new - 1) & 1] = f_new - 1;
        }
        c->fe_time = fe_time;
        c->ts0 = ts0;
        c->ts1 = ts1;
        c->f_new = f_new;
        c->f_next = f_next;
        c->ratio = ratio;
        c->dT_FE = ts0 - fe_time;
        c->max_ts = ts0 - fe_time;
      }
      c->step = S.step + 1;
      c->time = S.time + dT;
      c->dt_prev = S.dt;
      c->dt = dT;
      c->theta_init = 0;
      c->liquid += ld_volatile(&c->n_liq);
      c->n_liq = 0;
      c->n_hard = 0;
      c->minT_key = dkey(d.Tm);
      c->n_flag[par ^ 1] = 0;
      c->flagged += nf;
      if (exhausted) c->status = kRemeltFramesEnd;
      const unsigned long long t1 = now_ns();
      s_clk[kClkPhase + 4] += t1 - t_phase;
    }
    if (!(ok = grid_barrier(d, 4))) break;
    if (exhausted) break;  // uniform; block 0 recorded kRemeltFramesEnd
  }
  if (ok && blockIdx.x == 0) assign_new_grains(d, c);
  if (tid == 0)
    for (int i = 0; i < 6; ++i)
      if (s_busy[i]) atomicAdd(&c->ns_work_sum[i], s_busy[i]);
  if (tid == 0 && blockIdx.x == 0) {
    for (int k = 0; k < 5; ++k) c->ns_phase[k] += s_clk[kClkPhase + k];
    for (int k = 0; k < 6; ++k) c->ns_work_max[k] += s_clk[kClkWorkMax + k];
    c->ns_barrier += s_clk[kClkBarrier];
    c->ns_host += s_clk[kClkHost];
    c->host_calls += s_clk[kClkHostCalls];
    c->host_vel += s_clk[kClkHostVel];
    c->ns_newgrain += s_clk[kClkNewgrain];
    c->ns_nucleation += s_clk[kClkNucleation];
    c->ns_flags_max += s_clk[kClkFlagsMax];
    c->host_seq = s_host_seq;
  }
  if (tests) atomicAdd(&c->tests, tests);
  if (tests64) atomicAdd(&c->tests64, tests64);
  if (caps) atomicAdd(&c->captures, caps);
  if (exactT) atomicAdd(&c->exact_T, exactT);
  if (melts) atomicAdd(&c->melts, melts);
  if (visited) atomicAdd(&c->cells_visited, visited);
  if (eactive) atomicAdd(&c->elements_active, eactive);
}

}  // namespace

int remelt_persistent_grid(int device, int per_sm) {
  int sms = 0, per = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, remelt_kernel, kBlock, 0) != cudaSuccess) return 0;
  return sms * std::max(1, std::min(per, per_sm));
}

cudaError_t remelt_run_steps(const RemeltDevice &d, long long limit, int blocks, cudaStream_t s) {
  void *args[] = {(void *)&d, (void *)&limit};
  // the barrier's arrival counter starts every launch at zero
  const cudaError_t e = cudaMemsetAsync(d.ctrl, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  return cudaLaunchCooperativeKernel((const void *)remelt_kernel, dim3(blocks), dim3(kBlock), args, 0, s);
}

// ---------------------------------------------------------------------------
// Full state fields of the last completed step (reference arrays)
// ---------------------------------------------------------------------------
namespace {

__global__ void state_fields_kernel(RemeltDevice d, long long step, double dt_prev, double *T, uint8_t *cooling,
                                    uint8_t *flag) {
  // the last phase update ran at iStep_ = step - 1 with node temperatures
  // theta[(step - 1) % 3]; its cooling_ compared with theta[(step - 2) % 3]
  const long long k = step - 1;
  const double *th = d.theta[((k % 3) + 3) % 3];
  const double *thp = d.theta[(((k - 1) % 3) + 3) % 3];
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < d.ncells; c += (int64_t)gridDim.x * blockDim.x) {
    double t = -1.0;
    const bool withMat = eval_T(d, th, c, t);
    if (T) T[c] = t;
    if (cooling) {
      bool cool = false;
      if (k > 0) {
        double told = -1.0;
        eval_T(d, thp, c, told);
        double rate = 410;
        if (told > 0) rate = (t - told) / dt_prev;
        if (t <= 0) rate = 0;
        cool = withMat ? (rate < 0) : false;
      }
      cooling[c] = cool ? 1 : 0;
    }
    if (flag) flag[c] = (d.flagbits[c >> 5] >> (c & 31)) & 1u;
  }
}

}  // namespace

cudaError_t remelt_state_fields(const RemeltDevice &d, long long step, double dt_prev, double *T, uint8_t *cooling,
                                uint8_t *flag, cudaStream_t s) {
  const int blocks = (int)std::min<int64_t>((d.ncells + 255) / 256, 152 * 16);
  state_fields_kernel<<<blocks > 0 ? blocks : 1, 256, 0, s>>>(d, step, dt_prev, T, cooling, flag);
  return cudaGetLastError();
}

}  // namespace amca
