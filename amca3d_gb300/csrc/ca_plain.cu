// ca_plain.cu — the plain (uniform-cooling) CA step as one persistent,
// cooperative CUDA kernel for sm_103a.
//
// Reference semantics (CA/src/CellularAutomataManager_3D.cpp:441-669):
//   nucleate sites in ascending cell id, compute dt, grow every active
//   envelope, then walk the active list in ascending envelope id; each
//   envelope tests its 26 neighbours and captures every liquid one inside
//   its octahedron, appending the new envelope to the list it is walking.
//
// Parallel equivalent, per step:
//   The envelope list lives in one array in walk order: nucleation and
//   captures append to it, dead entries stay as tombstones until an
//   occasional compaction. Only what changes is touched:
//   wake    : growth is uniform, so each entry keeps a wake key, the
//             cumulative growth at which its half-diagonal may reach a lower
//             bound of |c'|_1 over its liquid neighbours. A scan of the keys
//             (4 B per entry) picks, in walk order, the entries that may
//             capture this step; the others are not read. Their half-diagonal
//             is brought up to date when they wake, by replaying the step
//             increments from a ring, the same FP64 sums in the same order.
//   deaths  : each entry keeps the count of its liquid neighbours; nucleation
//             and captures decrement the counts of the entries around the
//             cell. A sleeping entry whose count reaches zero leaves the list
//             in this step if every capture that emptied it came from an
//             earlier rank of generation 0, else in the next step (at its
//             turn a neighbour was still liquid), exactly as the reference's
//             walk deactivates it.
//   generation 0 = the woken entries, then this step's nuclei; generation
//   g+1 = the envelopes created while walking generation g (a contiguous id
//   range, because ids are handed out in walk order, appended to the list).
//   claim   : every envelope of the generation tests its liquid neighbours
//             (FP32 pre-test with a proven error margin, exact FP64 when the
//             margin is not enough) and atomicMin's a claim word
//             0x80000000 | parity<<30 | rank into each cell it contains.
//             rank order == walk order, so the smallest claim is the envelope
//             that reaches the cell first in the reference. An envelope of
//             generation g+1 first builds itself: the decentred octahedron of
//             its parent (FP64), and writes its orientation into its cell.
//             Each sets its liquid count and its next wake key.
//   resolve : an envelope captures the cells whose final claim is its own;
//             it stays active iff some neighbour was liquid at its turn and
//             not captured by it (unclaimed, or claimed by a later rank).
//             One decoupled look-back per block over (captures, survives)
//             gives the new envelope ids (walk order) and the child records
//             (parent rank, neighbour index); the others become tombstones.
// The resolve pass gives each block one contiguous chunk of the generation
// (its look-back runs once per block); claims and a separate marking pass
// need no order and hand out rank pieces dynamically (RankSched); nucleation
// sites sit one tile per block when they fit. Every phase boundary is a grid
// barrier; every wait is bounded in time and reports through an error flag.
//
// Loads use the default (L1-cached) path: a phase only reads values written
// before the barrier that opened it (the barrier's acquire makes them
// visible), or, for the cell field in the claim phase, values whose changes
// during the phase (claims, and claim words replaced by orientation ids)
// never change the liquid / solid answer the phase needs.
#include <math.h>
#include <stdio.h>

#include <mutex>

#include "../../include/amca3d.h"
#include "ca_plain.h"

namespace amca {

namespace {

constexpr int kBlock = 256;
constexpr int kWarps = kBlock / 32;
#ifndef AMCA_MIN_BLOCKS
#define AMCA_MIN_BLOCKS 4
#endif
constexpr int kMinBlocks = AMCA_MIN_BLOCKS;  // co-resident blocks per SM the register budget is sized for
constexpr unsigned long long kWaitNs = 5000000000ull;  // 5 s bound on any spin
constexpr long long kClaimBatch = 2 * kBlock;           // ranks a block takes per grab in the claim phase
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPrefix = 2ull << 62;
constexpr unsigned long long kPayload = (1ull << 62) - 1;

// The blocks that run one realm together (the team) and this block's rank in
// it: the whole grid for one realm, a slice of it in the batched launch.
__shared__ int t_nb;
__shared__ int t_b;

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
template <typename T>
__device__ __forceinline__ T ld_volatile(const T *p) {
  return *(const volatile T *)p;
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

// Thread 0's verdict on the block's last barrier.
__shared__ int s_bar_ok;

// Barrier of the t_nb blocks of the team on the adjacent words (count, gen),
// read as one 64-bit arrival counter that only grows: it is zero when the
// team's first barrier starts (host reset before every launch) and every
// arrival adds one, so barrier k of the launch ends when the counter reaches
// k x t_nb, the next multiple of the team size above the arrival's old
// value. An arrival is one acquire-release atomic (the block's writes,
// ordered before it by the block barrier, are released with it; the last
// arrival acquires the others' through it) and the others wait with acquire
// loads; no arrival has to open the next barrier (a second atomic on the
// critical path, about 0.65 us of a 2.2-2.3 us barrier with 152-456 blocks
// on GB300). Returns false when a wait ran out or thread 0 saw the error word
// set: sampled as it arrives (its latency hides behind the arrival) and
// while it waits. An error raised in this block before the barrier is always
// seen; one raised elsewhere at the latest at the next barrier, where every
// block still running waits on the blocks that stopped. The verdict reaches
// the block through shared memory (no global read after the release).
// Thread 0's part: arrive and wait; the verdict goes to s_bar_ok. Not
// inlined: one copy instead of one per barrier site keeps the step loop's
// register allocation free of it.
__device__ __noinline__ void barrier_arrive_wait(unsigned long long *w, int *error, unsigned long long wait_ns) {
  const int seen = ld_volatile(error);
  const unsigned long long old = atom_add_acq_rel64(w, 1ull);
  const unsigned long long nb = (unsigned long long)t_nb;
  const unsigned long long target = (old / nb + 1ull) * nb;
  bool ok = true;
  if (old + 1ull != target) {
    const unsigned long long t0 = now_ns();
    unsigned it = 0;
    while (ld_acquire64(w) < target) {
      if ((++it & 7u) == 0u) {
        if (ld_volatile(error) != 0) {
          ok = false;
          break;
        }
        if (now_ns() - t0 > wait_ns) {
          atomicCAS(error, 0, kErrBarrier);
          ok = false;
          break;
        }
      }
      __nanosleep(32);
    }
  }
  s_bar_ok = ok && seen == 0;
}
__device__ __forceinline__ bool team_barrier(unsigned *count, unsigned *gen_word, int *error,
                                             unsigned long long wait_ns = kWaitNs) {
  (void)gen_word;  // == count + 1
  __syncthreads();
  if (threadIdx.x == 0) barrier_arrive_wait((unsigned long long *)count, error, wait_ns);
  __syncthreads();
  return s_bar_ok != 0;
}

// Barrier over the blocks that run the realm; false when it failed. Block 0
// adds its time inside the barrier to ns_barrier_block0.
__device__ __forceinline__ bool grid_barrier(PlainCtrl *c) {
  const unsigned long long t0 = (t_b == 0 && threadIdx.x == 0) ? now_ns() : 0ull;
  const bool ok = team_barrier(&c->bar_count, &c->bar_gen, &c->error);
  if (t_b == 0 && threadIdx.x == 0) c->ns_barrier_block0 += now_ns() - t0;
  return ok;
}

// Exclusive scan of one u64 per thread over the block; *total = block sum.
__device__ unsigned long long block_exclusive_scan(unsigned long long v, unsigned long long *smem,
                                                   unsigned long long *total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) smem[warp] = x;
  __syncthreads();
  if (warp == 0) {
    unsigned long long w = lane < kWarps ? smem[lane] : 0ull;
#pragma unroll
    for (int o = 1; o < kWarps; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kWarps) smem[lane] = w;
  }
  __syncthreads();
  const unsigned long long before = warp > 0 ? smem[warp - 1] : 0ull;
  *total = smem[kWarps - 1];
  __syncthreads();
  return before + x - v;
}

// (a<<32 | b) <-> 62-bit payload (a<<31 | b); a, b < 2^31.
__device__ __forceinline__ unsigned long long to_payload(unsigned long long v) {
  return ((v >> 32) << 31) | (v & 0xffffffffull);
}
__device__ __forceinline__ unsigned long long from_payload(unsigned long long p) {
  return ((p >> 31) << 32) | (p & 0x7fffffffull);
}

// Exclusive prefix of this block's aggregate over the blocks before it
// (tile index = block index), by decoupled look-back with the whole block:
// thread 0 publishes the aggregate; each round every thread reads one of the
// kBlock nearest unread predecessor status words, each warp finds its nearest
// inclusive prefix and sums the payloads up to it, and the warps' results
// (shared memory, one barrier) give the block's answer: a round covers kBlock
// predecessors, so a team of a few hundred blocks needs at most a few rounds
// of one dependent load each. Returns ~0 (error flag set) when a wait ran out.
__device__ unsigned long long block_prefix(unsigned long long *status, unsigned long long agg,
                                           unsigned long long *smem, PlainCtrl *c) {
  (void)smem;
  __shared__ unsigned s_pre[kWarps], s_empty[kWarps];
  __shared__ unsigned long long s_part[kWarps];
  __shared__ int s_bail;
  const long long t = t_b;
  if (threadIdx.x == 0) atomicExch(status + t, (t == 0 ? kFlagPrefix : kFlagAgg) | to_payload(agg));
  if (t == 0) return 0ull;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long sum = 0;  // the same in every thread
  long long p = t - 1;
  const unsigned long long t0 = now_ns();
  for (;;) {
    const long long q = p - threadIdx.x;
    const unsigned long long s = q >= 0 ? ld_acquire(status + q) : kFlagPrefix;  // before tile 0: prefix 0
    const unsigned long long flag = s & ~kPayload;
    const unsigned pre = __ballot_sync(0xffffffffu, flag == kFlagPrefix);
    const unsigned empty = __ballot_sync(0xffffffffu, flag == 0);
    const unsigned upto = pre ? (((pre & (0u - pre)) << 1) - 1u) : 0xffffffffu;  // lanes up to the warp's prefix
    unsigned long long v = ((upto >> lane) & 1u) ? from_payload(s & kPayload) : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
      s_pre[warp] = pre;
      s_empty[warp] = empty & upto;
      s_part[warp] = v;
    }
    __syncthreads();
    // the nearest warp holding a prefix, and whether any word up to it is unpublished
    int wstar = kWarps;
    bool waiting = false;
    unsigned long long part = 0;
#pragma unroll
    for (int w = 0; w < kWarps; ++w) {
      if (wstar < kWarps) break;
      waiting = waiting || s_empty[w] != 0;
      part += s_part[w];
      if (s_pre[w]) wstar = w;
    }
    if (waiting) {
      if (threadIdx.x == 0)
        s_bail = (now_ns() - t0 > kWaitNs || ld_volatile(&c->error) != 0) ? (atomicCAS(&c->error, 0, kErrLookback), 1) : 0;
      __syncthreads();
      const int bail = s_bail;
      __syncthreads();  // s_pre and s_bail are rewritten next round
      if (bail) return ~0ull;
      continue;
    }
    sum += part;
    __syncthreads();  // s_pre, s_empty and s_part are rewritten next round
    if (wstar < kWarps) break;
    p -= kBlock;
  }
  if (threadIdx.x == 0) atomicExch(status + t, kFlagPrefix | to_payload(sum + agg));
  return sum;
}

// This block's contiguous share [b, e) of [0, n).
__device__ __forceinline__ void block_chunk(long long n, long long &b, long long &e) {
  const long long per = (n + t_nb - 1) / t_nb;
  b = per * t_b;
  if (b > n) b = n;
  e = b + per;
  if (e > n) e = n;
}

// Dynamic schedule of a pass over n ranks, taken warp by warp from a shared
// counter (warps never wait for each other inside the pass): chunks of up to
// 256 ranks first, then, over the last 32 ranks per warp of the team, chunks
// of 32 (one rank per lane), so the warps that finish last are at most one
// short chunk behind. Lane 0 calls it; returns (b, e), or b = -1 when none
// is left.
// A warp's first chunk is its own, numbered across blocks first (warp w of
// block b takes chunk w * blocks + b, so a small generation spreads over
// every SM) and taken without an atomic (a generation smaller than one chunk
// per warp costs no counter traffic); later ones come from the counter,
// numbered after those.
__device__ __noinline__ longlong2 next_warp_chunk(long long n, unsigned long long *counter, bool first) {
  const long long warps = (long long)t_nb * kWarps;
  long long big = (((n + 2 * warps - 1) / (2 * warps)) + 31) & ~31ll;
  big = big < 32 ? 32 : (big > 256 ? 256 : big);
  const long long head = n - 32 * warps;
  const long long nbig = head > 0 ? head / big : 0, split = nbig * big;
  // when every chunk is some warp's own, the counter has none to give
  if (!first && nbig + (n - split + 31) / 32 <= warps) return make_longlong2(-1, -1);
  const long long q =
      first ? (long long)(threadIdx.x >> 5) * t_nb + t_b : warps + (long long)atomicAdd(counter, 1ull);
  long long b, e;
  if (q < nbig) {
    b = q * big;
    e = b + big;
  } else {
    b = split + (q - nbig) * 32;
    e = b + 32;
  }
  if (b >= n) return make_longlong2(-1, -1);
  return make_longlong2(b, e < n ? e : n);
}

// Chunks of a pass over n ranks taken block by block: chunks of up to
// kClaimBatch ranks, then, over the last kBlock ranks per block of the team,
// chunks of at most one rank per thread (32-rank chunks for generations too
// small to give every block one). s_chunks = (big, small, number of big
// chunks, where the small ones start), set once per pass by thread 0.
__shared__ long long s_chunks[4];

__device__ __noinline__ void set_block_chunks(long long n) {
  long long small = (((n + t_nb - 1) / t_nb) + 31) & ~31ll;
  small = small < 32 ? 32 : (small > kBlock ? kBlock : small);
  long long big = (((n + 2ll * t_nb - 1) / (2ll * t_nb)) + 31) & ~31ll;
  big = big < small ? small : (big > kClaimBatch ? kClaimBatch : big);
  const long long head = n - small * t_nb;
  const long long nbig = head > 0 ? head / big : 0;
  s_chunks[0] = big;
  s_chunks[1] = small;
  s_chunks[2] = nbig;
  s_chunks[3] = nbig * big;
}

// Chunk q: (b, e), or b = -1 past the end.
__device__ __forceinline__ longlong2 block_chunk_range(long long n, long long q) {
  long long b, e;
  if (q < s_chunks[2]) {
    b = q * s_chunks[0];
    e = b + s_chunks[0];
  } else {
    b = s_chunks[3] + (q - s_chunks[2]) * s_chunks[1];
    e = b + s_chunks[1];
  }
  if (b >= n) return make_longlong2(-1, -1);
  return make_longlong2(b, e < n ? e : n);
}

// The block's pool of the current chunk, handed to its warps 32 ranks at a
// time: (chunk index << 32) | offset into the chunk.
__shared__ unsigned long long s_pool;

// Dynamic schedule of a pass over n ranks whose order does not matter, in
// pieces of 32 ranks per warp (lane i takes rank b + i). Teams of at most 64
// blocks, and small generations on larger teams, take their chunks warp by
// warp from the shared counter. Large generations on large teams take them
// block by block (one shared-counter atomic per block chunk: the counter
// serialises its atomics, about 3 ns each on GB300, and one per warp chunk
// of 600 blocks costs tens of us), and the block's warps share each chunk
// through the pool: a shared-memory atomic gives a warp its piece, the warp
// whose piece starts at the chunk's end takes the next chunk, and no warp
// waits for the others except while the pool is refilled.
struct RankSched {
  long long n;
  unsigned long long *counter;
  int *error;
  bool warp;
  bool own_chunk = true;  // warp mode: the first chunk is the warp's own
  __device__ RankSched(long long n_, unsigned long long *c, int *err, int warp_sched)
      : n(n_), counter(c), error(err), warp(t_nb <= 64 || n_ <= (long long)warp_sched * t_nb) {
    if (!warp) {
      if (threadIdx.x == 0) {
        set_block_chunks(n);
        s_pool = (unsigned long long)t_b << 32;  // the block's first chunk is its own index
      }
      __syncthreads();
    }
  }
  // The next piece [b, e) of this warp; false when none is left.
  __device__ __forceinline__ bool next(long long &b, long long &e) {
    const int lane = threadIdx.x & 31;
    if (warp) {
      longlong2 c = make_longlong2(0, 0);
      if (lane == 0) c = next_warp_chunk(n, counter, own_chunk);
      own_chunk = false;
      b = __shfl_sync(0xffffffffu, c.x, 0);
      e = __shfl_sync(0xffffffffu, c.y, 0);
      return b >= 0;
    }
    const unsigned long long t0 = now_ns();
    for (;;) {
      unsigned long long old = 0;
      if (lane == 0) old = atomicAdd(&s_pool, 32ull);
      old = __shfl_sync(0xffffffffu, old, 0);
      const long long q = (long long)(old >> 32), off = (long long)(old & 0xffffffffull);
      const longlong2 ch = block_chunk_range(n, q);
      if (ch.x < 0) return false;
      const long long len = ch.y - ch.x;
      if (off < len) {
        b = ch.x + off;
        e = b + 32 < ch.y ? b + 32 : ch.y;
        return true;
      }
      if (off < len + 32) {  // this warp's piece starts at the chunk's end: it takes the next chunk
        if (lane == 0) atomicExch(&s_pool, ((unsigned long long)t_nb + atomicAdd(counter, 1ull)) << 32);
        __syncwarp();
        continue;
      }
      // another warp is taking the next chunk: wait until the pool moves on
      int bail = 0;
      if (lane == 0) {
        while ((long long)(*(volatile unsigned long long *)&s_pool >> 32) == q) {
          if (now_ns() - t0 > kWaitNs || ld_volatile(error) != 0) {
            atomicCAS(error, 0, kErrBarrier);
            bail = 1;
            break;
          }
          __nanosleep(20);
        }
      }
      if (__shfl_sync(0xffffffffu, bail, 0)) return false;
    }
  }
  __device__ __forceinline__ int first() const { return (int)(threadIdx.x & 31); }
  __device__ __forceinline__ int stride() const { return 32; }
};

__device__ __forceinline__ int nbr_delta(const Grid &g, int n, int &di, int &dj, int &dk) {
  nbr_offset(n, di, dj, dk);
  return dk * g.nxyg + dj * g.nxg + di;
}

__device__ __forceinline__ void set_solid(uint32_t *solid, int cell) {
  atomicOr(solid + (cell >> 5), 1u << (cell & 31));
}

// Bits of a cell bitmap for the 26 neighbours of `cell`, in the reference's
// neighbour order (bit n of the result = neighbour n): one 64-bit window per
// row of three cells, nine rows.
__device__ __forceinline__ uint32_t neighbour_bits(const uint32_t *map, const Grid &g, int cell) {
  uint32_t m27 = 0;
#pragma unroll
  for (int dk = -1; dk <= 1; ++dk)
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
      const long long c0 = (long long)cell + dk * g.nxyg + dj * g.nxg - 1;  // the row's di = -1 cell
      const long long w = c0 >> 5;
      const unsigned long long two = ((unsigned long long)map[w + 1] << 32) | map[w];
      m27 |= ((uint32_t)(two >> (c0 & 31)) & 7u) << ((dk + 1) * 9 + (dj + 1) * 3);
    }
  return (m27 & 0x1fffu) | ((m27 >> 14) << 13);  // drop the centre cell (index 13 of 27)
}

__device__ __forceinline__ uint32_t liquid_neighbours(const uint32_t *solid, const Grid &g, int cell) {
  return ~neighbour_bits(solid, g, cell) & 0x03ffffffu;
}

// ---------------------------------------------------------------------------
// The envelope list: wake keys, grown half-diagonals, liquid counts.
// ---------------------------------------------------------------------------
// Whether an entry with wake key k is processed in a step whose cumulative
// growth is `grown` (all: every live entry, to bring its record up to date).
// Dead entries (NaN) never are. The test (double)k <= grown is made in FP32
// (the FP64 pipe is narrow), exactly: for a float k it holds iff k is at most
// grown rounded down to float, gf.
__device__ __forceinline__ float wake_bound(double grown) { return __double2float_rd(grown); }
__device__ __forceinline__ bool woken(float k, float gf, bool all) { return all ? !isnan(k) : k <= gf; }

// Wake key: the cumulative growth at which the half-diagonal L (grown up to
// `grown`, gf = grown rounded down to float) may reach t_lb: t_lb + (grown -
// L), every rounding downwards, less 2^-30 of the magnitudes involved (L is
// at most grown plus a few cells), which covers the rounding of the FP64 step
// sums over the at most kWakeAll steps before the entry is looked at again
// by a factor of thousands. One FP64 subtraction and one conversion; the rest
// in FP32. +inf when no liquid neighbour is left. Waking early only costs a
// test.
__device__ __forceinline__ float wake_key(float t_lb, double L, double grown, float gf) {
  if (!(t_lb < INFINITY)) return INFINITY;
  const float o = __double2float_rd(grown - L);
  const float slack = 9.313225746154785e-10f * (fabsf(t_lb) + fabsf(o) + 2.0f * gf);
  return __fsub_rd(__fadd_rd(t_lb, o), slack);
}

// Grain::grow (Grain.h:27) of the steps (from, to]: the same FP64 additions
// of each step's dt * vel, in order.
__device__ __forceinline__ double replay_growth(const double *dvh, double L, long long from, long long to) {
  for (long long t = from + 1; t <= to; ++t) L += dvh[t & (kDvRing - 1)];
  return L;
}

// A dead entry: never woken, and no longer found from its cell.
__device__ __forceinline__ void tombstone(const PlainDevice &d, int cur, long long q, int cell) {
  d.key[cur][q] = __int_as_float(0x7fc00000);
  d.cellw[cell] = kNoEntry;
}

// The list positions of a generation's ranks: generation 0 is the woken
// entries (wlist, in walk order) followed by the step's nuclei from `base`;
// a later generation is the contiguous run from `base`.
struct GenList {
  const int32_t *w;
  long long nw;
  long long base;
  __device__ __forceinline__ long long at(long long r) const { return r < nw ? (long long)w[r] : base + (r - nw); }
};

// A nucleus turned `cell` solid before the walk: one liquid neighbour fewer
// for every entry around it, and a sleeping entry left without one is
// deactivated at its turn (a woken one decides at its turn itself). Returns
// those entries.
__device__ __noinline__ unsigned nucleus_neighbours(const PlainDevice &d, int cur, int cell, double grown, bool all,
                                                    unsigned long long *stat_dec) {
  const Grid &g = d.grid;
  unsigned gone = 0;
  int di, dj, dk;
  // the 26 atomics issued before any result is used
  uint32_t w[26];
#pragma unroll
  for (int nb = 0; nb < 26; ++nb) w[nb] = atomicSub(d.cellw + cell + nbr_delta(g, nb, di, dj, dk), 1u);
  const float gf = wake_bound(grown);
#pragma unroll
  for (int nb = 0; nb < 26; ++nb) {
    if (!has_entry(w[nb])) continue;
    ++*stat_dec;
    const int q = (int)(w[nb] >> 5);
    if ((w[nb] & 31u) == 1u && !woken(d.key[cur][q], gf, all)) {
      tombstone(d, cur, q, cell + nbr_delta(g, nb, di, dj, dk));
      ++gone;
    }
  }
  return gone;
}

// Zero-count events a block gathers before adding them to a zero list.
constexpr int kZeroBuf = 512;
__shared__ int s_zero[kZeroBuf];
__shared__ unsigned s_nz;
__shared__ unsigned long long s_zbase;

// The liquid counts around the n cells that the previous generation captured
// (its child records, this generation's ranks, which name the capturers'
// list positions): one atomic decrement of the cell word of each
// neighbour cell, whose old value says which entry (if any) lives there and
// its count before. This generation's own entries still hold no-entry words
// (they set theirs in the resolve phase, from the bitmap, which has these
// captures), and a no-entry word never reaches a zero count. A decrement by
// a later rank (capturer beyond the entry) is recorded in late[]; a count
// reaching zero goes to the block's zero buffer (s_nz reset before), or to
// the zero list of parity zpar once the buffer is full. Capture k goes to
// the thread numbered k among `threads` ones; this thread is number t0. The
// 26 atomics of a capture are issued before any result is used.
__device__ __noinline__ void decrement_captures(const PlainDevice &d, int cur, long long n,
                                                long long step, int zpar, long long t0, long long threads,
                                                unsigned long long *stat_dec) {
  const Grid &g = d.grid;
  const EnvRec *act = d.act[cur];
  for (long long k = t0; k < n; k += threads) {
    const uint32_t rec = d.child[k];
    const int pc = (int)(rec >> 5);  // the capturer's list position
    int di, dj, dk;
    const int cell = act[pc].cell + nbr_delta(g, (int)(rec & 31u), di, dj, dk);
    uint32_t w[26];
#pragma unroll
    for (int nb = 0; nb < 26; ++nb) w[nb] = atomicSub(d.cellw + cell + nbr_delta(g, nb, di, dj, dk), 1u);
#pragma unroll
    for (int nb = 0; nb < 26; ++nb) {
      if (!has_entry(w[nb])) continue;
      ++*stat_dec;
      const int q = (int)(w[nb] >> 5);
      if (pc > q) d.late[q] = (int32_t)step;
      if ((w[nb] & 31u) != 1u) continue;
      const unsigned z = atomicAdd(&s_nz, 1u);
      if (z < (unsigned)kZeroBuf) {
        s_zero[z] = q;
      } else {
        const unsigned long long zi = atomicAdd(&d.ctrl->zn[zpar], 1ull);
        d.zlist[zpar][zi] = q;
      }
    }
  }
}

// The block's buffered zero events into the zero list of parity zpar (every
// thread of the block).
__device__ __noinline__ void flush_zero_buffer(const PlainDevice &d, int zpar) {
  __syncthreads();
  const unsigned nz = s_nz < (unsigned)kZeroBuf ? s_nz : (unsigned)kZeroBuf;
  if (threadIdx.x == 0 && nz) s_zbase = atomicAdd(&d.ctrl->zn[zpar], (unsigned long long)nz);
  __syncthreads();
  for (unsigned i = threadIdx.x; i < nz; i += kBlock) d.zlist[zpar][s_zbase + i] = s_zero[i];
}

// Nucleus number r (in site order) of this step on `cell`: orientation,
// envelope table entry and list record at position base_pos + r, grown from
// the previous step on (CellularAutomataManager.cpp:262-290). Returns the
// entries around it that leave the list at their turn.
__device__ __forceinline__ unsigned place_nucleus(const PlainDevice &d, int cur, long long base_pos,
                                                  long long base_orient, long long base_grain, long long r, int cell,
                                                  long long step, double grown, bool all,
                                                  unsigned long long *stat_dec) {
  const int oid = (int)(base_orient + r);
  const long long gid = base_grain + r;
  int I, J, K;
  cell_ijk(d.grid, cell, I, J, K);
  d.orient[cell] = (uint32_t)oid;
  set_solid(d.solid, cell);
  d.gx[gid] = centre_coord(d.grid.x0, d.grid.h, I);
  d.gy[gid] = centre_coord(d.grid.y0, d.grid.h, J);
  d.gz[gid] = centre_coord(d.grid.z0, d.grid.h, K);
  d.gori[gid] = oid;
  d.gcell[gid] = cell;
  EnvRec en;  // a nucleus: length 0, centred on its cell
  en.L = 0.0;
  en.dx = en.dy = en.dz = 0.f;
  en.cell = cell;
  en.ori = oid;
  en.id = (int32_t)gid;
  d.act[cur][base_pos + r] = en;
  d.lstep[cur][base_pos + r] = (int32_t)(step - 1);
  return nucleus_neighbours(d, cur, cell, grown, all, stat_dec);
}

// Sites are held as tiles of kBlock, one per block, when they fit: tile t =
// sites [t*kBlock, (t+1)*kBlock), thread i of block t owns site t*kBlock + i
// for the whole launch and keeps its cell (-1 once removed) and dTc in shared
// memory.
__device__ __forceinline__ bool site_tiles(const PlainDevice &d) { return d.nsites <= (long long)kBlock * t_nb; }

// ---------------------------------------------------------------------------
// Nucleation (CellularAutomataManager.cpp:219-297) in site order.
// Tiled sites: one pass, nucleus ranks from one block scan plus the look-back
// over the site tiles. Otherwise pass 1 marks sites (2 = nucleates now, 0 =
// removed) and pass 2 hands out orientation / envelope ids in site order.
// The counts that every block tracks itself (orientations, envelope ids,
// liquid cells) are not read here; the last site tile publishes the active
// count in the step's parity slot (a step without envelopes has no barrier
// before the next nucleation), which every block reads after the barrier.
// ---------------------------------------------------------------------------
// calculate_time_step (CellularAutomataManager_3D.cpp:449-507): one velocity
// for the uniform field; dt for "some active envelope" (da) and for "none"
// (dn: maxVelocity stays 1e-10), picked after nucleation. Every block
// evaluates it itself (the same FP64 operations, so the same values).
__device__ __forceinline__ void step_rates(const PlainDevice &d, double time, double &vel, double &da, double &dn) {
  const double T = d.T0 + d.Tdot * time;  // compute_cell_temperature (ProblemPhysics.cpp:164-169)
  vel = kgt_velocity(d.Tm, T, d.a1, d.a2, d.a3);
  const double maxV = vel > 1e-10 ? vel : 1e-10;
  const double a = d.tsf * d.grid.h / maxV, b = d.tsf * d.grid.h / 1e-10;
  da = (d.max_dt < a) ? d.max_dt : a;  // std::min (:507)
  dn = (d.max_dt < b) ? d.max_dt : b;
  if (d.dt_cap > 0) {  // setup_time_step_for_coupling of an external solver
    da = (d.dt_cap < da) ? d.dt_cap : da;
    dn = (d.dt_cap < dn) ? d.dt_cap : dn;
  }
}

// Nuclei go to the list from position base_pos on; `gone` counts the
// entries around them that leave the list at their turn.
__device__ __noinline__ bool nucleation_phase(const PlainDevice &d, int cur, double time, long long step, long long base_pos,
                                 long long base_orient, long long base_grain, double grown, bool all, int *s_cell,
                                 double *s_dtc, unsigned long long *smem, unsigned long long *stat_live,
                                 unsigned long long *stat_dec, unsigned *gone) {
  PlainCtrl *c = d.ctrl;
  unsigned long long *scan = d.scanA + (step & 1) * kStatusWords;
  const double T = d.T0 + d.Tdot * time;  // compute_cell_temperature (ProblemPhysics.cpp:164-169)
  const double dTu = d.Tm - T;
  // next step's look-back word starts cleared: it was last read in the
  // previous step's nucleation, which every block finished before that
  // phase's barrier
  if (threadIdx.x == 0) d.scanA[((step + 1) & 1) * kStatusWords + t_b] = 0ull;
  if (site_tiles(d)) {
    const long long ntiles = (d.nsites + kBlock - 1) / kBlock;
    if (t_b >= ntiles) {  // no sites in this block
      if (ntiles == 0 && t_b == 0 && threadIdx.x == 0) c->n_active_nuc[step & 1] = base_pos;
      return true;
    }
    const int cell = s_cell[threadIdx.x];
    unsigned nuc = 0;
    if (cell >= 0) {
      ++*stat_live;
      const bool liquid = d.orient[cell] == kLiquid;
      nuc = liquid && dTu > s_dtc[threadIdx.x];
      if (!liquid || nuc) {  // removed from the site list
        s_cell[threadIdx.x] = -1;
        d.site_live[(long long)t_b * kBlock + threadIdx.x] = 0;
      }
    }
    unsigned long long agg;
    const unsigned long long ex = block_exclusive_scan(nuc, smem, &agg);
    const unsigned long long pre = block_prefix(scan, agg, smem, c);
    if (pre == ~0ull) return false;
    if (nuc)
      *gone += place_nucleus(d, cur, base_pos, base_orient, base_grain, (long long)(pre + ex), cell, step, grown, all,
                             stat_dec);
    if (t_b == ntiles - 1 && threadIdx.x == 0) c->n_active_nuc[step & 1] = base_pos + (long long)(pre + agg);
    return true;
  }
  long long b, e;
  block_chunk(d.nsites, b, e);
  unsigned long long count = 0;
  for (long long i = b + threadIdx.x; i < e; i += kBlock) {
    if (!d.site_live[i]) continue;
    ++*stat_live;
    const bool liquid = d.orient[d.site_cell[i]] == kLiquid;
    const bool nuc = liquid && dTu > d.site_dtc[i];
    d.site_live[i] = nuc ? 2 : (liquid ? 1 : 0);
    count += nuc ? 1u : 0u;
  }
  unsigned long long agg;
  block_exclusive_scan(count, smem, &agg);
  const unsigned long long pre = block_prefix(scan, agg, smem, c);
  if (pre == ~0ull) return false;
  unsigned long long run = pre;
  for (long long i0 = b; i0 < e; i0 += kBlock) {
    const long long i = i0 + threadIdx.x;
    unsigned nuc = 0;
    int cell = 0;
    if (i < e && d.site_live[i] == 2) {
      nuc = 1;
      cell = d.site_cell[i];
      d.site_live[i] = 0;
    }
    unsigned long long tot;
    const unsigned long long ex = block_exclusive_scan(nuc, smem, &tot);
    if (nuc)
      *gone += place_nucleus(d, cur, base_pos, base_orient, base_grain, (long long)(run + ex), cell, step, grown, all,
                             stat_dec);
    run += tot;
  }
  if (t_b == t_nb - 1 && threadIdx.x == 0) c->n_active_nuc[step & 1] = base_pos + (long long)(pre + agg);
  return true;
}

// ---------------------------------------------------------------------------
// Ordered selections over the list: the wake scan and the compaction. The
// block takes a contiguous chunk of positions, each warp a contiguous piece
// of it: pass 1 counts (ballots), one block scan over the warps and one
// look-back over the blocks place the block, pass 2 writes in order.
// ---------------------------------------------------------------------------
struct WarpPiece {
  long long b, e;
  __device__ WarpPiece(long long n) {
    long long cb, ce;
    block_chunk(n, cb, ce);
    const long long per = ((((ce - cb) + kWarps - 1) / kWarps) + 31) & ~31ll;
    const long long w = threadIdx.x >> 5;
    b = cb + w * per < ce ? cb + w * per : ce;
    e = b + per < ce ? b + per : ce;
  }
};

// Offset of this warp's first selected position among all selected ones,
// given the warp's count (lane 0's value counts); ~0 on a look-back failure.
__device__ __forceinline__ unsigned long long warp_offset(unsigned cnt, unsigned long long *status,
                                                        unsigned long long *smem, unsigned long long *total,
                                                        PlainCtrl *c) {
  unsigned long long agg;
  const unsigned long long ex = block_exclusive_scan((threadIdx.x & 31) == 0 ? cnt : 0u, smem, &agg);
  const unsigned long long pre = block_prefix(status, agg, smem, c);
  if (pre == ~0ull) return ~0ull;
  *total = pre + agg;
  return pre + __shfl_sync(0xffffffffu, ex, 0);
}

// The entries among positions [0, n) that this step processes, in walk
// order, into wlist; the count goes to n_woken[step & 1]. Keys are read as
// float4, 128 positions per warp and iteration (the key arrays are padded to
// a whole number of these tiles); the team takes contiguous runs of tiles,
// each warp a contiguous run of its block's.
__device__ __forceinline__ unsigned woken4(const float4 v, long long p0, long long n, float gf, bool all) {
  return (p0 < n && woken(v.x, gf, all) ? 1u : 0u) | (p0 + 1 < n && woken(v.y, gf, all) ? 2u : 0u) |
         (p0 + 2 < n && woken(v.z, gf, all) ? 4u : 0u) | (p0 + 3 < n && woken(v.w, gf, all) ? 8u : 0u);
}
__device__ __noinline__ bool wake_scan(const PlainDevice &d, int cur, long long n, long long step, double grown, bool all,
                                       unsigned long long *smem) {
  PlainCtrl *c = d.ctrl;
  // the next step's words start cleared (last read in the previous step)
  if (threadIdx.x == 0) d.scanC[((step + 1) & 1) * kStatusWords + t_b] = 0ull;
  const float4 *k4 = (const float4 *)d.key[cur];
  const float gf = wake_bound(grown);
  const long long ntiles = (n + kKeyTile - 1) / kKeyTile;
  long long tb, te;
  block_chunk(ntiles, tb, te);
  const long long per = ((te - tb) + kWarps - 1) / kWarps;
  const long long wb = tb + (threadIdx.x >> 5) * per < te ? tb + (threadIdx.x >> 5) * per : te;
  const long long we = wb + per < te ? wb + per : te;
  const int lane = threadIdx.x & 31;
  unsigned cnt = 0;
#pragma unroll 4
  for (long long t = wb; t < we; ++t) {
    const long long p0 = t * kKeyTile + 4 * lane;
    cnt += __popc(woken4(k4[t * (kKeyTile / 4) + lane], p0, n, gf, all));
  }
  cnt = __reduce_add_sync(0xffffffffu, cnt);
  unsigned long long total = 0;
  unsigned long long off = warp_offset(cnt, d.scanC + (step & 1) * kStatusWords, smem, &total, c);
  if (off == ~0ull) return false;
  // a key read again here may have turned dead since (a nucleus next to a
  // sleeping entry), which the first pass counted as not woken all the same
#pragma unroll 2
  for (long long t = wb; t < we; ++t) {
    const long long p0 = t * kKeyTile + 4 * lane;
    const unsigned f = woken4(k4[t * (kKeyTile / 4) + lane], p0, n, gf, all);
    unsigned x = __popc(f);  // inclusive warp scan of the lanes' counts
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    unsigned long long at = off + x - __popc(f);
    for (unsigned bits = f; bits; bits &= bits - 1) d.wlist[at++] = (int32_t)(p0 + __ffs(bits) - 1);
    off += __shfl_sync(0xffffffffu, x, 31);
  }
  if (t_b == t_nb - 1 && threadIdx.x == 0) c->n_woken[step & 1] = (long long)total;
  return true;
}

// The live entries of list `cur` among [0, n), in order, into list cur ^ 1
// with their keys, grow steps and liquid counts; the cell map follows. The
// new length goes to compact_len.
__device__ __noinline__ bool compact_phase(const PlainDevice &d, int cur, long long n, unsigned par, unsigned long long *smem,
                              unsigned long long *stat_moved) {
  PlainCtrl *c = d.ctrl;
  if (threadIdx.x == 0) d.scanD[(par ^ 1u) * kStatusWords + t_b] = 0ull;  // the next compaction's words
  const float *key = d.key[cur];
  const WarpPiece wp(n);
  const int lane = threadIdx.x & 31;
  unsigned cnt = 0;
  for (long long p0 = wp.b; p0 < wp.e; p0 += 32) {
    const long long p = p0 + lane;
    cnt += __popc(__ballot_sync(0xffffffffu, p < wp.e && !isnan(key[p])));
  }
  unsigned long long total = 0;
  unsigned long long off = warp_offset(cnt, d.scanD + par * kStatusWords, smem, &total, c);
  if (off == ~0ull) return false;
  const int nxt = cur ^ 1;
  for (long long p0 = wp.b; p0 < wp.e; p0 += 32) {
    const long long p = p0 + lane;
    const bool live = p < wp.e && !isnan(key[p]);
    const unsigned bal = __ballot_sync(0xffffffffu, live);
    if (live) {
      const long long q = (long long)off + __popc(bal & ((1u << lane) - 1u));
      const EnvRec en = d.act[cur][p];
      d.act[nxt][q] = en;
      d.key[nxt][q] = key[p];
      d.lstep[nxt][q] = d.lstep[cur][p];
      d.late[q] = -1;
      d.cellw[en.cell] = ((uint32_t)q << 5) | (d.cellw[en.cell] & 31u);
      ++*stat_moved;
    }
    off += __popc(bal);
  }
  if (t_b == t_nb - 1 && threadIdx.x == 0) c->compact_len = (long long)total;
  return true;
}

// The list departures this thread decided, added to the step's slots (now:
// step % 3, next step: (step + 1) % 3), one atomic per warp that has any.
__device__ __forceinline__ void flush_departures(PlainCtrl *c, long long step, unsigned &now, unsigned &next) {
  const unsigned a = __reduce_add_sync(0xffffffffu, now), b = __reduce_add_sync(0xffffffffu, next);
  if ((threadIdx.x & 31) == 0) {
    if (a) atomicAdd((unsigned long long *)&c->deaths[step % 3], (unsigned long long)a);
    if (b) atomicAdd((unsigned long long *)&c->deaths[(step + 1) % 3], (unsigned long long)b);
  }
  now = next = 0;
}

// Entries whose liquid count reached zero through the previous generation's
// captures (zero list of parity zpar; gen0: those were generation 0's): each
// leaves the list now or in the next step, and becomes a tombstone. One that
// died at its own turn is one already; one processed this step outlived its
// turn (it goes next step); a sleeping one (emptied only by generation 0)
// goes now unless a capture by a later rank emptied it too.
__device__ __noinline__ void zero_decisions(const PlainDevice &d, int cur, int zpar, bool gen0, long long step,
                                            unsigned *now, unsigned *next) {
  const unsigned long long nz = ld_volatile(&d.ctrl->zn[zpar]);
  for (unsigned long long i = (unsigned long long)t_b * kBlock + threadIdx.x; i < nz;
       i += (unsigned long long)t_nb * kBlock) {
    const int q = d.zlist[zpar][i];
    if (isnan(d.key[cur][q])) continue;
    const bool later = d.lstep[cur][q] == (int32_t)step || !gen0 || d.late[q] == (int32_t)step;
    tombstone(d, cur, q, d.act[cur][q].cell);
    if (later)
      ++*next;
    else
      ++*now;
  }
}

// ---------------------------------------------------------------------------
// Claim: growth up to this step (generation 0) or self-construction
// (generation >= 1), neighbour tests, atomicMin claims and the entry's next
// wake key (its liquid count is set in the resolve phase).
// ---------------------------------------------------------------------------
// With `dec` (generations after the first) the liquid counts around the
// previous generation's captures are decremented in the same phase: the
// first dec_warps warps of every block do that first and then join the
// claims, whose dynamic hand-out balances the difference, so the memory
// latency of the decrements overlaps the FP64 decentring of the claims.
__device__ __noinline__ void claim_phase(const PlainDevice &d, int cur, int kind, long long lo, long long n, unsigned par,
                            const GenList &list, long long step, double grown, bool dec,
                            int zpar, unsigned long long *stat_tests, unsigned long long *stat_tests64,
                            unsigned long long *stat_dec) {
  const Grid &g = d.grid;
  if (threadIdx.x == 0) d.scanB[t_b] = 0ull;  // this block's look-back word of the resolve phase
  EnvRec *act = d.act[cur];
  int32_t *lstep = d.lstep[cur];
  const float gf = wake_bound(grown);
  unsigned tests = 0, tests64 = 0;  // this phase's, added to the launch totals at its end
  // Claims need no order: warps or blocks take chunks of consecutive ranks
  // from a shared counter until none is left, so those that drew cheap
  // envelopes (few liquid neighbours) take more chunks.
  if (dec) {
    if (threadIdx.x == 0) s_nz = 0u;
    __syncthreads();
  }
  RankSched sched(n, &d.ctrl->claim_next, &d.ctrl->error, d.warp_sched);
  // teams of the batched launch (at most 64 blocks) give the decrements more
  // of their warps (batched_64: 77 ms at four, 81 at two; the whole GPU on
  // one realm: 64.7 ms at two, 69 at four)
  const int dw = t_nb <= 64 ? kDecWarpsTeam : d.dec_warps;
  if (dec && (int)(threadIdx.x >> 5) < dw)
    decrement_captures(d, cur, n, step, zpar, ((long long)t_b * dw + (threadIdx.x >> 5)) * 32 + (threadIdx.x & 31),
                       (long long)t_nb * dw * 32, stat_dec);
  const int first = sched.first(), stride = sched.stride();
  long long b, e;
  while (sched.next(b, e)) {
  for (long long r = b + first; r < e; r += stride) {
    EnvRec en;
    double gxd = 0, gyd = 0, gzd = 0;
    bool have_centre = false;
    uint32_t liq = 0;
    const long long p = list.at(r);
    if (kind == 0) {
      en = act[p];
      liq = liquid_neighbours(d.solid, g, en.cell);
      // Grain::grow (Grain.h:27) for every step since the record was last
      // grown: L + dt * vel, the product rounded once per step
      en.L = replay_growth(d.dvh, en.L, (long long)lstep[p], step);
      act[p].L = en.L;
      lstep[p] = (int32_t)step;
    } else {
      // CellularAutomataManager_3D::capture_cell (:677-707) for the capture
      // recorded by the parent: decentred envelope from the parent's
      // (grown) envelope, same orientation.
      const uint32_t rec = d.child[r];
      const EnvRec pe = act[rec >> 5];  // the parent, by its list position
      const int pnb = (int)(rec & 31u);
      int di, dj, dk, I, J, K;
      en.cell = pe.cell + nbr_delta(g, pnb, di, dj, dk);
      en.ori = pe.ori;
      en.id = (int32_t)(lo + r);
      liq = liquid_neighbours(d.solid, g, en.cell);
      const double px = d.gx[pe.id], py = d.gy[pe.id], pz = d.gz[pe.id];
      cell_ijk(g, pe.cell, I, J, K);
      const double ccx = centre_coord(g.x0, g.h, I + di);
      const double ccy = centre_coord(g.y0, g.h, J + dj);
      const double ccz = centre_coord(g.z0, g.h, K + dk);
      double out[4];
      capture_f64(d.omat + 9 * pe.ori, ccx - px, ccy - py, ccz - pz, pe.L, g.h, d.trunc, out);
      gxd = out[0] + px;
      gyd = out[1] + py;
      gzd = out[2] + pz;
      en.L = out[3];
      en.dx = (float)(gxd - ccx);
      en.dy = (float)(gyd - ccy);
      en.dz = (float)(gzd - ccz);
      have_centre = true;
      act[p] = en;
      lstep[p] = (int32_t)step;
      d.gx[en.id] = gxd;
      d.gy[en.id] = gyd;
      d.gz[en.id] = gzd;
      d.gori[en.id] = en.ori;
      d.gcell[en.id] = en.cell;
      d.orient[en.cell] = (uint32_t)en.ori;  // the claim word of last generation becomes the orientation id
    }
    const int cell = en.cell, ori = en.ori, id = en.id;
    const double L = en.L;
    uint32_t con = 0;
    // lower bound of |c'|_1 over the liquid neighbours it does not contain
    float t_lb = INFINITY;
    // cell_is_captured is false for a zero half-diagonal (tested on the bits:
    // an integer compare instead of one on the narrow FP64 pipe); such an
    // entry is looked at again next step
    if (liq && (__double_as_longlong(L) << 1) == 0) t_lb = -INFINITY;
    if (liq && (__double_as_longlong(L) << 1) != 0) {
      int I, J, K;
      cell_ijk(g, cell, I, J, K);
      const float dxf = en.dx, dyf = en.dy, dzf = en.dz;
      const float errg = 4.76837158203125e-07f * (d.h32 + fabsf(dxf) + fabsf(dyf) + fabsf(dzf)) + d.coord_err;
      const float L32 = (float)L;
      float m32[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) m32[q] = __ldg(d.omat32 + 9 * ori + q);
      uint32_t bits = liq;
      while (bits) {
        const int nb = __ffs(bits) - 1;
        bits &= bits - 1;
        int di, dj, dk;
        nbr_offset(nb, di, dj, dk);
        ++tests;
        float lower;
        int f = captured_f32_lb(m32, (float)di * d.h32 - dxf, (float)dj * d.h32 - dyf, (float)dk * d.h32 - dzf, errg,
                                L32, &lower);
        if (f < 0) {
          ++tests64;
          if (!have_centre) {
            gxd = d.gx[id];
            gyd = d.gy[id];
            gzd = d.gz[id];
            have_centre = true;
          }
          const double ccx = centre_coord(g.x0, g.h, I + di);
          const double ccy = centre_coord(g.y0, g.h, J + dj);
          const double ccz = centre_coord(g.z0, g.h, K + dk);
          f = is_captured_f64(d.omat + 9 * ori, ccx - gxd, ccy - gyd, ccz - gzd, L) ? 1 : 0;
        }
        con |= (f ? 1u : 0u) << nb;
        if (!f) t_lb = fminf(t_lb, lower);
      }
      const uint32_t mine = claim_word(par, (uint32_t)r);
      bits = con;
      while (bits) {
        const int nb = __ffs(bits) - 1;
        bits &= bits - 1;
        int di, dj, dk;
        const int nc = cell + nbr_delta(g, nb, di, dj, dk);
        atomicMin(d.orient + nc, mine);
        atomicOr(d.claimed + (nc >> 5), 1u << (nc & 31));
      }
    }
    // growth is uniform: the entry can contain one of the neighbours left
    // only once the run's cumulative growth reaches this key
    d.key[cur][p] = t_lb == -INFINITY ? gf : wake_key(t_lb, L, grown, gf);
    d.liq[r] = liq;
    d.con[r] = con;
    d.cellr[r] = cell;
  }
  }
  *stat_tests += tests;
  *stat_tests64 += tests64;
  if (dec) flush_zero_buffer(d, zpar);
}

// ---------------------------------------------------------------------------
// Resolve: captures, deactivation, child records, liquid counts.
// ---------------------------------------------------------------------------
// Mark of one rank: the captured neighbours (final claim is its own) and
// whether it stays active, as captures | survives << 31.
__device__ __forceinline__ uint32_t mark_rank(const PlainDevice &d, long long r, unsigned par) {
  const Grid &g = d.grid;
  const uint32_t lm = d.liq[r], cm = d.con[r];
  uint32_t cap = 0, surv = 0;
  if (lm) {
    const int cell = d.cellr[r];
    const uint32_t mine = claim_word(par, (uint32_t)r);
    // a liquid neighbour this envelope does not contain and nobody claimed
    // keeps it active without a look at the cell field
    const uint32_t other = lm & ~cm;
    const uint32_t clm = neighbour_bits(d.claimed, g, cell);
    surv = (other & ~clm) ? 1u : 0u;
    // claim words are read for contained cells, and for claimed ones while
    // survival is still open
    const uint32_t need = cm | (surv ? 0u : (other & clm));
#pragma unroll
    for (int nb = 0; nb < 26; ++nb) {
      if (!((need >> nb) & 1u)) continue;
      int di, dj, dk;
      const uint32_t s = d.orient[cell + nbr_delta(g, nb, di, dj, dk)];
      if ((cm >> nb) & 1u) {
        cap |= (s == mine ? 1u : 0u) << nb;
      } else if (s == kLiquid || (s & kRankMask) > (uint32_t)r) {
        surv = 1;
      }
    }
  }
  return cap | (surv << 31);
}

// Marking pass for large generations: dynamic chunks of ranks, as in the
// claim phase, and write each rank's mark over its containment
// mask; a grid barrier then opens the scan.
__device__ __noinline__ void mark_phase(const PlainDevice &d, long long n, unsigned par) {
  RankSched sched(n, &d.ctrl->mark_next, &d.ctrl->error, d.warp_sched);
  const int first = sched.first(), stride = sched.stride();
  long long b, e;
  while (sched.next(b, e))
    for (long long r = b + first; r < e; r += stride) d.con[r] = mark_rank(d, r, par);
}

// Whether a generation of n ranks is marked inside the resolve pass (at most
// one rank per thread of the team: the barrier a separate pass needs would
// cost more than the imbalance of static chunks).
__device__ __forceinline__ bool mark_in_resolve(const PlainDevice &d, long long n) {
  return n <= (long long)d.mark_split * t_nb;
}

// Each block marks its contiguous chunk of ranks (the claim words are final
// after the claim phase's barrier), then one look-back per block over the
// chunk's marks gives new envelope ids (walk order) and child records; an
// entry that does not survive its turn becomes a tombstone, one that does
// gets its cell word (its position and the liquid neighbours it saw in the
// claim phase). Marking reads
// only claim words, the claimed bitmap, its own ranks' masks and cells, none
// of which another block's resolve writes, so no barrier separates the two
// passes. Every captured cell turns solid for the next generation (whose
// claim phase takes it off the liquid counts around it). The zero events
// that the claim phase found (parity zdec, -1: none; zgen0: of generation
// 0's captures) are decided here, and the list of parity zreset is emptied
// for the next claim phase. The last block publishes the generation's
// capture and survivor counts, which every block reads after the barrier.
__device__ __noinline__ bool resolve_phase(const PlainDevice &d, int cur, long long n, long long step, unsigned par,
                                           const GenList &list, int zdec, bool zgen0, int zreset,
                                           unsigned long long *smem,
                                           unsigned *gone_now, unsigned *gone_next) {
  PlainCtrl *c = d.ctrl;
  if (zdec >= 0) zero_decisions(d, cur, zdec, zgen0, step, gone_now, gone_next);
  if (t_b == 0 && threadIdx.x == 0) c->zn[zreset] = 0ull;  // last read in the previous resolve phase
  long long b, e;
  block_chunk(n, b, e);
  unsigned long long acc = 0;
  const bool marking = mark_in_resolve(d, n);
  // kMarkBatch ranks per thread marked before any mark is stored: a store
  // through one array could alias the next rank's loads, so storing each
  // mark at once would run the ranks' load chains one after another
  for (long long r0 = b + threadIdx.x; r0 < e; r0 += (long long)kBlock * kMarkBatch) {
    uint32_t word[kMarkBatch];
#pragma unroll
    for (int j = 0; j < kMarkBatch; ++j) {
      const long long r = r0 + (long long)j * kBlock;
      // marked here, or by mark_phase before the last barrier
      word[j] = r < e ? (marking ? mark_rank(d, r, par) : d.con[r]) : 0u;
    }
#pragma unroll
    for (int j = 0; j < kMarkBatch; ++j) {
      const long long r = r0 + (long long)j * kBlock;
      if (r >= e) continue;
      if (marking) d.con[r] = word[j];  // read back below by the same thread
      acc += ((unsigned long long)__popc(word[j] & 0x03ffffffu) << 32) | (word[j] >> 31);
    }
  }
  unsigned long long agg;
  block_exclusive_scan(acc, smem, &agg);
  const unsigned long long pre = block_prefix(d.scanB, agg, smem, c);
  if (pre == ~0ull) return false;
  const Grid &g = d.grid;
  unsigned long long run = pre;
  for (long long r0 = b; r0 < e; r0 += kBlock) {
    const long long r = r0 + threadIdx.x;
    const uint32_t word = r < e ? d.con[r] : 0u;
    const uint32_t cap = word & 0x03ffffffu, surv = word >> 31;
    // what the rank's entry needs, loaded before the scan (independent of it)
    const long long p = r < e ? list.at(r) : 0;
    const int cell = r < e ? d.cellr[r] : 0;
    const uint32_t lq = r < e ? d.liq[r] : 0u;
    unsigned long long tot;
    const unsigned long long ex = block_exclusive_scan(((unsigned long long)__popc(cap) << 32) | surv, smem, &tot);
    if (r < e) {
      if (!surv) {
        tombstone(d, cur, p, cell);  // deactivated at its turn
      } else {
        // its cell word: position and the liquid neighbours it saw in the
        // claim phase (this generation's captures come off in the next one)
        d.cellw[cell] = ((uint32_t)p << 5) | (uint32_t)__popc(lq);
      }
      long long slot = (long long)((run + ex) >> 32);  // rank of the first child in the next generation
      uint32_t bits = cap;
      while (bits) {
        const int nb = __ffs(bits) - 1;
        bits &= bits - 1;
        d.child[slot++] = ((uint32_t)p << 5) | (uint32_t)nb;  // parent's list position
        int di, dj, dk;
        set_solid(d.solid, cell + nbr_delta(g, nb, di, dj, dk));  // solid for the next generation
      }
    }
    run += tot;
  }
  if (t_b == t_nb - 1 && threadIdx.x == 0) {
    const unsigned long long total = pre + agg;
    c->gen_n = (long long)(total >> 32);
    c->gen_surv = (long long)(total & 0xffffffffull);
  }
  return true;
}

// Whole CA steps of one realm by the current team, until it is solid, its
// termination time, or step_limit.
//
// The realm's state (step, time, counts, list length, ...) is the same in
// every thread; it lives in shared memory, written by thread 0 right after
// the barriers at which its inputs become final and read by all after a
// block barrier, so that the registers stay free for the phases.
struct RealmState {
  long long step, n_act, a_len, n_orient, grain, liquid;
  double time, dt, grown, t_end;
  unsigned long long compactions;
  int cur, done;
  // the step in progress
  double da, dn, dv, grown_s;
  int all;
  long long nucs, n, lo, processed, gen_end, caps_all, died;
  unsigned gen;
  GenList list;  // this generation's list positions
  // thread 0's busy time per kind of work, added to the control block once
  // per launch; block 0's phase clock
  unsigned long long claim_busy, resolve_busy, nuc_busy, wake_busy, compact_busy, t_mark, t_work, w_mark;
};

__device__ void run_realm(const PlainDevice &d, long long step_limit, unsigned long long *smem) {
  // block 0's phase clock and step counters (its thread 0 only), added to
  // the control block once per launch
  enum { kNuc, kClaim, kClaim0, kResolve, kClaimMax, kResolveMax, kGens, kGrown, kProc, kCaps, kNucs, kScanned, kZero,
         kWalked, kNucMax, kClk };
  __shared__ unsigned long long s_clk[kClk];
  // this block's tile of sites when they are tiled (cell -1: removed, or no site)
  __shared__ int s_cell[kBlock];
  __shared__ double s_dtc[kBlock];
  __shared__ RealmState S;
  PlainCtrl *c = d.ctrl;
  unsigned long long tests = 0, tests64 = 0, live = 0, dec = 0, moved = 0;
  unsigned gone_now = 0, gone_next = 0;  // list departures this thread decided, added once per phase
  const bool timer = t_b == 0 && threadIdx.x == 0;
  if (threadIdx.x == 0) {
    S.step = ld_volatile(&c->step);
    S.time = ld_volatile(&c->time);
    S.dt = ld_volatile(&c->dt);
    S.n_act = ld_volatile(&c->n_active);
    S.a_len = ld_volatile(&c->a_len);
    S.n_orient = ld_volatile(&c->n_orient);
    S.grain = ld_volatile(&c->next_grain);
    S.liquid = ld_volatile(&c->liquid);
    S.compactions = ld_volatile(&c->compactions);
    S.grown = ld_volatile(&c->grown);
    S.cur = ld_volatile(&c->cur_list);
    S.done = ld_volatile(&c->done) != 0;
    S.t_end = (d.t_stop > 0 && d.t_stop < d.final_time) ? d.t_stop : d.final_time;
    S.claim_busy = S.resolve_busy = S.nuc_busy = S.wake_busy = S.compact_busy = 0ull;
    S.t_mark = now_ns();
  }
  if (site_tiles(d)) {
    const long long i = (long long)t_b * kBlock + threadIdx.x;
    const bool on = i < d.nsites && d.site_live[i] != 0;
    s_cell[threadIdx.x] = on ? d.site_cell[i] : -1;
    s_dtc[threadIdx.x] = on ? d.site_dtc[i] : 0.0;
  }
  if (timer)
    for (int k = 0; k < kClk; ++k) s_clk[k] = 0ull;
  __syncthreads();
  bool ok = true;
  while (!S.done && S.time < S.t_end && S.step < step_limit) {
    // the list is compacted once it is mostly tombstones
    if (S.a_len > 2 * S.n_act + d.compact_slack) {
      const unsigned long long tc = threadIdx.x == 0 ? now_ns() : 0ull;
      if (!(ok = compact_phase(d, S.cur, S.a_len, (unsigned)(S.compactions & 1ull), smem, &moved))) break;
      if (threadIdx.x == 0) S.compact_busy += now_ns() - tc;
      if (!(ok = grid_barrier(c))) break;
      if (threadIdx.x == 0) {
        S.cur ^= 1;
        S.a_len = ld_volatile(&c->compact_len);
        ++S.compactions;
      }
      __syncthreads();
    }
    // --- calculate_time_step (CellularAutomataManager_3D.cpp:441-511) ---
    if (threadIdx.x == 0) {
      double vel;
      step_rates(d, S.time, vel, S.da, S.dn);
      // growth of every envelope this step (when there is one); the wake
      // scan compares the keys with the cumulative growth
      S.dv = S.da * vel;
      S.grown_s = S.grown + S.dv;
      S.all = S.step % kWakeAll == 0;
      if (t_b == 0) d.dvh[S.step & (kDvRing - 1)] = S.dv;
    }
    __syncthreads();
    // the wake scan first: every block publishes its part of the scan at
    // once, while only the blocks holding sites take part in nucleation's.
    // A nucleus may turn a sleeping entry dead after the scan passed it,
    // which the scan's rule (dead or sleeping: not woken) already gave.
    const unsigned long long tn0 = threadIdx.x == 0 ? now_ns() : 0ull;
    if (!(ok = wake_scan(d, S.cur, S.a_len, S.step, S.grown_s, S.all != 0, smem))) break;
    const unsigned long long tn1 = threadIdx.x == 0 ? now_ns() : 0ull;
    if (!(ok = nucleation_phase(d, S.cur, S.time, S.step, S.a_len, S.n_orient, S.grain, S.grown_s, S.all != 0, s_cell,
                                s_dtc, smem, &live, &dec, &gone_now)))
      break;
    flush_departures(c, S.step, gone_now, gone_next);
    if (threadIdx.x == 0) {
      const unsigned long long tn2 = now_ns();
      S.wake_busy += tn1 - tn0;
      S.nuc_busy += tn2 - tn1;
      if (d.phase_detail && tn2 - tn0 > ld_volatile(&c->phase_max_scratch[2]))
        atomicMax(&c->phase_max_scratch[2], tn2 - tn0);
    }
    if (!(ok = grid_barrier(c))) break;
    if (threadIdx.x == 0) {
      const long long nA = ld_volatile(&c->n_active_nuc[S.step & 1]);
      const long long nucs = nA - S.a_len;  // nuclei of this step
      const long long nw = ld_volatile(&c->n_woken[S.step & 1]);
      if (timer) {
        const unsigned long long t_now = now_ns();
        s_clk[kNuc] += t_now - S.t_mark;
        S.t_mark = t_now;
        // the slot of step + 2 (last read at the end of step - 1)
        c->deaths[(S.step + 2) % 3] = 0;
        if (d.phase_detail) {
          s_clk[kNucMax] += ld_volatile(&c->phase_max_scratch[2]);
          c->phase_max_scratch[2] = 0ull;
        }
        s_clk[kNucs] += (unsigned long long)nucs;
        s_clk[kScanned] += (unsigned long long)S.a_len;
        s_clk[kGrown] += (unsigned long long)(nw + nucs);
        s_clk[kWalked] += (unsigned long long)(S.n_act + nucs);
      }
      S.dt = S.n_act + nucs > 0 ? S.da : S.dn;
      S.grown = S.grown_s;
      S.n_orient += nucs;
      S.grain += nucs;
      S.liquid -= nucs;
      // --- single_integration_step (CellularAutomataManager_3D.cpp:516-669) ---
      S.nucs = nucs;
      S.n = nw + nucs;
      S.lo = 0;
      S.processed = 0;
      S.gen_end = nA;
      S.caps_all = 0;
      S.died = 0;
      S.gen = 0;
      S.list = GenList{d.wlist, nw, S.a_len};
    }
    __syncthreads();
    while (S.n > 0) {
      if (threadIdx.x == 0) {
        S.processed += S.n;
        S.t_work = now_ns();
      }
      // (and the liquid counts around the previous generation's captures)
      claim_phase(d, S.cur, S.gen ? 1 : 0, S.lo, S.n, S.gen & 1u, S.list, S.step, S.grown, S.gen > 0,
                  (int)((S.gen - 1) & 1u), &tests, &tests64, &dec);
      __syncthreads();
      if (threadIdx.x == 0) {
        const unsigned long long w = now_ns() - S.t_work;
        S.claim_busy += w;
        if (d.phase_detail && w > ld_volatile(&c->phase_max_scratch[0])) atomicMax(&c->phase_max_scratch[0], w);
      }
      if (!(ok = grid_barrier(c))) break;
      if (threadIdx.x == 0) {
        if (timer) {
          const unsigned long long t_now = now_ns();
          s_clk[kClaim] += t_now - S.t_mark;
          if (S.gen == 0) s_clk[kClaim0] += t_now - S.t_mark;
          if (S.gen > 0) s_clk[kZero] += ld_volatile(&c->zn[(S.gen - 1) & 1u]);  // reset in this generation's resolve
          S.t_mark = t_now;
          if (d.phase_detail) {
            s_clk[kClaimMax] += ld_volatile(&c->phase_max_scratch[0]);
            c->phase_max_scratch[0] = 0ull;
          }
          c->claim_next = 0ull;  // the next claim phase is two barriers away
        }
        S.t_work = now_ns();
        S.w_mark = 0;  // busy time of a separate marking pass
      }
      __syncthreads();
      if (!mark_in_resolve(d, S.n)) {
        mark_phase(d, S.n, S.gen & 1u);
        __syncthreads();
        if (threadIdx.x == 0) S.w_mark = now_ns() - S.t_work;
        if (!(ok = grid_barrier(c))) break;
        if (timer) c->mark_next = 0ull;  // the next marking pass is two barriers away
        if (threadIdx.x == 0) S.t_work = now_ns();
        __syncthreads();
      }
      if (!(ok = resolve_phase(d, S.cur, S.n, S.step, S.gen & 1u, S.list, S.gen > 0 ? (int)((S.gen - 1) & 1u) : -1,
                               S.gen == 1, (int)(S.gen & 1u), smem, &gone_now, &gone_next)))
        break;
      flush_departures(c, S.step, gone_now, gone_next);
      if (threadIdx.x == 0) {
        const unsigned long long w = now_ns() - S.t_work + S.w_mark;
        S.resolve_busy += w;
        if (d.phase_detail && w > ld_volatile(&c->phase_max_scratch[1])) atomicMax(&c->phase_max_scratch[1], w);
      }
      if (!(ok = grid_barrier(c))) break;
      if (threadIdx.x == 0) {
        if (timer) {
          const unsigned long long t_now = now_ns();
          s_clk[kResolve] += t_now - S.t_mark;
          S.t_mark = t_now;
          if (d.phase_detail) {
            s_clk[kResolveMax] += ld_volatile(&c->phase_max_scratch[1]);
            c->phase_max_scratch[1] = 0ull;
          }
        }
        const long long caps = ld_volatile(&c->gen_n);  // envelopes of the next generation
        S.died += S.n - ld_volatile(&c->gen_surv);      // deactivated at their turn
        S.lo = S.grain;  // their ids follow on
        S.grain += caps;
        S.liquid -= caps;
        S.caps_all += caps;
        if (timer) s_clk[kCaps] += (unsigned long long)caps;
        S.n = caps;
        ++S.gen;
        S.list = GenList{nullptr, 0, S.gen_end};  // appended to the list after the previous generation
        S.gen_end += caps;
      }
      __syncthreads();
    }
    if (!ok) break;
    // step end (CellularAutomataManager_3D.cpp:653-659), from counts final
    // at the last barrier
    if (threadIdx.x == 0) {
      S.n_act = S.n_act + S.nucs + S.caps_all - S.died - (long long)ld_volatile(&c->deaths[S.step % 3]);
      S.a_len = S.gen_end;
      S.time = S.time + S.dt;
      ++S.step;
      S.done = S.liquid == 0;
      if (timer) {
        s_clk[kGens] += S.gen;
        s_clk[kProc] += (unsigned long long)S.processed;
      }
    }
    __syncthreads();
  }
  if (ok && timer) {
    // the realm's state for the host and the next launch
    c->step = S.step;
    c->time = S.time;
    c->dt = S.dt;
    c->n_active = S.n_act;
    c->a_len = S.a_len;
    c->grown = S.grown;
    c->compactions = S.compactions;
    c->n_orient = S.n_orient;
    c->next_grain = S.grain;
    c->liquid = S.liquid;
    c->cur_list = S.cur;
    c->done = S.done ? 1 : 0;
    c->keys_scanned += s_clk[kScanned];
    c->zero_events += s_clk[kZero];
    c->ref_walked += s_clk[kWalked];
    c->ns_nuc_work_max += s_clk[kNucMax];
    c->ns_nucleation += s_clk[kNuc];
    c->ns_claim += s_clk[kClaim];
    c->ns_claim_gen0 += s_clk[kClaim0];
    c->ns_resolve += s_clk[kResolve];
    c->ns_claim_work_max += s_clk[kClaimMax];
    c->ns_resolve_work_max += s_clk[kResolveMax];
    c->gens += s_clk[kGens];
    c->active_grown += s_clk[kGrown];
    c->grains_processed += s_clk[kProc];
    c->captures += s_clk[kCaps];
    c->nucleations += s_clk[kNucs];
    c->ns_step_end += now_ns() - S.t_mark;
  }
  // statistics: one atomic per warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    tests += __shfl_down_sync(0xffffffffu, tests, o);
    tests64 += __shfl_down_sync(0xffffffffu, tests64, o);
    live += __shfl_down_sync(0xffffffffu, live, o);
    dec += __shfl_down_sync(0xffffffffu, dec, o);
    moved += __shfl_down_sync(0xffffffffu, moved, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (threadIdx.x == 0) {
      if (S.claim_busy) atomicAdd(&c->ns_claim_work_sum, S.claim_busy);
      if (S.resolve_busy) atomicAdd(&c->ns_resolve_work_sum, S.resolve_busy);
      if (S.nuc_busy) atomicAdd(&c->ns_nuc_work_sum, S.nuc_busy);
      if (S.wake_busy) atomicAdd(&c->ns_wake_work_sum, S.wake_busy);
      if (S.compact_busy) atomicAdd(&c->ns_compact_work_sum, S.compact_busy);
    }
    if (tests) atomicAdd(&c->tests, tests);
    if (tests64) atomicAdd(&c->tests64, tests64);
    if (live) atomicAdd(&c->sites_scanned, live);
    if (dec) atomicAdd(&c->decrements, dec);
    if (moved) atomicAdd(&c->compacted, moved);
  }
}

__global__ void __launch_bounds__(kBlock, kMinBlocks) plain_persistent_kernel(PlainDevice d, long long step_limit) {
  __shared__ unsigned long long smem[kWarps + 2];
  // the descriptor in shared memory: the phases take it by reference, and a
  // reference to the kernel parameter would make every thread keep a copy of
  // it on its stack (local memory)
  __shared__ PlainDevice sd;
  if (threadIdx.x == 0) {
    t_nb = gridDim.x;
    t_b = blockIdx.x;
  }
  const int *src = (const int *)&d;
  int *dst = (int *)&sd;
  for (int w = threadIdx.x; w < (int)(sizeof(PlainDevice) / 4); w += blockDim.x) dst[w] = src[w];
  __syncthreads();
  run_realm(sd, step_limit, smem);
}

// One bitmap word (32 cells) of the initial field: cells past the grid count
// as solid.
__device__ __forceinline__ void init_field_word(uint32_t *orient, uint32_t *solid, uint32_t *claimed, uint32_t *cellw,
                                                const Grid &g, long long ncells, long long w) {
  uint32_t bits = 0;
  for (int b = 0; b < 32; ++b) {
    const long long i = w * 32 + b;
    bool ghost = true;
    if (i < ncells) {
      int I, J, K;
      cell_ijk(g, i, I, J, K);
      ghost = I == 0 || J == 0 || K == 0 || I == g.nxg - 1 || J == g.nyg - 1 || K == g.nzg - 1;
      orient[i] = ghost ? 0u : kLiquid;
      cellw[i] = kNoEntry;
    }
    bits |= (ghost ? 1u : 0u) << b;
  }
  solid[w] = bits;
  claimed[w] = 0u;
}

__global__ void init_field_kernel(uint32_t *orient, uint32_t *solid, uint32_t *claimed, uint32_t *cellw, Grid g,
                                  long long ncells) {
  const long long nwords = solid_words(ncells);
  for (long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += (long long)gridDim.x * blockDim.x)
    init_field_word(orient, solid, claimed, cellw, g, ncells, w);
}

// ---------------------------------------------------------------------------
// Batched launch: many independent realms in one cooperative launch. The
// grid is cut into teams of consecutive blocks (plan.blk gives each block
// its team and rank, plan.tsize each team's size); teams of one class share
// a queue over the class's slice of `order`. The first block of a team pulls
// the next queue position and publishes the realm in the team's slot (by
// round parity); after a team barrier every block of the team runs that
// realm with run_realm, the team standing in for the grid (its barriers
// count the team's arrivals on the realm's own control words). A realm's
// result does not depend on how many blocks run it, so team sizes, classes
// and queue order are free to tune.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock, kMinBlocks)
    plain_batched_kernel(const PlainDevice *insts, const int *order, int ninst, BatchPlanDev plan, unsigned *queues,
                         BatchTeam *teams, int *error, long long step_limit) {
  __shared__ unsigned long long smem[kWarps + 2];
  __shared__ PlainDevice sd;  // the descriptor of the realm this team runs
  __shared__ int s_idx;
  const int2 bt = plan.blk[blockIdx.x];
  const int team = bt.x;
  const int cls = plan.tclass[team];
  const int2 range = plan.crange[cls];  // (first position in order, realms) of the class
  if (threadIdx.x == 0) {
    t_nb = plan.tsize[team];
    t_b = bt.y;
  }
  __syncthreads();
  BatchTeam *tw = teams + team;
  for (int round = 0;; ++round) {
    // the slot written here was last read in round - 2, before every block
    // of the team arrived at the barrier of round - 1
    if (t_b == 0 && threadIdx.x == 0) {
      const unsigned q = atomicAdd(queues + cls, 1u);
      tw->slot[round & 1] = q < (unsigned)range.y ? order[range.x + (int)q] : -1;
    }
    if (!team_barrier(&tw->count, &tw->gen, error)) break;
    if (threadIdx.x == 0) s_idx = ld_volatile(&tw->slot[round & 1]);
    __syncthreads();
    const int idx = s_idx;
    if (idx < 0 || idx >= ninst) break;
    const int *src = (const int *)(insts + idx);
    int *dst = (int *)&sd;
    for (int w = threadIdx.x; w < (int)(sizeof(PlainDevice) / 4); w += blockDim.x) dst[w] = src[w];
    __syncthreads();
    run_realm(sd, step_limit, smem);
    __syncthreads();  // sd and s_idx are rewritten in the next round
  }
}

// Every realm of a batch back to its state right after initialize (site
// flags, look-back words, control block, field), and the queue and team
// words to zero. blockIdx.y is the realm.
__global__ void batch_reset_kernel(const PlainDevice *insts, int ninst, unsigned *queues, int nclasses,
                                   BatchTeam *teams, int nteams, int *error) {
  const int r = blockIdx.y;
  const PlainDevice &d = insts[r];
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (tid == 0) {
    PlainCtrl c{};
    c.liquid = d.gcap;  // every interior cell
    *d.ctrl = c;
  }
  if (r == 0) {
    if (tid == 0) *error = 0;
    for (long long q = tid; q < nclasses; q += stride) queues[q] = 0u;
    for (long long t = tid; t < nteams; t += stride) teams[t] = BatchTeam{0u, 0u, {-1, -1}};
  }
  for (long long i = tid; i < d.nsites; i += stride) d.site_live[i] = 1;
  for (long long i = tid; i < kStatusWords; i += stride) {
    d.scanA[i] = 0ull;
    d.scanA[kStatusWords + i] = 0ull;
    d.scanB[i] = 0ull;
    d.scanC[i] = 0ull;
    d.scanC[kStatusWords + i] = 0ull;
    d.scanD[i] = 0ull;
    d.scanD[kStatusWords + i] = 0ull;
  }
  const long long nwords = solid_words(d.ncells);
  for (long long w = tid; w < nwords; w += stride)
    init_field_word(d.orient, d.solid, d.claimed, d.cellw, d.grid, d.ncells, w);
}

// out[r] = realm r's control block.
__global__ void batch_gather_kernel(const PlainDevice *insts, int ninst, PlainCtrl *out) {
  const int r = blockIdx.x;
  if (r >= ninst) return;
  const unsigned *src = (const unsigned *)insts[r].ctrl;
  unsigned *dst = (unsigned *)(out + r);
  for (int w = threadIdx.x; w < (int)(sizeof(PlainCtrl) / 4); w += blockDim.x) dst[w] = src[w];
}

__global__ void grain_field_init_kernel(int32_t *out, const uint32_t *orient, Grid g, long long ncells) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < ncells; i += (long long)gridDim.x * blockDim.x) {
    int I, J, K;
    cell_ijk(g, i, I, J, K);
    const bool ghost = I == 0 || J == 0 || K == 0 || I == g.nxg - 1 || J == g.nyg - 1 || K == g.nzg - 1;
    out[i] = ghost ? 0 : -1;
  }
}

__global__ void grain_field_scatter_kernel(int32_t *out, const int32_t *gcell, long long ngrains) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < ngrains; i += (long long)gridDim.x * blockDim.x)
    out[gcell[i]] = (int32_t)i;
}

// One (envelope, cell) pair per thread: the FP64 containment test, the
// production decision (FP32 pre-test, FP64 when undecided) and, when
// captured, the decentred new envelope.
__global__ void envelope_eval_kernel(long long n, const double *l2g, const double *gc, const double *len, double h,
                                     const double *trunc, int32_t *cap64, int32_t *capfast, double *info) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double *m = l2g + 9 * i;
    const double gx = gc[3 * i], gy = gc[3 * i + 1], gz = gc[3 * i + 2], L = len[i];
    const bool c64 = is_captured_f64(m, gx, gy, gz, L);
    float m32[9];
    for (int q = 0; q < 9; ++q) m32[q] = (float)m[q];
    const float fx = (float)gx, fy = (float)gy, fz = (float)gz;
    const float err = 5.9604645e-08f * (fabsf(fx) + fabsf(fy) + fabsf(fz));  // conversion rounding of gc
    int f = L == 0 ? 0 : captured_f32(m32, fx, fy, fz, err, (float)L);
    if (f < 0) f = c64 ? 1 : 0;
    cap64[i] = c64 ? 1 : 0;
    capfast[i] = f;
    double out[4] = {0.0, 0.0, 0.0, 0.0};
    if (c64) capture_f64(m, gx, gy, gz, L, h, trunc[i], out);
    for (int q = 0; q < 4; ++q) info[4 * i + q] = out[q];
  }
}

// Set-up of the no-allocation entry point: clear the control block and the
// look-back words, mark every site live, round the orientation matrices to float.
// `bad` (preset to all ones) receives the smallest index of a site whose cell
// is not an interior cell or does not follow the previous site's cell; the
// host reads it before any kernel indexes the field with a site cell.
__global__ void noalloc_setup_kernel(PlainDevice d, long long liquid, unsigned long long *bad) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  if (tid == 0) {
    PlainCtrl c{};
    c.liquid = liquid;
    *d.ctrl = c;
  }
  const Grid g = d.grid;
  for (long long i = tid; i < d.nsites; i += stride) {
    d.site_live[i] = 1;
    const long long c = d.site_cell[i];
    bool ok = c >= 0 && c < d.ncells && (i == 0 || d.site_cell[i - 1] < c);
    if (ok) {
      const long long k = c / g.nxyg, r = c - k * g.nxyg, j = r / g.nxg, ii = r - j * g.nxg;
      ok = ii >= 1 && ii <= g.nx && j >= 1 && j <= g.ny && k >= 1 && k <= g.nz;
    }
    if (!ok) atomicMin(bad, (unsigned long long)i);
  }
  float *m32 = const_cast<float *>(d.omat32);
  for (long long i = tid; i < 9 * d.nsites; i += stride) m32[i] = (float)d.omat[i];
  for (long long i = tid; i < kStatusWords; i += stride) {
    d.scanA[i] = 0ull;
    d.scanA[kStatusWords + i] = 0ull;
    d.scanB[i] = 0ull;
    d.scanC[i] = 0ull;
    d.scanC[kStatusWords + i] = 0ull;
    d.scanD[i] = 0ull;
    d.scanD[kStatusWords + i] = 0ull;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Scratch of amca_plain_run_noalloc: one file-scope device array, held by
// every GPU that loads the library until the process exits. The entry point
// carves the envelope table, lists, masks, look-back words and control block
// out of it instead of calling cudaMalloc.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_base[kNoAllocMaxDevices];  // device address of g_noalloc_scratch, per device
bool g_noalloc_ready[kNoAllocMaxDevices];

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of every scratch buffer for a grid of n interior cells and s sites.
struct NoAllocLayout {
  size_t ctrl, check, live, omat32, scanA, gx, gy, gz, gori, gcell, act[2], key[2], lstep[2], late, cellw, wlist,
      zlist[2], dvh, liq, con, cellr, child, solid, claimed, scanB, scanC, scanD, total;
  // n interior cells, s sites, `cells` ghost-inclusive cells; the caller
  // bounds all three (see kNoAllocMaxCells) so that no size below wraps
  NoAllocLayout(long long n, long long s, long long cells) {
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o = align256(o + bytes);
      return at;
    };
    ctrl = take(sizeof(PlainCtrl));
    check = take(sizeof(unsigned long long));
    live = take((size_t)s);
    omat32 = take((size_t)s * 9 * sizeof(float));
    scanA = take((size_t)2 * kStatusWords * 8);
    gx = take((size_t)n * 8);
    gy = take((size_t)n * 8);
    gz = take((size_t)n * 8);
    gori = take((size_t)n * 4);
    gcell = take((size_t)n * 4);
    for (int b = 0; b < 2; ++b) {
      act[b] = take((size_t)n * sizeof(EnvRec));
      key[b] = take((size_t)(n + kKeyTile) * 4);  // the wake scan reads whole tiles
      lstep[b] = take((size_t)n * 4);
      zlist[b] = take((size_t)n * 4);
    }
    late = take((size_t)n * 4);
    wlist = take((size_t)n * 4);
    cellw = take((size_t)cells * 4);
    dvh = take((size_t)kDvRing * 8);
    liq = take((size_t)n * 4);
    cellr = take((size_t)n * 4);
    con = take((size_t)n * 4);
    child = take((size_t)n * 4);
    solid = take((size_t)solid_words(cells) * 4);
    claimed = take((size_t)solid_words(cells) * 4);
    scanB = take((size_t)kStatusWords * 8);
    scanC = take((size_t)2 * kStatusWords * 8);
    scanD = take((size_t)2 * kStatusWords * 8);
    total = o;
  }
};

// Largest grid edge and cell count the entry point considers. The edge bound
// keeps (nx+2)(ny+2)(nz+2) inside 63 bits; the cell bound (the scratch size
// in bytes: every interior cell takes more than a byte of scratch) keeps
// every buffer size of NoAllocLayout far from wrapping. Grids that pass both
// may still be rejected by the scratch size itself.
constexpr long long kNoAllocMaxEdge = 1ll << 20;
constexpr long long kNoAllocMaxCells = (long long)kNoAllocScratchBytes;

int noalloc_fail(char *err, size_t errlen, int code, const char *what, const char *detail) {
  if (err && errlen) snprintf(err, errlen, "amca_plain_run_noalloc: %s%s%s", what, detail ? ": " : "", detail ? detail : "");
  return code;
}

// Puts the caller's current device back on every return path.
struct DeviceRestore {
  int dev = -1;
  DeviceRestore() {
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
  }
  ~DeviceRestore() {
    if (dev >= 0) cudaSetDevice(dev);
  }
};
}  // namespace

}  // namespace amca

extern "C" int amca_plain_run_noalloc(int device, const amca_plain_params *p, const int32_t *site_cell,
                                      const double *site_dtc, int64_t nsites, const double *l2g, int32_t *orient,
                                      int max_steps, void *stream, amca_plain_result *res, char *err,
                                      size_t errlen) {
  using namespace amca;
  if (err && errlen) err[0] = '\0';
  if (!p || !orient || !res || (nsites > 0 && (!site_cell || !site_dtc || !l2g)) || nsites < 0)
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "null pointer or negative site count", nullptr);
  if (p->nx < 1 || p->ny < 1 || p->nz < 1 || !(p->h > 0))
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "grid dimensions and cell size must be positive", nullptr);
  if (device < 0 || device >= kNoAllocMaxDevices)
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "device ordinal out of range", nullptr);
  if (p->nx > kNoAllocMaxEdge || p->ny > kNoAllocMaxEdge || p->nz > kNoAllocMaxEdge)
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "grid too large for the static scratch", "an edge exceeds 2^20 cells");
  const long long n = (long long)p->nx * p->ny * p->nz;  // < 2^60: no overflow
  if (n > kNoAllocMaxCells)
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "grid too large for the static scratch", "too many interior cells");
  if (nsites > n)
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "more sites than interior cells", nullptr);
  const NoAllocLayout lay(n, nsites, (long long)(p->nx + 2) * (p->ny + 2) * (p->nz + 2));
  if (lay.total > kNoAllocScratchBytes) {
    char detail[160];
    snprintf(detail, sizeof detail, "needs %zu bytes of scratch for %lld cells and %lld sites, limit is %zu",
             lay.total, n, (long long)nsites, kNoAllocScratchBytes);
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "grid too large for the static scratch", detail);
  }
  DeviceRestore restore;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "cudaSetDevice", cudaGetErrorString(e));
  {
    // once per device, with that device current: the device address of the
    // static array (its host-side name is only a stand-in)
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ready[device]) {
      void *base = nullptr;
      e = cudaGetSymbolAddress(&base, g_noalloc_scratch);
      if (e != cudaSuccess)
        return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "cudaGetSymbolAddress", cudaGetErrorString(e));
      g_noalloc_base[device] = base;
      g_noalloc_ready[device] = true;
    }
  }
  unsigned char *base = (unsigned char *)g_noalloc_base[device];
  cudaStream_t s = (cudaStream_t)stream;
  PlainDevice d{};
  Grid &g = d.grid;
  g.nx = p->nx;
  g.ny = p->ny;
  g.nz = p->nz;
  g.nxg = p->nx + 2;
  g.nyg = p->ny + 2;
  g.nzg = p->nz + 2;
  g.nxyg = g.nxg * g.nyg;
  g.x0 = p->x0;
  g.y0 = p->y0;
  g.z0 = p->z0;
  g.h = p->h;
  d.T0 = p->T0;
  d.Tm = p->Tm;
  d.Tdot = p->Tdot;
  d.a1 = p->a1;
  d.a2 = p->a2;
  d.a3 = p->a3;
  d.max_dt = p->max_dt;
  d.final_time = p->final_time;
  d.tsf = p->time_step_factor;
  d.trunc = p->trunc_coeff;
  d.h32 = (float)p->h;
  double cmax = 0;
  const double o3[3] = {p->x0, p->y0, p->z0};
  const int n3[3] = {g.nxg, g.nyg, g.nzg};
  for (int a = 0; a < 3; ++a) cmax = fmax(cmax, fabs(o3[a]) + (n3[a] + 1) * p->h);
  d.coord_err = (float)(ldexp(cmax, -49) + 1e-30);
  d.ncells = (int64_t)g.nxyg * g.nzg;
  d.nsites = nsites;
  d.gcap = n;
  d.warp_sched = kWarpSched;
  d.mark_split = kMarkSplit;
  d.dec_warps = kDecWarps;
  d.compact_slack = kCompactSlack;
  d.orient = (uint32_t *)orient;
  d.site_cell = site_cell;
  d.site_dtc = site_dtc;
  d.omat = l2g;
  d.ctrl = (PlainCtrl *)(base + lay.ctrl);
  d.site_live = base + lay.live;
  d.omat32 = (const float *)(base + lay.omat32);
  d.scanA = (unsigned long long *)(base + lay.scanA);
  d.gx = (double *)(base + lay.gx);
  d.gy = (double *)(base + lay.gy);
  d.gz = (double *)(base + lay.gz);
  d.gori = (int32_t *)(base + lay.gori);
  d.gcell = (int32_t *)(base + lay.gcell);
  for (int b = 0; b < 2; ++b) {
    d.act[b] = (EnvRec *)(base + lay.act[b]);
    d.key[b] = (float *)(base + lay.key[b]);
    d.lstep[b] = (int32_t *)(base + lay.lstep[b]);
    d.zlist[b] = (int32_t *)(base + lay.zlist[b]);
  }
  d.late = (int32_t *)(base + lay.late);
  d.wlist = (int32_t *)(base + lay.wlist);
  d.cellw = (uint32_t *)(base + lay.cellw);
  d.dvh = (double *)(base + lay.dvh);
  d.liq = (uint32_t *)(base + lay.liq);
  d.cellr = (int32_t *)(base + lay.cellr);
  d.con = (uint32_t *)(base + lay.con);
  d.child = (uint32_t *)(base + lay.child);
  d.solid = (uint32_t *)(base + lay.solid);
  d.claimed = (uint32_t *)(base + lay.claimed);
  d.scanB = (unsigned long long *)(base + lay.scanB);
  d.scanC = (unsigned long long *)(base + lay.scanC);
  d.scanD = (unsigned long long *)(base + lay.scanD);
  // everything that must start at zero is cleared here: the array keeps the
  // previous call's contents
  unsigned long long *check = (unsigned long long *)(base + lay.check);
  if ((e = cudaMemsetAsync(check, 0xff, sizeof *check, s)) != cudaSuccess)
    return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "set-up", cudaGetErrorString(e));
  noalloc_setup_kernel<<<256, 256, 0, s>>>(d, n, check);
  if ((e = cudaGetLastError()) != cudaSuccess)
    return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "set-up launch", cudaGetErrorString(e));
  unsigned long long first_bad = 0;
  if ((e = cudaMemcpyAsync(&first_bad, check, sizeof first_bad, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "checking the site list", cudaGetErrorString(e));
  if (first_bad != ~0ull) {
    char detail[160];
    snprintf(detail, sizeof detail, "site %llu: its cell is not an interior cell of the grid or does not follow "
             "the previous site's cell", first_bad);
    return noalloc_fail(err, errlen, AMCA_ERR_ARG, "bad site list", detail);
  }
  if ((e = plain_init_field(d, s)) != cudaSuccess)
    return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "field launch", cudaGetErrorString(e));
  const int blocks = plain_persistent_grid(device);
  if (blocks <= 0) return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "no co-resident blocks", nullptr);
  if ((e = plain_run_steps(d, max_steps < 0 ? (1ll << 60) : (long long)max_steps, blocks, s)) != cudaSuccess)
    return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "step launch", cudaGetErrorString(e));
  PlainCtrl c;
  if ((e = cudaMemcpyAsync(&c, d.ctrl, sizeof c, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return noalloc_fail(err, errlen, AMCA_ERR_CUDA, "reading the control block", cudaGetErrorString(e));
  if (c.error) return noalloc_fail(err, errlen, AMCA_ERR_DEVICE, "a bounded device wait ran out", nullptr);
  res->steps = c.step;
  res->time = c.time;
  res->grains = c.next_grain;
  res->orientations = c.n_orient;
  res->liquid_cells = c.liquid;
  res->done = c.done;
  return AMCA_OK;
}

namespace amca {

cudaError_t plain_envelope_eval(long long n, const double *l2g, const double *gc, const double *len, double h,
                                const double *trunc, int32_t *cap64, int32_t *capfast, double *info, cudaStream_t s) {
  envelope_eval_kernel<<<256, 128, 0, s>>>(n, l2g, gc, len, h, trunc, cap64, capfast, info);
  return cudaGetLastError();
}

namespace {
// Self-test of the bounded barrier: `parties` arrivals expected from the
// launch's blocks (parties > blocks: one never comes and every wait must run
// out), with the error word preset to `preset`. verdict[b] = what block b's
// barrier returned.
__global__ void barrier_selftest_kernel(unsigned long long *word, int *error, int parties, unsigned long long wait_ns,
                                        int *verdict) {
  if (threadIdx.x == 0) {
    t_nb = parties;
    t_b = blockIdx.x;
  }
  __syncthreads();
  const bool ok = team_barrier((unsigned *)word, (unsigned *)word + 1, error, wait_ns);
  if (threadIdx.x == 0) verdict[blockIdx.x] = ok ? 1 : 0;
}
}  // namespace

cudaError_t plain_barrier_selftest(int blocks, int parties, long long wait_ns, int preset, int *error_out,
                                   int *verdicts) {
  unsigned long long *word = nullptr;
  int *dev = nullptr;
  cudaError_t e = cudaMalloc(&word, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&dev, sizeof(int) * (size_t)(blocks + 1));
  if (e == cudaSuccess) e = cudaMemset(word, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(dev, 0, sizeof(int) * (size_t)(blocks + 1));
  if (e == cudaSuccess) e = cudaMemcpy(dev, &preset, sizeof(int), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    int *error = dev, *verdict = dev + 1;
    unsigned long long w = (unsigned long long)wait_ns;
    void *args[] = {&word, &error, &parties, &w, &verdict};
    e = cudaLaunchCooperativeKernel((const void *)barrier_selftest_kernel, dim3(blocks), dim3(kBlock), args, 0, 0);
  }
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(error_out, dev, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(verdicts, dev + 1, sizeof(int) * (size_t)blocks, cudaMemcpyDeviceToHost);
  if (word) cudaFree(word);
  if (dev) cudaFree(dev);
  return e;
}

cudaError_t plain_init_field(const PlainDevice &d, cudaStream_t s) {
  init_field_kernel<<<1024, 256, 0, s>>>(d.orient, d.solid, d.claimed, d.cellw, d.grid, d.ncells);
  return cudaGetLastError();
}

int plain_persistent_grid(int device) {
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, plain_persistent_kernel, kBlock, 0) != cudaSuccess)
    return 0;
  const int blocks = sms * per_sm;
  return blocks < (int)kStatusWords ? blocks : (int)kStatusWords;
}

cudaError_t plain_run_steps(const PlainDevice &d, long long step_limit, int grid_blocks, cudaStream_t s) {
  PlainDevice dd = d;
  void *args[] = {(void *)&dd, (void *)&step_limit};
  // the barrier's arrival counter starts every launch at zero
  const cudaError_t e = cudaMemsetAsync(d.ctrl, 0, 2 * sizeof(unsigned), s);
  if (e != cudaSuccess) return e;
  return cudaLaunchCooperativeKernel((const void *)plain_persistent_kernel, dim3(grid_blocks), dim3(kBlock), args, 0,
                                     s);
}

int plain_batched_grid(int device) {
  int sms = 0, per_sm = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, plain_batched_kernel, kBlock, 0) != cudaSuccess)
    return 0;
  return sms * per_sm;
}

cudaError_t plain_batch_reset(const PlainDevice *insts, int ninst, unsigned *queues, int nclasses, BatchTeam *teams,
                              int nteams, int *error, cudaStream_t s) {
  if (ninst <= 0) return cudaSuccess;
  batch_reset_kernel<<<dim3(64, ninst), 256, 0, s>>>(insts, ninst, queues, nclasses, teams, nteams, error);
  return cudaGetLastError();
}

cudaError_t plain_batched_run(const PlainDevice *insts, const int *order, int ninst, const BatchPlanDev &plan,
                              int grid_blocks, unsigned *queues, BatchTeam *teams, int *error, long long step_limit,
                              cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid_blocks);
  cfg.blockDim = dim3(kBlock);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, plain_batched_kernel, insts, order, ninst, plan, queues, teams, error, step_limit);
}

cudaError_t plain_batch_gather(const PlainDevice *insts, int ninst, PlainCtrl *out, cudaStream_t s) {
  if (ninst <= 0) return cudaSuccess;
  batch_gather_kernel<<<ninst, 128, 0, s>>>(insts, ninst, out);
  return cudaGetLastError();
}

cudaError_t plain_grain_field(const PlainDevice &d, int32_t *out, long long ngrains, cudaStream_t s) {
  grain_field_init_kernel<<<1024, 256, 0, s>>>(out, d.orient, d.grid, d.ncells);
  if (ngrains > 0) grain_field_scatter_kernel<<<1024, 256, 0, s>>>(out, d.gcell, ngrains);
  return cudaGetLastError();
}

}  // namespace amca
