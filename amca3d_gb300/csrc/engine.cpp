// engine.cpp — the C ABI (include/amca3d.h) over the plain CA realm.
//
// Host side of CellularAutomataSolver / CellularAutomataManager_3D
// (CA/src/CellularAutomataSolver.cpp:40-201, CA/src/CellularAutomataManager_3D.cpp:366-379):
// parse the deck, draw sites and the orientation stream with the reference's
// libraries, move tables to HBM, run the persistent step kernel, write outputs.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/amca3d.h"
#include "ca_plain.h"
#include "deck.h"
#include "device_cache.h"
#include "engine_remelt.h"
#include "errors.h"
#include "host_init.h"
#include "writers.h"

using namespace amca;

namespace {

#define CK(call)                                                                                      \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));       \
  } while (0)

thread_local std::string g_create_error;

// Interior cells up to which a plain realm runs 2 (kTinyRealmCells) or 3
// (kSmallRealmCells) blocks per SM instead of the kernel's full occupancy
// (see initialize).
constexpr long long kTinyRealmCells = 4200000ll;
constexpr long long kSmallRealmCells = 8ll << 20;

}  // namespace

struct amca_t {
  std::string err;
  amca_opts opts{};
  std::string workdir;
  PlainConfig cfg;
  std::unique_ptr<RemeltRealm> rm;  // set for FE-coupled remelting decks
  bool initialized = false;
  // host tables
  SiteSet sites;
  OrientationTable otab;
  std::vector<int32_t> mapped_vtr;
  int64_t rand_draws_before_orient = 0;
  // device
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int grid_blocks = 0;
  PlainDevice dev{};
  std::vector<void *> allocs;
  int32_t *scratch_field = nullptr;
  PlainCtrl ctrl{};  // host copy after the last segment
  VtrSeries vtr;
  double kernel_ms = 0.0;
  int64_t launches = 0;

  ~amca_t() {
    if (stream) cudaStreamSynchronize(stream);
    if (arena_ptr) cache_give(device, arena_ptr, arena_bytes);
    for (void *p : allocs) cudaFree(p);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  template <typename T>
  T *alloc(size_t n) {
    void *p = nullptr;
    CK(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)));
    allocs.push_back(p);
    return (T *)p;
  }

  // The realm's buffers carved out of one allocation (one cudaMalloc and one
  // cudaFree per realm): a sizing pass, then the same sequence handing out
  // 256-byte-aligned pointers.
  struct Arena {
    char *base = nullptr;
    size_t off = 0;
    template <typename T>
    T *take(size_t n) {
      const size_t at = (off + 255) & ~(size_t)255;
      off = at + std::max<size_t>(n, 1) * sizeof(T);
      return base ? (T *)(base + at) : nullptr;
    }
  };

  std::string path(const std::string &p) const {
    if (p.empty() || p[0] == '/' || workdir.empty()) return p;
    return workdir + "/" + p;
  }

  int64_t h2d_bytes = 0, d2h_bytes = 0;
  void h2d(void *dst, const void *src, size_t bytes) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream));
    h2d_bytes += (int64_t)bytes;
  }
  void d2h(void *dst, const void *src, size_t bytes) {
    CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream));
    d2h_bytes += (int64_t)bytes;
  }

  void sync_ctrl() {
    d2h(&ctrl, dev.ctrl, sizeof(PlainCtrl));
    CK(cudaStreamSynchronize(stream));
    if (ctrl.error) {
      throw DeviceError(std::string("CA kernel stopped: ") +
                        (ctrl.error == kErrBarrier ? "grid barrier wait timed out" : "scan look-back wait timed out"));
    }
  }

  bool prepared = false;

  // Host half: sites, mapped ids, orientation stream (one glibc rand() stream).
  void prepare() {
    if (prepared) return;
    GlibcRand rng(opts.seed);
    sites = make_sites(cfg, rng);
    mapped_vtr = make_mapped_ids(sites.surface_sites + sites.bulk_sites, cfg.shuffle_vtr, rng);
    rand_draws_before_orient = rng.draws();
    otab = make_orientations((int64_t)sites.cell.size(), rng);
    prepared = true;
  }

  void initialize() {
    const PlainConfig &c = cfg;
    if ((long long)c.nx * c.ny * c.nz >= kMaxCells)
      throw std::invalid_argument("grid too large: fewer than 2^27 interior cells per realm");
    prepare();
    CK(cudaSetDevice(device));
    const int64_t nsites = (int64_t)sites.cell.size();
    // --- device ---
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    Grid g{};
    g.nx = c.nx;
    g.ny = c.ny;
    g.nz = c.nz;
    g.nxg = c.nx + 2;
    g.nyg = c.ny + 2;
    g.nzg = c.nz + 2;
    g.nxyg = g.nxg * g.nyg;
    g.x0 = c.x0;
    g.y0 = c.y0;
    g.z0 = c.z0;
    g.h = c.h;
    PlainDevice &d = dev;
    d.grid = g;
    d.T0 = c.T0;
    d.Tm = c.Tm;
    d.Tdot = c.Tdot;
    d.a1 = c.a1;
    d.a2 = c.a2;
    d.a3 = c.a3;
    d.max_dt = c.max_dt;
    d.final_time = c.final_time;
    d.tsf = c.time_step_factor;
    d.trunc = c.trunc_coeff;
    d.h32 = (float)c.h;
    double cmax = 0;
    const double o[3] = {c.x0, c.y0, c.z0};
    const int nn[3] = {g.nxg, g.nyg, g.nzg};
    for (int a = 0; a < 3; ++a) cmax = std::max(cmax, std::fabs(o[a]) + (nn[a] + 1) * c.h);
    d.coord_err = (float)(std::ldexp(cmax, -49) + 1e-30);
    // the slowest block's busy time per phase costs a global load per block
    // and phase, so it is gathered only on request
    const char *detail = getenv("AMCA_PHASE_DETAIL");
    d.phase_detail = detail && detail[0] && detail[0] != '0' ? 1 : 0;
    // claims are handed out warp by warp for generations up to this many
    // ranks per block of the team, block by block above (AMCA_WARP_SCHED)
    d.warp_sched = kWarpSched;
    if (const char *w = getenv("AMCA_WARP_SCHED")) d.warp_sched = std::max(1, atoi(w));
    // generations of up to this many ranks per block are marked inside the
    // resolve pass, larger ones in a pass of their own (AMCA_MARK_SPLIT)
    d.mark_split = kMarkSplit;
    if (const char *m = getenv("AMCA_MARK_SPLIT")) d.mark_split = std::max(1, atoi(m));
    // warps per block that start a claim phase with the decrements on a
    // realm run by the whole GPU (AMCA_DEC_WARPS, 1..8)
    d.dec_warps = kDecWarps;
    if (const char *w = getenv("AMCA_DEC_WARPS")) d.dec_warps = std::min(8, std::max(1, atoi(w)));
    // the list is compacted above 2 x active + this many entries (AMCA_COMPACT_SLACK)
    d.compact_slack = kCompactSlack;
    if (const char *cs = getenv("AMCA_COMPACT_SLACK")) d.compact_slack = std::max(0, atoi(cs));
    d.ncells = (int64_t)g.nxyg * g.nzg;
    d.nsites = nsites;
    d.gcap = (int64_t)c.nx * c.ny * c.nz;
    const int64_t ntA = 2 * kStatusWords, ntB = kStatusWords;
    int32_t *site_cell = nullptr;
    double *site_dtc = nullptr, *omat = nullptr;
    float *omat32 = nullptr;
    auto layout = [&](Arena &a) {
      d.orient = a.take<uint32_t>(d.ncells);
      site_cell = a.take<int32_t>(nsites);
      site_dtc = a.take<double>(nsites);
      d.site_live = a.take<uint8_t>(nsites);
      omat = a.take<double>(nsites * 9);
      omat32 = a.take<float>(nsites * 9);
      d.gx = a.take<double>(d.gcap);
      d.gy = a.take<double>(d.gcap);
      d.gz = a.take<double>(d.gcap);
      d.gori = a.take<int32_t>(d.gcap);
      d.gcell = a.take<int32_t>(d.gcap);
      for (int b = 0; b < 2; ++b) {
        d.act[b] = a.take<EnvRec>(d.gcap);
        d.key[b] = a.take<float>(d.gcap + kKeyTile);  // the wake scan reads whole tiles
        d.lstep[b] = a.take<int32_t>(d.gcap);
        d.zlist[b] = a.take<int32_t>(d.gcap);
      }
      d.late = a.take<int32_t>(d.gcap);
      d.wlist = a.take<int32_t>(d.gcap);
      d.cellw = a.take<uint32_t>(d.ncells);
      d.dvh = a.take<double>(kDvRing);
      d.liq = a.take<uint32_t>(d.gcap);
      d.cellr = a.take<int32_t>(d.gcap);
      d.con = a.take<uint32_t>(d.gcap);
      d.child = a.take<uint32_t>(d.gcap);
      d.solid = a.take<uint32_t>(solid_words(d.ncells));
      d.claimed = a.take<uint32_t>(solid_words(d.ncells));
      d.scanA = a.take<unsigned long long>(ntA);
      d.scanB = a.take<unsigned long long>(ntB);
      d.scanC = a.take<unsigned long long>(ntA);
      d.scanD = a.take<unsigned long long>(ntA);
      d.ctrl = a.take<PlainCtrl>(1);
    };
    Arena sizing;
    layout(sizing);
    Arena arena;
    arena_ptr = cache_take(device, sizing.off, &arena_bytes);
    if (!arena_ptr) throw CudaError("cudaMalloc of the realm arena failed");
    arena.base = (char *)arena_ptr;
    layout(arena);
    d.site_cell = site_cell;
    d.site_dtc = site_dtc;
    d.omat = omat;
    d.omat32 = omat32;
    ntA_ = ntA;
    ntB_ = ntB;
    if (nsites) {
      h2d(site_cell, sites.cell.data(), nsites * sizeof(int32_t));
      h2d(site_dtc, sites.dtc.data(), nsites * sizeof(double));
      h2d(omat, otab.l2g.data(), nsites * 9 * sizeof(double));
      h2d(omat32, otab.l2g32.data(), nsites * 9 * sizeof(float));
    }
    reset_device();
    grid_blocks = plain_persistent_grid(device);
    {
      // Blocks per SM of the persistent launch: a small realm's generations
      // are short, so its steps are set by barrier and look-back latency,
      // which fall with the number of blocks (GB300, blocks per SM 2 / 3 /
      // 4: 128^3 17.2 / 17.9 / 19.0 ms, 160^3 21.4 / 21.8, 200^3 29.0 /
      // 27.8, 256^3 44.6 / 42.4 / 41.9, 320^3 70.8 / 64.6 / 63.0).
      // AMCA_PLAIN_BLOCKS_PER_SM overrides the choice.
      const long long interior = (long long)c.nx * c.ny * c.nz;
      int per_sm = interior <= kTinyRealmCells ? 2 : interior <= kSmallRealmCells ? 3 : 0;
      if (const char *e = getenv("AMCA_PLAIN_BLOCKS_PER_SM")) per_sm = std::max(1, atoi(e));
      if (per_sm > 0) {
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
        grid_blocks = std::min(grid_blocks, sms * per_sm);
      }
    }
    if (grid_blocks <= 0) throw CudaError("no co-resident blocks for the persistent CA kernel");
    CK(cudaStreamSynchronize(stream));
    // VtrManager::initialize
    vtr.configure(c.output, workdir);
    if (opts.write_outputs) vtr.make_dirs();
    initialized = true;
  }

  int64_t ntA_ = 0, ntB_ = 0;
  void *arena_ptr = nullptr;  // the realm's buffers, from and back to the arena cache
  size_t arena_bytes = 0;

  // Device state right after initialize: liquid field with the ghost layer,
  // live sites, cleared scan words, zeroed control block.
  void reset_device() {
    PlainDevice &d = dev;
    if (d.nsites) CK(cudaMemsetAsync(d.site_live, 1, d.nsites, stream));
    CK(cudaMemsetAsync(d.scanA, 0, ntA_ * sizeof(unsigned long long), stream));
    CK(cudaMemsetAsync(d.scanB, 0, ntB_ * sizeof(unsigned long long), stream));
    CK(cudaMemsetAsync(d.scanC, 0, ntA_ * sizeof(unsigned long long), stream));
    CK(cudaMemsetAsync(d.scanD, 0, ntA_ * sizeof(unsigned long long), stream));
    PlainCtrl c0{};
    c0.liquid = (long long)cfg.nx * cfg.ny * cfg.nz;
    h2d(d.ctrl, &c0, sizeof c0);
    CK(plain_init_field(d, stream));
    ctrl = c0;
    kernel_ms = 0.0;
    launches = 0;
  }

  void reset() {
    if (!initialized) throw StateError("amca_reset before amca_initialize");
    reset_device();
    CK(cudaStreamSynchronize(stream));
    vtr = VtrSeries();
    vtr.configure(cfg.output, workdir);
  }

  double algorithmic_bytes() const {
    // The byte model of the reference's step (one figure for every
    // implementation of it): per step 12 B per live site (cell id + dTc),
    // 48 B per nucleation (new envelope 40 B + orientation id 4 B + cell write
    // 4 B), 16 B per active envelope (half-diagonal read + write), 216 B per
    // envelope and generation of the reference's walk (40 B envelope, 26 x 4 B
    // neighbour states, 72 B matrix), 44 B per capture (cell write + 40 B
    // envelope), 8 B per list entry. The walk's generation 0 is every active
    // envelope after nucleation, its later generations the captures; this
    // step processes only the envelopes that may change, so A counts the
    // reference's active envelopes, not the ones processed here.
    const double S = (double)ctrl.sites_scanned, N = (double)ctrl.nucleations, A = (double)ctrl.ref_walked;
    const double C = (double)ctrl.captures;
    return 12 * S + 48 * N + 16 * A + 216 * (A + C) + 44 * C + 8 * (A + C);
  }

  // Bytes this step moves by its own accounting: 4 B per wake key scanned,
  // 24 B per generation-0 entry processed (woken list write + read,
  // half-diagonal write, grow step read + write), 228 B per entry and
  // generation processed (40 B envelope, 26 x 4 B neighbour states, 72 B
  // matrix, key + cell word), 148 B per capture (cell write, 40 B envelope,
  // the 26 cell words around it), 8 B per liquid-count decrement, 48 B per
  // entry moved by a compaction, and the sites and nucleations as above.
  double step_bytes() const {
    const double S = (double)ctrl.sites_scanned, N = (double)ctrl.nucleations, A0 = (double)ctrl.active_grown;
    const double G = (double)ctrl.grains_processed, C = (double)ctrl.captures, K = (double)ctrl.keys_scanned;
    const double D = (double)ctrl.decrements, M = (double)ctrl.compacted;
    return 12 * S + 48 * N + 4 * K + 24 * A0 + 228 * G + 148 * C + 8 * D + 48 * M;
  }

  bool finished() const { return ctrl.done || !(ctrl.time < cfg.final_time); }

  // One step with dt also capped by dt_cap (<= 0: no cap).
  void step_coupled(double dt_cap) {
    dev.dt_cap = dt_cap > 0 ? dt_cap : 0.0;
    try {
      run(1);
    } catch (...) {
      dev.dt_cap = 0.0;
      throw;
    }
    dev.dt_cap = 0.0;
  }
  // Steps while time < t_end.
  void run_until(double t_end) {
    if (!(t_end > 0)) return;  // time starts at 0: no step starts before t_end
    dev.t_stop = t_end;
    try {
      run(-1);
    } catch (...) {
      dev.t_stop = 0.0;
      throw;
    }
    dev.t_stop = 0.0;
  }

  // Run up to `limit` (absolute step count) in one launch.
  void segment(long long limit) {
    CK(cudaEventRecord(ev0, stream));
    CK(plain_run_steps(dev, limit, grid_blocks, stream));
    CK(cudaEventRecord(ev1, stream));
    ++launches;
    sync_ctrl();
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev0, ev1));
    kernel_ms += ms;
  }

  void run(long long max_steps) {
    if (!initialized) throw StateError("amca_run before amca_initialize");
    const long long target = max_steps < 0 ? (1ll << 60) : ctrl.step + max_steps;
    while (!finished() && ctrl.step < target) {
      long long limit = target;
      if (opts.write_outputs) {
        if (cfg.output.frequency >= 1) {
          const long long f = cfg.output.frequency;
          limit = std::min(limit, (ctrl.step / f + 1) * f);  // stop at the next output step
        } else if (cfg.output.time_interval_set && cfg.output.time_interval > 0) {
          limit = std::min(limit, ctrl.step + 1);  // time-based outputs are checked every step
        }
      }
      const long long before = ctrl.step;
      segment(limit);
      if (ctrl.step == before) break;
      if (opts.write_outputs && vtr.due((int)ctrl.step, ctrl.time)) write_snapshot();
    }
  }

  std::vector<int32_t> orient_field() {
    std::vector<int32_t> h((size_t)dev.ncells);
    d2h(h.data(), dev.orient, h.size() * sizeof(int32_t));
    CK(cudaStreamSynchronize(stream));
    return h;
  }
  std::vector<int32_t> grain_field() {
    if (!scratch_field) scratch_field = alloc<int32_t>(dev.ncells);
    CK(plain_grain_field(dev, scratch_field, ctrl.next_grain, stream));
    std::vector<int32_t> h((size_t)dev.ncells);
    d2h(h.data(), scratch_field, h.size() * sizeof(int32_t));
    CK(cudaStreamSynchronize(stream));
    return h;
  }
  std::vector<double> site_field() {
    std::vector<uint8_t> live(sites.cell.size());
    if (!live.empty()) {
      d2h(live.data(), dev.site_live, live.size());
      CK(cudaStreamSynchronize(stream));
    }
    std::vector<double> f((size_t)dev.ncells, -1.0);
    for (size_t i = 0; i < live.size(); ++i) f[sites.cell[i]] = live[i] ? sites.dtc[i] : 0.0;
    return f;
  }

  OutputView view(const std::vector<int32_t> &orient) const {
    OutputView v{};
    v.nx = cfg.nx;
    v.ny = cfg.ny;
    v.nz = cfg.nz;
    v.x0 = cfg.x0;
    v.y0 = cfg.y0;
    v.z0 = cfg.z0;
    v.h = cfg.h;
    v.orient = orient.data();
    v.euler = otab.euler.data();
    v.n_orient = ctrl.n_orient;
    v.mapped_vtr = cfg.shuffle_vtr ? &mapped_vtr : nullptr;
    v.shuffle_vtk = cfg.shuffle_vtk;
    v.expected_grains = sites.surface_sites + sites.bulk_sites;
    return v;
  }

  // State after a batched run of this realm (which started from the state
  // reset_device gives): its control block and the launch's time.
  void adopt_batch_run(const PlainCtrl &c, double ms) {
    ctrl = c;
    kernel_ms = ms;
    launches = 1;
    vtr = VtrSeries();
    vtr.configure(cfg.output, workdir);
  }

  void write_snapshot() {
    std::vector<int32_t> o = orient_field();
    OutputView v = view(o);
    vtr.write(v, ctrl.time);
  }

  int final_grain_count(const std::vector<int32_t> &o) const {
    // get_amount_of_final_orientations: orientation ids present anywhere,
    // the ghost layer (id 0) included (CA/src/CellularAutomataManager_3D.cpp:2000-2034)
    const int64_t n = ctrl.n_orient;
    if (n <= 0) return 0;
    std::vector<char> seen((size_t)n, 0);
    for (int32_t v : o)
      if (v > -1 && v < n) seen[v] = 1;
    return (int)std::count(seen.begin(), seen.end(), 1);
  }

  void write_outputs() {
    if (!initialized) throw StateError("amca_write_outputs before amca_initialize");
    std::vector<int32_t> o = orient_field();
    OutputView v = view(o);
    std::vector<int32_t> grain;
    std::vector<double> dtc, gx, gy, gz;
    std::vector<int32_t> gori, gcell;
    // output_microstructure_information (after the time loop)
    if (cfg.micro_out) {
      grain = grain_field();
      dtc = site_field();
      const int64_t ng = ctrl.next_grain;
      gx.resize(ng);
      gy.resize(ng);
      gz.resize(ng);
      gori.resize(ng);
      gcell.resize(ng);
      if (ng) {
        d2h(gx.data(), dev.gx, ng * 8);
        d2h(gy.data(), dev.gy, ng * 8);
        d2h(gz.data(), dev.gz, ng * 8);
        d2h(gori.data(), dev.gori, ng * 4);
        d2h(gcell.data(), dev.gcell, ng * 4);
        CK(cudaStreamSynchronize(stream));
      }
      v.grain = grain.data();
      v.site_dtc = dtc.data();
      v.n_grains = ng;
      v.gx = gx.data();
      v.gy = gy.data();
      v.gz = gz.data();
      v.gori = gori.data();
      v.gcell = gcell.data();
      write_grain_info(v, path(cfg.micro_out_file));
    }
    // CellularAutomataSolver::finalize: last VTR snapshot (step 0), finalGrains.vtk
    std::vector<int32_t> mapped_vtk;
    if (cfg.shuffle_vtk) {
      int maxVal = -1;
      for (int k = 1; k <= cfg.nz; ++k)
        for (int j = 1; j <= cfg.ny; ++j)
          for (int i = 1; i <= cfg.nx; ++i)
            maxVal = std::max(maxVal, (int)o[((int64_t)k * (cfg.ny + 2) + j) * (cfg.nx + 2) + i]);
      // replay the glibc stream to where the reference's writeToFile shuffles
      GlibcRand rng(opts.seed);
      const int64_t skip = rand_draws_before_orient + 3 * ctrl.n_orient;
      for (int64_t i = 0; i < skip; ++i) rng.next();
      mapped_vtk = make_mapped_ids(maxVal + 1, true, rng);
      v.mapped_vtk = &mapped_vtk;
    }
    if (vtr.due(0, ctrl.time)) {
      vtr.make_dirs();
      vtr.write(v, ctrl.time);
    }
    write_final_grains(v, path("finalGrains.vtk"), vtr.pvd_path());
  }
};

// Many plain realms in one cooperative launch (amca_batch_*).
struct amca_batch {
  // One launch layout: teams (size, class) and, per class, its realms in
  // queue order. A uniform layout has one class.
  struct Plan {
    std::vector<int> tsize, tclass;
    std::vector<std::vector<int>> classes;
    int blocks() const {
      int n = 0;
      for (int t : tsize) n += t;
      return n;
    }
  };

  std::string err;
  std::vector<amca_t *> realms;
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  PlainDevice *d_insts = nullptr;
  int *d_order = nullptr;
  unsigned *d_queues = nullptr;
  BatchTeam *d_teams = nullptr;
  int *d_error = nullptr;
  int2 *d_blk = nullptr, *d_crange = nullptr;
  int *d_tsize = nullptr, *d_tclass = nullptr;
  PlainCtrl *d_ctrls = nullptr;
  PlainCtrl *h_ctrls = nullptr;  // pinned
  int *h_error = nullptr;        // pinned
  int max_blocks = 0;
  Plan plan;
  int grid = 0;
  std::vector<int> order;  // realms by measured time, longest first
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool graph_ok = true;     // capture works on this device / driver
  bool graph_stale = true;  // launch layout changed since the capture
  int64_t runs = 0, cell_updates = 0;
  double last_ms = 0.0, total_ms = 0.0, mixed_ms = 0.0;
  std::vector<std::pair<int, double>> tuned;

  ~amca_batch() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graph();
    for (void *p : {(void *)d_insts, (void *)d_order, (void *)d_queues, (void *)d_teams, (void *)d_error,
                    (void *)d_blk, (void *)d_crange, (void *)d_tsize, (void *)d_tclass, (void *)d_ctrls})
      if (p) cudaFree(p);
    if (h_ctrls) cudaFreeHost(h_ctrls);
    if (h_error) cudaFreeHost(h_error);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
  }

  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }

  int n() const { return (int)realms.size(); }

  void setup(int team) {
    const int nr = n();
    CK(cudaSetDevice(device));
    CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    max_blocks = plain_batched_grid(device);
    if (max_blocks <= 0) throw CudaError("no co-resident blocks for the batched CA kernel");
    std::vector<PlainDevice> descs((size_t)nr);
    for (int r = 0; r < nr; ++r) descs[r] = realms[r]->dev;
    CK(cudaMalloc(&d_insts, nr * sizeof(PlainDevice)));
    CK(cudaMalloc(&d_order, nr * sizeof(int)));
    CK(cudaMalloc(&d_queues, max_blocks * sizeof(unsigned)));
    CK(cudaMalloc(&d_teams, max_blocks * sizeof(BatchTeam)));
    CK(cudaMalloc(&d_error, sizeof(int)));
    CK(cudaMalloc(&d_blk, max_blocks * sizeof(int2)));
    CK(cudaMalloc(&d_crange, max_blocks * sizeof(int2)));
    CK(cudaMalloc(&d_tsize, max_blocks * sizeof(int)));
    CK(cudaMalloc(&d_tclass, max_blocks * sizeof(int)));
    CK(cudaMalloc(&d_ctrls, nr * sizeof(PlainCtrl)));
    CK(cudaMallocHost(&h_ctrls, nr * sizeof(PlainCtrl)));
    CK(cudaMallocHost(&h_error, sizeof(int)));
    CK(cudaMemcpyAsync(d_insts, descs.data(), nr * sizeof(PlainDevice), cudaMemcpyHostToDevice, stream));
    order.resize(nr);
    for (int r = 0; r < nr; ++r) order[r] = r;
    set_team(team > 0 ? team : 8);
  }

  Plan uniform(int team) const {
    if (team < 1 || team > max_blocks)
      throw std::invalid_argument("team size must be between 1 and the co-resident blocks (" +
                                  std::to_string(max_blocks) + ")");
    Plan p;
    const int nt = std::min(max_blocks / team, n());
    p.tsize.assign(nt, team);
    p.tclass.assign(nt, 0);
    p.classes.push_back(order);
    return p;
  }

  void set_team(int team) { apply(uniform(team)); }

  // Upload a layout; the next run captures a new graph.
  void apply(const Plan &p) {
    const int nt = (int)p.tsize.size(), nc = (int)p.classes.size();
    if (nt < 1 || nc < 1 || p.blocks() > max_blocks) throw std::logic_error("batch layout does not fit");
    std::vector<int2> blk;
    for (int t = 0; t < nt; ++t)
      for (int r = 0; r < p.tsize[t]; ++r) blk.push_back(make_int2(t, r));
    std::vector<int> ord;
    std::vector<int2> cr;
    for (const auto &c : p.classes) {
      cr.push_back(make_int2((int)ord.size(), (int)c.size()));
      ord.insert(ord.end(), c.begin(), c.end());
    }
    if ((int)ord.size() != n()) throw std::logic_error("batch layout must list every realm once");
    CK(cudaMemcpyAsync(d_blk, blk.data(), blk.size() * sizeof(int2), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_crange, cr.data(), cr.size() * sizeof(int2), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tsize, p.tsize.data(), nt * sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_tclass, p.tclass.data(), nt * sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d_order, ord.data(), ord.size() * sizeof(int), cudaMemcpyHostToDevice, stream));
    CK(cudaStreamSynchronize(stream));
    plan = p;
    grid = (int)blk.size();
    graph_stale = true;
  }

  void enqueue() {
    const int nr = n();
    const BatchPlanDev pd{d_blk, d_tsize, d_tclass, d_crange};
    CK(plain_batch_reset(d_insts, nr, d_queues, (int)plan.classes.size(), d_teams, (int)plan.tsize.size(), d_error,
                         stream));
    CK(plain_batched_run(d_insts, d_order, nr, pd, grid, d_queues, d_teams, d_error, 1ll << 60, stream));
    CK(plain_batch_gather(d_insts, nr, d_ctrls, stream));
    CK(cudaMemcpyAsync(h_ctrls, d_ctrls, nr * sizeof(PlainCtrl), cudaMemcpyDeviceToHost, stream));
    CK(cudaMemcpyAsync(h_error, d_error, sizeof(int), cudaMemcpyDeviceToHost, stream));
  }

  // Capture enqueue() into a graph; on a capture failure runs use plain launches.
  void capture() {
    drop_graph();
    graph_stale = false;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      cudaGetLastError();
      graph_ok = false;
      return;
    }
    bool ok = true;
    try {
      enqueue();
    } catch (const CudaError &) {
      ok = false;
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(stream, &g);
    if (!ok || e != cudaSuccess || !g || cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      exec = nullptr;
      cudaGetLastError();
      graph_ok = false;
      return;
    }
    graph = g;
  }

  double run() {
    if (graph_ok && graph_stale) capture();
    CK(cudaEventRecord(ev0, stream));
    if (graph_ok)
      CK(cudaGraphLaunch(exec, stream));
    else
      enqueue();
    CK(cudaEventRecord(ev1, stream));
    CK(cudaStreamSynchronize(stream));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, ev0, ev1));
    ++runs;
    last_ms = ms;
    total_ms += ms;
    if (*h_error) throw DeviceError("batched CA launch stopped: a team barrier wait timed out");
    cell_updates = 0;
    for (int r = 0; r < n(); ++r) {
      amca_t *h = realms[r];
      const PlainCtrl &c = h_ctrls[r];
      h->adopt_batch_run(c, ms);
      cell_updates += (int64_t)c.step * ((int64_t)h->cfg.nx * h->cfg.ny * h->cfg.nz);
      if (c.error)
        throw DeviceError("realm " + std::to_string(r) + " of the batch stopped: " +
                          (c.error == kErrBarrier ? "grid barrier wait timed out" : "scan look-back wait timed out"));
    }
    return ms;
  }

  // Block 0 of a realm's team timed every phase of its run; their sum is the
  // realm's time in the launch, ms.
  static double realm_ms(const PlainCtrl &c) {
    return 1e-6 * (double)(c.ns_nucleation + c.ns_claim + c.ns_resolve + c.ns_step_end);
  }

  // Mixed layout from per-realm times t[s][r] measured at uniform team sizes
  // sizes[s]: for a target makespan M each realm takes the team size with
  // the least block time (size x time) among those that finish it within M;
  // realms of one size share teams, counted by first-fit decreasing into
  // bins of M. The smallest M whose teams fit is found by bisection; blocks
  // left over then go, one team at a time, to the class with the largest
  // time per team. Each class's queue runs longest realm first.
  Plan mixed(const std::vector<int> &sizes, const std::vector<std::vector<double>> &t) const {
    const int nr = n(), ns = (int)sizes.size();
    auto choose = [&](double M, std::vector<int> &pick) {
      for (int r = 0; r < nr; ++r) {
        int best = -1;
        for (int s = 0; s < ns; ++s)
          if (t[s][r] <= M && (best < 0 || sizes[s] * t[s][r] < sizes[best] * t[best][r])) best = s;
        if (best < 0) return false;
        pick[r] = best;
      }
      return true;
    };
    auto teams_for = [&](double M, const std::vector<int> &pick, std::vector<int> &nteams) {
      nteams.assign(ns, 0);
      int blocks = 0;
      for (int s = 0; s < ns; ++s) {
        std::vector<double> items;
        for (int r = 0; r < nr; ++r)
          if (pick[r] == s) items.push_back(t[s][r]);
        std::sort(items.rbegin(), items.rend());
        std::vector<double> bins;
        for (double x : items) {
          bool placed = false;
          for (double &b : bins)
            if (b + x <= M) {
              b += x;
              placed = true;
              break;
            }
          if (!placed) bins.push_back(x);
        }
        nteams[s] = (int)bins.size();
        blocks += sizes[s] * nteams[s];
      }
      return blocks;
    };
    double lo = 0.0, hi = 0.0;
    for (int r = 0; r < nr; ++r) {
      double m = 1e300;
      for (int s = 0; s < ns; ++s) m = std::min(m, t[s][r]);
      lo = std::max(lo, m);
      hi += t[0][r];
    }
    std::vector<int> pick((size_t)nr), nteams;
    hi = std::max(hi, lo);
    if (!choose(hi, pick) || teams_for(hi, pick, nteams) > max_blocks) return Plan();
    for (int it = 0; it < 50; ++it) {
      const double M = 0.5 * (lo + hi);
      if (choose(M, pick) && teams_for(M, pick, nteams) <= max_blocks)
        hi = M;
      else
        lo = M;
    }
    choose(hi, pick);
    int blocks = teams_for(hi, pick, nteams);
    std::vector<double> load((size_t)ns, 0.0);
    for (int r = 0; r < nr; ++r) load[pick[r]] += t[pick[r]][r];
    std::vector<int> members((size_t)ns, 0);
    for (int r = 0; r < nr; ++r) members[pick[r]]++;
    for (;;) {
      int best = -1;
      for (int s = 0; s < ns; ++s)
        if (nteams[s] > 0 && nteams[s] < members[s] && blocks + sizes[s] <= max_blocks &&
            (best < 0 || load[s] / nteams[s] > load[best] / nteams[best]))
          best = s;
      if (best < 0) break;
      nteams[best]++;
      blocks += sizes[best];
    }
    Plan p;
    for (int s = ns - 1; s >= 0; --s) {
      if (nteams[s] == 0) continue;
      std::vector<int> rs;
      for (int r = 0; r < nr; ++r)
        if (pick[r] == s) rs.push_back(r);
      std::stable_sort(rs.begin(), rs.end(), [&](int a, int b) { return t[s][a] > t[s][b]; });
      const int cls = (int)p.classes.size();
      p.classes.push_back(rs);
      for (int k = 0; k < nteams[s]; ++k) {
        p.tsize.push_back(sizes[s]);
        p.tclass.push_back(cls);
      }
    }
    return p;
  }

  // Returns the uniform team size kept, or 0 when the mixed layout won.
  int tune(int repeats) {
    repeats = std::max(repeats, 1);
    set_team(plan.tsize.empty() ? 8 : plan.tsize[0]);
    run();
    std::vector<double> t0((size_t)n());
    for (int r = 0; r < n(); ++r) t0[r] = realm_ms(h_ctrls[r]);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return t0[a] > t0[b]; });
    tuned.clear();
    mixed_ms = 0.0;
    std::vector<int> sizes;
    for (int s = 1; s <= 128 && s <= max_blocks; s *= 2) sizes.push_back(s);
    std::vector<std::vector<double>> t(sizes.size(), std::vector<double>((size_t)n(), 1e300));
    int best = 8;
    double best_ms = 1e300;
    for (size_t k = 0; k < sizes.size(); ++k) {
      set_team(sizes[k]);
      double m = 1e300;
      for (int q = 0; q < repeats; ++q) {
        m = std::min(m, run());
        for (int r = 0; r < n(); ++r) t[k][r] = std::min(t[k][r], realm_ms(h_ctrls[r]));
      }
      if (tuned.size() < 8) tuned.emplace_back(sizes[k], m);
      if (m < best_ms) {
        best_ms = m;
        best = sizes[k];
      }
    }
    // Mixed layouts, refined: a realm's time on a small team measured with
    // few busy blocks per SM is optimistic once every SM is full, so each
    // round replaces the estimates of the sizes it used by the times the
    // realms took inside that layout and plans again.
    Plan best_mixed;
    for (int round = 0; round < 6; ++round) {
      Plan mp = mixed(sizes, t);
      if (mp.tsize.empty()) break;
      apply(mp);
      double m = 1e300;
      std::vector<double> took((size_t)n(), 1e300);
      for (int q = 0; q < repeats; ++q) {
        m = std::min(m, run());
        for (int r = 0; r < n(); ++r) took[r] = std::min(took[r], realm_ms(h_ctrls[r]));
      }
      if (mixed_ms == 0.0 || m < mixed_ms) {
        mixed_ms = m;
        best_mixed = mp;
      }
      for (size_t c = 0; c < mp.classes.size(); ++c) {
        int size = 0;
        for (size_t k = 0; k < mp.tsize.size(); ++k)
          if (mp.tclass[k] == (int)c) size = mp.tsize[k];
        const size_t si = std::find(sizes.begin(), sizes.end(), size) - sizes.begin();
        for (int r : mp.classes[c]) t[si][r] = took[r];
      }
    }
    if (mixed_ms > 0.0 && mixed_ms < best_ms) {
      apply(best_mixed);
      return 0;
    }
    set_team(best);
    return best;
  }
};

namespace {

template <typename H, typename F>
int guarded(H *h, F &&f) {
  try {
    f();
    if (h) h->err.clear();
    return AMCA_OK;
  } catch (const CudaError &e) {
    if (h) h->err = e.what();
    return AMCA_ERR_CUDA;
  } catch (const DeviceError &e) {
    if (h) h->err = e.what();
    return AMCA_ERR_DEVICE;
  } catch (const StateError &e) {
    if (h) h->err = e.what();
    return AMCA_ERR_STATE;
  } catch (const std::exception &e) {
    if (h) h->err = e.what();
    return AMCA_ERR_ARG;
  }
}

}  // namespace

extern "C" {

int amca_create(const char *yaml_text, const amca_opts *opts, amca_t **out) {
  if (!out || !yaml_text) {
    g_create_error = "amca_create: null argument";
    return AMCA_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<amca_t> h(new amca_t);
  if (opts) h->opts = *opts;
  h->device = h->opts.device;
  if (h->opts.workdir) h->workdir = h->opts.workdir;
  try {
    if (deck_is_coupled(yaml_text)) {
      RemeltConfig rc = parse_remelt_deck(yaml_text);
      h->cfg = rc.ca;
      h->rm.reset(new RemeltRealm(rc, h->opts, h->workdir));
    } else {
      h->cfg = parse_plain_deck(yaml_text);
    }
  } catch (const std::exception &e) {
    g_create_error = e.what();
    return AMCA_ERR_PARSE;
  }
  *out = h.release();
  return AMCA_OK;
}

int amca_get_grid(const amca_t *h, int32_t cells[3], double origin[3], double *cell_size) {
  if (!h) return AMCA_ERR_ARG;
  if (cells) {
    cells[0] = h->cfg.nx;
    cells[1] = h->cfg.ny;
    cells[2] = h->cfg.nz;
  }
  if (origin) {
    origin[0] = h->cfg.x0;
    origin[1] = h->cfg.y0;
    origin[2] = h->cfg.z0;
  }
  if (cell_size) *cell_size = h->cfg.h;
  return AMCA_OK;
}

int amca_prepare(amca_t *h) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->prepare(); });
  return guarded(h, [&] { h->prepare(); });
}

int amca_get_sites(const amca_t *h, int32_t *cells, double *dtc, size_t cap, size_t *n_out) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm ? !h->rm->prepared() : !h->prepared) return AMCA_ERR_STATE;
  const SiteSet &st = h->rm ? h->rm->sites() : h->sites;
  const size_t n = st.cell.size();
  if (n_out) *n_out = n;
  const size_t m = std::min(n, cap);
  if (cells && m) memcpy(cells, st.cell.data(), m * sizeof(int32_t));
  if (dtc && m) memcpy(dtc, st.dtc.data(), m * sizeof(double));
  return AMCA_OK;
}

int amca_initialize(amca_t *h) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->initialize(); });
  return guarded(h, [&] {
    if (h->initialized) throw StateError("amca_initialize called twice");
    h->initialize();
  });
}

int amca_step(amca_t *h, double *dt_out) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm)
    return guarded(h, [&] {
      h->rm->run(1);
      if (dt_out) *dt_out = h->rm->ctrl().dt;
    });
  return guarded(h, [&] {
    h->run(1);
    if (dt_out) *dt_out = h->ctrl.dt;
  });
}

int amca_step_coupled(amca_t *h, double dt_cap, double *dt_out) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm)
    return guarded(h, [&] {
      h->rm->step_coupled(dt_cap);
      if (dt_out) *dt_out = h->rm->ctrl().dt;
    });
  return guarded(h, [&] {
    if (!h->initialized) throw StateError("amca_step before amca_initialize");
    h->step_coupled(dt_cap);
    if (dt_out) *dt_out = h->ctrl.dt;
  });
}

int amca_run_until(amca_t *h, double t_end) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->run_until(t_end); });
  return guarded(h, [&] {
    if (!h->initialized) throw StateError("amca_run before amca_initialize");
    h->run_until(t_end);
  });
}

int amca_set_nodal_temperatures(amca_t *h, const double *theta, int64_t n) {
  if (!h || !theta || n <= 0) return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_set_nodal_temperatures needs an FE-coupled deck");
    h->rm->set_nodal_temperatures(theta, n);
  });
}

int amca_run(amca_t *h, int max_steps) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->run(max_steps); });
  return guarded(h, [&] { h->run(max_steps); });
}

int amca_set_fe_frames(amca_t *h, const int32_t nodes[3], const double *coords, int32_t nframes, const double *times,
                       const double *theta) {
  if (!h || !nodes || !coords || !times || !theta) return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_set_fe_frames needs an FE-coupled deck");
    h->rm->set_frames(nodes, coords, nframes, times, theta);
  });
}

int amca_set_microstructure(amca_t *h, const int32_t *grain, const int32_t *orient, const uint8_t *melted,
                            const double *dtc, int64_t norient, const double *euler, int64_t ngrains,
                            const int32_t *grain_cell, const int32_t *grain_orient, int64_t expected) {
  if (!h || !grain || !orient || norient < 0 || ngrains < 0 || (norient && !euler) ||
      (ngrains && (!grain_cell || !grain_orient)))
    return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_set_microstructure needs an FE-coupled deck");
    const PlainConfig &c = h->rm->config().ca;
    const int64_t N = (int64_t)(c.nx + 2) * (c.ny + 2) * (c.nz + 2);
    RestartData r;
    r.ncells = N;
    r.norient = norient;
    r.ngrains = ngrains;
    r.expected = expected;
    // the per-cell and per-grain arrays are copied in parallel chunks (a
    // pbf_500 microstructure is about 220 MB)
    r.grain.resize((size_t)N);
    r.orient.resize((size_t)N);
    r.melted.resize((size_t)N);  // zeros unless given
    r.gcell.resize((size_t)ngrains);
    r.gori.resize((size_t)ngrains);
    std::vector<std::pair<void *, const void *>> dst_src = {{r.grain.data(), grain}, {r.orient.data(), orient},
                                                            {r.gcell.data(), grain_cell}, {r.gori.data(), grain_orient}};
    const size_t sizes[4] = {(size_t)N * 4, (size_t)N * 4, (size_t)ngrains * 4, (size_t)ngrains * 4};
    if (melted) {
      dst_src.emplace_back(r.melted.data(), melted);
    }
    if (dtc) r.dtc.assign(dtc, dtc + N);  // kept for completeness: the realm draws its own sites
    r.euler.assign(euler, euler + 3 * norient);
    const int nt = (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
    std::atomic<int> bad{0};
    auto part = [&](int t) {
      for (size_t a = 0; a < dst_src.size(); ++a) {
        const size_t bytes = a < 4 ? sizes[a] : (size_t)N;
        const size_t lo = bytes * t / nt, hi = bytes * (t + 1) / nt;
        if (hi > lo) memcpy((char *)dst_src[a].first + lo, (const char *)dst_src[a].second + lo, hi - lo);
      }
      const int64_t g0 = ngrains * t / nt, g1 = ngrains * (t + 1) / nt;
      for (int64_t g = g0; g < g1; ++g)
        if (grain_orient[g] < 0 || grain_orient[g] >= norient) bad.store(1, std::memory_order_relaxed);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nt; ++t) th.emplace_back(part, t);
    part(0);
    for (auto &x : th) x.join();
    if (bad.load()) throw std::invalid_argument("grain orientation out of range");
    h->rm->set_microstructure(std::move(r));
  });
}

int amca_set_rosenthal_frames(amca_t *h, const amca_rosenthal *p) {
  if (!h || !p) return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_set_rosenthal_frames needs an FE-coupled deck");
    RosenthalParams r{};
    for (int a = 0; a < 3; ++a) {
      r.origin[a] = p->origin[a];
      r.nodes[a] = p->nodes[a];
    }
    r.spacing = p->spacing;
    r.length_scale = p->length_scale;
    r.frame_dt = p->frame_dt;
    r.time_scale = p->time_scale;
    r.power = p->power;
    r.absorptivity = p->absorptivity;
    r.speed = p->speed;
    r.conductivity = p->conductivity;
    r.diffusivity = p->diffusivity;
    r.t0 = p->t0;
    r.t_cap = p->t_cap;
    r.x_start = p->x_start;
    r.y_line = p->y_line;
    r.z_top = p->z_top;
    r.void_above_set = p->void_above_set;
    r.void_above = p->void_above;
    r.t_void = p->t_void;
    h->rm->set_rosenthal(r, p->frames, p->time_offset);
  });
}

int amca_set_scan_frames(amca_t *h, const amca_scan *p) {
  if (!h || !p) return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_set_scan_frames needs an FE-coupled deck");
    h->rm->set_scan(*p, nullptr, 0.0, 0.0, 0.0);
  });
}

int amca_set_thermal_frames(amca_t *h, amca_thermal *m, const amca_scan *p, double t_liq, double band,
                            double thresh) {
  if (!h || !m || !p) return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_set_thermal_frames needs an FE-coupled deck");
    if (!(band >= 0) || !(thresh >= 0)) throw std::invalid_argument("band and thresh must be >= 0");
    h->rm->set_scan(*p, thermal_model_of(m), t_liq, band, thresh);
  });
}

int amca_get_frame_stats(amca_t *h, int64_t out[5]) {
  if (!h || !out) return AMCA_ERR_ARG;
  return guarded(h, [&] {
    if (!h->rm) throw std::invalid_argument("amca_get_frame_stats needs an FE-coupled deck");
    h->rm->frame_stats(out);
  });
}

int amca_get_field(amca_t *h, int field, void *dst, size_t bytes) {
  if (!h || !dst) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->get_field(field, dst, bytes); });
  return guarded(h, [&] {
    if (!h->initialized) throw StateError("amca_get_field before amca_initialize");
    const size_t n = (size_t)h->dev.ncells;
    if (field == AMCA_FIELD_ORIENTATION_ID || field == AMCA_FIELD_GRAIN_ID) {
      if (bytes != n * 4) throw std::invalid_argument("amca_get_field: bytes must be cells*4");
      if (field == AMCA_FIELD_ORIENTATION_ID) {
        h->d2h(dst, h->dev.orient, n * 4);
        CK(cudaStreamSynchronize(h->stream));
      } else {
        std::vector<int32_t> g = h->grain_field();
        memcpy(dst, g.data(), n * 4);
      }
    } else if (field == AMCA_FIELD_SITE_UNDERCOOLING) {
      if (bytes != n * 8) throw std::invalid_argument("amca_get_field: bytes must be cells*8");
      std::vector<double> f = h->site_field();
      memcpy(dst, f.data(), n * 8);
    } else {
      throw std::invalid_argument("amca_get_field: unknown field");
    }
  });
}

int amca_get_orientations(amca_t *h, double *euler, size_t cap, size_t *n_out, int all) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm)
    return guarded(h, [&] {
      if (all && !h->rm->prepared()) throw StateError("amca_get_orientations(all=1) before amca_prepare");
      const size_t n = h->rm->orientations(euler, cap, all);
      if (n_out) *n_out = n;
    });
  return guarded(h, [&] {
    if (all && !h->prepared) throw StateError("amca_get_orientations(all=1) before amca_prepare");
    const size_t n = all ? h->otab.euler.size() / 3 : (size_t)std::max<long long>(0, h->ctrl.n_orient);
    if (n_out) *n_out = n;
    if (euler) memcpy(euler, h->otab.euler.data(), std::min(n, cap) * 3 * sizeof(double));
  });
}

int amca_write_outputs(amca_t *h) {
  if (!h) return AMCA_ERR_ARG;
  int rc = h->rm ? guarded(h, [&] { h->rm->write_outputs(); }) : guarded(h, [&] { h->write_outputs(); });
  if (rc == AMCA_ERR_ARG) rc = AMCA_ERR_IO;
  return rc;
}

int amca_get_stats(amca_t *h, amca_stats *s) {
  if (!h || !s) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->stats(s); });
  return guarded(h, [&] {
    memset(s, 0, sizeof *s);
    const PlainCtrl &c = h->ctrl;
    s->step = c.step;
    s->time = c.time;
    s->dt = c.dt;
    s->liquid_cells = c.liquid;
    s->grains = c.next_grain;
    s->orientations = c.n_orient;
    s->active = c.n_active;
    s->sites = (int64_t)h->sites.cell.size();
    s->cells = (int64_t)h->cfg.nx * h->cfg.ny * h->cfg.nz;
    s->tests = (int64_t)c.tests;
    s->tests_fp64 = (int64_t)c.tests64;
    s->generations = (int64_t)c.gens;
    s->done = c.done;
    s->kernel_ms = h->kernel_ms;
    s->launches = h->launches;
    s->sites_scanned = (int64_t)c.sites_scanned;
    s->nucleations = (int64_t)c.nucleations;
    s->captures = (int64_t)c.captures;
    s->active_grown = (int64_t)c.active_grown;
    s->grains_processed = (int64_t)c.grains_processed;
    s->keys_scanned = (int64_t)c.keys_scanned;
    s->decrements = (int64_t)c.decrements;
    s->zero_events = (int64_t)c.zero_events;
    s->compactions = (int64_t)c.compactions;
    s->reference_walked = (int64_t)c.ref_walked;
    s->step_bytes = h->step_bytes();
    s->algorithmic_bytes = h->algorithmic_bytes();
    s->h2d_bytes = h->h2d_bytes;
    s->d2h_bytes = h->d2h_bytes;
    s->phase_ms[0] = c.ns_nucleation * 1e-6;
    s->phase_ms[1] = c.ns_claim * 1e-6;
    s->phase_ms[2] = c.ns_resolve * 1e-6;
    s->phase_ms[3] = c.ns_step_end * 1e-6;
    s->phase_ms[4] = c.ns_claim_gen0 * 1e-6;
    const double nb = h->grid_blocks > 0 ? h->grid_blocks : 1;
    s->phase_ms[5] = c.ns_claim_work_sum * 1e-6 / nb;
    s->phase_ms[6] = c.ns_claim_work_max * 1e-6;
    s->phase_ms[7] = c.ns_resolve_work_sum * 1e-6 / nb;
    s->phase_ms[8] = c.ns_resolve_work_max * 1e-6;
    s->detail_ms[0] = c.ns_nuc_work_sum * 1e-6 / nb;
    s->detail_ms[1] = c.ns_wake_work_sum * 1e-6 / nb;
    s->detail_ms[2] = c.ns_compact_work_sum * 1e-6 / nb;
    s->detail_ms[3] = c.ns_nuc_work_max * 1e-6;
    s->detail_ms[4] = c.ns_barrier_block0 * 1e-6;
  });
}

int amca_final_grain_count(amca_t *h, int32_t *count) {
  if (!h || !count) return AMCA_ERR_ARG;
  if (h->rm)
    return guarded(h, [&] {
      if (!h->rm->initialized()) throw StateError("amca_final_grain_count before amca_initialize");
      *count = h->rm->final_grain_count();
    });
  return guarded(h, [&] {
    if (!h->initialized) throw StateError("amca_final_grain_count before amca_initialize");
    *count = h->final_grain_count(h->orient_field());
  });
}

int amca_reset(amca_t *h) {
  if (!h) return AMCA_ERR_ARG;
  if (h->rm) return guarded(h, [&] { h->rm->reset(); });
  return guarded(h, [&] { h->reset(); });
}

int amca_host_alloc(size_t bytes, void **out) {
  if (!out) return AMCA_ERR_ARG;
  *out = nullptr;
  cudaError_t e = cudaMallocHost(out, std::max<size_t>(bytes, 1));
  if (e != cudaSuccess) {
    g_create_error = std::string("cudaMallocHost: ") + cudaGetErrorString(e);
    return AMCA_ERR_CUDA;
  }
  return AMCA_OK;
}

int amca_host_free(void *p) {
  if (p && cudaFreeHost(p) != cudaSuccess) return AMCA_ERR_CUDA;
  return AMCA_OK;
}

int amca_envelope_eval(int device, size_t n, const double *l2g, const double *gc, const double *length, double h,
                       const double *trunc, int32_t *captured, int32_t *captured_fast, double *info) {
  if (!l2g || !gc || !length || !trunc || !captured || !captured_fast || !info) {
    g_create_error = "amca_envelope_eval: null argument";
    return AMCA_ERR_ARG;
  }
  std::vector<void *> bufs;
  int rc = AMCA_OK;
  try {
    CK(cudaSetDevice(device));
    auto up = [&](const void *src, size_t bytes) {
      void *p = nullptr;
      CK(cudaMalloc(&p, std::max<size_t>(bytes, 1)));
      bufs.push_back(p);
      if (src && bytes) CK(cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice));
      return p;
    };
    double *dm = (double *)up(l2g, n * 9 * 8), *dg = (double *)up(gc, n * 3 * 8), *dl = (double *)up(length, n * 8);
    double *dt = (double *)up(trunc, n * 8);
    int32_t *c64 = (int32_t *)up(nullptr, n * 4), *cf = (int32_t *)up(nullptr, n * 4);
    double *di = (double *)up(nullptr, n * 4 * 8);
    if (n) {
      CK(plain_envelope_eval((long long)n, dm, dg, dl, h, dt, c64, cf, di, 0));
      CK(cudaMemcpy(captured, c64, n * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(captured_fast, cf, n * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(info, di, n * 4 * 8, cudaMemcpyDeviceToHost));
    }
  } catch (const std::exception &e) {
    g_create_error = e.what();
    rc = AMCA_ERR_CUDA;
  }
  for (void *p : bufs) cudaFree(p);
  return rc;
}

int amca_release_cached_memory(int device) {
  if (!cache_release(device)) {
    g_create_error = "amca_release_cached_memory: cudaFree failed";
    return AMCA_ERR_CUDA;
  }
  return AMCA_OK;
}

int amca_selftest_barrier(int device, int blocks, int parties, int64_t wait_ns, int32_t preset_error,
                          int32_t *error_out, int32_t *verdicts) {
  if (!error_out || !verdicts || blocks < 1 || blocks > 64 || parties < 1 || wait_ns < 1000 ||
      wait_ns > 2000000000ll) {
    g_create_error = "amca_selftest_barrier: bad argument (1 <= blocks <= 64, 1 us <= wait_ns <= 2 s)";
    return AMCA_ERR_ARG;
  }
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = plain_barrier_selftest(blocks, parties, (long long)wait_ns, preset_error, error_out,
                                                   verdicts);
  if (e != cudaSuccess) {
    g_create_error = std::string("amca_selftest_barrier: ") + cudaGetErrorString(e);
    return AMCA_ERR_CUDA;
  }
  return AMCA_OK;
}

int amca_batch_create(amca_t *const *realms, int n, int team_size, amca_batch **out) {
  if (!out || !realms || n < 1 || n > 65535) {
    g_create_error = "amca_batch_create: null argument, or not 1 to 65535 realms";
    return AMCA_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<amca_batch> b(new amca_batch);
  try {
    for (int r = 0; r < n; ++r) {
      amca_t *h = realms[r];
      if (!h) throw std::invalid_argument("amca_batch_create: null realm handle");
      if (h->rm) throw std::invalid_argument("amca_batch_create: batches run plain realms only");
      if (!h->initialized) throw StateError("amca_batch_create: realm " + std::to_string(r) + " is not initialized");
      if (r > 0 && h->device != realms[0]->device)
        throw std::invalid_argument("amca_batch_create: realms on different devices");
      if (std::find(b->realms.begin(), b->realms.end(), h) != b->realms.end())
        throw std::invalid_argument("amca_batch_create: a realm appears twice");
      b->realms.push_back(h);
    }
    b->device = realms[0]->device;
    for (amca_t *h : b->realms) CK(cudaStreamSynchronize(h->stream));
    b->setup(team_size);
  } catch (const StateError &e) {
    g_create_error = e.what();
    return AMCA_ERR_STATE;
  } catch (const CudaError &e) {
    g_create_error = e.what();
    return AMCA_ERR_CUDA;
  } catch (const std::exception &e) {
    g_create_error = e.what();
    return AMCA_ERR_ARG;
  }
  *out = b.release();
  return AMCA_OK;
}

int amca_batch_run(amca_batch *b, double *device_ms) {
  if (!b) return AMCA_ERR_ARG;
  return guarded(b, [&] {
    const double ms = b->run();
    if (device_ms) *device_ms = ms;
  });
}

int amca_batch_tune(amca_batch *b, int repeats, int *team_size_out) {
  if (!b) return AMCA_ERR_ARG;
  return guarded(b, [&] {
    const int t = b->tune(repeats);
    if (team_size_out) *team_size_out = t;
  });
}

int amca_batch_set_layout(amca_batch *b, int nclasses, const int32_t *team_size, const int32_t *teams,
                          const int32_t *realm_class, const int32_t *queue_order) {
  if (!b) return AMCA_ERR_ARG;
  return guarded(b, [&] {
    if (nclasses < 1 || nclasses > b->max_blocks || !team_size || !teams || !realm_class)
      throw std::invalid_argument("amca_batch_set_layout: need 1 or more classes and three arrays");
    amca_batch::Plan p;
    p.classes.resize(nclasses);
    long long blocks = 0;
    for (int c = 0; c < nclasses; ++c) {
      if (team_size[c] < 1 || teams[c] < 1)
        throw std::invalid_argument("amca_batch_set_layout: every class needs at least one team of one block");
      blocks += (long long)team_size[c] * teams[c];
      if (blocks > b->max_blocks)
        throw std::invalid_argument("amca_batch_set_layout: the teams need more blocks than fit on the device (" +
                                    std::to_string(b->max_blocks) + ")");
      for (int k = 0; k < teams[c]; ++k) {
        p.tsize.push_back(team_size[c]);
        p.tclass.push_back(c);
      }
    }
    std::vector<int> q = b->order;
    if (queue_order) {
      q.assign(queue_order, queue_order + b->n());
      std::vector<char> seen((size_t)b->n(), 0);
      for (int r : q) {
        if (r < 0 || r >= b->n() || seen[r])
          throw std::invalid_argument("amca_batch_set_layout: queue_order is not a permutation of the realms");
        seen[r] = 1;
      }
    }
    for (int r : q) {
      const int c = realm_class[r];
      if (c < 0 || c >= nclasses) throw std::invalid_argument("amca_batch_set_layout: realm class out of range");
      p.classes[c].push_back(r);
    }
    b->apply(p);
    if (queue_order) b->order = q;
  });
}

int amca_batch_get_layout(const amca_batch *b, int cap, int32_t *team_size, int32_t *teams, int32_t *realm_class,
                          int32_t *queue_order, int *nclasses) {
  if (!b) return AMCA_ERR_ARG;
  const amca_batch::Plan &p = b->plan;
  const int nc = (int)p.classes.size();
  if (nclasses) *nclasses = nc;
  for (int c = 0; c < nc && c < cap; ++c) {
    int size = 0, count = 0;
    for (size_t t = 0; t < p.tsize.size(); ++t)
      if (p.tclass[t] == c) {
        size = p.tsize[t];
        ++count;
      }
    if (team_size) team_size[c] = size;
    if (teams) teams[c] = count;
  }
  int k = 0;
  for (int c = 0; c < nc; ++c)
    for (int r : p.classes[c]) {
      if (realm_class) realm_class[r] = c;
      if (queue_order) queue_order[k] = r;
      ++k;
    }
  return AMCA_OK;
}

int amca_batch_get_stats(const amca_batch *b, amca_batch_stats *s) {
  if (!b || !s) return AMCA_ERR_ARG;
  memset(s, 0, sizeof *s);
  s->realms = b->n();
  const amca_batch::Plan &p = b->plan;
  s->teams = (int32_t)p.tsize.size();
  s->team_size = p.classes.size() == 1 && !p.tsize.empty() ? p.tsize[0] : 0;
  s->grid_blocks = b->grid;
  s->max_blocks = b->max_blocks;
  s->n_classes = (int32_t)std::min<size_t>(p.classes.size(), 8);
  for (int c = 0; c < s->n_classes; ++c) {
    s->class_realms[c] = (int32_t)p.classes[c].size();
    for (size_t t = 0; t < p.tsize.size(); ++t)
      if (p.tclass[t] == c) {
        s->class_team[c] = p.tsize[t];
        s->class_teams[c]++;
      }
  }
  s->mixed_ms = b->mixed_ms;
  s->graph = b->graph_ok ? 1 : 0;
  s->runs = b->runs;
  s->last_ms = b->last_ms;
  s->total_ms = b->total_ms;
  s->cell_updates = b->cell_updates;
  const int nt = std::min<int>((int)b->tuned.size(), 8);
  s->n_tuned = nt;
  for (int i = 0; i < nt; ++i) {
    s->tuned_team[i] = b->tuned[i].first;
    s->tuned_ms[i] = b->tuned[i].second;
  }
  return AMCA_OK;
}

const char *amca_batch_last_error(const amca_batch *b) {
  if (!b) return g_create_error.c_str();
  return b->err.c_str();
}

void amca_batch_destroy(amca_batch *b) { delete b; }

const char *amca_last_error(const amca_t *h) {
  if (!h) return g_create_error.c_str();
  return h->err.c_str();
}

void amca_destroy(amca_t *h) { delete h; }

}  // extern "C"
