// engine_remelt.cpp — see engine_remelt.h.
#include "engine_remelt.h"

#include "device_cache.h"
#include "errors.h"

#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <atomic>
#include <cmath>
#include <fstream>
#include <stdexcept>
#include <thread>

namespace amca {

namespace {

#define RCK(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess) throw CudaError(std::string(#call) + ": " + cudaGetErrorString(e_));   \
  } while (0)

inline bool is_ghost(int I, int J, int K, int nxg, int nyg, int nzg) {
  return I == 0 || I == nxg - 1 || J == 0 || J == nyg - 1 || K == 0 || K == nzg - 1;
}

// the device's ordered key of a double (atomicMin of minimum temperatures)
unsigned long long host_dkey(double x) {
  unsigned long long b;
  memcpy(&b, &x, 8);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// The largest float at most t and the smallest float at least t.
void float_bounds(double t, float &lo, float &hi) {
  lo = hi = (float)t;
  if ((double)lo > t) lo = std::nextafter(lo, -INFINITY);
  if ((double)hi < t) hi = std::nextafter(hi, INFINITY);
}

}  // namespace

RemeltRealm::RemeltRealm(RemeltConfig cfg, const amca_opts &opts, std::string workdir)
    : cfg_(std::move(cfg)), opts_(opts), workdir_(std::move(workdir)) {
  device_ = opts_.device;
}

RemeltRealm::~RemeltRealm() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (const auto &a : allocs_) cache_give(device_, a.first, a.second);
  if (hostvel_) cudaFreeHost(hostvel_);
  if (staging_) cudaFreeHost(staging_);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  if (stream_) cudaStreamDestroy(stream_);
}

template <typename T>
T *RemeltRealm::alloc(size_t n) {
  size_t got = 0;
  void *p = cache_take(device_, std::max<size_t>(n, 1) * sizeof(T), &got);
  if (!p) throw CudaError("cudaMalloc failed for a remelting realm buffer");
  allocs_.emplace_back(p, got);
  return (T *)p;
}

void RemeltRealm::h2d(void *dst, const void *src, size_t bytes) {
  if (!bytes) return;
  RCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, stream_));
  h2d_bytes_ += (int64_t)bytes;
}
void RemeltRealm::d2h(void *dst, const void *src, size_t bytes) {
  if (!bytes) return;
  RCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream_));
  d2h_bytes_ += (int64_t)bytes;
}

std::string RemeltRealm::path(const std::string &p) const {
  if (p.empty() || p[0] == '/' || workdir_.empty()) return p;
  return workdir_ + "/" + p;
}

void RemeltRealm::set_frames(const int32_t nodes[3], const double *coords, int64_t nframes, const double *times,
                             const double *theta) {
  if (initialized_) throw StateError("frames must be set before amca_initialize");
  frames_ = fe_frames_from_arrays(nodes, coords, nframes, times, theta, cfg_.fe);
  frames_src_ = 1;
}

void RemeltRealm::set_rosenthal(const RosenthalParams &p, int nframes, double time_offset) {
  if (initialized_) throw StateError("frames must be set before amca_initialize");
  if (nframes < 2) throw std::invalid_argument("at least two frames");
  for (int a = 0; a < 3; ++a)
    if (p.nodes[a] < 2) throw std::invalid_argument("at least 2 nodes per axis");
  ros_ = p;
  ros_nframes_ = nframes;
  ros_toff_ = time_offset;
  const int32_t nodes[3] = {p.nodes[0], p.nodes[1], p.nodes[2]};
  synthetic_grid(p.origin, p.spacing, nodes, nframes, p.frame_dt, time_offset);
  frames_src_ = 2;
}

// Node coordinates and frame times of generated frames, exactly as the text
// reader would hold them for the same file.
void RemeltRealm::synthetic_grid(const double origin[3], double spacing, const int32_t nodes[3], int nframes,
                                 double frame_dt, double time_offset) {
  FeFrames fr;
  for (int a = 0; a < 3; ++a) fr.nn[a] = nodes[a];
  fr.nnodes = (int64_t)nodes[0] * nodes[1] * nodes[2];
  fr.coord.resize(3 * (size_t)fr.nnodes);
  for (int64_t n = 0; n < fr.nnodes; ++n) {
    const int64_t I[3] = {n % nodes[0], (n / nodes[0]) % nodes[1], n / ((int64_t)nodes[0] * nodes[1])};
    for (int d = 0; d < 3; ++d) {
      double x = origin[d] + spacing * (double)I[d];
      x += cfg_.fe.offset[d];
      x *= cfg_.fe.length_scale;
      fr.coord[3 * n + d] = x;
    }
  }
  fr.times.resize((size_t)nframes);
  const double t0 = time_offset + 0 * frame_dt;
  fr.times[0] = 0.0;
  for (int f = 1; f < nframes; ++f) fr.times[f] = ((time_offset + f * frame_dt) - t0) * cfg_.fe.time_scale;
  fr.nframes = nframes;
  frames_ = std::move(fr);
}

void RemeltRealm::set_scan(const amca_scan &scan, ThermalModel *model, double t_liq, double band, double thresh) {
  if (initialized_) throw StateError("frames must be set before amca_initialize");
  if (scan.frames < 2) throw std::invalid_argument("at least two frames");
  for (int a = 0; a < 3; ++a)
    if (scan.nodes[a] < 2) throw std::invalid_argument("at least 2 nodes per axis");
  if (!(scan.spacing > 0) || !(scan.length_scale > 0) || !(scan.frame_dt > 0) || !(scan.time_scale > 0))
    throw std::invalid_argument("scan: spacing, length_scale, frame_dt and time_scale must be positive");
  if (scan.ntracks > 1 && !(scan.track_time > 0)) throw std::invalid_argument("scan: track_time must be positive");
  scan_ = scan;
  model_ = model;
  t_liq_ = t_liq;
  band_ = band;
  thresh_ = thresh;
  synthetic_grid(scan.origin, scan.spacing, scan.nodes, scan.frames, scan.frame_dt, scan.time_offset);
  frames_src_ = 3;
}

// Frames avail_ .. upto - 1 into the ring: generated on the GPU (scan or
// model frames) or read from the text file (streamed text frames), with
// their times in the ring of times.
void RemeltRealm::fill_frames(int upto) {
  upto = std::min<int>(upto, (int)nframes_);
  if (upto <= avail_) return;
  const int64_t nn = dev_.nnodes;
  if (text_stream_) {
    int f = avail_;
    double t = 0;
    while (f < upto) {
      double *dst = staging_ + (size_t)(f - avail_) * nn;
      if (!reader_->next(dst, t)) {  // end of the file, or a malformed frame: the frame count is known now
        nframes_ = f;
        dev_.nframes = f;
        if (reader_->bad()) dev_.bad_frame = f;
        break;
      }
      times_read_.push_back(t);
      ++f;
    }
    for (int g = avail_; g < f; ++g) {
      RCK(cudaMemcpyAsync(ring_ + (size_t)(g % slots_) * nn, staging_ + (size_t)(g - avail_) * nn, (size_t)nn * 8,
                          cudaMemcpyHostToDevice, stream_));
      RCK(cudaMemcpyAsync(ftime_ + g % slots_, &times_read_[g], 8, cudaMemcpyHostToDevice, stream_));
    }
    RCK(cudaStreamSynchronize(stream_));
    h2d_bytes_ += (int64_t)(f - avail_) * nn * 8;
    upto = f;
  } else {
    fill_scan_frames(&scan_, model_, t_liq_, band_, thresh_, avail_, upto - avail_, ring_, slots_, fcount_, stream_);
    for (int g = avail_; g < upto; ++g)
      RCK(cudaMemcpyAsync(ftime_ + g % slots_, &frames_.times[g], 8, cudaMemcpyHostToDevice, stream_));
    RCK(cudaStreamSynchronize(stream_));
  }
  produced_ += upto - avail_;
  ++fills_;
  avail_ = upto;
  dev_.frames_avail = avail_;
}

// A fresh reader at the start of the text frames (frame 0 and the grid).
void RemeltRealm::open_text_frames() {
  reader_.reset(new FrameReader(path(cfg_.fe.mesh), cfg_.fe));
  times_read_.assign(1, reader_->head().times[0]);
  nframes_ = 1 << 30;  // unknown until the reader reaches the end of the file
  dev_.nframes = (int)nframes_;
  dev_.bad_frame = -1;
  avail_ = 0;
  dev_.frames_avail = 0;
}

void RemeltRealm::frame_stats(int64_t out[5]) {
  out[0] = produced_;
  out[1] = fills_;
  unsigned long long c[4] = {0, 0, 0, 0};
  if (fcount_) {
    RCK(cudaMemcpyAsync(c, fcount_, sizeof c, cudaMemcpyDeviceToHost, stream_));
    RCK(cudaStreamSynchronize(stream_));
  }
  for (int i = 0; i < 3; ++i) out[2 + i] = (int64_t)c[i];
}

void RemeltRealm::set_microstructure(RestartData r) {
  if (prepared_) throw StateError("amca_set_microstructure after amca_prepare");
  const PlainConfig &c = cfg_.ca;
  const int64_t N = (int64_t)(c.nx + 2) * (c.ny + 2) * (c.nz + 2);
  if (r.ncells != N) throw std::invalid_argument("microstructure arrays must cover the ghost-inclusive grid");
  micro_.reset(new RestartData(std::move(r)));
}

void RemeltRealm::prepare() {
  if (prepared_) return;
  const PlainConfig &c = cfg_.ca;
  if (cfg_.load_seeds) throw std::invalid_argument("load_microstructure_information.load_seeds is not supported");
  rng_.reset(new GlibcRand(opts_.seed));  // srand in the CA manager's constructor (CellularAutomataManager_3D.cpp:40)
  const int nxg = c.nx + 2, nyg = c.ny + 2, nzg = c.nz + 2;
  const int64_t nxyg = (int64_t)nxg * nyg, N = nxyg * nzg;
  site_field_.clear();  // built on first use (site_field())
  grain_cell_.clear();
  grain_ori0_.clear();
  if (cfg_.random_micro && !micro_) {
    orient0_.assign((size_t)N, -1);
    grain0_.assign((size_t)N, -1);
    melted0_.assign((size_t)N, cfg_.initial_melted ? 1 : 0);
    gori0_.assign((size_t)N, -1);
    // random_microstructure_information (CellularAutomataManager_3D.cpp:1929-1984):
    // one orientation and one grain per interior cell, in cell order
    const int64_t M = (int64_t)c.nx * c.ny * c.nz;
    otab_ = make_orientations(M, *rng_);
    int64_t q = 0;
    grain_cell_.reserve((size_t)M);
    grain_ori0_.reserve((size_t)M);
    for (int K = 1; K < nzg - 1; ++K)
      for (int J = 1; J < nyg - 1; ++J)
        for (int I = 1; I < nxg - 1; ++I) {
          const int64_t cell = K * nxyg + (int64_t)J * nxg + I;
          orient0_[cell] = (int32_t)q;
          grain0_[cell] = (int32_t)q;
          gori0_[cell] = (int32_t)q;
          grain_cell_.push_back((int32_t)cell);
          grain_ori0_.push_back((int32_t)q);
          ++q;
        }
    n_init_orient_ = M;
    n_init_grains_ = M;
    if (c.shuffle_vtr) mapped_vtr_ = make_mapped_ids(N, true, *rng_);
    expected_grains_ = 0;
  } else {
    // load_microstructure_information + retrieve_grain_information_before_simulation
    // (CellularAutomataManager_3DRemelting.cpp:164-332)
    RestartData loaded;
    if (!micro_) loaded = read_restart(path(cfg_.micro_file));
    RestartData &r = micro_ ? *micro_ : loaded;  // consumed here: its arrays move into the initial state
    if (r.ncells != N)
      throw std::runtime_error("Error : microstructure information file is not fit the current domain size");
    if (!cfg_.nucleation && c.shuffle_vtr) mapped_vtr_ = make_mapped_ids(r.expected, true, *rng_);
    otab_ = orientations_from_euler(r.euler);
    orient0_ = std::move(r.orient);
    grain0_ = std::move(r.grain);
    melted0_ = std::move(r.melted);
    grain_cell_ = std::move(r.gcell);
    grain_ori0_ = std::move(r.gori);
    n_init_orient_ = r.norient;
    n_init_grains_ = r.ngrains;
    expected_grains_ = r.expected;
    micro_.reset();
    gori0_.assign((size_t)N, -1);
    // per cell, in parallel over z slabs: a grain belongs to the one interior
    // cell its record names (a second cell naming it fails that test), and a
    // cell without an orientation takes its grain's; the error reported is
    // that of the first offending cell in cell order, as a serial pass would
    const int64_t ngr = n_init_grains_;
    const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<int64_t> bad_cell((size_t)nt, INT64_MAX);
    std::vector<int> bad_kind((size_t)nt, 0);
    std::vector<std::thread> th;
    auto slab = [&](int t) {
      const int k0 = (int)((int64_t)nzg * t / nt), k1 = (int)((int64_t)nzg * (t + 1) / nt);
      for (int K = k0; K < k1; ++K)
        for (int J = 0; J < nyg; ++J)
          for (int I = 0; I < nxg; ++I) {
            const int64_t cell = K * nxyg + (int64_t)J * nxg + I;
            if (is_ghost(I, J, K, nxg, nyg, nzg)) {
              orient0_[cell] = -1;
              continue;
            }
            const int32_t g = grain0_[cell];
            int kind = 0;
            if (g >= 0) {
              if (g >= ngr) {
                kind = 1;
              } else if (grain_cell_[g] != cell) {
                kind = 2;
              } else {
                // the grain's centre is reset to its cell centre, length 0
                // (:289-296): remelt_init_records on the device
                gori0_[cell] = grain_ori0_[g];
              }
            }
            if (!kind && orient0_[cell] <= -1) {
              if (g < 0) kind = 3;
              else orient0_[cell] = grain_ori0_[g];
            }
            if (kind) {
              bad_cell[t] = cell;
              bad_kind[t] = kind;
              return;
            }
          }
    };
    for (int t = 1; t < nt; ++t) th.emplace_back(slab, t);
    slab(0);
    for (auto &x : th) x.join();
    for (int t = 0; t < nt; ++t) {
      if (bad_cell[t] == INT64_MAX) continue;
      if (bad_kind[t] == 1) throw std::runtime_error("restart cell refers to a grain that is not listed");
      if (bad_kind[t] == 2)
        throw std::runtime_error("restart grains must each belong to the one interior cell that refers to them");
      throw std::runtime_error("restart cell has neither an orientation nor a grain");
    }
  }
  init_draws_ = rng_->draws();
  if (cfg_.nucleation) {
    sites_ = make_sites(c, *rng_);
    if (c.shuffle_vtr) {  // global_mapped_grain_ID_plus (CellularAutomataManager_3DRemelting.cpp:873-931)
      const int64_t surf = ((int64_t)c.nx * c.ny + (int64_t)c.nx * (c.nz - 2) + (int64_t)(c.ny - 2) * (c.nz - 2)) * 2;
      const int64_t bulk = (int64_t)c.nx * c.ny * c.nz;
      const int ss = (int)(std::round(c.ns * surf * (c.h * c.h)) + 0.5);
      const int sb = (int)(std::round(c.nv * bulk * (c.h * c.h * c.h)) + 0.5);
      mapped_vtr_ = make_mapped_ids((int64_t)ss + sb + expected_grains_, true, *rng_);
    }
    expected_grains_ += sites_.surface_sites + sites_.bulk_sites;
    init_draws_ = rng_->draws();
    // the nucleation orientation stream, extended on demand
    const int64_t K = std::max<int64_t>(4 * (int64_t)sites_.cell.size(), 1024);
    append_orientations(otab_, make_orientations(K, *rng_));
  }
  prepared_ = true;
}

const std::vector<double> &RemeltRealm::site_field() {
  if (site_field_.empty()) {
    site_field_.assign((size_t)dev_.ncells > 0 ? (size_t)dev_.ncells : orient0_.size(), -1.0);
    for (size_t i = 0; i < sites_.cell.size(); ++i) site_field_[sites_.cell[i]] = sites_.dtc[i];
  }
  return site_field_;
}

void RemeltRealm::upload_initial_state() {
  const int64_t N = dev_.ncells;
  h2d(dev_.orient, orient0_.data(), N * 4);
  h2d(dev_.grain, grain0_.data(), N * 4);
  h2d(dev_.melted, melted0_.data(), N);
  RCK(remelt_init_records(dev_, stream_));  // from the grain field just uploaded
  h2d(dev_.gori, gori0_.data(), N * 4);
  RCK(cudaMemsetAsync(dev_.gdx, 0, N * 4, stream_));
  RCK(cudaMemsetAsync(dev_.gdy, 0, N * 4, stream_));
  RCK(cudaMemsetAsync(dev_.gdz, 0, N * 4, stream_));
  RCK(cudaMemsetAsync(dev_.flagbits, 0, ((N + 31) / 32) * 4, stream_));
  RCK(cudaMemsetAsync(dev_.eliq, 0, std::max<int64_t>(dev_.nelem, 1) * 4, stream_));
  RCK(remelt_init_theta(dev_, stream_));
  hostvel_->seq_req = 0;
  hostvel_->seq_done = 0;
  h2d(dev_.ctrl, &ctrl0_, sizeof ctrl0_);
  ctrl_ = ctrl0_;
  RCK(cudaStreamSynchronize(stream_));
  // the host vectors above are staged through pageable memory; the sync keeps them alive
}

void RemeltRealm::initialize() {
  if (initialized_) throw StateError("amca_initialize called twice");
  prepare();
  const PlainConfig &c = cfg_.ca;
  RCK(cudaSetDevice(device_));
  RCK(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  RCK(cudaEventCreate(&ev0_));
  RCK(cudaEventCreate(&ev1_));
  if (frames_src_ == 0) {
    // text frames are read whole, or (files over 4 GiB, or AMCA_FRAME_STREAM=1) a window at a time
    const std::string fpath = path(cfg_.fe.mesh);
    std::ifstream probe(fpath.c_str(), std::ios::binary | std::ios::ate);
    const long long bytes = probe ? (long long)probe.tellg() : 0;
    const char *se = getenv("AMCA_FRAME_STREAM");
    text_stream_ = se ? atoi(se) != 0 : bytes > (4ll << 30);
    if (text_stream_) {
      reader_.reset(new FrameReader(fpath, cfg_.fe));
      frames_ = reader_->head();
    } else {
      frames_ = read_fe_frames(fpath, cfg_.fe);
    }
  }
  nframes_ = frames_src_ == 2 ? ros_nframes_ : (text_stream_ ? (1 << 30) : frames_.nframes);
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
  RemeltDevice &d = dev_;
  d.g = g;
  d.ncells = (int64_t)g.nxyg * g.nzg;
  const int64_t N = d.ncells;
  d.Tm = c.Tm;
  float_bounds(c.Tm, d.tm_lo, d.tm_hi);
  float_bounds(-1.0 + 0.01, d.np_lo, d.np_hi);  // nullMatTemp_ + 0.01
  d.Ts = c.Ts;
  d.Tnuc = c.Tmin_nuc;
  d.a1 = c.a1;
  d.a2 = c.a2;
  d.a3 = c.a3;
  d.b1 = (int)c.b1;
  d.b2 = (int)c.b2;
  d.b3 = (int)c.b3;
  d.tsf_ca = c.time_step_factor;
  d.h = c.h;
  d.trunc = c.trunc_coeff;
  d.cutoff = c.length_cutoff_factor * c.h;  // cellGrainLegnthCutoff_ *= h_ (Remelting.cpp:89)
  d.final_time = c.final_time;
  d.void_t = cfg_.tr.void_temperature;
  d.h32 = (float)c.h;
  {
    double cmax = 0;
    const double o[3] = {c.x0, c.y0, c.z0};
    const int nn[3] = {g.nxg, g.nyg, g.nzg};
    for (int a = 0; a < 3; ++a) cmax = std::max(cmax, std::fabs(o[a]) + (nn[a] + 1) * c.h);
    d.coord_err = (float)(std::ldexp(cmax, -49) + 1e-30);
  }
  // --- FE -> CA map (MapVoxelManager::execute_with_focus_on_CA_region) ---
  for (int a = 0; a < 3; ++a) d.nn[a] = frames_.nn[a];
  d.nnodes = frames_.nnodes;
  d.nelem = frames_.nelem();
  int32_t *tag = alloc<int32_t>(N);
  double *pc = alloc<double>(3 * N);
  unsigned long long *tcount = alloc<unsigned long long>(2);
  {
    VoxelMapPlan plan = plan_voxel_map(frames_, c, cfg_.tr);
    std::vector<void *> tmp;
    auto up = [&](const void *src, size_t bytes) {
      void *p = nullptr;
      RCK(cudaMalloc(&p, std::max<size_t>(bytes, 1)));
      tmp.push_back(p);
      h2d(p, src, bytes);
      return p;
    };
    TagPlan tp{};
    memcpy(tp.mm, plan.mm, sizeof tp.mm);
    memcpy(tp.dbin, plan.dbin, sizeof tp.dbin);
    memcpy(tp.nbin, plan.nbin, sizeof tp.nbin);
    tp.bin_start = (const int64_t *)up(plan.bin_start.data(), plan.bin_start.size() * 8);
    tp.bin_elems = (const int32_t *)up(plan.bin_elems.data(), plan.bin_elems.size() * 4);
    tp.erange = (const double *)up(plan.erange.data(), plan.erange.size() * 8);
    tp.coord = (const double *)up(frames_.coord.data(), frames_.coord.size() * 8);
    for (int a = 0; a < 3; ++a) tp.nn[a] = frames_.nn[a];
    tp.tolerance = cfg_.tr.tolerance;
    tp.max_iter = cfg_.tr.max_iter;
    tp.counts = tcount;
    RCK(cudaMemsetAsync(tcount, 0, 16, stream_));
    RCK(remelt_tag_voxels(g, tp, tag, pc, stream_));
    unsigned long long counts[2] = {0, 0};
    d2h(counts, tcount, 16);
    RCK(cudaStreamSynchronize(stream_));
    for (void *p : tmp) cudaFree(p);
    if (counts[0] == 0)
      throw std::runtime_error(
          "Error: a proc has no corrsponding FEM mesh!! Maybe decrease the number of multi-core parallel can help.");
    d.force_exact = counts[1] ? 1 : 0;
  }
  {
    // the slowest block's busy time per barrier costs a global load per block
    // and barrier, so it is gathered only on request
    const char *detail = getenv("AMCA_PHASE_DETAIL");
    d.detail = detail && detail[0] && detail[0] != '0' ? 1 : 0;
  }
  d.tag = tag;
  d.pc = pc;
  {
    float *pc32 = alloc<float>(3 * N);
    RCK(remelt_round_coords(pc, pc32, 3 * N, stream_));
    d.pc32 = pc32;
  }
  {  // element -> interior cells (CSR), for the phase-update pass over active elements
    std::vector<int32_t> htag((size_t)N);
    d2h(htag.data(), tag, N * 4);
    RCK(cudaStreamSynchronize(stream_));
    // counts per element and thread over z slabs of the interior, then each
    // thread fills its slab's cells: every element's list stays in ascending
    // cell order, as a serial pass gives
    const int64_t ne = d.nelem;
    int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if ((int64_t)nt * (ne + 1) > (64ll << 20)) nt = 1;  // bound the per-thread count arrays
    const int kz = g.nzg - 2;
    nt = std::max(1, std::min(nt, kz));
    std::vector<std::vector<int32_t>> cnt((size_t)nt, std::vector<int32_t>((size_t)ne, 0));
    auto slab_of = [&](int t, int &k0, int &k1) {
      k0 = 1 + (int)((int64_t)kz * t / nt);
      k1 = 1 + (int)((int64_t)kz * (t + 1) / nt);
    };
    auto run_threads = [&](auto body) {
      std::vector<std::thread> th;
      for (int t = 1; t < nt; ++t) th.emplace_back(body, t);
      body(0);
      for (auto &x : th) x.join();
    };
    run_threads([&](int t) {
      int k0, k1;
      slab_of(t, k0, k1);
      int32_t *ct = cnt[(size_t)t].data();
      for (int K = k0; K < k1; ++K)
        for (int J = 1; J < g.nyg - 1; ++J) {
          const int32_t *row = htag.data() + (int64_t)K * g.nxyg + (int64_t)J * g.nxg;
          for (int I = 1; I < g.nxg - 1; ++I)
            if (row[I] >= 0) ++ct[row[I]];
        }
    });
    std::vector<int64_t> start((size_t)ne + 1, 0);
    for (int64_t e = 0; e < ne; ++e) {
      int64_t sum = 0;
      for (int t = 0; t < nt; ++t) sum += cnt[(size_t)t][(size_t)e];
      start[(size_t)e + 1] = start[(size_t)e] + sum;
    }
    std::vector<int32_t> list((size_t)std::max<int64_t>(start[(size_t)ne], 1));
    // thread t's first slot of element e: start[e] plus the counts of the slabs before it
    for (int64_t e = 0; e < ne; ++e) {
      int64_t at = start[(size_t)e];
      for (int t = 0; t < nt; ++t) {
        const int32_t n_te = cnt[(size_t)t][(size_t)e];
        cnt[(size_t)t][(size_t)e] = (int32_t)(at - start[(size_t)e]);
        at += n_te;
      }
    }
    run_threads([&](int t) {
      int k0, k1;
      slab_of(t, k0, k1);
      int32_t *ct = cnt[(size_t)t].data();
      for (int K = k0; K < k1; ++K)
        for (int J = 1; J < g.nyg - 1; ++J) {
          const int64_t base = (int64_t)K * g.nxyg + (int64_t)J * g.nxg;
          const int32_t *row = htag.data() + base;
          for (int I = 1; I < g.nxg - 1; ++I) {
            const int32_t e = row[I];
            if (e >= 0) list[(size_t)(start[(size_t)e] + ct[e]++)] = (int32_t)(base + I);
          }
        }
    });
    int64_t *es = alloc<int64_t>(start.size());
    int32_t *el = alloc<int32_t>(list.size());
    h2d(es, start.data(), start.size() * 8);
    h2d(el, list.data(), list.size() * 4);
    RCK(cudaStreamSynchronize(stream_));
    d.ecell_start = es;
    d.ecell = el;
  }
  // --- frames ---
  d.nframes = (int)nframes_;
  d.bad_frame = (int)frames_.bad_frame;
  d.dt_cap = INFINITY;
  d.t_stop = INFINITY;
  d.external = 0;
  if (frames_src_ == 3 || text_stream_) {
    // a ring of window + 4 frame slots (and their times), refilled a window at a
    // time as the run reaches its end
    window_ = 32;
    if (const char *e = getenv("AMCA_FRAME_WINDOW")) window_ = std::max(2, atoi(e));
    slots_ = (int)std::min<int64_t>(nframes_, window_ + 4);
    ring_ = alloc<double>((size_t)slots_ * d.nnodes);
    ftime_ = alloc<double>((size_t)slots_);
    d.frames = ring_;
    d.frame_time = ftime_;
    d.frame_slots = slots_;
    if (text_stream_) {
      void *st = nullptr;
      RCK(cudaHostAlloc(&st, (size_t)(window_ + 2) * d.nnodes * 8, cudaHostAllocDefault));
      staging_ = (double *)st;
      // frame 0 came with the grid; the reader continues from frame 1
      times_read_.assign(1, frames_.times[0]);
      RCK(cudaMemcpyAsync(ring_, frames_.theta.data(), (size_t)d.nnodes * 8, cudaMemcpyHostToDevice, stream_));
      RCK(cudaMemcpyAsync(ftime_, &times_read_[0], 8, cudaMemcpyHostToDevice, stream_));
      RCK(cudaStreamSynchronize(stream_));
      avail_ = 1;
      d.frames_avail = 1;
    } else {
      fcount_ = alloc<unsigned long long>(4);
      RCK(cudaMemsetAsync(fcount_, 0, 4 * sizeof(unsigned long long), stream_));
      avail_ = 0;
    }
    fill_frames(window_ + 2);  // sets d.frames_avail (d is dev_)
    if (avail_ < 2) throw std::runtime_error(dev_.bad_frame == 1 ? std::string(
        "fail to read next step temperature file, please check title of line!!") :
        std::string("the temperature file holds fewer than two frames"));
    if (text_stream_) frames_.times = times_read_;  // the first window's times (ts0, ts1 below)
  } else {
    double *ftime = alloc<double>(nframes_);
    h2d(ftime, frames_.times.data(), nframes_ * 8);
    d.frame_time = ftime;
    double *frames = alloc<double>((size_t)nframes_ * d.nnodes);
    if (frames_src_ == 2) {
      RCK(remelt_rosenthal_frames(ros_, (int)nframes_, frames, stream_));
    } else {
      h2d(frames, frames_.theta.data(), frames_.theta.size() * 8);
    }
    d.frames = frames;
    d.frame_slots = (int)nframes_;
    d.frames_avail = (int)nframes_;
  }
  for (int i = 0; i < 3; ++i) {
    d.theta[i] = alloc<double>(d.nnodes);
    d.theta32[i] = alloc<float>(d.nnodes);
  }
  d.emax = alloc<double>(d.nelem);
  d.emin = alloc<double>(d.nelem);
  d.evoid = alloc<uint8_t>(d.nelem);
  d.eliq = alloc<int32_t>(d.nelem);
  for (int sl = 0; sl < 2; ++sl) {
    d.fmax[sl] = alloc<double>(d.nelem);
    d.fmin[sl] = alloc<double>(d.nelem);
    d.fnear[sl] = alloc<uint8_t>(d.nelem);
  }
  d.eact[0] = alloc<int32_t>(d.nelem);
  d.eact[1] = alloc<int32_t>(d.nelem);
  // --- cells ---
  d.orient = alloc<int32_t>(N);
  d.grain = alloc<int32_t>(N);
  d.melted = alloc<uint8_t>(N);
  d.flagbits = alloc<uint32_t>((N + 31) / 32);
  d.tcls = alloc<uint8_t>(N);
  d.gx = alloc<double>(N);
  d.gy = alloc<double>(N);
  d.gz = alloc<double>(N);
  d.glen = alloc<double>(N);
  d.gori = alloc<int32_t>(N);
  d.gdx = alloc<float>(N);
  d.gdy = alloc<float>(N);
  d.gdz = alloc<float>(N);
  d.list_cap = N;
  d.liq = alloc<int32_t>(N);
  d.flagged[0] = alloc<int32_t>(N);
  d.flagged[1] = alloc<int32_t>(N);
  d.claimed = alloc<int32_t>(N);
  d.newkey = alloc<unsigned long long>(kNewGrainCap);
  d.newcell = alloc<int32_t>(kNewGrainCap);
  d.fvel = alloc<double>(N);
  d.hard_idx = alloc<int32_t>(N);
  d.hard_T = alloc<double>(N);
  {
    void *hv = nullptr;
    RCK(cudaHostAlloc(&hv, sizeof(HostVelocity), cudaHostAllocMapped));
    hostvel_ = (HostVelocity *)hv;
    memset(hostvel_, 0, sizeof(HostVelocity));
    void *dv = nullptr;
    RCK(cudaHostGetDevicePointer(&dv, hv, 0));
    d.host = (HostVelocity *)dv;
    // entries one request may use; AMCA_HOST_VEL_CAP (tests) makes it small
    // so that steps take the chunked path
    d.host_cap = kHostVelCap;
    if (const char *e = getenv("AMCA_HOST_VEL_CAP")) d.host_cap = std::min(kHostVelCap, std::max(2, atoi(e)));
  }
  // --- orientations and sites ---
  orient_cap_ = (int64_t)otab_.euler.size() / 3;
  omat_ = alloc<double>(9 * orient_cap_);
  omat32_ = alloc<float>(9 * orient_cap_);
  h2d(omat_, otab_.l2g.data(), otab_.l2g.size() * 8);
  h2d(omat32_, otab_.l2g32.data(), otab_.l2g32.size() * 4);
  d.omat = omat_;
  d.omat32 = omat32_;
  d.orient_cap = orient_cap_;
  d.nsites = (int)sites_.cell.size();
  int32_t *sc = alloc<int32_t>(d.nsites);
  double *sd = alloc<double>(d.nsites);
  h2d(sc, sites_.cell.data(), sites_.cell.size() * 4);
  h2d(sd, sites_.dtc.data(), sites_.dtc.size() * 8);
  d.site_cell = sc;
  d.site_dtc = sd;
  d.snuc = alloc<uint8_t>(d.nsites);
  d.ctrl = alloc<RemeltCtrl>(1);
  // --- control block: CafeSolver::time_integration_weak_coupling set-up (CafeSolver.cpp:182-184) ---
  RemeltCtrl c0{};
  c0.ts1 = frames_.times[0];
  c0.ts0 = frames_.times[1];
  c0.f_new = 1;
  c0.f_next = 2;
  c0.theta_init = 1;
  c0.dT_FE = c0.ts0 - c0.ts1;  // FiniteElementManager::setup_integration
  c0.max_ts = c0.dT_FE;        // CellularAutomataManager::setup_integration
  c0.n_orient = n_init_orient_;
  c0.n_grains = n_init_grains_;
  c0.minT_key = host_dkey(c.Tm);
  c0.fstat_frame[0] = c0.fstat_frame[1] = -1;
  ctrl0_ = c0;
  upload_initial_state();
  {
    // blocks per SM of the persistent kernel; AMCA_REMELT_BLOCKS_PER_SM overrides the default for tuning
    int per_sm = 1;
    if (const char *e = getenv("AMCA_REMELT_BLOCKS_PER_SM")) per_sm = std::max(1, atoi(e));
    blocks_ = remelt_persistent_grid(device_, per_sm);
  }
  if (blocks_ <= 0) throw CudaError("no co-resident blocks for the persistent remelting kernel");
  vtr_.configure(c.output, workdir_);
  if (opts_.write_outputs) vtr_.make_dirs();  // VtrManager::initialize
  initialized_ = true;
}

void RemeltRealm::reset() {
  if (!initialized_) throw StateError("amca_reset before amca_initialize");
  if (text_stream_) {  // read the file again from its start
    open_text_frames();
    RCK(cudaMemcpyAsync(ring_, reader_->head().theta.data(), (size_t)dev_.nnodes * 8, cudaMemcpyHostToDevice,
                        stream_));
    RCK(cudaMemcpyAsync(ftime_, &times_read_[0], 8, cudaMemcpyHostToDevice, stream_));
    RCK(cudaStreamSynchronize(stream_));
    avail_ = 1;
    dev_.frames_avail = 1;
    fill_frames(window_ + 2);
  } else if (frames_src_ == 3 && avail_ > window_ + 2) {  // the ring has moved on: produce the first window again
    avail_ = 0;
    dev_.frames_avail = 0;
    fill_frames(window_ + 2);
  }
  dev_.external = 0;
  dev_.dt_cap = INFINITY;
  dev_.t_stop = INFINITY;
  ext_ready_ = false;
  upload_initial_state();
  kernel_ms_ = 0.0;
  launches_ = 0;
  vtr_ = VtrSeries();
  vtr_.configure(cfg_.ca.output, workdir_);
}

void RemeltRealm::sync_ctrl() {
  d2h(&ctrl_, dev_.ctrl, sizeof ctrl_);
  RCK(cudaStreamSynchronize(stream_));
  if (ctrl_.error) {
    static const char *msg[] = {"",
                                "grid barrier wait timed out",
                                "fail to read next step temperature file, please check title of line!!",
                                "more new grain objects in one step than the library supports (16384)",
                                "time ratio error: timeRatio is less then 0",
                                "work list overflow",
                                "the host did not answer a velocity request in time",
                                "a frame was needed before it was loaded"};
    const int e = ctrl_.error;
    throw DeviceError(std::string("remelting kernel stopped: ") + (e > 0 && e < 8 ? msg[e] : "unknown error"));
  }
}

void RemeltRealm::extend_orientations() {
  const int64_t K = std::max<int64_t>(4 * (int64_t)sites_.cell.size(), 1024);
  OrientationTable more = make_orientations(K, *rng_);
  append_orientations(otab_, more);
  const int64_t cap = (int64_t)otab_.euler.size() / 3;
  double *m = alloc<double>(9 * cap);
  float *m32 = alloc<float>(9 * cap);
  RCK(cudaMemcpyAsync(m, omat_, 9 * orient_cap_ * 8, cudaMemcpyDeviceToDevice, stream_));
  RCK(cudaMemcpyAsync(m32, omat32_, 9 * orient_cap_ * 4, cudaMemcpyDeviceToDevice, stream_));
  h2d(m + 9 * orient_cap_, more.l2g.data(), more.l2g.size() * 8);
  h2d(m32 + 9 * orient_cap_, more.l2g32.data(), more.l2g32.size() * 4);
  RCK(cudaStreamSynchronize(stream_));
  omat_ = m;
  omat32_ = m32;
  orient_cap_ = cap;
  dev_.omat = m;
  dev_.omat32 = m32;
  dev_.orient_cap = cap;
}

// The reference's growth velocity with glibc's pow
// (ProblemPhysics_RappazGandin1993::compute_growth_velocity_with_temperature_input,
// CA/src/ProblemPhysics.cpp:142-158), for the arguments the kernel cannot round itself.
static double reference_velocity(const PlainConfig &c, double T) {
  const double dT = c.Tm - T;
  double v = 0.0;
  if (dT > 0) {
    v = c.a1 * std::pow(dT, c.b1) + c.a2 * std::pow(dT, c.b2) + c.a3 * std::pow(dT, c.b3);
    if (v < 0.0) v = 0.0;
  }
  return v;
}

// Runs beside a kernel launch: answers the kernel's velocity requests.
void RemeltRealm::serve_velocities(const volatile int *stop, int w, int workers, VelocityJob *job, unsigned last) {
  HostVelocity *hv = hostvel_;
  // worker 0 watches the device's request word and hands each request to all
  // workers; every worker spins (yielding when idle for long) on the job word.
  // `last` is what each has served before the launch (read before any thread
  // starts: a worker that started after the first request was posted would
  // otherwise take that request as served and never count it off)
  unsigned idle = 0;
  while (!*stop) {
    unsigned r;
    if (w == 0) {
      r = __atomic_load_n(&hv->seq_req, __ATOMIC_ACQUIRE);
      if (r != last) {
        const unsigned n = std::min(__atomic_load_n(&hv->n, __ATOMIC_ACQUIRE), (unsigned)kHostVelCap);
        // small requests are not worth waking the others
        const int use = n >= 64u ? workers : 1;
        job->n.store(n, std::memory_order_relaxed);
        job->left.store((unsigned)use, std::memory_order_relaxed);
        if (use > 1) job->seq.store(r, std::memory_order_release);
        for (unsigned i = 0; i < n; i += (unsigned)use) hv->v[i] = reference_velocity(cfg_.ca, hv->T[i]);
        if (job->left.fetch_sub(1, std::memory_order_acq_rel) != 1)
          while (job->left.load(std::memory_order_acquire) != 0 && !*stop) {
          }
        __atomic_store_n(&hv->seq_done, r, __ATOMIC_RELEASE);
        last = r;
        idle = 0;
        continue;
      }
    } else {
      r = job->seq.load(std::memory_order_acquire);
      if (r != last) {
        const unsigned n = job->n.load(std::memory_order_relaxed);
        for (unsigned i = (unsigned)w; i < n; i += (unsigned)workers) hv->v[i] = reference_velocity(cfg_.ca, hv->T[i]);
        job->left.fetch_sub(1, std::memory_order_acq_rel);
        last = r;
        idle = 0;
        continue;
      }
    }
    if (++idle > 4096) std::this_thread::yield();
  }
}

void RemeltRealm::set_nodal_temperatures(const double *theta, int64_t n) {
  if (!initialized_) throw StateError("amca_set_nodal_temperatures before amca_initialize");
  if (n != dev_.nnodes)
    throw std::invalid_argument("amca_set_nodal_temperatures: " + std::to_string(dev_.nnodes) + " node values needed");
  if (!ext_theta_) ext_theta_ = alloc<double>((size_t)dev_.nnodes);
  h2d(ext_theta_, theta, (size_t)n * 8);
  const int par = (int)(ctrl_.step & 1);
  RCK(cudaMemsetAsync(&dev_.ctrl->n_eact[par], 0, sizeof(unsigned), stream_));
  RCK(remelt_external_theta(dev_, ctrl_.step, ext_theta_, stream_));
  RCK(cudaStreamSynchronize(stream_));
  dev_.external = 1;
  ext_ready_ = true;
}

void RemeltRealm::step_coupled(double dt_cap) {
  if (!initialized_) throw StateError("amca_step before amca_initialize");
  const double cap = dt_cap > 0 ? dt_cap : INFINITY;
  if (dev_.external) {
    // the external solver's step is the FE time step of the coupling (dT_FE and the CA's maxTimestep_)
    h2d(&dev_.ctrl->dT_FE, &cap, sizeof cap);
    h2d(&dev_.ctrl->max_ts, &cap, sizeof cap);
  }
  dev_.dt_cap = cap;
  try {
    run(1);
  } catch (...) {
    dev_.dt_cap = INFINITY;
    throw;
  }
  dev_.dt_cap = INFINITY;
}

void RemeltRealm::run_until(double t_end) {
  if (!initialized_) throw StateError("amca_run before amca_initialize");
  if (dev_.external) throw StateError("node temperatures come from the caller: advance step by step");
  dev_.t_stop = t_end;
  try {
    run(-1);
  } catch (...) {
    dev_.t_stop = INFINITY;
    throw;
  }
  dev_.t_stop = INFINITY;
}

void RemeltRealm::run(long long max_steps) {
  if (!initialized_) throw StateError("amca_run before amca_initialize");
  if (dev_.external) {
    if (!ext_ready_) throw StateError("call amca_set_nodal_temperatures before each step");
    if (max_steps != 1) throw StateError("node temperatures come from the caller: advance step by step");
  }
  if (ctrl_.status == kRemeltTimeStop) ctrl_.status = kRemeltRunning;
  const long long target = max_steps < 0 ? (1ll << 60) : ctrl_.step + max_steps;
  const OutputConfig &oc = cfg_.ca.output;
  while (ctrl_.status != kRemeltFinalTime && ctrl_.status != kRemeltFramesEnd && ctrl_.status != kRemeltTimeStop &&
         ctrl_.step < target) {
    long long limit = target;
    if (opts_.write_outputs) {  // VtrManager::execute after every step (Remelting.cpp:640)
      if (oc.frequency >= 1)
        limit = std::min(limit, (ctrl_.step / oc.frequency + 1) * (long long)oc.frequency);
      else if (oc.time_interval_set && oc.time_interval > 0)
        limit = std::min(limit, ctrl_.step + 1);
    }
    const long long before = ctrl_.step;
    launch(limit);
    if (ctrl_.status == kRemeltNeedOrient) {
      extend_orientations();
      continue;
    }
    if (ctrl_.status == kRemeltNeedFrames) {
      fill_frames(avail_ + window_);
      continue;
    }
    if (opts_.write_outputs && ctrl_.step != before && vtr_.due((int)ctrl_.step, ctrl_.time)) write_snapshot();
  }
  if (dev_.external) ext_ready_ = false;  // the handed-in node temperatures are used up
}

void RemeltRealm::launch(long long limit) {
  {
    const int running = kRemeltRunning;
    h2d(&dev_.ctrl->status, &running, sizeof running);
    volatile int stop = 0;
    // the hard velocities of one step (a few hundred glibc pow calls) are
    // split over a few spinning host threads
    const int hw = (int)std::thread::hardware_concurrency();
    const int workers = std::max(1, std::min(8, hw / 2));
    VelocityJob job;
    const unsigned done0 = __atomic_load_n(&hostvel_->seq_done, __ATOMIC_ACQUIRE);
    std::vector<std::thread> servers;
    for (int w = 0; w < workers; ++w)
      servers.emplace_back([&, w] { serve_velocities(&stop, w, workers, &job, w == 0 ? done0 : 0u); });
    RCK(cudaEventRecord(ev0_, stream_));
    cudaError_t le = remelt_run_steps(dev_, limit, blocks_, stream_);
    if (le == cudaSuccess) le = cudaEventRecord(ev1_, stream_);
    if (le == cudaSuccess) le = cudaStreamSynchronize(stream_);
    stop = 1;
    for (std::thread &t : servers) t.join();
    if (le != cudaSuccess) throw CudaError(std::string("remelting kernel: ") + cudaGetErrorString(le));
    ++launches_;
    sync_ctrl();
    float ms = 0.f;
    RCK(cudaEventElapsedTime(&ms, ev0_, ev1_));
    kernel_ms_ += ms;
  }
}

void RemeltRealm::get_field(int field, void *dst, size_t bytes) {
  if (!initialized_) throw StateError("amca_get_field before amca_initialize");
  const size_t N = (size_t)dev_.ncells;
  auto need = [&](size_t b) {
    if (bytes != b) throw std::invalid_argument("amca_get_field: wrong byte count for this field");
  };
  switch (field) {
    case AMCA_FIELD_ORIENTATION_ID:
      need(N * 4);
      d2h(dst, dev_.orient, N * 4);
      RCK(cudaStreamSynchronize(stream_));
      return;
    case AMCA_FIELD_GRAIN_ID:
      need(N * 4);
      d2h(dst, dev_.grain, N * 4);
      RCK(cudaStreamSynchronize(stream_));
      return;
    case AMCA_FIELD_SITE_UNDERCOOLING:
      need(N * 8);
      memcpy(dst, site_field().data(), N * 8);
      return;
    case AMCA_FIELD_MELTED:
      need(N);
      d2h(dst, dev_.melted, N);
      RCK(cudaStreamSynchronize(stream_));
      return;
    case AMCA_FIELD_TEMPERATURE:
    case AMCA_FIELD_COOLING:
    case AMCA_FIELD_LIQUID_NEIGHBOUR: {
      const bool t = field == AMCA_FIELD_TEMPERATURE;
      need(t ? N * 8 : N);
      if (ctrl_.step == 0) {  // before the first step: nullMatTemp_, false, false
        if (t) {
          double *o = (double *)dst;
          for (size_t i = 0; i < N; ++i) o[i] = -1.0;
        } else {
          memset(dst, 0, N);
        }
        return;
      }
      void *buf = nullptr;
      RCK(cudaMalloc(&buf, t ? N * 8 : N));
      cudaError_t e = remelt_state_fields(dev_, ctrl_.step, ctrl_.dt_prev, t ? (double *)buf : nullptr,
                                          field == AMCA_FIELD_COOLING ? (uint8_t *)buf : nullptr,
                                          field == AMCA_FIELD_LIQUID_NEIGHBOUR ? (uint8_t *)buf : nullptr, stream_);
      if (e == cudaSuccess) e = cudaMemcpyAsync(dst, buf, t ? N * 8 : N, cudaMemcpyDeviceToHost, stream_);
      if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
      cudaFree(buf);
      if (e != cudaSuccess) throw CudaError(std::string("state fields: ") + cudaGetErrorString(e));
      d2h_bytes_ += (int64_t)(t ? N * 8 : N);
      return;
    }
    default:
      throw std::invalid_argument("amca_get_field: unknown field");
  }
}

size_t RemeltRealm::orientations(double *euler, size_t cap, int all) const {
  const size_t n = all ? otab_.euler.size() / 3 : (size_t)std::max<long long>(0, ctrl_.n_orient);
  if (euler) memcpy(euler, otab_.euler.data(), std::min(n, cap) * 3 * sizeof(double));
  return n;
}

double RemeltRealm::algorithmic_bytes() const {
  // 8 B per cell the phase update visits (orientation + element tag); per
  // exact temperature 33 B (parametric coordinates 24, temperature 8, flag 1);
  // per listed liquid cell 104 B (26 neighbour states); per flagged cell
  // 364 B (grain record 48, 26 x (state 4 + temperature 8)); per capture 80 B
  // (winner record 36, new record 36, state 8); per step and node 24 B (two
  // frame values, one write) and per element 21 B (bounds, void flag, liquid
  // count).
  const double steps = (double)ctrl_.step;
  return 8 * (double)ctrl_.cells_visited + 33 * (double)ctrl_.exact_T + 104 * (double)ctrl_.liquid +
         364 * (double)ctrl_.flagged + 80 * (double)ctrl_.captures +
         (24 * (double)dev_.nnodes + 21 * (double)dev_.nelem) * steps;
}

void RemeltRealm::stats(amca_stats *s) const {
  memset(s, 0, sizeof *s);
  const RemeltCtrl &c = ctrl_;
  s->step = c.step;
  s->time = c.time;
  s->dt = c.dt;
  s->liquid_cells = -1;
  s->grains = c.n_grains;
  s->orientations = c.n_orient;
  s->active = (int64_t)c.flagged;
  s->sites = (int64_t)sites_.cell.size();
  s->cells = (int64_t)cfg_.ca.nx * cfg_.ca.ny * cfg_.ca.nz;
  s->tests = (int64_t)c.tests;
  s->tests_fp64 = (int64_t)c.tests64;
  s->generations = (int64_t)c.exact_T;
  s->done = (c.status == kRemeltFinalTime || c.status == kRemeltFramesEnd) ? 1 : 0;
  s->kernel_ms = kernel_ms_;
  s->launches = launches_;
  s->sites_scanned = (int64_t)c.elements_active;
  s->nucleations = (int64_t)c.nucleations;
  s->captures = (int64_t)c.captures;
  s->active_grown = (int64_t)c.cells_visited;
  s->grains_processed = (int64_t)c.liquid;
  s->reserved = (int32_t)std::min<unsigned long long>(c.host_calls, 0x7fffffff);
  s->algorithmic_bytes = algorithmic_bytes();
  s->h2d_bytes = h2d_bytes_;
  s->d2h_bytes = d2h_bytes_;
  for (int i = 0; i < 5; ++i) s->phase_ms[i] = c.ns_phase[i] * 1e-6;
  s->phase_ms[5] = c.ns_host * 1e-6;
  s->phase_ms[6] = c.ns_barrier * 1e-6;
  const double nb = blocks_ > 0 ? (double)blocks_ : 1.0;
  for (int i = 0; i < 6; ++i) {
    s->detail_ms[i] = c.ns_work_sum[i] * 1e-6 / nb;
    s->detail_ms[6 + i] = c.ns_work_max[i] * 1e-6;
  }
  s->detail_ms[12] = c.ns_newgrain * 1e-6;
  s->detail_ms[13] = c.ns_nucleation * 1e-6;
  s->detail_ms[14] = c.ns_flags_max * 1e-6;
}

int RemeltRealm::final_grain_count() {
  std::vector<int32_t> o((size_t)dev_.ncells);
  get_field(AMCA_FIELD_ORIENTATION_ID, o.data(), o.size() * 4);
  const int64_t n = ctrl_.n_orient;
  if (n <= 0) return 0;
  std::vector<char> seen((size_t)n, 0);
  for (int32_t v : o)
    if (v > -1 && v < n) seen[v] = 1;
  return (int)std::count(seen.begin(), seen.end(), 1);
}

RemeltRealm::Fields RemeltRealm::fetch_fields(bool grain) {
  Fields f;
  const size_t N = (size_t)dev_.ncells;
  f.orient.resize(N);
  get_field(AMCA_FIELD_ORIENTATION_ID, f.orient.data(), N * 4);
  f.melted.resize(N);
  get_field(AMCA_FIELD_MELTED, f.melted.data(), N);
  f.temperature.resize(N);
  get_field(AMCA_FIELD_TEMPERATURE, f.temperature.data(), N * 8);
  if (grain) {
    f.grain.resize(N);
    get_field(AMCA_FIELD_GRAIN_ID, f.grain.data(), N * 4);
  }
  return f;
}

OutputView RemeltRealm::view(const Fields &f) const {
  const PlainConfig &c = cfg_.ca;
  OutputView v{};
  v.nx = c.nx;
  v.ny = c.ny;
  v.nz = c.nz;
  v.x0 = c.x0;
  v.y0 = c.y0;
  v.z0 = c.z0;
  v.h = c.h;
  v.orient = f.orient.data();
  v.euler = otab_.euler.data();
  v.n_orient = ctrl_.n_orient;
  v.mapped_vtr = (c.shuffle_vtr && !mapped_vtr_.empty()) ? &mapped_vtr_ : nullptr;
  v.shuffle_vtk = c.shuffle_vtk;
  v.expected_grains = expected_grains_;
  v.melted = f.melted.data();
  v.temperature = f.temperature.data();
  return v;
}

void RemeltRealm::write_snapshot() {
  Fields f = fetch_fields(false);
  vtr_.make_dirs();
  vtr_.write(view(f), ctrl_.time);
}

// CafeSolver::finalize (CA/src/CafeSolver.cpp:224-261): the restart file when
// asked for, the last VTR snapshot (output_last_step_result), finalGrains.vtk
// and finalResult.txt (output_orientations).
void RemeltRealm::write_outputs() {
  if (!initialized_) throw StateError("amca_write_outputs before amca_initialize");
  const PlainConfig &c = cfg_.ca;
  Fields f = fetch_fields(c.micro_out);
  OutputView v = view(f);
  std::vector<double> gx, gy, gz;
  std::vector<int32_t> gori, gcell;
  if (c.micro_out) {
    // grain table: a grain's record lives with the interior cell that owns it
    const size_t N = (size_t)dev_.ncells;
    std::vector<double> x(N), y(N), z(N);
    std::vector<int32_t> o(N);
    d2h(x.data(), dev_.gx, N * 8);
    d2h(y.data(), dev_.gy, N * 8);
    d2h(z.data(), dev_.gz, N * 8);
    d2h(o.data(), dev_.gori, N * 4);
    RCK(cudaStreamSynchronize(stream_));
    const int64_t ng = ctrl_.n_grains;
    gcell.assign((size_t)ng, -1);
    for (int64_t g = 0; g < (int64_t)grain_cell_.size() && g < ng; ++g) gcell[g] = grain_cell_[g];
    const int nxg = c.nx + 2, nyg = c.ny + 2, nzg = c.nz + 2;
    const int64_t nxyg = (int64_t)nxg * nyg;
    std::vector<char> owned((size_t)ng, 0);
    for (size_t cell = 0; cell < N; ++cell) {
      const int32_t g = f.grain[cell];
      const int K = (int)(cell / nxyg), J = (int)((cell % nxyg) / nxg), I = (int)((cell % nxyg) % nxg);
      if (g < 0 || g >= ng || is_ghost(I, J, K, nxg, nyg, nzg)) continue;
      gcell[g] = (int32_t)cell;
      owned[g] = 1;
    }
    gx.resize((size_t)ng);
    gy.resize((size_t)ng);
    gz.resize((size_t)ng);
    gori.resize((size_t)ng);
    for (int64_t g = 0; g < ng; ++g) {
      const int64_t cell = gcell[g];
      if (owned[g]) {
        gx[g] = x[cell];
        gy[g] = y[cell];
        gz[g] = z[cell];
        gori[g] = o[cell];
      } else {  // never touched: as loaded, centred on its cell
        const int K = (int)(cell / nxyg), J = (int)((cell % nxyg) / nxg), I = (int)((cell % nxyg) % nxg);
        gx[g] = centre_coord(c.x0, c.h, I);
        gy[g] = centre_coord(c.y0, c.h, J);
        gz[g] = centre_coord(c.z0, c.h, K);
        gori[g] = g < (int64_t)grain_ori0_.size() ? grain_ori0_[g] : -1;
      }
    }
    v.grain = f.grain.data();
    v.site_dtc = site_field().data();
    v.n_grains = ng;
    v.gx = gx.data();
    v.gy = gy.data();
    v.gz = gz.data();
    v.gori = gori.data();
    v.gcell = gcell.data();
    write_grain_info(v, path(c.micro_out_file));
  }
  std::vector<int32_t> mapped_vtk;
  if (c.shuffle_vtk) {  // writeToFile's shuffle draws from the glibc stream where the run left it
    int maxVal = -1;
    for (int k = 1; k <= c.nz; ++k)
      for (int j = 1; j <= c.ny; ++j)
        for (int i = 1; i <= c.nx; ++i)
          maxVal = std::max(maxVal, (int)f.orient[((int64_t)k * (c.ny + 2) + j) * (c.nx + 2) + i]);
    GlibcRand rng(opts_.seed);
    const int64_t skip = init_draws_ + 3 * (ctrl_.n_orient - n_init_orient_);
    for (int64_t i = 0; i < skip; ++i) rng.next();
    mapped_vtk = make_mapped_ids(maxVal + 1, true, rng);
    v.mapped_vtk = &mapped_vtk;
  }
  if (vtr_.due(0, ctrl_.time)) {
    vtr_.make_dirs();
    vtr_.write(v, ctrl_.time);
  }
  write_final_grains(v, path("finalGrains.vtk"), vtr_.pvd_path());
}

}  // namespace amca
