// engine_remelt.h — host side of the FE-coupled remelting realm behind the C ABI.
//
// CafeSolver (CA/src/CafeSolver.cpp:40-219) with a finite_element realm that
// replays frames and a cellular_automata_remelting realm: parse the deck, read
// the frames and the restart file, draw the orientation stream and the sites
// with the reference's libraries, build the FE -> CA map on the GPU, run the
// persistent step kernel, and hand the reference's arrays back.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "../../include/amca3d.h"
#include "deck.h"
#include "fe_input.h"
#include "host_init.h"
#include "remelt.h"
#include "surrogate.h"
#include "writers.h"

namespace amca {

class RemeltRealm {
 public:
  RemeltRealm(RemeltConfig cfg, const amca_opts &opts, std::string workdir);
  ~RemeltRealm();

  const RemeltConfig &config() const { return cfg_; }
  // frame sources other than the deck's mesh file (before initialize)
  void set_frames(const int32_t nodes[3], const double *coords, int64_t nframes, const double *times,
                  const double *theta);
  void set_rosenthal(const RosenthalParams &p, int nframes, double time_offset);
  // frames of a raster scan produced on the GPU a window at a time: the FE
  // field (model == nullptr) or a thermal model with its fallback rule
  void set_scan(const amca_scan &scan, ThermalModel *model, double t_liq, double band, double thresh);
  // frames produced so far, window fills, and (model frames) nodes evaluated,
  // nodes near the liquidus, fallbacks
  void frame_stats(int64_t out[5]);
  // restart microstructure from memory (before prepare)
  void set_microstructure(RestartData r);

  void prepare();     // host tables: microstructure, sites, orientation stream
  void initialize();  // device state, frames, FE -> CA map
  void reset();       // back to the state right after initialize
  void run(long long max_steps);
  // coupling with an external solver: one step with dt also capped by dt_cap;
  // steps while time < t_end; node temperatures for the next step
  void step_coupled(double dt_cap);
  void run_until(double t_end);
  void set_nodal_temperatures(const double *theta, int64_t n);
  bool prepared() const { return prepared_; }
  bool initialized() const { return initialized_; }

  void get_field(int field, void *dst, size_t bytes);
  size_t orientations(double *euler, size_t cap, int all) const;
  void stats(amca_stats *s) const;
  int final_grain_count();
  void write_outputs();
  const SiteSet &sites() const { return sites_; }
  const RemeltCtrl &ctrl() const { return ctrl_; }
  int64_t frames_count() const { return nframes_; }

 private:
  template <typename T>
  T *alloc(size_t n);
  void h2d(void *dst, const void *src, size_t bytes);
  void d2h(void *dst, const void *src, size_t bytes);
  void sync_ctrl();
  void extend_orientations();
  void upload_initial_state();
  // Host side of the velocity requests: worker w of `workers` evaluates
  // entries w, w + workers, ... of each request; the last to finish answers.
  struct VelocityJob {
    std::atomic<unsigned> seq{0};   // request being served
    std::atomic<unsigned> n{0};     // its entry count
    std::atomic<unsigned> left{0};  // workers still evaluating it
  };
  void serve_velocities(const volatile int *stop, int w, int workers, VelocityJob *job, unsigned last);
  void launch(long long limit);
  void write_snapshot();
  // host copies of the output fields of the current state
  struct Fields {
    std::vector<int32_t> orient, grain;
    std::vector<uint8_t> melted;
    std::vector<double> temperature;
  };
  Fields fetch_fields(bool grain);
  OutputView view(const Fields &f) const;
  std::string path(const std::string &p) const;
  double algorithmic_bytes() const;

  RemeltConfig cfg_;
  amca_opts opts_{};
  std::string workdir_;
  bool prepared_ = false, initialized_ = false;
  // frame source
  int frames_src_ = 0;  // 0 deck file, 1 arrays, 2 Rosenthal generator, 3 scan (FE field or model), on a ring
  FeFrames frames_;
  RosenthalParams ros_{};
  int ros_nframes_ = 0;
  double ros_toff_ = 0.0;
  int64_t nframes_ = 0;
  // frame ring of source 3
  amca_scan scan_{};
  ThermalModel *model_ = nullptr;
  double t_liq_ = 0, band_ = 0, thresh_ = 0;
  double *ring_ = nullptr;
  int slots_ = 0, window_ = 0, avail_ = 0;
  int64_t fills_ = 0, produced_ = 0;
  unsigned long long *fcount_ = nullptr;  // device: model nodes evaluated, near the liquidus, fallbacks
  void synthetic_grid(const double origin[3], double spacing, const int32_t nodes[3], int nframes, double frame_dt,
                      double time_offset);
  void fill_frames(int upto);
  double *ext_theta_ = nullptr;  // device copy of the host's node temperatures
  // text frames read while the run goes on (large files, or AMCA_FRAME_STREAM=1)
  std::unique_ptr<FrameReader> reader_;
  bool text_stream_ = false;
  double *ftime_ = nullptr;        // device: frame times, slot f % slots_ on a ring
  double *staging_ = nullptr;      // page-locked: one window of text frames
  std::vector<double> times_read_;  // host: times of the text frames read so far
  void open_text_frames();
  bool ext_ready_ = false;       // node temperatures handed in for the next step
  std::unique_ptr<RestartData> micro_;  // set_microstructure
  // host tables
  std::unique_ptr<GlibcRand> rng_;
  OrientationTable otab_;          // initial orientations, then the nucleation stream
  int64_t n_init_orient_ = 0;
  int64_t n_init_grains_ = 0;
  SiteSet sites_;
  std::vector<int32_t> mapped_vtr_;
  std::vector<int32_t> orient0_, grain0_;  // initial cell fields
  std::vector<uint8_t> melted0_;
  std::vector<int32_t> gori0_;
  std::vector<int32_t> grain_cell_;  // grain id -> owning cell (restart + created)
  std::vector<int32_t> grain_ori0_;  // grain id -> initial orientation
  int64_t init_draws_ = 0;           // glibc rand() values consumed before the nucleation stream
  std::vector<double> site_field_;   // cellNucleationDT_, built on first use
  const std::vector<double> &site_field();
  int64_t expected_grains_ = 0;
  int64_t restart_sites_ = 0;
  // device
  int device_ = 0;
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  std::vector<std::pair<void *, size_t>> allocs_;  // device buffers and sizes, back to the device cache at the end
  RemeltDevice dev_{};
  RemeltCtrl ctrl_{};
  RemeltCtrl ctrl0_{};
  int blocks_ = 0;
  double kernel_ms_ = 0.0;
  long long launches_ = 0;
  int64_t h2d_bytes_ = 0, d2h_bytes_ = 0;
  HostVelocity *hostvel_ = nullptr;  // mapped page-locked buffer of the velocity service
  double *omat_ = nullptr;
  float *omat32_ = nullptr;
  int64_t orient_cap_ = 0;
  VtrSeries vtr_;
};

}  // namespace amca
