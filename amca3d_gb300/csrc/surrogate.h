// surrogate.h — the learned thermal model of the FE-coupled path: a
// Fourier-feature MLP that maps (along-track offset from the laser, lateral
// offset, depth below the top surface, laser power, scan speed) to a
// temperature and an error estimate, trained and evaluated on the tensor
// cores by the kernels of surrogate.cu.
//
// Network: u = (raw - shift) * scale (5 inputs); 64 phases f_j = B_j . u
// (in turns, B fixed from the seed); features [sin 2 pi f_j, cos 2 pi f_j]
// (128); four hidden layers 128 -> 256 -> 256 -> 256 -> 256 with SiLU; head
// 256 -> 2 giving mu and s. Temperature T = t_shift + t_scale * mu (or
// t_shift + t_scale * exp(mu)); error estimate 2 * |dT/dmu| * exp(s) (K).
// Hidden-layer GEMMs take bf16 operands and accumulate in FP32; the head runs
// in FP32 on the FP32 activations.
//
// What it stands in for: the nodal temperatures the FE realm hands to
// MapVoxelManager::evaluate_temperature (CA/src/MapVoxelManager.cpp:746-799)
// at every CA step (CA/src/CafeSolver.cpp:179-219); the reference has no
// learned component.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/amca3d.h"

namespace amca {

constexpr int kSurIn = 5, kSurFreq = 64, kSurEnc = 128, kSurHid = 256, kSurLayers = 4, kSurOut = 2;

// Offsets of the FP32 master parameters (one vector, Adam state alike).
struct SurParamLayout {
  int64_t W[kSurLayers], b[kSurLayers], Wh, bh, total;
  __host__ __device__ static constexpr int in_dim(int l) { return l == 0 ? kSurEnc : kSurHid; }
  __host__ __device__ SurParamLayout() {
    int64_t o = 0;
    for (int l = 0; l < kSurLayers; ++l) {
      W[l] = o;
      o += (int64_t)kSurHid * in_dim(l);
      b[l] = o;
      o += kSurHid;
    }
    Wh = o;
    o += (int64_t)kSurOut * kSurHid;
    bh = o;
    o += kSurOut;
    total = o;
  }
};

// Device view of a model for the kernels.
struct SurModelDev {
  const float *fourier;                 // kSurFreq x kSurIn
  const float *p;                       // FP32 master parameters (SurParamLayout)
  const __nv_bfloat16 *Wb[kSurLayers];  // bf16 copies, [out][in]
  float in_shift[kSurIn], in_scale[kSurIn];
  float t_shift, t_scale;
  int log_out;  // T = t_shift + t_scale * exp(mu) instead of t_shift + t_scale * mu
};

// The moving source of the synthetic FE field and of the model's inputs: a
// raster of ntracks passes along x with alternating direction, track k at
// y_line + k * hatch, each track_time long; on even tracks the source moves
// in +x from x_start, on odd tracks in -x from x_turn. The Rosenthal field of
// the current pass (t0 + A P / (2 pi k R) exp(-v (R + xi) / (2 alpha)),
// xi = (x - x_laser) * direction, capped at t_cap) is the FE field.
struct ScanSource {
  double power, absorptivity, speed, conductivity, diffusivity, t0, t_cap;
  double x_start, x_turn, y_line, z_top, hatch, track_time;
  int ntracks;
};

struct ThermalModel;  // surrogate.cu

// Frames f0 .. f0 + nf - 1 of a scan into ring slots (frame f at slot
// f % slots of nnodes doubles each) on stream s: the FE field of the scan
// (model == nullptr) or the model's frames with the fallback rule (nodes whose
// model temperature is within band of t_liq and whose error estimate exceeds
// thresh take the FE field). counters (device, 4 words, may be null for the
// FE field) accumulate: nodes evaluated by the model, near the liquidus,
// fallbacks.
void fill_scan_frames(const amca_scan *scan, ThermalModel *model, double t_liq, double band, double thresh, int f0,
                      int nf, double *ring, int slots, unsigned long long *counters, cudaStream_t s);
// The model behind an amca_thermal handle.
ThermalModel *thermal_model_of(void *handle);

// Laser position, direction and track at time t (s).
__host__ __device__ inline void scan_position(const ScanSource &s, double t, double &xl, double &yl, double &dir) {
  int k = 0;
  double tl = t;
  if (s.ntracks > 1 && s.track_time > 0) {
    k = (int)(t / s.track_time);
    if (k < 0) k = 0;
    if (k > s.ntracks - 1) k = s.ntracks - 1;
    tl = t - k * s.track_time;
  }
  dir = (k & 1) ? -1.0 : 1.0;
  xl = (k & 1) ? s.x_turn - s.speed * tl : s.x_start + s.speed * tl;
  yl = s.y_line + k * s.hatch;
}

}  // namespace amca
