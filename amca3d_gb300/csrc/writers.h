// writers.h — AMCA3D's ASCII grain output, byte for byte.
//
//   VTR piece / PVTR / PVD collection   CA/src/VtrManager.cpp:186-561, CA/src/VtkManager.cpp:67-262
//   finalGrains.vtk + finalResult.txt   CA/src/CellularAutomataManager_3D.cpp:1221-1639
//   grainInfo<rank>.txt                 CA/src/CellularAutomataManager_3D.cpp:1836-1913
#pragma once

#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "deck.h"

namespace amca {

// Everything the writers read about one realm, on the host.
struct OutputView {
  int nx, ny, nz;
  double x0, y0, z0, h;
  const int32_t *orient;  // ghost-inclusive cellOrientationID_
  const int32_t *grain;   // ghost-inclusive cellGrainID_ (grainInfo only)
  const double *site_dtc; // ghost-inclusive cellNucleationDT_ (grainInfo only)
  const double *euler;    // 3 per orientation
  int64_t n_orient;
  const std::vector<int32_t> *mapped_vtr;  // shuffled ids, or nullptr
  bool shuffle_vtk;
  const std::vector<int32_t> *mapped_vtk;  // shuffle for finalGrains.vtk, or nullptr
  // grainInfo: envelope table (host copies)
  int64_t n_grains;
  const double *gx, *gy, *gz;
  const int32_t *gori, *gcell;
  int64_t expected_grains;  // numSitesSurface_ + numSitesBulk_
  // remelting realm: hasBeenMelted_ and cellTemperature_ (ghost-inclusive);
  // nullptr for the plain realm (melted flags report 1, no temperature output)
  const uint8_t *melted = nullptr;
  const double *temperature = nullptr;
};

// VtrManager state across calls (numOutputStep_, timeVec_, time threshold).
class VtrSeries {
 public:
  void configure(const OutputConfig &o, const std::string &workdir);
  // VtkManager::output_result: whether step/time triggers an output
  bool due(int step, double time);
  // Creates the directories VtrManager::initialize makes (when frequency != 0).
  void make_dirs() const;
  // VtrManager::execute body for a due step
  void write(const OutputView &v, double time);
  const std::string &pvd_path() const { return pvd_path_; }

 private:
  OutputConfig cfg_;
  bool by_freq_ = true;
  double threshold_ = 1.0e8;
  int num_output_ = 0;
  int pvtk_num_ = 0;
  std::string pvd_path_, pvd_name_;
  std::vector<std::pair<int, double>> times_;
};

// finalGrains.vtk (at `vtk_path`) and <pvd_path>/finalResult.txt
void write_final_grains(const OutputView &v, const std::string &vtk_path, const std::string &pvd_path);

// grainInfo<rank>.txt next to `file_name` (rank 0)
void write_grain_info(const OutputView &v, const std::string &file_name);

}  // namespace amca
