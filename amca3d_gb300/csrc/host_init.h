// host_init.h — host-side set-up of a plain CA realm: nucleation sites and
// the orientation stream.
//
// These steps draw from glibc's rand() stream and libstdc++'s
// std::normal_distribution, exactly as the reference does, so they run on
// the host with the same libraries rather than on the GPU:
//   create_nucleation_sites   CA/src/CellularAutomataManager.cpp:153-213
//   get_surface_cells / bulk  CA/src/CellularAutomataManager_3D.cpp:935-1000
//   global_mapped_grain_ID    CA/src/CellularAutomataManager.cpp:471-518
//   orientation angles        CA/src/CellularAutomataManager_3D.cpp:839-850
//   rotation matrix           CA/src/Octahedron.cpp:282-310
#pragma once

#include <stdint.h>
#include <stdlib.h>

#include <vector>

#include "deck.h"

namespace amca {

// glibc rand() with private state: random_r over a TYPE_3 state seeded like
// srand(seed), so the library never touches the process-wide rand() state.
class GlibcRand {
 public:
  explicit GlibcRand(unsigned seed);
  int next();
  int64_t draws() const { return draws_; }

 private:
  int64_t draws_ = 0;
  struct random_data data_;
  char state_[128];
};

struct SiteSet {
  std::vector<int32_t> cell;  // ascending ghost-inclusive cell id
  std::vector<double> dtc;    // critical undercooling
  int64_t surface_sites = 0;  // numSitesSurface_
  int64_t bulk_sites = 0;     // numSitesBulk_
};

struct OrientationTable {
  std::vector<double> euler;  // 3 per orientation
  std::vector<double> l2g;    // 9 per orientation (transMatrixLocal2Global)
  std::vector<float> l2g32;   // the same, rounded to float
};

// Sites of one realm, drawn surface first, then bulk, from `rng`.
SiteSet make_sites(const PlainConfig &c, GlibcRand &rng);

// mappedGrainID (identity, shuffled with std::random_shuffle's loop when the
// deck asks for shuffled VTR ids); consumes rand() values like the reference.
std::vector<int32_t> make_mapped_ids(int64_t n, bool shuffle, GlibcRand &rng);

// Orientation stream: n orientations, 3 rand() values each, in draw order.
OrientationTable make_orientations(int64_t n, GlibcRand &rng);

// Matrices of given Euler angles (restart files).
OrientationTable orientations_from_euler(const std::vector<double> &euler);
void append_orientations(OrientationTable &t, const OrientationTable &more);

// Octahedron::set_coordinate_transformation_matrix for one orientation.
void orientation_matrix(const double euler[3], double l2g[9], float l2g32[9]);

}  // namespace amca
