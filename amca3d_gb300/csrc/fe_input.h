// fe_input.h — host-side inputs of the FE-coupled remelting realm.
//
//   temperature frames   FiniteElementManager::load_mesh_and_first_two_steps_results_from_txt_file,
//                        load_next_step_nodal_data (CA/src/LoadDataFromFile.cpp:21-191)
//   restart file         CellularAutomataManager_3DRemelting::load_microstructure_information
//                        (CA/src/CellularAutomataManager_3DRemelting.cpp:164-307)
//   FE -> CA map set-up  MapVoxelManager::get_CA_domain_xyz_min_max, attach_elements
//                        (CA/src/MapVoxelManager.cpp:140-352); the per-voxel search
//                        (tag_voxels / is_in_element) runs on the GPU.
#pragma once

#include <stdint.h>

#include <memory>
#include <string>
#include <vector>

#include "deck.h"

namespace amca {

// A structured hex mesh and its temperature frames, as the reference holds
// them after reading: coordinates are (file value + offset) * length_scale;
// frame f's time is (t_f - t_0) * time_scale (inTimeSeries_); theta is
// frame-major (nframes x nnodes).
struct FeFrames {
  int nn[3] = {0, 0, 0};
  int64_t nnodes = 0;
  std::vector<double> coord;   // 3 per node, x fastest node order
  std::vector<double> times;   // per frame
  std::vector<double> theta;   // per frame, per node
  int64_t nframes = 0;
  // A malformed frame stops the reference with an exception when it is
  // reached; bad_frame is its index (-1: none) and bad_msg the message.
  int64_t bad_frame = -1;
  std::string bad_msg;

  int64_t nelem() const { return (int64_t)(nn[0] - 1) * (nn[1] - 1) * (nn[2] - 1); }
};

// Read the whole frame file. Throws std::runtime_error when the first two
// frames cannot be read (the reference fails in load()).
FeFrames read_fe_frames(const std::string &path, const FeConfig &fe);

// The same reader a frame at a time, for files read while the run goes on:
// the constructor reads the title, the node grid and frame 0 (head()); next()
// reads the following frame (load_next_step_nodal_data,
// CA/src/LoadDataFromFile.cpp:143-191) into out (nnodes values) with its
// scaled time, and returns false at the end of the file or at a malformed
// frame (then bad() is true and bad_msg() has the reference's message).
class FrameReader {
 public:
  FrameReader(const std::string &path, const FeConfig &fe);
  ~FrameReader();
  const FeFrames &head() const { return head_; }
  bool next(double *out, double &t);
  bool bad() const { return bad_; }
  const std::string &bad_msg() const { return bad_msg_; }
  int64_t frames_read() const { return read_; }

 private:
  struct Impl;
  std::unique_ptr<Impl> impl_;
  FeFrames head_;
  int64_t read_ = 0;
  bool done_ = false, bad_ = false;
  std::string bad_msg_;
};

// Frames from memory, in file units (same transformation as the reader).
FeFrames fe_frames_from_arrays(const int32_t nodes[3], const double *coords, int64_t nframes, const double *times,
                               const double *theta, const FeConfig &fe);

// Node ids of element e (LoadDataFromFile.cpp:104-131).
inline void fe_elem_nodes(const int nn[3], int64_t e, int64_t nid[8]) {
  const int64_t ncx = nn[0] - 1, ncy = nn[1] - 1;
  const int64_t i = e % ncx, j = (e / ncx) % ncy, k = e / (ncx * ncy);
  const int64_t nxy = (int64_t)nn[0] * nn[1];
  nid[0] = nxy * k + (int64_t)nn[0] * j + i;
  nid[1] = nid[0] + 1;
  nid[2] = nid[1] + nn[0];
  nid[3] = nid[2] - 1;
  for (int l = 4; l < 8; l++) nid[l] = nid[l - 4] + nxy;
}

// The restart file grainInfo<rank>.txt.
struct RestartData {
  int64_t ncells = 0, norient = 0, ngrains = 0, expected = 0;
  std::vector<int32_t> grain, orient;  // per ghost-inclusive cell
  std::vector<uint8_t> melted;
  std::vector<double> dtc;             // nucleation undercooling column (-1: none)
  std::vector<double> euler;           // 3 per orientation
  std::vector<int32_t> gcell, gori;    // per grain
};

// Reads "<stem>0.txt" for the stem of `file_name` (text before the last dot).
RestartData read_restart(const std::string &file_name);

// Bins and the element list of the FE -> CA map (MapVoxelManager.cpp:140-352).
struct VoxelMapPlan {
  double mm[6];                  // xyzMinMax_ after get_CA_domain_xyz_min_max
  double dbin[3];
  int nbin[3];
  std::vector<int64_t> bin_start;   // CSR over bins (x fastest)
  std::vector<int32_t> bin_elems;   // attach order kept
  std::vector<double> erange;       // 6 per element: get_cell_xyz_min_max
  std::vector<uint8_t> around;      // Node::grainAround_
};

VoxelMapPlan plan_voxel_map(const FeFrames &fr, const PlainConfig &ca, const TransferConfig &tr);

}  // namespace amca
