/*
 * State probe for the shimmed reference build (test infrastructure only).
 *
 * Linked into oracle/_ref/amca3d_np1_dump together with the UNMODIFIED
 * reference objects, with -Wl,--wrap=_ZN10VtrManager7executeEid: the
 * reference calls VtrManager::execute(iStep_, time_) at the end of every CA
 * step (CellularAutomataManager_3DRemelting.cpp:640,
 * CellularAutomataManager_3D.cpp single_integration_step), so the wrapper sees
 * the realm's complete state after each step. When AMCA_DUMP is set it
 * appends that state to the file it names; the reference's own VTR output
 * then runs unchanged.
 *
 * Record layout (little-endian, one record per CA step):
 *   char[4] "AMCD"; i32 step; f64 time, dT_, maxTimestep_;
 *   i32 ncells, ngrains, norient, nnodes;
 *   i32 orient[ncells]; i32 grain[ncells]; f64 T[ncells];
 *   u8 cooling[ncells]; u8 melted[ncells]; u8 liquid_neigh[ncells];
 *   per grain: i32 id, cell, orient; u8 active; f64 xc, yc, zc, length;
 *   f64 euler[3*norient]; f64 theta[nnodes]  (FE nodal temperatures used
 *   by this step's phase update).
 * The first record is preceded by "AMCT", i32 ncells, i32 tag[ncells],
 * f64 parcoords[3*ncells] (MapVoxelManager element tags and parametric
 * coordinates).
 *
 * Member access: the reference keeps this state protected/private, so the
 * reference headers are included with the access keywords mapped to public.
 * This changes no layout (GCC lays out members in declaration order
 * regardless of access) and no reference source.
 */
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <list>
#include <map>
#include <random>
#include <sstream>
#include <string>
#include <vector>

#include "mpi.h"
#include "yaml-cpp/yaml.h"
#include "boost/filesystem.hpp"
#include "boost/program_options.hpp"

#define private public
#define protected public
#include "CellularAutomataManager_3DRemelting.h"
#include "FiniteElementManager.h"
#include "Grain.h"
#include "MapVoxelManager.h"
#include "Orientation.h"
#include "VtrManager.h"
#undef private
#undef protected

/* VtrManager::execute(int, double) under its linker name; `this` is the first
 * argument in the x86-64 and AArch64 C++ ABIs. */
extern "C" bool __real__ZN10VtrManager7executeEid(VtrManager *self, int numStep, double time);

static void put(FILE *f, const void *p, size_t n) {
  if (n && fwrite(p, 1, n, f) != n) {
    fprintf(stderr, "state_dump: write failed\n");
    exit(3);
  }
}

static bool g_tags_written = false;

static void dump_state(CellularAutomataManager_3D *ca, FILE *f) {
  const int n = ca->numLocGhostCells_;
  MapVoxelManager *mv = ca->mapVoxelManager_;
  if (!g_tags_written) {
    g_tags_written = true;
    put(f, "AMCT", 4);
    put(f, &n, 4);
    std::vector<int32_t> tag(n, -1);
    std::vector<double> pc(3 * (size_t)n, -2.0);
    if (mv && mv->elementTagList_) {
      for (int i = 0; i < n; ++i) tag[i] = mv->elementTagList_[i];
      for (size_t i = 0; i < 3 * (size_t)n; ++i) pc[i] = mv->parCoordsList_[i];
    }
    put(f, tag.data(), 4 * (size_t)n);
    put(f, pc.data(), 8 * 3 * (size_t)n);
  }
  put(f, "AMCD", 4);
  int32_t step = ca->iStep_;
  put(f, &step, 4);
  put(f, &ca->time_, 8);
  put(f, &ca->dT_, 8);
  put(f, &ca->maxTimestep_, 8);
  int32_t ng = (int32_t)ca->grainVector_.size();
  int32_t no = (int32_t)ca->orientationVector_.size();
  FiniteElementManager *fe = mv ? mv->feManager_ : 0;
  int32_t nn = (fe && fe->thetaArray_) ? fe->numNodes_ : 0;
  put(f, &n, 4);
  put(f, &ng, 4);
  put(f, &no, 4);
  put(f, &nn, 4);
  put(f, ca->cellOrientationID_, 4 * (size_t)n);
  put(f, ca->cellGrainID_, 4 * (size_t)n);
  std::vector<double> T(n, 0.0);
  std::vector<uint8_t> b(n, 0);
  if (ca->cellTemperature_)
    for (int i = 0; i < n; ++i) T[i] = ca->cellTemperature_[i];
  put(f, T.data(), 8 * (size_t)n);
  for (int i = 0; i < n; ++i) b[i] = ca->cooling_ ? (uint8_t)ca->cooling_[i] : 0;
  put(f, b.data(), n);
  for (int i = 0; i < n; ++i) b[i] = (i < (int)ca->hasBeenMelted_.size()) ? (uint8_t)ca->hasBeenMelted_[i] : 0;
  put(f, b.data(), n);
  for (int i = 0; i < n; ++i) b[i] = (i < (int)ca->cellLiquidNeigh.size()) ? (uint8_t)ca->cellLiquidNeigh[i] : 0;
  put(f, b.data(), n);
  for (int g = 0; g < ng; ++g) {
    Grain *gr = ca->grainVector_[g];
    int32_t rec[3] = {gr->id_, gr->cell_, gr->orientation_ ? gr->orientation_->id_ : -1};
    uint8_t act = gr->active_ ? 1 : 0;
    double geo[4] = {gr->xc_, gr->yc_, gr->zc_, gr->length_};
    put(f, rec, sizeof rec);
    put(f, &act, 1);
    put(f, geo, sizeof geo);
  }
  for (int o = 0; o < no; ++o) put(f, ca->orientationVector_[o]->EulerAngle_, 24);
  if (nn) put(f, fe->thetaArray_, 8 * (size_t)nn);
}

/* Which calls to record. By default every call. For runs too large to record
 * every step, AMCA_DUMP_EVERY=N keeps only the CA steps that are multiples of
 * N and AMCA_DUMP_FINAL=1 keeps the call that output_last_step_result makes
 * at the end (VtrManager::execute(0, time) once the realm has stepped,
 * CellularAutomataManager_3D.cpp:1990-1993); with either set, only the
 * selected calls are recorded. */
static bool selected(CellularAutomataManager_3D *ca, int numStep) {
  const char *every = getenv("AMCA_DUMP_EVERY");
  const char *fin = getenv("AMCA_DUMP_FINAL");
  const long n = every ? atol(every) : 0;
  const bool want_final = fin && *fin == '1';
  if (n <= 0 && !want_final) return true;
  if (numStep == 0 && ca->iStep_ > 0) return want_final;
  return n > 0 && ca->iStep_ % n == 0;
}

extern "C" bool __wrap__ZN10VtrManager7executeEid(VtrManager *self, int numStep, double time) {
  const char *path = getenv("AMCA_DUMP");
  if (path && *path && selected(self->caManager_, numStep)) {
    FILE *f = fopen(path, "ab");
    if (!f) {
      fprintf(stderr, "state_dump: cannot open %s\n", path);
      exit(3);
    }
    dump_state(self->caManager_, f);
    fclose(f);
  }
  return __real__ZN10VtrManager7executeEid(self, numStep, time);
}
