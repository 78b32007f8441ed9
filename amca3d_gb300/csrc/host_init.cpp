// host_init.cpp — see host_init.h. Built with -ffp-contract=off.
#include "host_init.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>

namespace amca {

GlibcRand::GlibcRand(unsigned seed) {
  std::memset(&data_, 0, sizeof data_);
  std::memset(state_, 0, sizeof state_);
  // 128 bytes selects TYPE_3, the state rand() uses; srandom_r(seed) as srand
  if (initstate_r(seed, state_, sizeof state_, &data_) != 0) throw std::runtime_error("initstate_r failed");
}

int GlibcRand::next() {
  int32_t r = 0;
  random_r(&data_, &r);
  ++draws_;
  return (int)r;
}

SiteSet make_sites(const PlainConfig &c, GlibcRand &rng) {
  const int nxg = c.nx + 2, nyg = c.ny + 2, nzg = c.nz + 2;
  const int64_t nxyg = (int64_t)nxg * nyg, ncells = nxyg * nzg;
  std::vector<double> dtc_of;  // cellNucleationDT_, -1 = no site (allocated lazily)
  std::vector<int32_t> sites;
  SiteSet out;
  auto population = [&](double density, double mean, double sigma, bool surface) {
    std::vector<int32_t> ids;
    if (surface) {
      // every ghost-inclusive cell; a face cell is listed once per face it lies
      // on. The y test compares against nxLocGhost_-1 as the reference does.
      for (int64_t i = 0; i < ncells; ++i) {
        const int K = (int)(i / nxyg);
        if (K == 0 || K == nzg - 1) continue;
        const int I = (int)((i % nxyg) % nxg);
        if (I == 0 || I == nxg - 1) continue;
        const int J = (int)((i % nxyg) / nxg);
        if (J == 0 || J == nxg - 1) continue;
        if (K == 1 || K == c.nz)
          if (I != 0 && I != c.nx + 1 && J != 0 && J != c.ny + 1) ids.push_back((int32_t)i);
        if (I == 1 || I == c.nx)
          if (J != 0 && J != c.ny + 1 && K != 0 && K != c.nz + 1) ids.push_back((int32_t)i);
        if (J == 1 || J == c.ny)
          if (I != 0 && I != c.nx + 1 && K != 0 && K != c.nz + 1) ids.push_back((int32_t)i);
      }
    } else {
      ids.reserve((size_t)c.nx * c.ny * c.nz);
      for (int k = 1; k < nzg - 1; ++k)
        for (int j = 1; j < nyg - 1; ++j)
          for (int i = 1; i < nxg - 1; ++i) ids.push_back((int32_t)(k * nxyg + (int64_t)j * nxg + i));
    }
    const double per_cell = surface ? c.h * c.h : c.h * c.h * c.h;
    const int numCells = (int)ids.size();
    const int numSites = round(per_cell * density * numCells) + 0.5;
    std::default_random_engine generator;
    std::normal_distribution<double> distribution(mean, sigma);
    int64_t generated = 0;
    if (numSites > 0 && numCells == 0) throw std::runtime_error("nucleation sites requested on an empty cell set");
    for (int s = 0; s < numSites; ++s) {
      const int cell = ids[rng.next() % numCells];
      double dT = distribution(generator);
      dT = (dT < 0) ? 0 : dT;
      if (dtc_of.empty()) dtc_of.assign((size_t)ncells, -1.0);
      const double cur = dtc_of[cell];
      if (cur < 0) {
        sites.push_back(cell);
        dtc_of[cell] = dT;
        ++generated;
      } else if (dT < cur) {
        dtc_of[cell] = dT;
      }
    }
    std::sort(sites.begin(), sites.end());
    (surface ? out.surface_sites : out.bulk_sites) = generated;
  };
  population(c.ns, c.mu_s, c.sigma_s, true);
  population(c.nv, c.mu_v, c.sigma_v, false);
  out.cell = sites;
  out.dtc.resize(sites.size());
  for (size_t i = 0; i < sites.size(); ++i) out.dtc[i] = dtc_of[sites[i]];
  return out;
}

std::vector<int32_t> make_mapped_ids(int64_t n, bool shuffle, GlibcRand &rng) {
  std::vector<int32_t> m((size_t)n);
  for (int64_t i = 0; i < n; ++i) m[i] = (int32_t)i;
  if (shuffle && n > 1) {
    // libstdc++ std::random_shuffle(first, last): j = rand() % (i + 1)
    for (int64_t i = 1; i < n; ++i) {
      const int64_t j = rng.next() % (i + 1);
      if (i != j) std::swap(m[i], m[j]);
    }
  }
  return m;
}

OrientationTable make_orientations(int64_t n, GlibcRand &rng) {
  const double kPi = 3.14159265358979323846;  // CellularAutomataManager_3D.cpp:24
  OrientationTable t;
  t.euler.resize((size_t)n * 3);
  t.l2g.resize((size_t)n * 9);
  t.l2g32.resize((size_t)n * 9);
  for (int64_t o = 0; o < n; ++o) {
    double U, V;
    U = static_cast<double>(rng.next()) / RAND_MAX;
    V = static_cast<double>(rng.next()) / RAND_MAX;
    double *a = &t.euler[o * 3];
    a[0] = U * 2 * kPi;
    a[1] = std::acos(2 * V - 1);
    a[2] = static_cast<double>(rng.next()) / RAND_MAX * 0.5 * kPi;
    const double ca = std::cos(a[0]), sa = std::sin(a[0]);
    const double cb = std::cos(a[1]), sb = std::sin(a[1]);
    const double cg = std::cos(a[2]), sg = std::sin(a[2]);
    double *m = &t.l2g[o * 9];
    m[0] = ca * cg - sa * cb * sg;
    m[1] = -ca * sg - sa * cb * cg;
    m[2] = sa * sb;
    m[3] = sa * cg + ca * cb * sg;
    m[4] = -sa * sg + ca * cb * cg;
    m[5] = -ca * sb;
    m[6] = sb * sg;
    m[7] = sb * cg;
    m[8] = cb;
    for (int q = 0; q < 9; ++q) t.l2g32[o * 9 + q] = (float)m[q];
  }
  return t;
}

}  // namespace amca
