// host_init.cpp — see host_init.h. Built with -ffp-contract=off.
#include "host_init.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <stdexcept>
#include <thread>
#include <unordered_map>

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
  // every draw in draw order: (cell, dTc, population); a cell keeps the
  // smallest dTc of its draws and counts for the population of its first
  // draw (create_nucleation_sites' map of chosen cells, shared by both
  // populations)
  struct Draw {
    int32_t cell;
    int32_t pop;  // 0 surface, 1 bulk
    double dtc;
  };
  std::vector<Draw> draws;
  SiteSet out;
  auto population = [&](double density, double mean, double sigma, bool surface) {
    // Surface list (CA/src/CellularAutomataManager_3D.cpp:958-1000): ascending
    // ghost-inclusive id, a face cell listed once per face it lies on (z, x,
    // y faces). Rows with J == nx+1 are skipped: the reference tests
    // locGhostJ against nxLocGhost_-1. A row that touches a z or y face lists
    // all its cells, the others only their two x ends. Entry q is found from
    // per-row counts instead of materialising the list.
    std::vector<int64_t> row_end;  // cumulative entry count after each (K, J) row, K outer
    int64_t numCells64 = 0;
    auto row_base = [&](int K, int J) { return (K == 1 || K == c.nz ? 1 : 0) + (J == 1 || J == c.ny ? 1 : 0); };
    if (surface && density != 0.0) {  // a zero density draws no site whatever the list holds
      row_end.reserve((size_t)c.nz * c.ny);
      for (int K = 1; K <= c.nz; ++K)
        for (int J = 1; J <= c.ny; ++J) {
          int64_t m = 0;
          if (J != nxg - 1) {
            const int bb = row_base(K, J);
            m = bb > 0 ? (int64_t)bb * c.nx + (c.nx == 1 ? 1 : 2) : (c.nx == 1 ? 1 : 2);
          }
          numCells64 += m;
          row_end.push_back(numCells64);
        }
    } else if (!surface) {
      // the bulk list is every interior cell in k, j, i order; entry q is
      // computed instead of stored
      numCells64 = (int64_t)c.nx * c.ny * c.nz;
    }
    auto surface_cell = [&](int64_t q) {
      const int64_t r = std::upper_bound(row_end.begin(), row_end.end(), q) - row_end.begin();
      const int K = (int)(r / c.ny) + 1, J = (int)(r % c.ny) + 1;
      const int64_t p = q - (r > 0 ? row_end[r - 1] : 0);
      const int bb = row_base(K, J);
      int I;
      if (bb == 0 || c.nx == 1) {
        I = (p == 0 || c.nx == 1) ? 1 : c.nx;  // the two x ends (one cell when nx == 1)
      } else if (p < bb + 1) {
        I = 1;  // bb + 1 entries at I = 1
      } else if (p - (bb + 1) < (int64_t)bb * (c.nx - 2)) {
        I = 2 + (int)((p - (bb + 1)) / bb);  // bb entries at each inner I
      } else {
        I = c.nx;
      }
      return (int32_t)(K * nxyg + (int64_t)J * nxg + I);
    };
    auto bulk_cell = [&](int64_t q) {
      const int64_t k = q / ((int64_t)c.nx * c.ny) + 1, j = (q / c.nx) % c.ny + 1, i = q % c.nx + 1;
      return (int32_t)(k * nxyg + j * nxg + i);
    };
    const double per_cell = surface ? c.h * c.h : c.h * c.h * c.h;
    const int numCells = (int)numCells64;
    const int numSites = density == 0.0 ? 0 : (int)(round(per_cell * density * numCells) + 0.5);
    std::default_random_engine generator;
    std::normal_distribution<double> distribution(mean, sigma);
    if (numSites > 0 && numCells == 0) throw std::runtime_error("nucleation sites requested on an empty cell set");
    draws.reserve(draws.size() + (size_t)std::max(numSites, 0));
    for (int s = 0; s < numSites; ++s) {
      const int q = rng.next() % numCells;
      const int32_t cell = surface ? surface_cell(q) : bulk_cell(q);
      double dT = distribution(generator);
      dT = (dT < 0) ? 0 : dT;
      draws.push_back(Draw{cell, surface ? 0 : 1, dT});
    }
  };
  (void)ncells;
  population(c.ns, c.mu_s, c.sigma_s, true);
  population(c.nv, c.mu_v, c.sigma_v, false);
  // ascending cell id; within a cell, draw order: a least-significant-digit
  // radix sort on the cell id (0 <= cell < 2^33 covered by three stable 11-bit
  // passes), which keeps equal cells in draw order like a stable sort
  {
    std::vector<Draw> tmp(draws.size());
    std::vector<size_t> count(2049);
    for (int pass = 0; pass < 3; ++pass) {
      const int shift = 11 * pass;
      std::fill(count.begin(), count.end(), 0);
      for (const Draw &x : draws) ++count[(((uint32_t)x.cell >> shift) & 2047u) + 1];
      for (size_t b = 1; b < count.size(); ++b) count[b] += count[b - 1];
      for (const Draw &x : draws) tmp[count[((uint32_t)x.cell >> shift) & 2047u]++] = x;
      draws.swap(tmp);
    }
  }
  out.surface_sites = 0;
  out.bulk_sites = 0;
  out.cell.reserve(draws.size());
  out.dtc.reserve(draws.size());
  for (size_t i = 0; i < draws.size();) {
    size_t j = i + 1;
    double dtc = draws[i].dtc;
    for (; j < draws.size() && draws[j].cell == draws[i].cell; ++j) dtc = std::min(dtc, draws[j].dtc);
    out.cell.push_back(draws[i].cell);
    out.dtc.push_back(dtc);
    (draws[i].pop == 0 ? out.surface_sites : out.bulk_sites) += 1;
    i = j;
  }
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

void orientation_matrix(const double a[3], double m[9], float m32[9]) {
  // Octahedron::set_coordinate_transformation_matrix (CA/src/Octahedron.cpp:282-310)
  const double ca = std::cos(a[0]), sa = std::sin(a[0]);
  const double cb = std::cos(a[1]), sb = std::sin(a[1]);
  const double cg = std::cos(a[2]), sg = std::sin(a[2]);
  m[0] = ca * cg - sa * cb * sg;
  m[1] = -ca * sg - sa * cb * cg;
  m[2] = sa * sb;
  m[3] = sa * cg + ca * cb * sg;
  m[4] = -sa * sg + ca * cb * cg;
  m[5] = -ca * sb;
  m[6] = sb * sg;
  m[7] = sb * cg;
  m[8] = cb;
  for (int q = 0; q < 9; ++q) m32[q] = (float)m[q];
}

namespace {
// Run body(lo, hi) over [0, n) on up to hardware_concurrency threads.
template <typename F>
void parallel_ranges(int64_t n, F body) {
  // one thread per 2048 items at most: the per-item work (glibc libm
  // trigonometry) is a few hundred ns, a thread start a few tens of us
  unsigned nt = std::max(1u, std::thread::hardware_concurrency());
  nt = (unsigned)std::min<int64_t>(nt, std::max<int64_t>(1, n / 2048));
  nt = (unsigned)std::min<int64_t>(nt, 64);
  std::vector<std::thread> th;
  const int64_t chunk = (n + nt - 1) / nt;
  for (unsigned t = 1; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo < hi) th.emplace_back([=] { body(lo, hi); });
  }
  body(0, std::min(n, chunk));
  for (auto &x : th) x.join();
}
}  // namespace

OrientationTable make_orientations(int64_t n, GlibcRand &rng) {
  const double kPi = 3.14159265358979323846;  // CellularAutomataManager_3D.cpp:24
  OrientationTable t;
  t.euler.resize((size_t)n * 3);
  t.l2g.resize((size_t)n * 9);
  t.l2g32.resize((size_t)n * 9);
  // get_random_orientation_angle (CellularAutomataManager_3D.cpp:839-850):
  // three rand() per orientation, in draw order; the trigonometry is
  // independent per orientation and runs on all host threads.
  std::vector<int32_t> r((size_t)n * 3);
  for (int64_t q = 0; q < 3 * n; ++q) r[q] = rng.next();
  parallel_ranges(n, [&](int64_t lo, int64_t hi) {
    for (int64_t o = lo; o < hi; ++o) {
      double U, V;
      U = static_cast<double>(r[3 * o]) / RAND_MAX;
      V = static_cast<double>(r[3 * o + 1]) / RAND_MAX;
      double *a = &t.euler[o * 3];
      a[0] = U * 2 * kPi;
      a[1] = std::acos(2 * V - 1);
      a[2] = static_cast<double>(r[3 * o + 2]) / RAND_MAX * 0.5 * kPi;
      orientation_matrix(a, &t.l2g[o * 9], &t.l2g32[o * 9]);
    }
  });
  return t;
}

OrientationTable orientations_from_euler(const std::vector<double> &euler) {
  OrientationTable t;
  const int64_t n = (int64_t)euler.size() / 3;
  t.euler = euler;
  t.l2g.resize((size_t)n * 9);
  t.l2g32.resize((size_t)n * 9);
  parallel_ranges(n, [&](int64_t lo, int64_t hi) {
    for (int64_t o = lo; o < hi; ++o) orientation_matrix(&t.euler[o * 3], &t.l2g[o * 9], &t.l2g32[o * 9]);
  });
  return t;
}

void append_orientations(OrientationTable &t, const OrientationTable &more) {
  t.euler.insert(t.euler.end(), more.euler.begin(), more.euler.end());
  t.l2g.insert(t.l2g.end(), more.l2g.begin(), more.l2g.end());
  t.l2g32.insert(t.l2g32.end(), more.l2g32.begin(), more.l2g32.end());
}

}  // namespace amca
