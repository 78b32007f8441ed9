// ca_math.h — envelope arithmetic of the CA step, shared by the CUDA kernels
// and the host engine.
//
// The FP64 routines reproduce AMCA3D's octahedron arithmetic bit for bit:
// the same operations in the same order, no fused multiply-add (device code
// is built with -fmad=false, host code with -ffp-contract=off), float square
// roots where the reference calls sqrtf on doubles.
//
//   cell centre        CA/src/CellularAutomataManager_3D.cpp:877-888
//   containment test   CA/src/Octahedron.cpp:99-128
//   decentred capture  CA/src/Octahedron.cpp:134-275, CA/src/CellularAutomataManager_3D.cpp:677-707
//   KGT velocity       CA/src/ProblemPhysics.cpp:118-135
//
// The FP32 containment pre-test decides a (cell, envelope) pair only when its
// rounding-error bound keeps it on one side of the FP64 boundary; otherwise
// the caller runs the FP64 test. Decisions therefore equal the FP64 ones.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define AMCA_HD __host__ __device__ __forceinline__
#else
#define AMCA_HD inline
#endif

#include <math.h>
#include <string.h>

namespace amca {

constexpr double kTheodorus = 1.732050807568877;  // CA/src/Octahedron.cpp:13

// Liquid cells hold -1 in the orientation field; during one generation of
// the capture sweep a liquid cell may instead hold a claim
// 0x80000000 | parity << 30 | rank (rank = position of the claiming envelope
// in the generation, which is ascending envelope id). Solid cells and the
// ghost layer hold an orientation id >= 0.
constexpr uint32_t kLiquid = 0xFFFFFFFFu;
constexpr uint32_t kClaimBit = 0x80000000u;
constexpr uint32_t kParityBit = 0x40000000u;
constexpr uint32_t kRankMask = 0x3FFFFFFFu;

AMCA_HD uint32_t claim_word(uint32_t parity, uint32_t rank) { return kClaimBit | (parity ? kParityBit : 0u) | rank; }
// liquid at the start of the current generation: -1, or a claim made in it
AMCA_HD bool is_liquid_now(uint32_t s, uint32_t parity) {
  return s == kLiquid || ((s & kClaimBit) && (((s & kParityBit) != 0) == (parity != 0)));
}

struct Grid {
  int nx, ny, nz;     // interior cells
  int nxg, nyg, nzg;  // with the ghost layer
  int nxyg;
  double x0, y0, z0, h;
};

// get_cell_center: x0 + h*(I - 0.5) with the ghost-inclusive index I.
AMCA_HD double centre_coord(double o, double h, int I) { return o + h * (I - 0.5); }

AMCA_HD void cell_ijk(const Grid &g, int64_t id, int &I, int &J, int &K) {
  K = (int)(id / g.nxyg);
  int r = (int)(id - (int64_t)K * g.nxyg);
  J = r / g.nxg;
  I = r - J * g.nxg;
}

// Neighbour n in 0..25 in the reference's k, j, i loop order
// (CA/src/CellularAutomataManager_3D.cpp:913-925).
AMCA_HD void nbr_offset(int n, int &di, int &dj, int &dk) {
  int m = n < 13 ? n : n + 1;  // skip the centre (index 13 of 27)
  dk = m / 9 - 1;
  dj = (m / 3) % 3 - 1;
  di = m % 3 - 1;
}

// cell_is_captured in FP64. l2g is transMatrixLocal2Global (row-major);
// the global->local matrix is its transpose, summed from 0 in component order.
AMCA_HD bool is_captured_f64(const double *l2g, double gcx, double gcy, double gcz, double length) {
  if (length == 0) return false;
  double cx = 0, cy = 0, cz = 0;
  cx += gcx * l2g[0];
  cy += gcx * l2g[1];
  cz += gcx * l2g[2];
  cx += gcy * l2g[3];
  cy += gcy * l2g[4];
  cz += gcy * l2g[5];
  cx += gcz * l2g[6];
  cy += gcz * l2g[7];
  cz += gcz * l2g[8];
  return fabs(cx) + fabs(cy) + fabs(cz) <= 1.0 * length;
}

// FP32 pre-test. Returns +1 (captured), 0 (not captured) or -1 (too close to
// the boundary for FP32: use is_captured_f64). gc* are the cell-centre offsets
// from the envelope centre in FP32; err is an absolute bound on their error
// per component; m32 is l2g rounded to float.
//
// Bound: |m_ij| <= 1, so each local coordinate is a 3-term dot product whose
// FP32 evaluation errs by at most 3*u*(|gx|+|gy|+|gz|) + 3*err (u = 2^-24),
// and the final sum of three absolute values adds 2*u*(its magnitude). The
// margin used is 2^-14 relative plus 8*err per component — orders of
// magnitude above that bound and the FP64 evaluation's own error.
//
// *lower receives a lower bound of the FP64 |c'|_1 (the same FP32 estimate
// less the margin's terms for the estimate itself, plus 2^-14 of it): an
// envelope whose half-diagonal stays below it cannot contain the cell.
AMCA_HD int captured_f32_lb(const float *m32, float gx, float gy, float gz, float err, float length, float *lower) {
  float cx = gx * m32[0] + gy * m32[3] + gz * m32[6];
  float cy = gx * m32[1] + gy * m32[4] + gz * m32[7];
  float cz = gx * m32[2] + gy * m32[5] + gz * m32[8];
  float s = fabsf(cx) + fabsf(cy) + fabsf(cz);
  float scale = fabsf(gx) + fabsf(gy) + fabsf(gz);
  float margin = 6.103515625e-05f * (3.0f * scale + length) + 24.0f * err;  // 2^-14
  *lower = s - (6.103515625e-05f * (3.0f * scale + s) + 24.0f * err);
  if (s < length - margin) return 1;
  if (s > length + margin) return 0;
  return -1;
}
AMCA_HD int captured_f32(const float *m32, float gx, float gy, float gz, float err, float length) {
  float lower;
  return captured_f32_lb(m32, gx, gy, gz, err, length, &lower);
}

// CA/src/Octahedron.cpp:27-84 tables
AMCA_HD double face_normal(int q, int i) {
  // normalVector[8][3]: (+x +y +z), (-x +y +z), (-x -y +z), (+x -y +z), then z negated
  const int sx = (q == 1 || q == 2 || q == 5 || q == 6) ? -1 : 1;
  const int sy = (q == 2 || q == 3 || q == 6 || q == 7) ? -1 : 1;
  const int sz = q >= 4 ? -1 : 1;
  return (double)(i == 0 ? sx : (i == 1 ? sy : sz));
}
AMCA_HD int face_corner(int q, int i) {
  // surfaceCorner[8][3] = {0,1,4},{1,2,4},{2,3,4},{3,0,4},{0,1,5},{1,2,5},{2,3,5},{3,0,5}
  const int f = q & 3;
  if (i == 2) return q < 4 ? 4 : 5;
  return (f + i) & 3;
}
AMCA_HD double corner_unit(int c, int j) {
  // cornerCoord[6][3] = +x, +y, -x, -y, +z, -z
  switch (c) {
    case 0: return j == 0 ? 1.0 : 0.0;
    case 1: return j == 1 ? 1.0 : 0.0;
    case 2: return j == 0 ? -1.0 : 0.0;
    case 3: return j == 1 ? -1.0 : 0.0;
    case 4: return j == 2 ? 1.0 : 0.0;
    default: return j == 2 ? -1.0 : 0.0;
  }
}
// Axis of corner c (+x +y -x -y +z -z).
AMCA_HD int corner_axis(int c) { return c < 4 ? (c & 1) : 2; }
AMCA_HD double dmin_ref(double a, double b) { return (b < a) ? b : a; }  // std::min
AMCA_HD double dmax_ref(double a, double b) { return (a < b) ? b : a; }  // std::max

// Octahedron::capture_cell: the new, decentred envelope for a captured cell.
// gc = cell centre - parent centre (FP64). Writes the new centre offset
// (global frame) into out[0..2] and the new half-diagonal into out[3].
// Helpers that keep exact FP64 bookkeeping off the narrow FP64 pipe.
AMCA_HD long long f64_bits(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  long long b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}
// plus_zero(x) == x + 0.0 (a zero of either sign becomes +0).
AMCA_HD double plus_zero(double x) {
  const long long b = f64_bits(x);
  return b == (long long)0x8000000000000000ull ? 0.0 : x;
}
// nonneg(x) == (x >= 0) for x not NaN (-0 included).
AMCA_HD bool nonneg(double x) {
  const long long b = f64_bits(x);
  return b >= 0 || b == (long long)0x8000000000000000ull;
}
// corner_unit(c, corner_axis(c)) * length: +-length (exact: a sign flip).
AMCA_HD double corner_length(int c, double length) { return (c == 2 || c == 3 || c == 5) ? -length : length; }

// Octahedron::capture decentring (CA/src/Octahedron.cpp) in the reference's
// operation order. Where a term is a product with a corner coordinate (+-1 on
// one axis, 0 on the others) the zero terms are dropped and the +-1 products
// taken as sign flips; every such rewrite is bit-identical: a sum accumulated
// from +0.0 does not depend on the signs of its zero terms (+0 + -0 = +0,
// x + -0 = x), and squares and products of zeros are zeros.
AMCA_HD void capture_f64(const double *l2g, double gcx, double gcy, double gcz, double length, double h,
                         double trunc_coeff, double out[4]) {
  double cx = plus_zero(gcx * l2g[0]);  // 0 + p
  double cy = plus_zero(gcx * l2g[1]);
  double cz = plus_zero(gcx * l2g[2]);
  cx += gcy * l2g[3];
  cy += gcy * l2g[4];
  cz += gcy * l2g[5];
  cx += gcz * l2g[6];
  cy += gcz * l2g[7];
  cz += gcz * l2g[8];
  const double interception = fabs(cx) + fabs(cy) + fabs(cz);
  int quad = 0;
  const bool px = nonneg(cx), py = nonneg(cy);
  if (nonneg(cz)) {
    if (px && py) quad = 0;
    else if (px && !py) quad = 3;
    else if (!px && py) quad = 1;
    else quad = 2;
  } else {
    if (px && py) quad = 4;
    else if (px && !py) quad = 7;
    else if (!px && py) quad = 5;
    else quad = 6;
  }
  const double pC[3] = {cx, cy, cz};
  const double perp = length - interception;
  // (perp * n_i) / 3 with n_i = +-1 equals +-(perp / 3) exactly (IEEE
  // division is sign-symmetric), so one division serves all three terms
  const double third = perp / 3;
  double pA[3];
  for (int i = 0; i < 3; i++) pA[i] = pC[i] + (face_normal(quad, i) > 0 ? third : -third);
  // dist[i] = ((0 + d0^2) + d1^2) + d2^2 with d_j = pA[j] - corner_j * length:
  // on corner i's axis a, d_a = pA[a] -+ length; elsewhere d_j = pA[j]
  const double sq[3] = {pA[0] * pA[0], pA[1] * pA[1], pA[2] * pA[2]};
  double dist[3];
  for (int i = 0; i < 3; i++) {
    const int id = face_corner(quad, i);
    const int a = corner_axis(id);
    const double da = pA[a] - corner_length(id, length);
    const double t0 = a == 0 ? da * da : sq[0];
    const double t1 = a == 1 ? da * da : sq[1];
    const double t2 = a == 2 ? da * da : sq[2];
    dist[i] = (t0 + t1) + t2;
  }
  // distances are +0 or positive: their order is the order of their bits
  const long long b1 = f64_bits(dist[1]), b2 = f64_bits(dist[2]);
  int cid0 = face_corner(quad, 0), cid1, cid2;
  long long mind = f64_bits(dist[0]);
  // i = 1
  if (mind > b1) {
    mind = b1;
    cid1 = cid0;
    cid0 = face_corner(quad, 1);
  } else {
    cid1 = face_corner(quad, 1);
  }
  // i = 2
  if (mind > b2) {
    mind = b2;
    cid2 = cid0;
    cid0 = face_corner(quad, 2);
  } else {
    cid2 = face_corner(quad, 2);
  }
  // |S1S2|^2 = |S1S3|^2: the three corners of a face lie on three different
  // axes, so each edge vector is +-length on two axes and +0 on the third and
  // both sums are exactly fl(L*L) + fl(L*L). S1A . S1S2 and S1A . S1S3 keep
  // their two non-zero terms, in order.
  const int a0 = corner_axis(cid0), a1 = corner_axis(cid1), a2 = corner_axis(cid2);
  const double c1v = corner_length(cid0, length);  // S1 on its axis
  const double e1 = corner_length(cid1, length);   // S2 on its axis
  const double e2 = corner_length(cid2, length);   // S3 on its axis
  const double ll = length * length;
  double n12 = ll + ll;
  double d12 = 0.0, d13 = 0.0;
  for (int i = 0; i < 3; i++) {
    const double s1a = i == a0 ? pA[i] - c1v : pA[i];
    // S2 - S1 (and S3 - S1) on axis i: +e on S2's axis, -c1 on S1's, +0 elsewhere
    if (i == a1) d12 += s1a * e1;
    else if (i == a0) d12 += s1a * (0.0 - c1v);
    if (i == a2) d13 += s1a * e2;
    else if (i == a0) d13 += s1a * (0.0 - c1v);
  }
  n12 = (double)sqrtf((float)n12);
  const double n13 = n12;
  double I0 = d12 / n12, I1 = n12 - I0;
  const double J0 = d13 / n13, J1 = n13 - J0;
  const double tv = trunc_coeff * h;
  if (I0 < tv && I1 < tv) {
    I0 = n12 * 0.5;  // == n12 / 2 exactly
    I1 = n13 * 0.5;
  }
  const double L1 = 0.5 * (dmin_ref(I0, tv) + dmin_ref(I1, tv));
  const double L2 = 0.5 * (dmin_ref(J0, tv) + dmin_ref(J1, tv));
  const double Lnew = (double)sqrtf(2.0f) * (dmax_ref(L1, L2));
  const double mag = (length - Lnew);
  // (mag * c_i) / (length * T) for the corner S1 = c: non-zero on S1's axis
  // only; the rotated offset o_k = sum_i comp_i * l2g[i + 3k] is that term + 0
  const double comp = mag * c1v / (length * kTheodorus);
  out[0] = plus_zero(comp * l2g[a0 + 0]);
  out[1] = plus_zero(comp * l2g[a0 + 3]);
  out[2] = plus_zero(comp * l2g[a0 + 6]);
  out[3] = Lnew;
}

// Hexahedral (8-node) interpolation of MapVoxelManager::evaluate_temperature
// (CA/src/MapVoxelManager.cpp:746-799) in FP64: the shape functions in the
// reference's factor order, summed from 0 in node order.
AMCA_HD double hex8_interp64(const double t[8], double xi, double eta, double zeta) {
  double s[8];
  s[0] = 0.125 * (1.0 - eta) * (1.0 - xi) * (1.0 - zeta);
  s[1] = 0.125 * (1.0 - eta) * (1.0 + xi) * (1.0 - zeta);
  s[2] = 0.125 * (1.0 + eta) * (1.0 + xi) * (1.0 - zeta);
  s[3] = 0.125 * (1.0 + eta) * (1.0 - xi) * (1.0 - zeta);
  s[4] = 0.125 * (1.0 - eta) * (1.0 - xi) * (1.0 + zeta);
  s[5] = 0.125 * (1.0 - eta) * (1.0 + xi) * (1.0 + zeta);
  s[6] = 0.125 * (1.0 + eta) * (1.0 + xi) * (1.0 + zeta);
  s[7] = 0.125 * (1.0 + eta) * (1.0 - xi) * (1.0 + zeta);
  double v = 0.0;
  for (int i = 0; i < 8; i++) v += s[i] * t[i];
  return v;
}

// FP32 estimate of hex8_interp64 from the node values and parametric
// coordinates rounded to float. The shape functions are convex weights
// (coordinates in [-1, 1]), so its error stays below 2e-6 of the largest node
// magnitude; hex8_err32 gives the bound the kernels decide with: 2^-16 of that
// magnitude plus 2^-16 absolute.
AMCA_HD float hex8_interp32(const float t[8], float xi, float eta, float zeta) {
  const float a0 = 1.0f - eta, a1 = 1.0f + eta, b0 = 1.0f - xi, b1 = 1.0f + xi, c0 = 1.0f - zeta, c1 = 1.0f + zeta;
  return 0.125f * (a0 * b0 * c0 * t[0] + a0 * b1 * c0 * t[1] + a1 * b1 * c0 * t[2] + a1 * b0 * c0 * t[3] +
                   a0 * b0 * c1 * t[4] + a0 * b1 * c1 * t[5] + a1 * b1 * c1 * t[6] + a1 * b0 * c1 * t[7]);
}
AMCA_HD float hex8_err32(const float t[8]) {
  float mg = 0.0f;
  for (int i = 0; i < 8; ++i) mg = fmaxf(mg, fabsf(t[i]));
  return ldexpf(mg, -16) + 1.52587890625e-05f;
}

// ProblemPhysics_RappazGandin1993::compute_growth_velocity for a uniform field
AMCA_HD double kgt_velocity(double Tm, double T, double a1, double a2, double a3) {
  const double dT = Tm - T;
  double v = 0.0;
  if (dT > 0) {
    v = a1 * dT + a2 * dT * dT + a3 * dT * dT * dT;
    if (v < 0.0) v = 0.0;
  }
  return v;
}

}  // namespace amca
