// Host driver for tests/test_fp32_margins.py: adversarial checks of the two
// places where the kernels decide an FP64 comparison from an FP32 estimate
// with a margin, compiled from the same source the CUDA kernels use
// (amca3d_gb300/csrc/ca_math.h, no contraction), plus a differential of the
// rewritten decentring arithmetic against the C restatement of the
// reference's Octahedron (oracle/amca_oracle.c).
//
//   containment  captured_f32 (with the plain kernel's own inputs: FP32 cell
//                offsets from the stored envelope centre, its error bound and
//                the grid's coordinate error) must return -1 or agree with
//                is_captured_f64 on (envelope, neighbour) pairs whose |c'|_1
//                lies within a few ulps of the half-diagonal L: tiny, unit
//                and huge L, grids far from the origin, every octant and
//                every neighbour direction.
//   lower        the lower bound of |c'|_1 that captured_f32_lb returns with
//                the same inputs (the plain kernel's wake keys) must never
//                exceed the FP64 |c'|_1 of is_captured_f64, on the same pairs.
//   interp       the FP32 interpolation of the remelting kernel and its bound
//                (ends rounded outwards, thresholds inwards to float) must
//                decide T < thr exactly as the FP64 interpolation does, or be
//                undecided, for node values whose FP64 interpolation lies
//                within a few ulps of the liquidus, nullMatTemp_ (-1) and
//                nullMatTemp_ + 0.01.
//   capture      capture_f64 (ca_math.h) against amca_oracle_capture, bit for
//                bit, on random captured pairs.
// Each FP32 check runs three tiers of distance from the threshold: a few
// ulps, 2^-30..2^-16 relative, and 2^-14..2^-6 relative.
// Usage: fp32_margins <cases> <seed>; prints one line per check:
//   <name><tier> <cases> <undecided> <wrong>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../amca3d_gb300/csrc/ca_math.h"

extern "C" {
#include "../oracle/amca_oracle.h"
}

namespace {

uint64_t g_state = 1;
uint64_t next_u64() {  // splitmix64
  uint64_t z = (g_state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double uni() { return (double)(next_u64() >> 11) * 0x1.0p-53; }
double uni(double lo, double hi) { return lo + (hi - lo) * uni(); }

void rotation(double a, double b, double g, double m[9]) {
  const double ca = cos(a), sa = sin(a), cb = cos(b), sb = sin(b), cg = cos(g), sg = sin(g);
  const double r[9] = {ca * cg - sa * cb * sg, -ca * sg - sa * cb * cg, sa * sb,
                       sa * cg + ca * cb * sg, -sa * sg + ca * cb * cg, -ca * sb,
                       sb * sg, sb * cg, cb};
  memcpy(m, r, sizeof r);
}

// |c'|_1 of an offset exactly as is_captured_f64 evaluates it
double l1_local(const double *m, double gx, double gy, double gz) {
  double cx = 0, cy = 0, cz = 0;
  cx += gx * m[0];
  cy += gx * m[1];
  cz += gx * m[2];
  cx += gy * m[3];
  cy += gy * m[4];
  cz += gy * m[5];
  cx += gz * m[6];
  cy += gz * m[7];
  cz += gz * m[8];
  return fabs(cx) + fabs(cy) + fabs(cz);
}

void containment(long n, int tier) {
  long undecided = 0, wrong = 0, lower_wrong = 0;
  const double origins[4] = {0.0, 1.0e-2, -0.37, 2.5};
  const double hs[2] = {2.0e-6, 5.0e-4};
  const double lscale[4] = {1.0e-9, 0.7, 1.5, 1.0e3};  // L relative to h: tiny, unit, unit, huge
  for (long i = 0; i < n; ++i) {
    const double h = hs[next_u64() & 1];
    double o[3];
    for (int a = 0; a < 3; ++a) o[a] = origins[next_u64() & 3] * (next_u64() & 1 ? 1.0 : -1.0);
    const int nxyz = 400;
    double cmax = 0;
    for (int a = 0; a < 3; ++a) cmax = fmax(cmax, fabs(o[a]) + (nxyz + 3) * h);
    const float coord_err = (float)(ldexp(cmax, -49) + 1e-30);
    const int I = 1 + (int)(next_u64() % nxyz), J = 1 + (int)(next_u64() % nxyz), K = 1 + (int)(next_u64() % nxyz);
    int di, dj, dk;
    amca::nbr_offset((int)(next_u64() % 26), di, dj, dk);
    double m[9];
    rotation(uni(0, 2 * M_PI), uni(0, M_PI), uni(0, 2 * M_PI), m);
    float m32[9];
    for (int q = 0; q < 9; ++q) m32[q] = (float)m[q];
    const double ls = lscale[next_u64() & 3];
    // envelope centre: its own cell centre plus an offset of the order of L
    const double own[3] = {amca::centre_coord(o[0], h, I), amca::centre_coord(o[1], h, J),
                           amca::centre_coord(o[2], h, K)};
    double c[3];
    for (int a = 0; a < 3; ++a) c[a] = own[a] + uni(-1, 1) * fmin(ls, 2.0) * h;
    if (ls < 1e-3) {  // tiny envelopes: centre within a few L of the neighbour's centre
      const double nbc[3] = {amca::centre_coord(o[0], h, I + di), amca::centre_coord(o[1], h, J + dj),
                             amca::centre_coord(o[2], h, K + dk)};
      for (int a = 0; a < 3; ++a) c[a] = nbc[a] + uni(-1, 1) * ls * h;
    }
    const double ccx = amca::centre_coord(o[0], h, I + di), ccy = amca::centre_coord(o[1], h, J + dj),
                 ccz = amca::centre_coord(o[2], h, K + dk);
    const double s = l1_local(m, ccx - c[0], ccy - c[1], ccz - c[2]);
    if (!(s > 0)) continue;
    // L within a few ulps of |c'|_1 (tier 0), within 2^-30..2^-16 of it
    // relative (tier 1) or within 2^-14..2^-6 (tier 2)
    double L = s;
    if (tier == 0) {
      const int k = (int)(next_u64() % 17) - 8;
      for (int t = 0; t < abs(k); ++t) L = nextafter(L, k > 0 ? INFINITY : 0.0);
    } else {
      const double e = tier == 1 ? uni(-30, -16) : uni(-14, -6);
      L = s * (1.0 + (next_u64() & 1 ? 1.0 : -1.0) * exp2(e));
    }
    // the kernel's FP32 inputs: stored offset of the centre from its own cell
    // centre, the neighbour offset in FP32 and the error bound
    const float dxf = (float)(c[0] - own[0]), dyf = (float)(c[1] - own[1]), dzf = (float)(c[2] - own[2]);
    const float h32 = (float)h;
    const float errg = 4.76837158203125e-07f * (h32 + fabsf(dxf) + fabsf(dyf) + fabsf(dzf)) + coord_err;
    float lower;
    const int f = amca::captured_f32_lb(m32, (float)di * h32 - dxf, (float)dj * h32 - dyf, (float)dk * h32 - dzf,
                                        errg, (float)L, &lower);
    if ((double)lower > s) ++lower_wrong;
    const bool exact = amca::is_captured_f64(m, ccx - c[0], ccy - c[1], ccz - c[2], L);
    if (f < 0)
      ++undecided;
    else if ((f == 1) != exact)
      ++wrong;
  }
  printf("containment%d %ld %ld %ld\n", tier, n, undecided, wrong);
  printf("lower%d %ld 0 %ld\n", tier, n, lower_wrong);
}

// float rounding of a double downwards / upwards (a sum of two floats is
// exact in double, so this is the FP32 addition with that rounding)
float round_down(double x) {
  float f = (float)x;
  if ((double)f > x) f = nextafterf(f, -INFINITY);
  return f;
}
float round_up(double x) {
  float f = (float)x;
  if ((double)f < x) f = nextafterf(f, INFINITY);
  return f;
}
float below_of(double t) { return round_down(t); }
float above_of(double t) { return round_up(t); }

void interp(long n, int tier) {
  long undecided = 0, wrong = 0;
  const double thr[3] = {1700.0, -1.0, -1.0 + 0.01};
  for (long i = 0; i < n; ++i) {
    const double T0 = thr[i % 3];
    double pc[3];
    for (int a = 0; a < 3; ++a) pc[a] = uni(-1, 1);
    // node values spread around the threshold (up to +-40% of the scale, at least 300 K wide)
    const double spread = fmax(fabs(T0), 300.0) * uni(0.0, 0.4);
    double t[8];
    for (int q = 0; q < 7; ++q) t[q] = T0 + uni(-1, 1) * spread;
    // last node chosen so that the interpolation lands on the threshold, then nudged by ulps
    double s[8];
    {
      double one[8];
      for (int q = 0; q < 8; ++q) {
        for (int r = 0; r < 8; ++r) one[r] = r == q ? 1.0 : 0.0;
        s[q] = amca::hex8_interp64(one, pc[0], pc[1], pc[2]);
      }
    }
    if (s[7] < 1e-3) continue;
    double partial = 0.0;
    for (int q = 0; q < 7; ++q) partial += s[q] * t[q];
    t[7] = (T0 - partial) / s[7];
    if (tier == 0) {  // within a few ulps of the threshold
      const int k = (int)(next_u64() % 33) - 16;
      for (int u = 0; u < abs(k); ++u) t[7] = nextafter(t[7], k > 0 ? INFINITY : -INFINITY);
    } else {  // 2^-30..2^-16 (tier 1) or 2^-14..2^-6 (tier 2) of the node scale away from it
      const double e = tier == 1 ? uni(-30, -16) : uni(-14, -6);
      t[7] += (next_u64() & 1 ? 1.0 : -1.0) * exp2(e) * fmax(fabs(T0), 300.0) / s[7];
    }
    const double T = amca::hex8_interp64(t, pc[0], pc[1], pc[2]);
    float t32[8];
    for (int q = 0; q < 8; ++q) t32[q] = (float)t[q];
    const float v = amca::hex8_interp32(t32, (float)pc[0], (float)pc[1], (float)pc[2]);
    const float err = amca::hex8_err32(t32);
    // the kernel's decision rule (phase_update's `below`): the ends of the
    // bound rounded outwards to float, the threshold inwards
    int b = -1;
    if (round_up((double)v + (double)err) < below_of(T0)) b = 1;
    else if (round_down((double)v - (double)err) >= above_of(T0)) b = 0;
    if (b < 0)
      ++undecided;
    else if ((b == 1) != (T < T0))
      ++wrong;
  }
  printf("interp%d %ld %ld %ld\n", tier, n, undecided, wrong);
}

void capture(long n) {
  long done = 0, wrong = 0;
  for (long i = 0; i < n; ++i) {
    const double h = next_u64() & 1 ? 2.0e-6 : 5.0e-4;
    double m[9];
    rotation(uni(0, 2 * M_PI), uni(0, M_PI), uni(0, 2 * M_PI), m);
    double gc[3];
    for (int a = 0; a < 3; ++a) gc[a] = uni(-1.5, 1.5) * h;
    const double L = uni(0.3, 3.0) * h;
    const double trunc = (double)sqrtf(3.0f);
    if (!amca::is_captured_f64(m, gc[0], gc[1], gc[2], L)) continue;
    double a[4], b[4];
    amca::capture_f64(m, gc[0], gc[1], gc[2], L, h, trunc, a);
    amca_oracle_capture(m, gc, L, h, trunc, b);
    ++done;
    if (memcmp(a, b, sizeof a) != 0) ++wrong;
  }
  printf("capture %ld 0 %ld\n", done, wrong);
}

}  // namespace

int main(int argc, char **argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  g_state = argc > 2 ? strtoull(argv[2], nullptr, 10) : 1;
  for (int tier = 0; tier < 3; ++tier) containment(n, tier);
  for (int tier = 0; tier < 3; ++tier) interp(n, tier);
  capture(n);
  return 0;
}
