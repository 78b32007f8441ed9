// thermal_field.cuh — the synthetic FE temperature field of a scanning point
// source (the Rosenthal quasi-steady solution of the current pass), shared by
// the multi-track frame generator, the thermal model's training labels and
// its fallback. IEEE add/mul/div/sqrt only, exp by a fixed polynomial, so
// host and device give the same doubles; for one track it is the field of
// amca_set_rosenthal_frames operation for operation.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "surrogate.h"

namespace amca {

// exp(a) for a <= 0: k = rint(a / ln 2), r = a - k ln 2, degree-13 Taylor
// polynomial in r (Horner), times 2^k built from the exponent bits.
__host__ __device__ inline double field_exp(double a) {
  const double c[14] = {0x1.0000000000000p+0, 0x1.0000000000000p+0, 0x1.0000000000000p-1, 0x1.5555555555555p-3,
                        0x1.5555555555555p-5, 0x1.1111111111111p-7, 0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-13,
                        0x1.a01a01a01a01ap-16, 0x1.71de3a556c734p-19, 0x1.27e4fb7789f5cp-22, 0x1.ae64567f544e4p-26,
                        0x1.1eed8eff8d898p-29, 0x1.6124613a86d09p-33};
  const double kLn2 = 0x1.62e42fefa39efp-1, kInvLn2 = 0x1.71547652b82fep+0;
  a = (a < -700.0) ? -700.0 : a;
  const double k = rint(a * kInvLn2);
  const double r = a - k * kLn2;
  double p = c[13];
  for (int n = 12; n >= 0; --n) p = p * r + c[n];
  const long long ki = (long long)k;
  const unsigned long long bits = (unsigned long long)(ki + 1023) << 52;
  double scale;
  memcpy(&scale, &bits, sizeof scale);
  return p * scale;
}

// Field value at (x, y, z) (m) and time t (s).
__host__ __device__ inline double scan_field(const ScanSource &s, double x, double y, double z, double t) {
  double xl, yl, dir;
  scan_position(s, t, xl, yl, dir);
  const double xi = (x - xl) * dir;
  const double dy = y - yl;
  const double dz = z - s.z_top;
  double r = sqrt((xi * xi + dy * dy) + dz * dz);
  r = (r < 1e-9) ? 1e-9 : r;
  const double qv = (s.absorptivity * s.power) / ((2.0 * 3.141592653589793 * s.conductivity) * r);
  const double T = s.t0 + qv * field_exp(-(s.speed * (r + xi)) / (2.0 * s.diffusivity));
  return (s.t_cap < T) ? s.t_cap : T;
}

// The model's raw inputs for a point: along-track offset (m, positive ahead of
// the source), lateral offset (m), depth below the top surface (m), power (W),
// speed (m/s).
__host__ __device__ inline void scan_inputs(const ScanSource &s, double x, double y, double z, double t, float in[5]) {
  double xl, yl, dir;
  scan_position(s, t, xl, yl, dir);
  in[0] = (float)((x - xl) * dir);
  in[1] = (float)(y - yl);
  in[2] = (float)(s.z_top - z);
  in[3] = (float)s.power;
  in[4] = (float)s.speed;
}

}  // namespace amca
