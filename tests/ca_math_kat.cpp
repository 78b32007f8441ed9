// Host driver for tests/test_ca_math_host.py: evaluates the envelope
// arithmetic of amca3d_gb300/csrc/ca_math.h (the same source the CUDA kernels
// compile) on known-answer cases produced by the reference's own Octahedron
// class. Input (binary, little endian): int32 n, then n rows of 20 doubles:
// l2g[9], gc[3], L, h, trunc, captured, info[4]. Prints the mismatch count.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../amca3d_gb300/csrc/ca_math.h"

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  int n = 0;
  if (fread(&n, 4, 1, f) != 1) return 2;
  std::vector<double> in((size_t)n * 20);
  if (fread(in.data(), 8, in.size(), f) != in.size()) return 2;
  fclose(f);
  int bad = 0, caps = 0;
  for (int i = 0; i < n; ++i) {
    const double *r = &in[(size_t)i * 20];
    const double *m = r, *gc = r + 9;
    const double L = r[12], h = r[13], tr = r[14];
    const bool want = r[15] != 0;
    const bool got = amca::is_captured_f64(m, gc[0], gc[1], gc[2], L);
    if (got != want) {
      ++bad;
      continue;
    }
    if (got) {
      ++caps;
      double out[4];
      amca::capture_f64(m, gc[0], gc[1], gc[2], L, h, tr, out);
      if (memcmp(out, r + 16, sizeof out) != 0) ++bad;
    }
  }
  printf("%d %d %d\n", n, caps, bad);
  return 0;
}
