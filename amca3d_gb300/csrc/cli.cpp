// cli.cpp — the amca3d command: the reference's program (CA/src/Cafe.cpp:33-120)
// over the C ABI. Reads the deck given by -i (default cafe.i), runs the realm
// it selects (plain or FE-coupled remelting) on one GPU to its end, writes the
// reference's output files, and a short run log to -o (default: standard
// output). Options beyond the reference's: --device N, --seed S, --no-outputs.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <iostream>
#include <sstream>
#include <string>

#include "amca3d.h"

namespace {

void usage(std::ostream &o) {
  o << "amca3d supported options:\n"
       "  -h [ --help ]                 Help message\n"
       "  -v [ --version ]              Code Version 1.0\n"
       "  -i [ --input-deck ] arg (=cafe.i)  Analysis input file\n"
       "  -o [ --log-file ] arg         Analysis log file\n"
       "  --device arg (=0)             CUDA device\n"
       "  --seed arg (=0)               glibc srand() offset (the reference seeds srand(0) at np=1)\n"
       "  --no-outputs                  skip VTR snapshots and final output files\n";
}

int fail(std::ostream &log, const char *what, amca_t *h) {
  log << "error: " << what << ": " << amca_last_error(h) << std::endl;
  std::cerr << "error: " << what << ": " << amca_last_error(h) << std::endl;
  if (h) amca_destroy(h);
  return 1;
}

}  // namespace

int main(int argc, char **argv) {
  std::string input = "cafe.i", logname;
  int device = 0, outputs = 1;
  unsigned seed = 0;
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    auto next = [&](const char *name) -> std::string {
      if (a + 1 >= argc) {
        std::cerr << "missing value for " << name << std::endl;
        exit(2);
      }
      return argv[++a];
    };
    if (s == "-h" || s == "--help") {
      usage(std::cerr);
      return 0;
    } else if (s == "-v" || s == "--version") {
      std::cerr << "Version: Cafe1.0 (GB300)" << std::endl;
      return 0;
    } else if (s == "-i" || s == "--input-deck") {
      input = next("-i");
    } else if (s == "-o" || s == "--log-file") {
      logname = next("-o");
    } else if (s == "--device") {
      device = atoi(next("--device").c_str());
    } else if (s == "--seed") {
      seed = (unsigned)strtoul(next("--seed").c_str(), nullptr, 10);
    } else if (s == "--no-outputs") {
      outputs = 0;
    } else {
      std::cerr << "unknown option " << s << std::endl;
      usage(std::cerr);
      return 2;
    }
  }
  std::ifstream fin(input.c_str());
  if (!fin.good()) {
    std::cerr << "Input file is not specified or does not exist: user specified or (default) name= " << input
              << std::endl;
    return 0;
  }
  std::stringstream deck;
  deck << fin.rdbuf();
  std::ofstream logf;
  if (!logname.empty()) logf.open(logname.c_str());
  std::ostream &log = logname.empty() ? std::cout : logf;

  amca_opts o = {device, seed, outputs, nullptr};
  amca_t *h = nullptr;
  if (amca_create(deck.str().c_str(), &o, &h) != AMCA_OK) return fail(log, "parsing the deck", nullptr);
  int32_t cells[3];
  double origin[3], hcell;
  amca_get_grid(h, cells, origin, &hcell);
  log << "Domain: " << cells[0] << " x " << cells[1] << " x " << cells[2] << " cells of " << hcell << std::endl;
  if (amca_initialize(h) != AMCA_OK) return fail(log, "initialize", h);
  if (amca_run(h, -1) != AMCA_OK) return fail(log, "time integration", h);
  amca_stats st;
  amca_get_stats(h, &st);
  int32_t grains = 0;
  if (amca_final_grain_count(h, &grains) != AMCA_OK) return fail(log, "final grain count", h);
  if (outputs && amca_write_outputs(h) != AMCA_OK) return fail(log, "writing outputs", h);
  log << "Time Step Count: " << st.step << "\n"
      << "Final time: " << st.time << "\n"
      << " Final Number of Grains:\n"
      << "             " << grains << "\n"
      << "GPU time (ms): " << st.kernel_ms << std::endl;
  amca_destroy(h);
  return 0;
}
