// TEST INFRASTRUCTURE ONLY: command-line driver of the CPU oracle.
//   dmrg_oracle <dmrg.conf> [--threads T] [--verbose V] [--noreorder]
//   dmrg_oracle --synthetic norb nelec nchol seed d2h M sweeps [...]
// Prints one JSON line with the final energies.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "cpu_engine.h"

using namespace bgpu;

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s dmrg.conf [--threads T] [--verbose V]\n", argv[0]);
    return 2;
  }
  int threads = 0, verbose = 0;
  std::string reorder_override, write_dump;
  for (int i = 2; i < argc; ++i) {
    if (!std::strcmp(argv[i], "--threads") && i + 1 < argc) threads = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--verbose") && i + 1 < argc) verbose = std::atoi(argv[++i]);
    else if (!std::strcmp(argv[i], "--noreorder")) reorder_override = "noreorder";
    else if (!std::strcmp(argv[i], "--write-fcidump") && i + 1 < argc) write_dump = argv[++i];
  }
  try {
    Config c = parse_config(argv[1]);
    if (!reorder_override.empty()) c.reorder = reorder_override;
    Integrals I = load_integrals(c);
    if (!write_dump.empty()) {  // integrals in the orbital order used by the sweep
      write_fcidump(I, write_dump);
      return 0;
    }
    oracle::CpuEngine eng(threads);
    DriverOptions opt;
    opt.verbose = verbose;
    SweepDriver drv(I, c, eng, opt);
    SweepResult r = drv.run();
    std::printf("{\"energies\": [");
    for (size_t i = 0; i < r.energies.size(); ++i) std::printf("%s%.12f", i ? ", " : "", r.energies[i]);
    std::printf("], \"sweep_energies\": [");
    for (size_t i = 0; i < r.sweep_energies.size(); ++i) std::printf("%s%.12f", i ? ", " : "", r.sweep_energies[i]);
    std::printf("], \"sweeps\": %d, \"sigma_calls\": %ld, \"sigma_seconds\": %.3f}\n", r.sweeps, eng.sigma_calls,
                eng.sigma_seconds);
  } catch (std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
