// `gen_boards OUTPUT N SEED MIN_EMPTIES [MAX_EMPTIES]` -- writes N positions
// of the seeded random-playout stream (gpo_generate, on the GPU) as a board
// file in the reference's input format (README.md:27-41), in generation
// order (duplicates kept; the solver removes them, main.cu:64-65).
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "boardfile.h"
#include "gpuothello2.h"

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: %s OUTPUT N SEED MIN_EMPTIES [MAX_EMPTIES]\n", argv[0]);
    return 1;
  }
  const long n = std::strtol(argv[2], nullptr, 10);
  const unsigned long long seed = std::strtoull(argv[3], nullptr, 10);
  const int lo = std::atoi(argv[4]);
  const int hi = argc > 5 ? std::atoi(argv[5]) : lo;
  if (n < 0 || n > (1L << 30)) {
    std::fprintf(stderr, "N out of range\n");
    return 1;
  }
  std::vector<uint64_t> p(n), o(n);
  const int rc = gpo_generate(seed, 0, static_cast<int>(n), lo, hi, p.data(), o.data());
  if (rc != GPO_OK) {
    std::fprintf(stderr, "generate failed: %s\n", gpo_strerror(rc));
    return 1;
  }
  std::vector<gpo_host::Board> boards(n);
  for (long i = 0; i < n; ++i) boards[i] = {p[i], o[i]};
  std::string err;
  if (!gpo_host::write_boards(argv[1], boards, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return 1;
  }
  solve_shutdown();
  return 0;
}
