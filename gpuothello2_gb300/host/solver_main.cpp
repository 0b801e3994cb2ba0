// `solver INPUT OUTPUT DEPTH` -- the reference CLI's solve mode
// (main.cu:123-185) over the C ABI.
//
// Same arguments, input format, sort + dedup, output lines and stderr lines
// as the reference; additionally prints throughput.  Differences: errors
// (unreadable file, bad board line, a position with more empties than
// DEPTH, CUDA failures) end with a message and a nonzero exit instead of
// undefined behaviour, and the 5-argument think mode (main.cu:69-121) is
// rejected because its pattern weights (value/value52, main.cu:75) are not
// part of the reference.
//
// Environment: GPO_METHOD=plain selects the plain thread-per-board kernel
// (default: batched).
#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "boardfile.h"
#include "gpuothello2.h"

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s INPUT OUTPUT DEPTH [THINK_DEPTH]\n", argv[0]);
    return 1;
  }
  if (argc >= 5) {
    std::fprintf(stderr,
                 "think mode (THINK_DEPTH) is not supported: it needs the pattern weights "
                 "value/value52, which the reference does not ship\n");
    return 2;
  }
  char* end = nullptr;
  const long depth = std::strtol(argv[3], &end, 10);
  if (!end || *end != '\0' || depth < 1 || depth > 32) {
    std::fprintf(stderr, "DEPTH must be an integer in [1, 32]\n");
    return 1;
  }
  std::vector<gpo_host::Board> boards;
  std::string err;
  if (!gpo_host::load_boards(argv[1], boards, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return EXIT_FAILURE;
  }
  const size_t n = boards.size();
  std::fprintf(stderr, "n = %zu\n", n);
  std::vector<uint64_t> p(n), o(n);
  for (size_t i = 0; i < n; ++i) {
    p[i] = boards[i].p;
    o[i] = boards[i].o;
  }
  std::vector<int8_t> score(n, 0);
  gpo_options opt;
  gpo_default_options(&opt);
  const char* method = std::getenv("GPO_METHOD");
  if (method && std::strcmp(method, "plain") == 0) opt.method = GPO_METHOD_PLAIN;
  gpo_stats st;
  std::memset(&st, 0, sizeof(st));
  std::fprintf(stderr, "start!\n");
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = solve_batch_ex(p.data(), o.data(), static_cast<int>(n), static_cast<int>(depth),
                                score.data(), nullptr, nullptr, &opt, &st);
  const auto t1 = std::chrono::steady_clock::now();
  const long ms = static_cast<long>(
      std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count());
  std::fprintf(stderr,
               "%s (%s), elapsed: %ldms, table update count: %" PRIu64 ", table hit: %" PRIu64
               ", table find: %" PRIu64 "\n",
               rc == GPO_OK ? "cudaSuccess" : "error", rc == GPO_OK ? "no error" : gpo_strerror(rc),
               ms, st.table_updates, st.table_hits, st.table_probes);
  if (rc != GPO_OK) return EXIT_FAILURE;
  const double sec = std::chrono::duration<double>(t1 - t0).count();
  std::fprintf(stderr, "positions/s: %.0f, nodes/s: %.4g, kernel: %.3fms\n",
               sec > 0 ? n / sec : 0.0, sec > 0 ? st.nodes / sec : 0.0, st.kernel_ms);
  if (!gpo_host::write_results(argv[2], boards, score, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return EXIT_FAILURE;
  }
  std::fprintf(stderr, "total nodes: %" PRIu64 "\n", st.nodes);
  solve_shutdown();
  return 0;
}
