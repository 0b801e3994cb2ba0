// `solver INPUT OUTPUT DEPTH [THINK_DEPTH]` -- the reference CLI
// (main.cu:69-185) over the C ABI.
//
// Solve mode (3 arguments, main.cu:123-173) and think mode (4 arguments,
// main.cu:69-121): same arguments, input format, sort + dedup, output lines
// and stderr lines as the reference; additionally prints throughput.  Think
// mode reads the pattern evaluator from "subboard.txt" and "value/value52"
// in the working directory, as the reference does (main.cu:74); the
// environment variables GPO_FEATURES_FILE and GPO_VALUES_FILE override the
// two paths.  DEPTH is read but unused in think mode, as in the reference.
// Differences: errors (unreadable file, bad board line, a position with more
// empties than DEPTH, a missing evaluator file, CUDA failures) end with a
// message and a nonzero exit instead of undefined behaviour.
//
// Environment (solve mode):
//   GPO_METHOD=plain      the plain thread-per-board kernel (default: batched)
//   GPO_TABLE=0           no transposition table (default: on; the stderr line
//                         "table update count / hit / find" reports its counters,
//                         the reference's Table counters, main.cu:158-162)
//   GPO_TABLE_BITS=n      a table of 2^n entries (default: from the device memory)
//   GPO_WEIGHTS=FILE      learned move-orderer weights (gpo_mlp_load); default: the
//                         weights shipped beside the binary (../data/orderer.f32),
//                         used when present; GPO_WEIGHTS=none turns the orderer off
#include <unistd.h>

#include <chrono>
#include <cinttypes>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "boardfile.h"
#include "gpuothello2.h"

namespace {

long parse_int(const char* s) {
  char* end = nullptr;
  const long v = std::strtol(s, &end, 10);
  return (end && *end == '\0' && end != s) ? v : -1;
}

// Directory of the running binary (Linux), with a trailing slash; "" if unknown.
std::string exe_dir() {
  char buf[4096];
  const ssize_t k = readlink("/proc/self/exe", buf, sizeof(buf) - 1);
  if (k <= 0) return "";
  buf[k] = '\0';
  std::string s(buf);
  const size_t slash = s.rfind('/');
  return slash == std::string::npos ? "" : s.substr(0, slash + 1);
}

// Loads move-orderer weights from `path` (gpo_mlp_param_count() floats);
// false if the file is missing or short.
bool load_weights(const std::string& path) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::vector<float> w(static_cast<size_t>(gpo_mlp_param_count()));
  const size_t got = std::fread(w.data(), sizeof(float), w.size(), f);
  std::fclose(f);
  return got == w.size() && gpo_mlp_load(w.data()) == GPO_OK;
}

int think_main(char** argv) {
  const long depth = parse_int(argv[4]);
  if (depth < 4 || depth > 24) {
    std::fprintf(stderr, "THINK_DEPTH must be an integer in [4, 24]\n");
    return 1;
  }
  std::vector<gpo_host::Board> boards;
  std::string err;
  if (!gpo_host::load_boards(argv[1], boards, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return EXIT_FAILURE;
  }
  const char* fpath = std::getenv("GPO_FEATURES_FILE");
  const char* vpath = std::getenv("GPO_VALUES_FILE");
  if (!fpath) fpath = "subboard.txt";
  if (!vpath) vpath = "value/value52";
  const int lrc = gpo_eval_load_files(fpath, vpath);
  if (lrc != GPO_OK) {
    std::fprintf(stderr, "cannot load the pattern evaluator from %s and %s: %s\n", fpath, vpath,
                 gpo_strerror(lrc));
    return EXIT_FAILURE;
  }
  const size_t n = boards.size();
  std::fprintf(stderr, "n = %zu\n", n);
  std::vector<uint64_t> p(n), o(n);
  for (size_t i = 0; i < n; ++i) {
    p[i] = boards[i].p;
    o[i] = boards[i].o;
  }
  std::vector<int8_t> score(n, 0), best(n, 0);
  gpo_stats st;
  std::memset(&st, 0, sizeof(st));
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = think_batch(p.data(), o.data(), static_cast<int>(n), static_cast<int>(depth),
                             score.data(), best.data(), nullptr, &st);
  const auto t1 = std::chrono::steady_clock::now();
  const long ms = static_cast<long>(
      std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count());
  std::fprintf(stderr,
               "%s (%s), elapsed: %ldms, table update count: 0, table hit: 0, table find: 0\n",
               rc == GPO_OK ? "cudaSuccess" : "error", rc == GPO_OK ? "no error" : gpo_strerror(rc),
               ms);
  if (rc != GPO_OK) return EXIT_FAILURE;
  const double sec = std::chrono::duration<double>(t1 - t0).count();
  std::fprintf(stderr, "positions/s: %.0f, nodes/s: %.4g, kernel: %.3fms\n",
               sec > 0 ? n / sec : 0.0, sec > 0 ? st.nodes / sec : 0.0, st.kernel_ms);
  if (!gpo_host::write_think_results(argv[2], boards, score, best, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return EXIT_FAILURE;
  }
  std::fprintf(stderr, "total nodes: %" PRIu64 "\n", st.nodes);
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s INPUT OUTPUT DEPTH [THINK_DEPTH]\n", argv[0]);
    return 1;
  }
  if (argc == 5) return think_main(argv);
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
  const char* table = std::getenv("GPO_TABLE");
  if (table && std::strcmp(table, "0") == 0) opt.use_table = 0;
  const char* bits = std::getenv("GPO_TABLE_BITS");
  if (bits) opt.table_bits = static_cast<int>(parse_int(bits));
  const char* weights = std::getenv("GPO_WEIGHTS");
  opt.use_learned = 0;
  if (opt.method == GPO_METHOD_BATCHED && !(weights && std::strcmp(weights, "none") == 0)) {
    const std::string wpath = weights ? std::string(weights) : exe_dir() + "../data/orderer.f32";
    if (load_weights(wpath)) {
      opt.use_learned = 1;
    } else if (weights) {
      std::fprintf(stderr, "cannot load move-orderer weights from %s\n", wpath.c_str());
      return EXIT_FAILURE;
    }
  }
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
