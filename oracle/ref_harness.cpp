/*
 * Reference-run harness (test infrastructure only; never shipped, never
 * timed as the product).
 *
 * Links the reference's own, unmodified search code (solver.cu, board.cu,
 * table.cu, node.cuh compiled for the CPU through refshim/prelude.h) and its
 * x86 base81 codec (to_board.cpp), and drives them exactly as the reference
 * CLI's solve path does (main.cu:49-67 load/sort/unique, main.cu:123-173
 * BatchedTask fill, launch, result read-back and "%s %d\n" output lines).
 *
 * Differences from main.cu, none of which reach the search:
 *   - the transposition table is built with 1 slot instead of 50,000,001
 *     (main.cu:133-134): no search code calls it (solver.cu:119-144 and 182
 *     are commented out), only its pointers are passed through;
 *   - the kernel runs as one CPU "thread" (blockDim = gridDim = 1), so its
 *     per-block fetch (solver.cu:289-292, 172) visits problems in order;
 *   - `--per-board` runs one BatchedTask per board and appends the task's
 *     step counter (solver.cu:273-275, 308-309) to each output line, giving
 *     per-position loop-step counts instead of only the batch total.
 *
 * Usage: refsolve INPUT OUTPUT DEPTH [--per-board]
 *        refsolve --codec N SEED
 * The second form prints N random disjoint boards built as test.cpp:25-31
 * does (p = x & y, o = x & ~y), with a fixed mt19937_64 seed instead of
 * random_device, as "<p hex> <o hex> <fromBoard string>" lines, and exits 1
 * if toBoard(fromBoard(b)) != b for any of them (test.cpp:32-38).
 */
#include <cinttypes>
#include <cstdio>
#include <random>
#include <string>
#include <vector>

#include "node.cuh"
#include "solver.cuh"
#include "to_board.hpp"

refshim_dim3 threadIdx = {0, 0, 0};
refshim_dim3 blockIdx = {0, 0, 0};
refshim_dim3 blockDim = {1, 1, 1};
refshim_dim3 gridDim = {1, 1, 1};

// Backing store for `extern __shared__ Node nodes_stack[]` (solver.cu:11):
// lower_stack_depth + 1 = 10 frames for the single emulated thread
// (solver.cu:9, 331).
Node nodes_stack[10];

static std::vector<Board> load_boards(const char* filename) {
  FILE* fp = std::fopen(filename, "r");
  if (!fp) {
    std::fprintf(stderr, "cannot open %s\n", filename);
    std::exit(EXIT_FAILURE);
  }
  int n = 0;
  if (std::fscanf(fp, "%d\n", &n) != 1) {
    std::fprintf(stderr, "Failed to load boards\n");
    std::exit(EXIT_FAILURE);
  }
  std::vector<Board> vboard(n);
  for (int i = 0; i < n; ++i) {
    char buf[33] = {};
    if (std::fgets(buf, 32, fp) == nullptr) {
      std::fprintf(stderr, "Failed to load boards\n");
      std::exit(EXIT_FAILURE);
    }
    vboard[i] = toBoard(buf);
  }
  std::fclose(fp);
  std::sort(vboard.begin(), vboard.end());
  vboard.erase(std::unique(vboard.begin(), vboard.end()), vboard.end());
  return vboard;
}

static int codec_vectors(size_t n, unsigned long long seed) {
  std::mt19937_64 mt(seed);
  std::uniform_int_distribution<uint64_t> dis;
  int bad = 0;
  char buf[17] = {};
  for (size_t i = 0; i < n; ++i) {
    const uint64_t x = dis(mt), y = dis(mt);
    const Board b(x & y, x & ~y);
    fromBoard(b, buf);
    if (toBoard(buf) != b) ++bad;
    std::printf("%016llx %016llx %s\n", static_cast<unsigned long long>(b.first),
                static_cast<unsigned long long>(b.second), buf);
  }
  return bad ? 1 : 0;
}

int main(int argc, char** argv) {
  if (argc == 4 && std::string(argv[1]) == "--codec") {
    return codec_vectors(std::stoul(argv[2]), std::stoull(argv[3]));
  }
  if (argc < 4) {
    std::fprintf(stderr, "usage: %s INPUT OUTPUT DEPTH [--per-board]\n", argv[0]);
    return 1;
  }
  const bool per_board = argc > 4 && std::string(argv[4]) == "--per-board";
  const auto vboard = load_boards(argv[1]);
  const size_t max_depth = std::stoul(argv[3]);
  if (max_depth < 10) {
    std::fprintf(stderr, "DEPTH must be >= 10 (solver.cu:9, 322)\n");
    return 1;
  }
  FILE* fp_out = std::fopen(argv[2], "w");
  if (!fp_out) return 1;
  const size_t n = vboard.size();
  std::fprintf(stderr, "n = %zu\n", n);
  Table table(1);
  unsigned long long total = 0;
  char buf[17];
  const size_t batch = per_board ? 1 : 2000000;
  for (size_t base = 0; base < n; base += batch) {
    const size_t size = std::min(batch, n - base);
    BatchedTask bt(size, max_depth, table);
    for (size_t j = 0; j < size; ++j) {
      bt.abp[j] = AlphaBetaProblem(vboard[base + j].first, vboard[base + j].second);
    }
    bt.launch();
    total += *bt.total;
    for (size_t j = 0; j < size; ++j) {
      fromBoard(Board(bt.abp[j].player, bt.abp[j].opponent), buf);
      if (per_board) {
        std::fprintf(fp_out, "%s %d %llu\n", buf, bt.result[j],
                     static_cast<unsigned long long>(*bt.total));
      } else {
        std::fprintf(fp_out, "%s %d\n", buf, bt.result[j]);
      }
    }
  }
  std::fclose(fp_out);
  std::fprintf(stderr, "total nodes: %llu\n", total);
  return 0;
}
