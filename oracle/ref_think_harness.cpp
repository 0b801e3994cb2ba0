/*
 * Reference think-mode harness (test infrastructure only; never shipped,
 * never timed as the product).
 *
 * Links the reference's own, unmodified pattern evaluator and think-mode
 * search (eval.cu, thinker.cu, node.cuh, board.cu, table.cu compiled for the
 * CPU through refshim/prelude.h) and its x86 base81 codec (to_board.cpp),
 * and drives them as the reference CLI's think path does (main.cu:69-121:
 * load/sort/unique, Evaluator(features, values), BatchedThinkTask fill,
 * launch, "%s %d %s\n" output lines with hand_to_s, main.cu:31-39).
 *
 * Differences from main.cu, none of which reach the search:
 *   - the feature and value files are arguments instead of the fixed
 *     "subboard.txt" and "value/value52" (main.cu:74);
 *   - the transposition table has 1 slot (thinker.cu never calls it: its
 *     find/update calls are commented out, thinker.cu:68-92, 187, 256-265);
 *   - the kernel runs as one CPU "thread", so problems are visited in order;
 *   - `--per-board` runs one task per board and appends that task's
 *     loop-step counter (thinker.cu:324-326, 367-368) to each line.
 *
 * Usage: refthink FEATURES VALUES INPUT OUTPUT THINK_DEPTH [--per-board]
 *        refthink --eval FEATURES VALUES INPUT
 * The second form prints, for every board of INPUT (sorted, unique),
 * "<p hex> <o hex> <float bits hex>" of Evaluator::eval (eval.cu:129-141).
 */
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "eval.cuh"
#include "node.cuh"
#include "thinker.cuh"
#include "to_board.hpp"

refshim_dim3 threadIdx = {0, 0, 0};
refshim_dim3 blockIdx = {0, 0, 0};
refshim_dim3 blockDim = {1, 1, 1};
refshim_dim3 gridDim = {1, 1, 1};

// Backing store for `extern __shared__ Node nodes_stack[]` (thinker.cu:10):
// think_lower_stack_depth + 1 frames for the single emulated thread.
Node nodes_stack[8];

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

// main.cu:31-39
static std::string move_string(hand move) {
  if (move == hand::PASS) return "ps";
  std::string res(1, static_cast<char>(static_cast<int>(move) % 8 + 'A'));
  res += static_cast<char>(static_cast<int>(move) / 8 + '1');
  return res;
}

int main(int argc, char** argv) {
  if (argc == 5 && std::string(argv[1]) == "--eval") {
    Evaluator ev(argv[2], argv[3]);
    for (const auto& b : load_boards(argv[4])) {
      const float v = ev.eval(b.first, b.second);
      uint32_t bits = 0;
      std::memcpy(&bits, &v, sizeof(bits));
      std::printf("%016llx %016llx %08x\n", static_cast<unsigned long long>(b.first),
                  static_cast<unsigned long long>(b.second), bits);
    }
    return 0;
  }
  if (argc < 6) {
    std::fprintf(stderr, "usage: %s FEATURES VALUES INPUT OUTPUT THINK_DEPTH [--per-board]\n",
                 argv[0]);
    return 1;
  }
  const bool per_board = argc > 6 && std::string(argv[6]) == "--per-board";
  const size_t depth = std::stoul(argv[5]);
  if (depth < 4) {
    std::fprintf(stderr, "THINK_DEPTH must be >= 4 (thinker.cu:8, 362)\n");
    return 1;
  }
  Evaluator ev(argv[1], argv[2]);
  const auto vboard = load_boards(argv[3]);
  FILE* fp_out = std::fopen(argv[4], "w");
  if (!fp_out) return 1;
  const size_t n = vboard.size();
  std::fprintf(stderr, "n = %zu\n", n);
  Table table(1);
  unsigned long long total = 0;
  char buf[17];
  const size_t batch = per_board ? 1 : 2000000;
  for (size_t base = 0; base < n; base += batch) {
    const size_t size = std::min(batch, n - base);
    BatchedThinkTask bt(size, depth, table, ev);
    for (size_t j = 0; j < size; ++j) {
      bt.abp[j] = AlphaBetaProblem(vboard[base + j].first, vboard[base + j].second);
    }
    bt.launch();
    total += *bt.total;
    for (size_t j = 0; j < size; ++j) {
      fromBoard(Board(bt.abp[j].player, bt.abp[j].opponent), buf);
      if (per_board) {
        std::fprintf(fp_out, "%s %d %s %llu\n", buf, bt.result[j],
                     move_string(bt.bestmove[j]).c_str(),
                     static_cast<unsigned long long>(*bt.total));
      } else {
        std::fprintf(fp_out, "%s %d %s\n", buf, bt.result[j],
                     move_string(bt.bestmove[j]).c_str());
      }
    }
  }
  std::fclose(fp_out);
  std::fprintf(stderr, "total nodes: %llu\n", total);
  return 0;
}
