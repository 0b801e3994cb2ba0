// `diff_results A B` -- compares two result files of the solver's output
// format ("<base81> <score>" per line, main.cu:164-171) by board: line order
// and duplicate lines do not matter, a board with two different scores in one
// file is an error.  Prints each board whose score differs or that only one
// file holds, then a summary line; exits 0 when the files agree on every
// board, 1 when they differ, 2 on a read or parse error.  Compares results of
// this solver with the reference's, or two runs with different options.
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>

#include "boardfile.h"

namespace {

bool read_results(const char* path, std::map<gpo_host::Board, int>& out, std::string& err) {
  FILE* f = std::fopen(path, "r");
  if (!f) {
    err = std::string("cannot open ") + path;
    return false;
  }
  char line[256];
  long lineno = 0;
  bool ok = true;
  while (std::fgets(line, sizeof(line), f)) {
    ++lineno;
    std::string s(line);
    while (!s.empty() && (s.back() == '\n' || s.back() == '\r' || s.back() == ' ')) s.pop_back();
    if (s.empty()) continue;
    const size_t sp = s.find(' ');
    uint64_t p = 0, o = 0;
    char* end = nullptr;
    const long v = sp == std::string::npos ? 0 : std::strtol(s.c_str() + sp + 1, &end, 10);
    if (sp != 16 || !gpo_host::decode(s.c_str(), p, o) || !end || end == s.c_str() + sp + 1) {
      err = std::string(path) + ":" + std::to_string(lineno) + ": not a \"<board> <score>\" line";
      ok = false;
      break;
    }
    const gpo_host::Board b{p, o};
    auto it = out.find(b);
    if (it != out.end() && it->second != static_cast<int>(v)) {
      err = std::string(path) + ":" + std::to_string(lineno) + ": board " + s.substr(0, 16) +
            " listed with two scores";
      ok = false;
      break;
    }
    out[b] = static_cast<int>(v);
  }
  std::fclose(f);
  return ok;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s RESULTS_A RESULTS_B\n", argv[0]);
    return 2;
  }
  std::map<gpo_host::Board, int> a, b;
  std::string err;
  if (!read_results(argv[1], a, err) || !read_results(argv[2], b, err)) {
    std::fprintf(stderr, "%s\n", err.c_str());
    return 2;
  }
  long differ = 0, only_a = 0, only_b = 0;
  char enc[17];
  for (const auto& kv : a) {
    gpo_host::encode(kv.first.p, kv.first.o, enc);
    auto it = b.find(kv.first);
    if (it == b.end()) {
      std::printf("only in A: %s %d\n", enc, kv.second);
      ++only_a;
    } else if (it->second != kv.second) {
      std::printf("differs: %s %d %d\n", enc, kv.second, it->second);
      ++differ;
    }
  }
  for (const auto& kv : b) {
    if (a.count(kv.first)) continue;
    gpo_host::encode(kv.first.p, kv.first.o, enc);
    std::printf("only in B: %s %d\n", enc, kv.second);
    ++only_b;
  }
  std::printf("%zu boards in A, %zu in B: %ld differ, %ld only in A, %ld only in B\n", a.size(),
              b.size(), differ, only_a, only_b);
  return (differ || only_a || only_b) ? 1 : 0;
}
