#include "boardfile.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>

namespace gpo_host {

void encode(uint64_t p, uint64_t o, char out[17]) {
  static const int w[4] = {1, 3, 9, 32};
  for (int i = 0; i < 16; ++i) {
    int v = 33;
    for (int j = 0; j < 4; ++j) {
      const int sq = 4 * i + j;
      if ((p >> sq) & 1) v += w[j];
      if ((o >> sq) & 1) v += 2 * w[j];
    }
    out[i] = static_cast<char>(v);
  }
  out[16] = '\0';
}

bool decode(const char* s, uint64_t& p, uint64_t& o) {
  uint64_t pp = 0, oo = 0;
  for (int i = 0; i < 16; ++i) {
    const int v = static_cast<int>(static_cast<unsigned char>(s[i])) - 33;
    if (v < 0 || v > 90) return false;
    const int hi = v >> 5, lo = v & 31;
    if (hi > 2 || lo > 26) return false;
    const int digit[4] = {lo % 3, (lo / 3) % 3, lo / 9, hi};
    for (int j = 0; j < 4; ++j) {
      const uint64_t b = 1ULL << (4 * i + j);
      if (digit[j] == 1) pp |= b;
      if (digit[j] == 2) oo |= b;
    }
  }
  p = pp;
  o = oo;
  return true;
}

namespace {
bool read_line(std::FILE* fp, std::string& line) {
  line.clear();
  int c;
  while ((c = std::fgetc(fp)) != EOF) {
    if (c == '\n') return true;
    line.push_back(static_cast<char>(c));
  }
  return !line.empty();
}
}  // namespace

bool load_boards(const std::string& path, std::vector<Board>& out, std::string& err) {
  std::FILE* fp = std::fopen(path.c_str(), "r");
  if (!fp) {
    err = "cannot open " + path;
    return false;
  }
  long n = -1;
  if (std::fscanf(fp, "%ld", &n) != 1 || n < 0) {
    std::fclose(fp);
    err = "bad board count in " + path;
    return false;
  }
  int c;
  while ((c = std::fgetc(fp)) != EOF && (c == ' ' || c == '\t' || c == '\r' || c == '\n')) {
  }
  if (c != EOF) std::ungetc(c, fp);
  out.clear();
  out.reserve(static_cast<size_t>(n));
  std::string line;
  for (long i = 0; i < n; ++i) {
    if (!read_line(fp, line)) {
      std::fclose(fp);
      err = "Failed to load boards";
      return false;
    }
    Board b;
    if (line.size() < 16 || !decode(line.c_str(), b.p, b.o)) {
      std::fclose(fp);
      err = "bad board on line " + std::to_string(i + 2) + " of " + path;
      return false;
    }
    out.push_back(b);
  }
  std::fclose(fp);
  std::sort(out.begin(), out.end());
  out.erase(std::unique(out.begin(), out.end()), out.end());
  return true;
}

bool write_results(const std::string& path, const std::vector<Board>& boards,
                   const std::vector<int8_t>& score, std::string& err) {
  std::FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) {
    err = "cannot open " + path + " for writing";
    return false;
  }
  char buf[17];
  for (size_t i = 0; i < boards.size(); ++i) {
    encode(boards[i].p, boards[i].o, buf);
    std::fprintf(fp, "%s %d\n", buf, static_cast<int>(score[i]));
  }
  if (std::fclose(fp) != 0) {
    err = "write failed: " + path;
    return false;
  }
  return true;
}

std::string move_string(int move) {
  if (move == 64) return "ps";
  std::string s(1, static_cast<char>('A' + move % 8));
  s += static_cast<char>('1' + move / 8);
  return s;
}

bool write_think_results(const std::string& path, const std::vector<Board>& boards,
                         const std::vector<int8_t>& score, const std::vector<int8_t>& best,
                         std::string& err) {
  std::FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) {
    err = "cannot open " + path + " for writing";
    return false;
  }
  char buf[17];
  for (size_t i = 0; i < boards.size(); ++i) {
    encode(boards[i].p, boards[i].o, buf);
    std::fprintf(fp, "%s %d %s\n", buf, static_cast<int>(score[i]),
                 move_string(best[i]).c_str());
  }
  if (std::fclose(fp) != 0) {
    err = "write failed: " + path;
    return false;
  }
  return true;
}

bool write_boards(const std::string& path, const std::vector<Board>& boards, std::string& err) {
  std::FILE* fp = std::fopen(path.c_str(), "w");
  if (!fp) {
    err = "cannot open " + path + " for writing";
    return false;
  }
  char buf[17];
  std::fprintf(fp, "%zu\n", boards.size());
  for (const Board& b : boards) {
    encode(b.p, b.o, buf);
    std::fprintf(fp, "%s\n", buf);
  }
  if (std::fclose(fp) != 0) {
    err = "write failed: " + path;
    return false;
  }
  return true;
}

}  // namespace gpo_host
