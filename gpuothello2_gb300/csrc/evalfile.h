// Host side of the pattern evaluator: reading the reference's two evaluator
// files and building the tables the think kernels use.
//
// Feature file (eval.cu:14-24): the feature count, then for each feature 8
// rows, each read like a std::bitset<8> (after optional whitespace, up to 8
// characters '0'/'1', the first one the highest bit); row j is byte j of
// the feature's square mask.  Value file (eval.cu:26-51): for each feature
// in order, 3^k doubles (k = the mask's square count, native byte order),
// then one double, the offset.  Values are used as float, as the reference
// stores them.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gpuothello2.h"
#include "think.cuh"

namespace gpo {
namespace think {

struct EvalHost {
  EvalMeta meta;
  std::vector<unsigned> digits;  // meta.npairs tables of 256 entries
  std::vector<float> values;
};

inline unsigned pow3u(int k) {
  unsigned r = 1;
  while (k-- > 0) r *= 3u;
  return r;
}

// Tables for `n` features; `values` holds every feature's 3^k entries in
// order.  Returns GPO_OK or GPO_ERR_ARG (too many features, squares or
// byte tables).
inline int build_eval(const uint64_t* features, int n, const double* values, double offset,
                      EvalHost* out) {
  if (n < 1 || n > kMaxFeatures || !features || !values || !out) return GPO_ERR_ARG;
  EvalMeta m = {};
  m.nf = n;
  m.offset = static_cast<float>(offset);
  std::vector<unsigned> digits;
  size_t total = 0;
  int pairs = 0;
  for (int j = 0; j < n; ++j) {
    const uint64_t mask = features[j];
    const int k = __builtin_popcountll(mask);
    if (k > kMaxFeatureBits) return GPO_ERR_ARG;
    m.value_off[j] = static_cast<unsigned>(total);
    total += pow3u(k);
    m.pair_begin[j] = static_cast<unsigned char>(pairs);
    int rank = 0;  // squares of the mask below the current byte
    for (int b = 0; b < 8; ++b) {
      const unsigned byte_mask = static_cast<unsigned>((mask >> (8 * b)) & 0xFF);
      if (!byte_mask) continue;
      if (pairs == kMaxPairs) return GPO_ERR_ARG;
      m.pair_byte[pairs] = static_cast<unsigned char>(b);
      for (unsigned v = 0; v < 256; ++v) {
        unsigned w = 0;
        int r = rank;
        for (int i = 0; i < 8; ++i) {
          if (!((byte_mask >> i) & 1)) continue;
          if ((v >> i) & 1) w += pow3u(r);
          ++r;
        }
        digits.push_back(w);
      }
      rank += __builtin_popcount(byte_mask);
      ++pairs;
    }
  }
  m.pair_begin[n] = static_cast<unsigned char>(pairs);
  m.npairs = pairs;
  out->meta = m;
  out->digits.swap(digits);
  out->values.resize(total);
  for (size_t i = 0; i < total; ++i) out->values[i] = static_cast<float>(values[i]);
  return GPO_OK;
}

inline bool read_text(const char* path, std::string* text) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[4096];
  size_t got;
  text->clear();
  while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) text->append(buf, got);
  std::fclose(f);
  return true;
}

inline bool is_space(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t' || c == '\f' || c == '\v'; }

// Returns GPO_OK, GPO_ERR_IO (unreadable) or GPO_ERR_ARG (malformed).
inline int read_feature_file(const char* path, std::vector<uint64_t>* masks) {
  std::string s;
  if (!path || !read_text(path, &s)) return GPO_ERR_IO;
  size_t pos = 0;
  while (pos < s.size() && is_space(s[pos])) ++pos;
  size_t count = 0;
  const size_t start = pos;
  while (pos < s.size() && s[pos] >= '0' && s[pos] <= '9') count = count * 10 + (s[pos++] - '0');
  if (pos == start || count < 1 || count > static_cast<size_t>(kMaxFeatures)) return GPO_ERR_ARG;
  masks->assign(count, 0);
  for (size_t f = 0; f < count; ++f) {
    for (int row = 0; row < 8; ++row) {
      while (pos < s.size() && is_space(s[pos])) ++pos;
      unsigned v = 0;
      int got = 0;
      while (got < 8 && pos < s.size() && (s[pos] == '0' || s[pos] == '1')) {
        v = (v << 1) | static_cast<unsigned>(s[pos++] - '0');
        ++got;
      }
      if (got == 0) return GPO_ERR_ARG;
      (*masks)[f] |= static_cast<uint64_t>(v) << (8 * row);
    }
  }
  return GPO_OK;
}

// Reads the value file for `masks`; GPO_ERR_IO if it is missing or short.
inline int read_value_file(const char* path, const std::vector<uint64_t>& masks,
                           std::vector<double>* values, double* offset) {
  size_t total = 0;
  for (uint64_t m : masks) {
    const int k = __builtin_popcountll(m);
    if (k > kMaxFeatureBits) return GPO_ERR_ARG;
    total += pow3u(k);
  }
  FILE* f = path ? std::fopen(path, "rb") : nullptr;
  if (!f) return GPO_ERR_IO;
  values->resize(total);
  const size_t got = std::fread(values->data(), sizeof(double), total, f);
  const size_t got_off = std::fread(offset, sizeof(double), 1, f);
  std::fclose(f);
  return (got == total && got_off == 1) ? GPO_OK : GPO_ERR_IO;
}

}  // namespace think
}  // namespace gpo
