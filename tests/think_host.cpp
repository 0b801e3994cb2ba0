// Host build of the think-mode search and evaluator (test infrastructure).
//
// gpuothello2_gb300/csrc/think.cuh is written once for the device and the
// host; the CUDA kernels in think.cu run it per thread.  Compiled here as
// plain C++, the same search, evaluator and file readers (evalfile.h) can be
// checked against the oracle and the reference's fixtures on a machine
// without a GPU.  The product never links this file.
#include <cstdint>
#include <vector>

#include "../gpuothello2_gb300/csrc/evalfile.h"
#include "../gpuothello2_gb300/csrc/think.cuh"

namespace th = gpo::think;

static th::EvalHost g_eval;
static bool g_loaded = false;

extern "C" {

int th_load(const uint64_t* features, int n, const double* values, double offset) {
  g_loaded = false;
  const int rc = th::build_eval(features, n, values, offset, &g_eval);
  g_loaded = rc == GPO_OK;
  return rc;
}

int th_load_files(const char* features_path, const char* values_path) {
  std::vector<uint64_t> masks;
  int rc = th::read_feature_file(features_path, &masks);
  if (rc != GPO_OK) return rc;
  std::vector<double> values;
  double offset = 0.0;
  rc = th::read_value_file(values_path, masks, &values, &offset);
  if (rc != GPO_OK) return rc;
  return th_load(masks.data(), static_cast<int>(masks.size()), values.data(), offset);
}

// Masks of a feature file: returns the count, or a negative status.
int th_read_features(const char* path, uint64_t* masks, int cap) {
  std::vector<uint64_t> m;
  const int rc = th::read_feature_file(path, &m);
  if (rc != GPO_OK) return rc;
  for (size_t i = 0; i < m.size() && static_cast<int>(i) < cap; ++i) masks[i] = m[i];
  return static_cast<int>(m.size());
}

int th_evaluate(const uint64_t* p, const uint64_t* o, int n, float* out) {
  if (!g_loaded) return GPO_ERR_ARG;
  for (int i = 0; i < n; ++i)
    out[i] = th::evaluate(p[i], o[i], g_eval.meta, g_eval.digits.data(), g_eval.values.data());
  return GPO_OK;
}

int th_think(const uint64_t* p, const uint64_t* o, int n, int depth, int8_t* score, int8_t* best,
             uint64_t* nodes) {
  if (!g_loaded) return GPO_ERR_ARG;
  if (depth < th::kMinDepth || depth > th::kMaxDepth) return GPO_ERR_DEPTH;
  th::Frame fr[th::kMaxDepth];
  unsigned char lists[th::kMaxDepth - 3][th::kMaxMoves];
  for (int i = 0; i < n; ++i) {
    int bm = th::kMoveNone;
    unsigned long long nd = 0;
    score[i] = static_cast<int8_t>(th::search(p[i], o[i], depth, g_eval.meta,
                                              g_eval.digits.data(), g_eval.values.data(), fr,
                                              lists, &bm, &nd));
    best[i] = static_cast<int8_t>(bm);
    nodes[i] = nd;
  }
  return GPO_OK;
}

uint64_t th_transpose(uint64_t x) { return th::transpose(x); }
uint64_t th_flip_rows(uint64_t x) { return th::flip_rows(x); }
uint64_t th_mobility(uint64_t p, uint64_t o) { return th::mobility(p, o); }
uint64_t th_flips(uint64_t p, uint64_t o, int sq) { return th::flips(p, o, sq); }

}  // extern "C"
