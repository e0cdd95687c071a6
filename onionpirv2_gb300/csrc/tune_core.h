// tune_core.h -- host-side decisions of the autotuner (opir_autotune),
// free of CUDA so that they can be tested on the CPU.
//
// The tuner times, on the device and for one resident database, every
// compiled tile configuration of the single-query scan and every
// first-dimension engine (one scan per query, integer GEMM, tensor-core limb
// GEMM) at the batch sizes 2, 4, ..., max_batch.  These functions turn the
// measured times into the database's choices.
#pragma once

#include <cstdint>

namespace opir {
namespace tune {

constexpr int kMaxPoints = 8;  // batch sizes 2^1 .. 2^8
constexpr int kEngines = 3;    // OPIR_ENGINE_SCAN, _IMAD, _TENSOR (1, 2, 3)

// index of the fastest of n measurements; entries < 0 are unavailable;
// -1 if none is available.  Ties keep the lower index.
inline int pick(const float *ms, int n) {
  int best = -1;
  for (int i = 0; i < n; i++)
    if (ms[i] >= 0 && (best < 0 || ms[i] < ms[best])) best = i;
  return best;
}

// Launch forms and ring shapes timed on their own, outside the pipeline,
// replace the default only when at least this much faster.
constexpr float kTuneMargin = 0.03f;
// A form timed inside its stage's whole launch sequence replaces the
// default when the sequence gets at least this much faster.
constexpr float kSeqMargin = 0.01f;

// the fastest of n measurements if it beats measurement `dflt` by more than
// `margin` (a fraction of dflt's time), else dflt; pick() when dflt is
// unavailable
inline int pick_over(const float *ms, int n, int dflt, float margin) {
  const int best = pick(ms, n);
  if (dflt < 0 || dflt >= n || ms[dflt] < 0 || best < 0) return best;
  return ms[best] < ms[dflt] * (1.0f - margin) ? best : dflt;
}

// batch sizes measured for max_batch: 2, 4, ... up to the largest power of
// two <= max_batch (at most kMaxPoints); returns how many
inline int batch_points(uint32_t max_batch, uint32_t *out) {
  int n = 0;
  for (uint32_t b = 2; b <= max_batch && n < kMaxPoints; b *= 2) out[n++] = b;
  return n;
}

struct EngineTable {
  int points = 0;                 // 0: not tuned
  uint32_t batch[kMaxPoints] = {};
  int engine[kMaxPoints] = {};    // OPIR_ENGINE_* chosen at batch[i]
};

// The engine for a batch of `batch` queries: the choice at the largest
// measured size not above it (the smallest point below it); 0 when the table
// is empty or batch < 2.
inline int engine_at(const EngineTable &t, int batch) {
  if (t.points == 0 || batch < 2) return 0;
  int e = t.engine[0];
  for (int i = 0; i < t.points; i++)
    if ((uint32_t)batch >= t.batch[i]) e = t.engine[i];
  return e;
}

// fill the table from ms[point][engine - 1] (engine 1..3; < 0 = unavailable)
inline void build_table(EngineTable &t, const uint32_t *batch, int points,
                        const float (*ms)[kEngines]) {
  t.points = points;
  for (int i = 0; i < points; i++) {
    t.batch[i] = batch[i];
    const int k = pick(ms[i], kEngines);
    t.engine[i] = k < 0 ? 1 : k + 1;
  }
}

}  // namespace tune
}  // namespace opir
