// CPU checks of the autotuner's decisions (onionpirv2_gb300/csrc/tune_core.h):
// the fastest measurement wins, unavailable ones never do, batch sizes map to
// the nearest measured size below them.
#include <cstdio>

#include "tune_core.h"

using namespace opir::tune;

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);  \
      ++failures;                                                  \
    }                                                              \
  } while (0)

int main() {
  const float a[] = {3.0f, 1.5f, -1.0f, 1.5f};
  CHECK(pick(a, 4) == 1);  // fastest, first of a tie
  const float none[] = {-1.0f, -2.0f};
  CHECK(pick(none, 2) == -1);
  const float only_last[] = {-1.0f, -1.0f, 9.0f};
  CHECK(pick(only_last, 3) == 2);

  uint32_t pts[kMaxPoints];
  CHECK(batch_points(1, pts) == 0);
  CHECK(batch_points(2, pts) == 1 && pts[0] == 2);
  CHECK(batch_points(48, pts) == 5 && pts[4] == 32);
  CHECK(batch_points(64, pts) == 6 && pts[5] == 64);
  CHECK(batch_points(100000, pts) == kMaxPoints && pts[kMaxPoints - 1] == 256);

  // scan wins at 2, tensor from 4, tensor unavailable at 64 -> integer GEMM
  const uint32_t b[] = {2, 4, 8, 16, 32, 64};
  const float ms[6][kEngines] = {{1.3f, 2.0f, 1.4f}, {2.6f, 2.1f, 1.5f}, {5.2f, 2.3f, 1.7f},
                                 {10.4f, 2.9f, 2.0f}, {20.8f, 4.4f, 3.6f}, {41.6f, 8.0f, -1.0f}};
  EngineTable t;
  CHECK(engine_at(t, 32) == 0);  // untuned
  build_table(t, b, 6, ms);
  CHECK(t.points == 6);
  CHECK(engine_at(t, 1) == 0);
  CHECK(engine_at(t, 2) == 1 && engine_at(t, 3) == 1);
  CHECK(engine_at(t, 4) == 3 && engine_at(t, 7) == 3 && engine_at(t, 63) == 3);
  CHECK(engine_at(t, 64) == 2 && engine_at(t, 1000) == 2);
  // a point where nothing ran falls back to one scan per query
  const float dead[1][kEngines] = {{-1.0f, -1.0f, -1.0f}};
  EngineTable u;
  build_table(u, b, 1, dead);
  CHECK(engine_at(u, 2) == 1);

  // a form or ring timed on its own replaces the default only when more than
  // kTuneMargin faster
  const float near[3] = {1.00f, 0.98f, 1.20f}, far[3] = {1.00f, 0.90f, 1.20f};
  CHECK(pick_over(near, 3, 0, kTuneMargin) == 0);
  CHECK(pick_over(far, 3, 0, kTuneMargin) == 1);
  const float gone[3] = {-1.0f, 0.98f, 1.20f};
  CHECK(pick_over(gone, 3, 0, kTuneMargin) == 1);  // default unavailable
  CHECK(pick_over(near, 3, -1, kTuneMargin) == 1);

  // tree forms, timed inside their stage's whole launch sequence, take the
  // smaller kSeqMargin; a form the GPU cannot place (the ten-CTA cluster)
  // is -1 and never chosen
  const float seq[4] = {0.2504f, 0.2480f, 0.2530f, -1.0f};
  CHECK(pick_over(seq, 4, 2, kSeqMargin) == 1);   // 2 % faster than the default
  const float seq_near[4] = {0.2504f, 0.2500f, 0.2510f, 0.2499f};
  CHECK(pick_over(seq_near, 4, 1, kSeqMargin) == 1);  // within 1 %: keep the default
  const float seq_wide[4] = {0.2811f, 0.2647f, 0.2536f, 0.2503f};
  CHECK(pick_over(seq_wide, 4, 2, kSeqMargin) == 3);  // the ten-CTA form, 1.3 % faster

  if (failures) return 1;
  std::printf("all checks passed\n");
  return 0;
}
