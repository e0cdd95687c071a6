// CPU checks of the serving policy (onionpirv2_gb300/csrc/serve_core.h):
// per-database FIFOs, the continuous-batching dispatch rule, least-recently-
// used key residency with pins, and nearest-rank percentiles.
#include <cstdio>
#include <cstdlib>
#include <set>

#include "serve_core.h"

using namespace opir::serve;

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);  \
      ++failures;                                                  \
    }                                                              \
  } while (0)

static void queue_tests() {
  BatchQueue q;
  CHECK(q.size() == 0);
  CHECK(q.pop_batch(8).empty());
  // db 2's first request is the oldest
  q.push({1, 1, 10, 5.0});
  q.push({2, 2, 11, 1.0});
  q.push({3, 1, 12, 6.0});
  q.push({4, 2, 13, 7.0});
  q.push({5, 2, 14, 8.0});
  CHECK(q.size() == 5);
  CHECK(q.oldest() == 1.0);
  uint32_t db = 0;
  CHECK(q.next_db(&db) && db == 2);
  auto b = q.pop_batch(2);  // db 2, arrival order, capped at 2
  CHECK(b.size() == 2 && b[0].ticket == 2 && b[1].ticket == 4);
  CHECK(q.size() == 3 && q.pending_for(2) == 1 && q.pending_for(1) == 2);
  b = q.pop_batch(8);  // now db 1 holds the oldest (t = 5)
  CHECK(b.size() == 2 && b[0].ticket == 1 && b[1].ticket == 3);
  b = q.pop_batch(8);
  CHECK(b.size() == 1 && b[0].ticket == 5 && b[0].client == 14);
  CHECK(q.size() == 0 && q.pop_batch(8).empty());
}

static void dispatch_tests() {
  // nothing pending / no free lane
  CHECK(!should_dispatch(0, 32, 0, 2, 0, 0.002));
  CHECK(!should_dispatch(5, 32, 2, 0, 1.0, 0.002));
  // idle device: go at once
  CHECK(should_dispatch(1, 32, 0, 2, 0.0, 0.002));
  // busy device: wait for a full batch or the deadline
  CHECK(!should_dispatch(5, 32, 1, 1, 0.001, 0.002));
  CHECK(should_dispatch(32, 32, 1, 1, 0.0, 0.002));
  CHECK(should_dispatch(5, 32, 1, 1, 0.0025, 0.002));
}

static void lru_tests() {
  KeyLru lru(2);
  uint64_t ev;
  bool fresh;
  CHECK(lru.admit(100, &ev, &fresh) == 0 && fresh && ev == KeyLru::kNone);
  CHECK(lru.admit(200, &ev, &fresh) == 1 && fresh);
  CHECK(lru.admit(100, &ev, &fresh) == 0 && !fresh);  // resident: touch only
  CHECK(lru.used() == 2);
  // 200 is now least recently used
  int s = lru.admit(300, &ev, &fresh);
  CHECK(s == 1 && ev == 200 && fresh && lru.slot_of(200) == -1 && lru.slot_of(300) == 1);
  // pinned clients are never evicted
  lru.pin(100);
  lru.pin(300);
  CHECK(lru.admit(400, &ev, &fresh) == -1);
  lru.unpin(300);
  s = lru.admit(400, &ev, &fresh);
  CHECK(s == 1 && ev == 300);
  CHECK(lru.pinned(100) && !lru.pinned(400));
  lru.unpin(100);
  lru.touch(100);  // 400 becomes the oldest
  s = lru.admit(500, &ev, &fresh);
  CHECK(s == 1 && ev == 400);
  lru.erase(100);
  CHECK(lru.slot_of(100) == -1 && lru.used() == 1);
  s = lru.admit(600, &ev, &fresh);
  CHECK(s == 0 && ev == KeyLru::kNone && fresh);
  // a randomised run: occupancy never exceeds the slots, pins always hold
  KeyLru r(5);
  std::set<uint64_t> pinned;
  srand(3);
  for (int i = 0; i < 20000; ++i) {
    const uint64_t c = (uint64_t)(rand() % 23);
    const int op = rand() % 4;
    if (op == 0 && !pinned.count(c) && r.slot_of(c) >= 0 && pinned.size() < 4) {
      r.pin(c);
      pinned.insert(c);
    } else if (op == 1 && pinned.count(c)) {
      r.unpin(c);
      pinned.erase(c);
    } else {
      const int slot = r.admit(c, &ev, &fresh);
      CHECK(slot >= 0);  // at most 4 of 5 slots are pinned
      CHECK(!pinned.count(ev));
    }
    CHECK(r.used() <= 5);
    for (uint64_t p : pinned) CHECK(r.slot_of(p) >= 0);
  }
}

static void percentile_tests() {
  CHECK(percentile({}, 50) == 0.0);
  std::vector<double> v;
  for (int i = 100; i >= 1; --i) v.push_back(i);
  CHECK(percentile(v, 50) == 50.0);
  CHECK(percentile(v, 99) == 99.0);
  CHECK(percentile(v, 100) == 100.0);
  CHECK(percentile(v, 0) == 1.0);
  CHECK(percentile({7.0}, 99) == 7.0);
}

int main() {
  queue_tests();
  dispatch_tests();
  lru_tests();
  percentile_tests();
  if (failures) {
    std::printf("%d checks failed\n", failures);
    return 1;
  }
  std::printf("serve_core: all checks passed\n");
  return 0;
}
