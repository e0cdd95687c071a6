// serve_core.h -- host-side policy of the serving loop (no CUDA): request
// queues per database, the continuous-batching dispatch rule, least-recently-
// used residency of client keys in a fixed pool of device slots, and latency
// percentiles.  capi.cu drives the GPU with it; tests/cpp/test_serve_core.cpp
// checks it on the CPU.
//
// The reference answers one query at a time (PirServer::make_query,
// server.cpp:520-579, keys in std::map members, server.h:58-59); this layer
// has no counterpart there.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <deque>
#include <limits>
#include <map>
#include <unordered_map>
#include <vector>

namespace opir {
namespace serve {

struct Pending {
  uint64_t ticket;
  uint32_t db;
  uint64_t client;
  double t_submit;  // seconds, any monotonic origin
};

// FIFO of pending requests per database.  A batch always serves one
// database: the one whose oldest request has waited longest, taking up to
// max_batch of its requests in arrival order.
class BatchQueue {
 public:
  void push(const Pending &p) {
    q_[p.db].push_back(p);
    ++n_;
  }
  size_t size() const { return n_; }
  size_t pending_for(uint32_t db) const {
    auto it = q_.find(db);
    return it == q_.end() ? 0 : it->second.size();
  }
  // submission time of the oldest pending request (+inf when empty)
  double oldest() const {
    double t = std::numeric_limits<double>::infinity();
    for (const auto &kv : q_)
      if (!kv.second.empty()) t = std::min(t, kv.second.front().t_submit);
    return t;
  }
  // database of the oldest pending request (the next batch's database)
  bool next_db(uint32_t *db) const {
    double t = std::numeric_limits<double>::infinity();
    bool found = false;
    for (const auto &kv : q_)
      if (!kv.second.empty() && kv.second.front().t_submit < t) {
        t = kv.second.front().t_submit;
        *db = kv.first;
        found = true;
      }
    return found;
  }
  std::vector<Pending> pop_batch(size_t max_batch) {
    std::vector<Pending> out;
    uint32_t db;
    if (!max_batch || !next_db(&db)) return out;
    auto &dq = q_[db];
    while (!dq.empty() && out.size() < max_batch) {
      out.push_back(dq.front());
      dq.pop_front();
    }
    n_ -= out.size();
    if (dq.empty()) q_.erase(db);
    return out;
  }

 private:
  std::map<uint32_t, std::deque<Pending>> q_;
  size_t n_ = 0;
};

// Continuous-batching rule: a free lane takes a batch at once when the device
// is otherwise idle; while another batch runs it waits for a full batch or
// until the oldest request has waited max_wait seconds.
inline bool should_dispatch(size_t pending, size_t max_batch, int busy_lanes, int free_lanes,
                            double oldest_wait, double max_wait) {
  if (!pending || free_lanes <= 0) return false;
  if (busy_lanes == 0) return true;
  if (pending >= max_batch) return true;
  return oldest_wait >= max_wait;
}

// Residency of client keys in `slots` fixed-size device slots, least recently
// used first out.  Pinned clients (keys read by a batch in flight) are never
// evicted.
class KeyLru {
 public:
  static constexpr uint64_t kNone = std::numeric_limits<uint64_t>::max();
  explicit KeyLru(int slots = 0) { reset(slots); }
  void reset(int slots) {
    slots_ = slots;
    tick_ = 0;
    by_client_.clear();
    owner_.assign(slots > 0 ? slots : 0, kNone);
  }
  int slots() const { return slots_; }
  int used() const { return (int)by_client_.size(); }
  int slot_of(uint64_t client) const {
    auto it = by_client_.find(client);
    return it == by_client_.end() ? -1 : it->second.slot;
  }
  // Make `client` resident.  Returns its slot (a free one, or the least
  // recently used unpinned one, whose client goes to *evicted), or -1 when
  // every slot is pinned.  *fresh tells whether the slot must be (re)filled.
  int admit(uint64_t client, uint64_t *evicted, bool *fresh) {
    *evicted = kNone;
    *fresh = false;
    auto it = by_client_.find(client);
    if (it != by_client_.end()) {
      it->second.last = ++tick_;
      return it->second.slot;
    }
    int slot = -1;
    for (int s = 0; s < slots_; ++s)
      if (owner_[s] == kNone) {
        slot = s;
        break;
      }
    if (slot < 0) {
      uint64_t best = kNone, best_tick = kNone;
      for (const auto &kv : by_client_)
        if (kv.second.pins == 0 && kv.second.last < best_tick) {
          best_tick = kv.second.last;
          best = kv.first;
        }
      if (best == kNone) return -1;
      slot = by_client_[best].slot;
      by_client_.erase(best);
      *evicted = best;
    }
    owner_[slot] = client;
    by_client_[client] = Entry{slot, ++tick_, 0};
    *fresh = true;
    return slot;
  }
  void touch(uint64_t client) {
    auto it = by_client_.find(client);
    if (it != by_client_.end()) it->second.last = ++tick_;
  }
  void pin(uint64_t client) {
    auto it = by_client_.find(client);
    if (it != by_client_.end()) it->second.pins++;
  }
  void unpin(uint64_t client) {
    auto it = by_client_.find(client);
    if (it != by_client_.end() && it->second.pins > 0) it->second.pins--;
  }
  bool pinned(uint64_t client) const {
    auto it = by_client_.find(client);
    return it != by_client_.end() && it->second.pins > 0;
  }
  void erase(uint64_t client) {
    auto it = by_client_.find(client);
    if (it == by_client_.end()) return;
    owner_[it->second.slot] = kNone;
    by_client_.erase(it);
  }

 private:
  struct Entry {
    int slot;
    uint64_t last;
    int pins;
  };
  int slots_ = 0;
  uint64_t tick_ = 0;
  std::unordered_map<uint64_t, Entry> by_client_;
  std::vector<uint64_t> owner_;
};

// Nearest-rank percentile (pct in [0, 100]) of v; 0 for an empty sample.
inline double percentile(std::vector<double> v, double pct) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double rank = std::ceil(pct / 100.0 * (double)v.size());
  size_t i = rank < 1 ? 0 : (size_t)rank - 1;
  if (i >= v.size()) i = v.size() - 1;
  return v[i];
}

}  // namespace serve
}  // namespace opir
