// CPU test of the staging ring's bookkeeping (natural_number_gb300/csrc/
// stage_ring.h) with host-side fake events: a region may be handed out again
// only once the copy that reads it is done.  Random sizes (including ones
// that wrap around the end of the ring) and random completion orders;
// exits non-zero on the first violation.
#include <cstdint>
#include <cstdio>
#include <random>
#include <set>

#include "stage_ring.h"

struct FakeEvents {
  using event = int;
  std::set<int> finished;  // copies that completed
  std::set<int> recycled;
  int waits = 0;
  bool done(int e) { return finished.count(e) != 0; }
  void wait(int e) {
    ++waits;
    finished.insert(e);
  }
  void recycle(int e) { recycled.insert(e); }
};

struct Copy {  // a queued copy reading [off, off + len)
  uint64_t off, len;
  int ev;
};

int main() {
  std::mt19937_64 rng(7);
  for (int trial = 0; trial < 200; ++trial) {
    FakeEvents ev;
    nn::RegionRing<FakeEvents> ring;
    ring.cap = 256ull << (2 + rng() % 6);  // 1 KiB .. 32 KiB
    std::vector<Copy> pending;
    int next_ev = 1;
    for (int step = 0; step < 400; ++step) {
      const uint64_t want = 1 + rng() % (ring.cap / 2);
      const uint64_t n = ring.granule(want);
      if (n > ring.cap) continue;
      const uint64_t off = ring.place(n, ev);
      if (off + n > ring.cap || off % 256) {
        std::printf("region [%llu, +%llu) outside the ring of %llu\n", (unsigned long long)off,
                    (unsigned long long)n, (unsigned long long)ring.cap);
        return 1;
      }
      for (const Copy& c : pending) {
        const bool busy = !ev.done(c.ev);
        if (busy && c.off < off + n && off < c.off + c.len) {
          std::printf("trial %d step %d: region [%llu, +%llu) handed out while copy %d reads [%llu, +%llu)\n", trial,
                      step, (unsigned long long)off, (unsigned long long)n, c.ev, (unsigned long long)c.off,
                      (unsigned long long)c.len);
          return 1;
        }
      }
      if (rng() % 10 == 0) {  // the copy could not be queued
        ring.drop();
      } else {
        ring.seal(next_ev);
        pending.push_back(Copy{off, n, next_ev});
        ++next_ev;
      }
      // some copies finish, in any order
      for (const Copy& c : pending)
        if (rng() % 3 == 0) ev.finished.insert(c.ev);
    }
    ring.drain(ev);
    if (!ring.live.empty()) return 1;
    for (const Copy& c : pending)
      if (!ev.recycled.count(c.ev)) {
        std::printf("event %d never recycled\n", c.ev);
        return 1;
      }
  }
  std::printf("ok\n");
  return 0;
}
