// stage_ring.h — the bookkeeping of the context's page-locked staging ring
// (engine.cpp, Stager): regions of a fixed buffer handed out in order, each
// reused only after the event recorded behind the copy that reads it.  The
// event operations are a policy, so that the same code runs with CUDA events
// in the library and with host-side fakes in the CPU tests.
#pragma once

#include <cstdint>
#include <vector>

namespace nn {

// Events must provide: using event = ...; bool done(event) (the copy
// finished: cudaEventQuery), void wait(event) (cudaEventSynchronize) and
// void recycle(event) (the event may be recorded again).
template <class Events>
struct RegionRing {
  using event = typename Events::event;
  struct Region {
    uint64_t off, len;
    event done;
  };
  uint64_t cap = 0, head = 0;
  std::vector<Region> live;  // oldest first

  static uint64_t granule(uint64_t n) { return (n + 255) & ~255ull; }

  void retire_front(Events& ev) {
    ev.recycle(live.front().done);
    live.erase(live.begin());
  }
  // Waits for every region still read by a copy.
  void drain(Events& ev) {
    while (!live.empty()) {
      ev.wait(live.front().done);
      retire_front(ev);
    }
  }
  // The offset of a region of n bytes (a multiple of 256, at most cap),
  // after waiting for the copies that still read any of it; the region
  // stays live until `seal` gives it its event (or `drop` removes it).
  uint64_t place(uint64_t n, Events& ev) {
    const uint64_t off = head + n <= cap ? head : 0;
    for (;;) {
      while (!live.empty() && ev.done(live.front().done)) retire_front(ev);
      bool overlap = false;
      for (const Region& r : live) overlap = overlap || (r.off < off + n && off < r.off + r.len);
      if (!overlap) break;
      ev.wait(live.front().done);
      retire_front(ev);
    }
    head = off + n;
    live.push_back(Region{off, n, event{}});
    return off;
  }
  // The region last placed is read by the copy that `e` follows.
  void seal(event e) { live.back().done = e; }
  // The region last placed is not read by any copy.
  void drop() { live.pop_back(); }
};

}  // namespace nn
