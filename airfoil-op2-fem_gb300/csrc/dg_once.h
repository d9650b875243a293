// Per-(device, order) set-up bookkeeping (host only).
//
// __constant__ and file-scope __device__ tables, and the dynamic shared-memory limits set with
// cudaFuncSetAttribute, belong to one device: each GPU that loads the library holds its own copy,
// written only by uploads made while that device is current.  A process that drives two GPUs
// must therefore run the uploads once per (device, order) pair, not once per order.  OnceTable
// records which pairs are done and serialises the uploads: ensure() runs the loader for a pair at
// most once until it succeeds, and two host threads that ask for the same pair at the same time
// both return only after the one upload has finished (its writes are visible to both through
// the lock).
#pragma once

#include <mutex>

namespace dg {

constexpr int kMaxDevices = 64;

class OnceTable {
 public:
  // Slot 0..kSlots-1 per device (orders 1..6 use their own index; 0 is free for other set-up).
  static constexpr int kSlots = 7;

  // Runs load() for (dev, slot) unless an earlier call for that pair succeeded; returns load()'s
  // code (0 = success, then the pair is recorded), or -1 for a pair out of range.
  template <class F>
  int ensure(int dev, int slot, F &&load) {
    if (dev < 0 || dev >= kMaxDevices || slot < 0 || slot >= kSlots) return -1;
    std::lock_guard<std::mutex> g(mu_);
    if (done_[dev][slot]) return 0;
    const int rc = load();
    if (rc == 0) done_[dev][slot] = 1;
    return rc;
  }

  // 1 if (dev, slot) is set up, 0 if not, -1 out of range.
  int done(int dev, int slot) const {
    if (dev < 0 || dev >= kMaxDevices || slot < 0 || slot >= kSlots) return -1;
    std::lock_guard<std::mutex> g(mu_);
    return done_[dev][slot];
  }

 private:
  mutable std::mutex mu_;
  unsigned char done_[kMaxDevices][kSlots] = {};
};

}  // namespace dg
