// Per-device, per-kernel cache of the dynamic shared-memory limit.
//
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) is a per-device property
// of a kernel that every later launch on that device is checked against.
// Several host threads launch the same kernel at different sizes (one
// red-black level's compressions run on worker threads, each at its own
// tree level), so the limit may only ever grow: a thread that set a smaller
// value between another thread's set and launch would make that launch fail
// with "invalid argument".  SmemLimit raises the limit under one mutex and
// never lowers it.  Host-only, so the rule is testable without a GPU.
#pragma once
#include <cstddef>
#include <map>
#include <mutex>
#include <utility>

namespace slu {

class SmemLimit {
 public:
  // Calls set(bytes) when (dev, kernel) has been given less than bytes, and
  // remembers bytes only if set() succeeded (returned 0).  Returns set()'s
  // result, or 0 when no call was needed.
  template <typename Setter>
  int raise(int dev, const void* kernel, std::size_t bytes, Setter set) {
    if (bytes <= kDefault) return 0;
    std::lock_guard<std::mutex> lock(mu_);
    std::size_t& cur = done_[std::make_pair(dev, kernel)];
    if (cur >= bytes) return 0;
    int rc = set(bytes);
    if (rc == 0) cur = bytes;
    return rc;
  }
  std::size_t current(int dev, const void* kernel) {
    std::lock_guard<std::mutex> lock(mu_);
    auto it = done_.find(std::make_pair(dev, kernel));
    return it == done_.end() ? 0 : it->second;
  }
  static constexpr std::size_t kDefault = 48 * 1024;

 private:
  std::mutex mu_;
  std::map<std::pair<int, const void*>, std::size_t> done_;
};

}  // namespace slu
