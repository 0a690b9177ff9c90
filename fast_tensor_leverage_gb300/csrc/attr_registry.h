// Bookkeeping of per-device kernel attributes (pure host C++, no CUDA).
//
// A kernel's dynamic shared-memory limit is a per-device setting:
// cudaFuncSetAttribute changes it for the current device only, so a process
// that launches the same kernel on two GPUs must raise it on each.  Setting
// it again on every call is not free either (it can wait for running
// launches of that kernel).  AttrRegistry remembers, per (kernel, device),
// the largest limit already set, and calls the setter only when a launch
// needs more.  It is thread-safe: the setter runs under the registry's lock,
// so two host threads never race on the same (kernel, device).
#pragma once

#include <map>
#include <mutex>
#include <utility>

namespace ftl {

class AttrRegistry {
  public:
    // Calls set(bytes) unless (func, dev) already holds a limit >= bytes;
    // records the limit only when set returns 0.  Returns 0 when nothing was
    // needed, else set's return value.
    template <class SetFn>
    int ensure(const void *func, int dev, int bytes, SetFn &&set) {
        std::lock_guard<std::mutex> lock(mu_);
        const auto key = std::make_pair(func, dev);
        const auto it = done_.find(key);
        if (it != done_.end() && it->second >= bytes) return 0;
        const int rc = set(bytes);
        if (rc == 0) done_[key] = bytes;
        return rc;
    }

    // The limit recorded for (func, dev), 0 when none.
    int limit(const void *func, int dev) {
        std::lock_guard<std::mutex> lock(mu_);
        const auto it = done_.find(std::make_pair(func, dev));
        return it == done_.end() ? 0 : it->second;
    }

  private:
    std::mutex mu_;
    std::map<std::pair<const void *, int>, int> done_;
};

}  // namespace ftl
