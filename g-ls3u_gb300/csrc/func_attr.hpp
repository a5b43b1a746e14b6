// func_attr.hpp -- per-device bookkeeping of kernel attributes (host only).
//
// cudaFuncSetAttribute (the dynamic shared-memory limit of a kernel) applies
// to the device that is current when it is called.  A process that drives
// several GPUs, or several host threads making their first launch at the
// same time, therefore needs the record of "already raised" kept per
// (kernel, device) and under a lock.  The class is plain C++ so that it can
// be tested without a GPU.
#pragma once

#include <map>
#include <mutex>
#include <utility>

namespace glsu {

class FuncAttrCache {
public:
    // True when the limit of `func` on `device` is below `bytes` (the caller
    // then raises it and calls done()); false when a limit of at least
    // `bytes` was recorded for that device.
    bool needs(const void *func, int device, int bytes)
    {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = set_.find(std::make_pair(func, device));
        return it == set_.end() || it->second < bytes;
    }
    // Record that `func` on `device` now accepts `bytes` of dynamic shared memory.
    void done(const void *func, int device, int bytes)
    {
        std::lock_guard<std::mutex> lock(mu_);
        int &v = set_[std::make_pair(func, device)];
        if (v < bytes) v = bytes;
    }
    int recorded(const void *func, int device)
    {
        std::lock_guard<std::mutex> lock(mu_);
        auto it = set_.find(std::make_pair(func, device));
        return it == set_.end() ? 0 : it->second;
    }

private:
    std::mutex mu_;
    std::map<std::pair<const void *, int>, int> set_;
};

}  // namespace glsu
