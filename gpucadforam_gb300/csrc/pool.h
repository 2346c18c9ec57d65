// First-fit range allocator over one pre-reserved region (device pool or
// pinned host arena).  Host-only logic: it hands out offsets, never touches
// the memory, and is usable (and tested) without a GPU.
#pragma once

#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <iterator>
#include <map>
#include <mutex>

namespace gcm {

class RangePool {
 public:
  explicit RangePool(size_t size = 0, size_t align = 256) { reset(size, align); }

  void reset(size_t size, size_t align = 256) {
    std::lock_guard<std::mutex> lock(m_);
    size_ = size;
    align_ = align;
    used_ = peak_ = 0;
    free_.clear();
    if (size) free_[0] = size;
  }

  // Reserves `bytes` (rounded up to the alignment); false when no free range
  // is large enough right now.
  bool try_alloc(size_t bytes, size_t* off) {
    std::lock_guard<std::mutex> lock(m_);
    return alloc_locked(bytes, off);
  }

  // Waits until the reservation succeeds, the request can never fit
  // (returns false), `stop()` returns true, or timeout_ms elapses.
  template <class Stop>
  bool alloc_wait(size_t bytes, size_t* off, Stop stop, int64_t timeout_ms) {
    std::unique_lock<std::mutex> lock(m_);
    const size_t need = round(bytes);
    if (need > size_) return false;
    auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
    while (!alloc_locked(bytes, off)) {
      if (stop()) return false;
      if (cv_.wait_until(lock, deadline) == std::cv_status::timeout) return alloc_locked(bytes, off);
    }
    return true;
  }

  void release(size_t off, size_t bytes) {
    {
      std::lock_guard<std::mutex> lock(m_);
      const size_t n = round(bytes);
      used_ -= n;
      auto it = free_.emplace(off, n).first;
      // merge with the next range
      auto nx = std::next(it);
      if (nx != free_.end() && it->first + it->second == nx->first) {
        it->second += nx->second;
        free_.erase(nx);
      }
      // merge with the previous range
      if (it != free_.begin()) {
        auto pv = std::prev(it);
        if (pv->first + pv->second == it->first) {
          pv->second += it->second;
          free_.erase(it);
        }
      }
    }
    cv_.notify_all();
  }

  void wake() { cv_.notify_all(); }

  size_t size() const { return size_; }
  size_t used() {
    std::lock_guard<std::mutex> lock(m_);
    return used_;
  }
  size_t peak() {
    std::lock_guard<std::mutex> lock(m_);
    return peak_;
  }
  size_t free_ranges() {
    std::lock_guard<std::mutex> lock(m_);
    return free_.size();
  }
  size_t largest_free() {
    std::lock_guard<std::mutex> lock(m_);
    size_t best = 0;
    for (auto& kv : free_) best = kv.second > best ? kv.second : best;
    return best;
  }
  size_t round(size_t bytes) const { return (bytes + align_ - 1) / align_ * align_ + (bytes == 0 ? align_ : 0); }

 private:
  bool alloc_locked(size_t bytes, size_t* off) {
    const size_t n = round(bytes);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        const size_t rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used_ += n;
        if (used_ > peak_) peak_ = used_;
        return true;
      }
    }
    return false;
  }

  std::mutex m_;
  std::condition_variable cv_;
  std::map<size_t, size_t> free_;  // offset -> length
  size_t size_ = 0, align_ = 256, used_ = 0, peak_ = 0;
};

}  // namespace gcm
