// Host-side parallel loops over independent items (instances of a batch).
#pragma once

#include <atomic>
#include <cstddef>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace amr {

// Runs body(worker, item) for items 0..n-1 on up to `threads` host threads
// (dynamic assignment); returns the first exception's message, if any.
template <typename F>
inline std::string parallel_items(size_t n, size_t threads, F body) {
  std::atomic<size_t> next{0};
  std::mutex mu;
  std::string err;
  auto work = [&](size_t w) {
    for (;;) {
      const size_t q = next.fetch_add(1);
      if (q >= n) break;
      try {
        body(w, q);
      } catch (const std::exception &ex) {
        std::lock_guard<std::mutex> g(mu);
        if (err.empty()) err = ex.what();
      }
    }
  };
  if (threads > n) threads = n;
  if (threads <= 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (size_t w = 1; w < threads; w++) th.emplace_back(work, w);
    work(0);
    for (auto &t : th) t.join();
  }
  return err;
}

inline size_t host_threads(size_t work_blocks) {
  if (work_blocks < 2048) return 1;  // thread start-up would cost more than the work
  const unsigned hw = std::thread::hardware_concurrency();
  const size_t n = hw ? hw : 1;
  return n > 32 ? 32 : n;
}

}  // namespace amr
