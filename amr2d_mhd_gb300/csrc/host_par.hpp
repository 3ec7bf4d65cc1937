// Host-side parallel loops over independent items (instances of a batch).
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <exception>
#include <functional>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace amr {

// Host worker threads kept for the life of an engine, so that a parallel loop
// costs a wake-up instead of thread creation.  run(n, body) calls body(w) for
// w in [0, n), w = 0 on the calling thread, and returns when all have
// returned.  One job at a time (an engine is driven by one thread).
class HostPool {
 public:
  HostPool() = default;
  HostPool(const HostPool &) = delete;
  HostPool &operator=(const HostPool &) = delete;
  ~HostPool() {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : threads_) t.join();
  }

  void run(size_t n, const std::function<void(size_t)> &body) {
    if (n <= 1) {
      body(0);
      return;
    }
    {
      std::lock_guard<std::mutex> g(m_);
      while (threads_.size() + 1 < n) {
        const size_t idx = threads_.size() + 1;
        threads_.emplace_back([this, idx] { worker(idx); });
      }
      job_ = &body;
      want_ = n - 1;
      pending_ = n - 1;
      gen_++;
    }
    cv_.notify_all();
    std::exception_ptr ex;
    try {
      body(0);
    } catch (...) {
      ex = std::current_exception();
    }
    {
      std::unique_lock<std::mutex> g(m_);
      done_.wait(g, [this] { return pending_ == 0; });
      job_ = nullptr;
    }
    if (ex) std::rethrow_exception(ex);
  }

 private:
  void worker(size_t idx) {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> g(m_);
    for (;;) {
      cv_.wait(g, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      if (idx > want_) continue;  // not needed for this job
      const std::function<void(size_t)> *job = job_;
      g.unlock();
      try {
        (*job)(idx);
      } catch (...) {
      }
      g.lock();
      if (--pending_ == 0) done_.notify_all();
    }
  }

  std::mutex m_;
  std::condition_variable cv_, done_;
  std::vector<std::thread> threads_;
  const std::function<void(size_t)> *job_ = nullptr;
  size_t want_ = 0, pending_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

// Runs body(worker, item) for items 0..n-1 on up to `threads` threads of
// `pool` (dynamic assignment); returns the first exception's message, if any.
template <typename F>
inline std::string parallel_items(HostPool &pool, size_t n, size_t threads, F body) {
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
    pool.run(threads, work);
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
