// Host-side bulk work split over threads: comparing a caller's sparsity
// pattern with the resident one, copying patterns into output containers, and
// the first touch of large output arrays.  One thread moves about 16 GB/s on
// the GB300's Grace host, eight to sixteen about 90 GB/s (sixteen map fresh
// pages fastest); host-device copies of pageable memory that is already
// mapped run at about 180 GB/s there, so on the drop-ins' path these host
// loops, not the copies, set the time.
#pragma once

#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <cstddef>
#include <cstring>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace lace {

// Parked host threads for the bulk loops below: waking one costs a few
// microseconds where creating and joining one costs tens, and a drop-in call
// runs several of these loops.  One region runs at a time.  A region asked
// for while another runs (from another thread, or from inside a region) and
// any region in a forked child (whose copy of the pool has no threads) get
// threads of their own instead.  The pool lives until the process exits.
class HostPool {
 public:
  static HostPool *get() {
    static HostPool *pool = new HostPool(
        (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency())) - 1);
    return pool;
  }
  // f(t) for t in [0, nt) on the caller (t = 0) and nt - 1 parked threads;
  // false (nothing run) when the pool cannot take the region now
  bool try_run(int nt, const std::function<void(int)> &f) {
    if (nt - 1 > workers_ || getpid() != pid_) return false;
    std::unique_lock<std::mutex> busy(run_mu_, std::try_to_lock);
    if (!busy.owns_lock()) return false;
    {
      std::lock_guard<std::mutex> l(mu_);
      job_ = &f;
      nt_ = nt;
      left_ = nt - 1;
      ++gen_;
    }
    wake_.notify_all();
    f(0);
    std::unique_lock<std::mutex> l(mu_);
    done_.wait(l, [&] { return left_ == 0; });
    job_ = nullptr;
    return true;
  }

 private:
  // the workers that could be started (none when the process may start no
  // more threads: every region then takes the path without the pool)
  explicit HostPool(int workers) : pid_(getpid()) {
    for (int t = 1; t <= workers; ++t) {
      try {
        std::thread([this, t] { loop(t); }).detach();
      } catch (...) {
        break;
      }
      workers_ = t;
    }
  }
  void loop(int id) {
    unsigned long seen = 0;
    std::unique_lock<std::mutex> l(mu_);
    for (;;) {
      wake_.wait(l, [&] { return gen_ != seen; });
      seen = gen_;
      if (id >= nt_) continue;
      const std::function<void(int)> *f = job_;
      l.unlock();
      (*f)(id);
      l.lock();
      if (--left_ == 0) done_.notify_one();
    }
  }
  int workers_ = 0;
  const pid_t pid_;
  std::mutex run_mu_, mu_;
  std::condition_variable wake_, done_;
  const std::function<void(int)> *job_ = nullptr;
  int nt_ = 0, left_ = 0;
  unsigned long gen_ = 0;
};

// f(t) for t in [0, nt): on the pool, else on threads started for it
inline void par_run(int nt, const std::function<void(int)> &f) {
  if (nt <= 1) {
    f(0);
    return;
  }
  if (HostPool::get()->try_run(nt, f)) return;
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(f, t);
  f(0);
  for (auto &x : th) x.join();
}

// threads for a bulk operation over `bytes`: one per 4 MB, at most 16
inline int host_threads(size_t bytes) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t want = bytes / ((size_t)4 << 20);
  return (int)std::max<size_t>(1, std::min<size_t>({want, (size_t)16, (size_t)hw}));
}

// f(offset, length) over `bytes` cut into 64-byte aligned ranges, the calling
// thread taking the first
template <typename F>
void par_ranges(size_t bytes, F f) {
  const int nt = host_threads(bytes);
  if (nt <= 1) {
    if (bytes) f((size_t)0, bytes);
    return;
  }
  const size_t per = ((bytes + nt - 1) / nt + 63) & ~(size_t)63;
  par_run(nt, [&](int t) {
    const size_t o = per * t;
    if (o < bytes) f(o, std::min(per, bytes - o));
  });
}

// f(begin, end) over [0, count) cut into one range per thread (`grain`
// items per thread at least), the calling thread taking the first
template <typename F>
void par_for(size_t count, size_t grain, F f) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::max<size_t>(1, std::min<size_t>({(size_t)16, (size_t)hw, count / std::max<size_t>(1, grain)}));
  if (nt <= 1) {
    if (count) f((size_t)0, count);
    return;
  }
  const size_t per = (count + nt - 1) / nt;
  par_run((int)nt, [&](int t) {
    const size_t b = per * t;
    if (b < count) f(b, std::min(count, b + per));
  });
}

inline bool par_equal(const void *a, const void *b, size_t bytes) {
  const int nt = host_threads(bytes);
  std::vector<char> diff(nt + 1, 0);
  const size_t per = ((bytes + nt - 1) / nt + 63) & ~(size_t)63;
  par_ranges(bytes, [&](size_t o, size_t len) {
    diff[o / per] = memcmp((const char *)a + o, (const char *)b + o, len) != 0;
  });
  for (char d : diff)
    if (d) return false;
  return true;
}

inline void par_copy(void *dst, const void *src, size_t bytes) {
  par_ranges(bytes, [&](size_t o, size_t len) { memcpy((char *)dst + o, (const char *)src + o, len); });
}

// zero (and so map) fresh memory before the GPU writes into it: faults taken
// inside a device-to-host copy cost several times more
inline void par_zero(void *dst, size_t bytes) {
  par_ranges(bytes, [&](size_t o, size_t len) { memset((char *)dst + o, 0, len); });
}

}  // namespace lace
