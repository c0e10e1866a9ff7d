// Host-side bulk work split over threads: comparing a caller's sparsity
// pattern with the resident one, copying patterns into output containers, and
// the first touch of large output arrays.  One thread moves about 16 GB/s on
// the GB300's Grace host, eight to sixteen about 90 GB/s (sixteen map fresh
// pages fastest); host-device copies of pageable memory that is already
// mapped run at about 180 GB/s there, so on the drop-ins' path these host
// loops, not the copies, set the time.
#pragma once

#include <algorithm>
#include <cstddef>
#include <cstring>
#include <thread>
#include <vector>

namespace lace {

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
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) {
    const size_t o = per * t;
    if (o >= bytes) break;
    th.emplace_back(f, o, std::min(per, bytes - o));
  }
  f((size_t)0, std::min(per, bytes));
  for (auto &x : th) x.join();
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
  std::vector<std::thread> th;
  for (size_t t = 1; t < nt; ++t) {
    const size_t b = per * t;
    if (b >= count) break;
    th.emplace_back(f, b, std::min(count, b + per));
  }
  f((size_t)0, std::min(count, per));
  for (auto &x : th) x.join();
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
