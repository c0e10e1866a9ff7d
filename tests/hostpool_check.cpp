// Checks of the host thread pool in lace_gb300/csrc/hostpar.h: regions on the
// pool, regions asked for while another runs (two threads at once, and one
// nested inside a region), and a region in a forked child, each writing every
// slot of its range exactly once.  Prints "ok" and exits 0 when all hold.
#include <sys/wait.h>

#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

#include "hostpar.h"

static bool covered(const std::vector<int> &v, int want) {
  for (int x : v)
    if (x != want) return false;
  return true;
}

static bool one_pass(size_t count) {
  std::vector<int> hits(count, 0);
  lace::par_for(count, 1024, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) ++hits[i];
  });
  return covered(hits, 1);
}

int main() {
  // plain regions, of several sizes, many times (the parked threads reused)
  for (int rep = 0; rep < 200; ++rep)
    if (!one_pass(1 + (size_t)rep * 977)) return printf("plain region %d\n", rep), 1;
  // two threads at once: one gets the pool, the other its own threads
  std::atomic<int> bad{0};
  std::vector<std::thread> th;
  for (int t = 0; t < 4; ++t)
    th.emplace_back([&] {
      for (int rep = 0; rep < 100; ++rep)
        if (!one_pass(50000 + rep)) ++bad;
    });
  for (auto &x : th) x.join();
  if (bad) return printf("concurrent regions\n"), 1;
  // a region inside a region
  std::vector<int> outer(64, 0);
  lace::par_for(64, 4, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) outer[i] = one_pass(4096 + i) ? 1 : -1;
  });
  if (!covered(outer, 1)) return printf("nested regions\n"), 1;
  // a forked child: the parent's parked threads do not exist there
  const pid_t pid = fork();
  if (pid == 0) _exit(one_pass(100000) && one_pass(3) ? 0 : 3);
  int st = 0;
  if (pid < 0 || waitpid(pid, &st, 0) != pid || !WIFEXITED(st) || WEXITSTATUS(st) != 0)
    return printf("forked child\n"), 1;
  // byte ranges
  std::vector<char> a(10'000'003, 1), b(a.size(), 0);
  lace::par_copy(b.data(), a.data(), a.size());
  for (char c : b)
    if (c != 1) return printf("par_copy\n"), 1;
  printf("ok\n");
  return 0;
}
