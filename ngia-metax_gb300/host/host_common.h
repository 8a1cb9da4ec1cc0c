// host_common.h — shared helpers of the host half of libngia (error state,
// makeDB record geometry).  Internal header: not part of the C ABI.
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/ngia.h"

namespace ngia {

// Records the calling thread's last error; returns `code` so call sites can
// write `return fail(NGIA_E_IO, "...")`.
int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

// Residue-count words and bit planes per record (makeDB/src/makeDB.cpp:110,155).
inline int count_words(int type) { return type == 0 ? 4 : 28; }
inline int header_words(int type) { return 2 + count_words(type); }
inline int plane_count(int type) { return type == 0 ? 2 : 5; }
// Words of one record with raw length `len` (makeDB.cpp:282-286, func.cu:120-122).
inline int64_t record_words(int type, int64_t len) {
  return header_words(type) + (len + 31) / 32 * plane_count(type);
}

// Maximum raw length makeDB keeps (makeDB.cpp:92).
constexpr int kMaxLen = 65536;

// Runs body(i) for i in [0, n) on all hardware threads, handing out chunks of
// `grain` indices from an atomic counter.  body(i, thread) when it takes two
// arguments (per-thread scratch).
template <class F>
void parallel_for(int64_t n, int64_t grain, F body) {
  if (n <= 0) return;
  const int64_t nchunks = (n + grain - 1) / grain;
  int nt = (int)std::min<int64_t>(std::max(1u, std::thread::hardware_concurrency()), nchunks);
  std::atomic<int64_t> next{0};
  auto work = [&](int t) {
    for (;;) {
      const int64_t c = next.fetch_add(1);
      if (c >= nchunks) break;
      const int64_t e = std::min(n, (c + 1) * grain);
      for (int64_t i = c * grain; i < e; i++) {
        if constexpr (std::is_invocable_v<F, int64_t, int>)
          body(i, t);
        else
          body(i);
      }
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; t++) th.emplace_back(work, t);
  work(0);
  for (auto &x : th) x.join();
}
inline int hardware_threads() { return (int)std::max(1u, std::thread::hardware_concurrency()); }

}  // namespace ngia
