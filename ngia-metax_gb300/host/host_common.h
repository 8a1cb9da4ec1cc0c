// host_common.h — shared helpers of the host half of libngia (error state,
// makeDB record geometry).  Internal header: not part of the C ABI.
#pragma once
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>

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

}  // namespace ngia
