// errors.cpp — thread-local error state behind ngia_last_error, plus the
// parameter clamps of the reference loader.
#include <algorithm>
#include <cstring>

#include "host_common.h"

namespace ngia {

static thread_local int t_code = 0;
static thread_local char t_msg[512] = {0};

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
  va_end(ap);
  t_code = code;
  return code;
}

void clear_error() {
  t_code = 0;
  t_msg[0] = 0;
}

}  // namespace ngia

extern "C" int ngia_last_error(char *buf, size_t len) {
  if (buf && len) {
    std::strncpy(buf, ngia::t_msg, len - 1);
    buf[len - 1] = 0;
  }
  return ngia::t_code;
}

extern "C" const char *ngia_version(void) { return "ngia-gb300 1.0"; }

extern "C" void ngia_free(void *p) { std::free(p); }

// Parameter clamps of readIndex, CUDA/signalNode/src/func.cu:57-75: the
// similarity is clamped to [0.1, 1.0], precise to {0,1}; DNA word length to
// [4,8] and lowered step-wise for low similarity (precise forced below 0.75);
// protein word length to [2,3] (2 below 0.7; precise forced below 0.5).
// All comparisons are single-precision, as in the reference.
extern "C" int ngia_params_clamp(int32_t type, ngia_params *p) {
  if (!p) return ngia::fail(NGIA_E_ARG, "ngia_params_clamp: null params");
  if (type != 0 && type != 1)
    return ngia::fail(NGIA_E_ARG, "ngia_params_clamp: type %d not 0/1", type);
  float s = p->similarity;
  s = s < 0.1f ? 0.1f : s;   // max(0.1f, s)
  s = s > 1.0f ? 1.0f : s;   // min(1.0f, s)
  int precise = std::min(1, std::max(0, (int)p->precise));
  int w = p->word_length;
  if (type == 0) {
    if (s < 0.75f) precise = 1;
    w = std::max(4, w);
    w = std::min(8, w);
    if (s < 0.88f) w = std::min(7, w);
    if (s < 0.86f) w = std::min(6, w);
    if (s < 0.84f) w = std::min(5, w);
    if (s < 0.81f) w = std::min(4, w);
  } else {
    if (s < 0.5f) precise = 1;
    w = std::max(2, w);
    w = std::min(3, w);
    if (s < 0.7f) w = std::min(2, w);
  }
  p->similarity = s;
  p->precise = precise;
  p->word_length = w;
  return NGIA_OK;
}
