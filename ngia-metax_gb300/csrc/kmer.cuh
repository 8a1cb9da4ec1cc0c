// kmer.cuh — the per-candidate filter tests shared by the filter (filter.cu)
// and the serving kernels (serve.cu): residue codes, the composition sum and
// the short-word (k-mer) count against a representative's k-mer bitset.
#pragma once
#include <stdint.h>

#include "common.cuh"

namespace ngia {

// Residue code of net position q of a record's planes.
template <int P>
__device__ __forceinline__ uint32_t code_at(const uint32_t *planes, int q) {
  const uint32_t *b = planes + (q >> 5) * P;
  uint32_t c = 0;
#pragma unroll
  for (int p = 0; p < P; p++) c |= ((b[p] >> (q & 31)) & 1u) << p;
  return c;
}

// ---- short-word count of one candidate (kernel_wordFilter job body) ----------
template <int P>
__device__ int word_count(const uint32_t *__restrict__ planes, int net2, int w, const uint32_t *list) {
  constexpr int bits = P == 2 ? 2 : 5;
  const uint32_t mask = (1u << (w * bits)) - 1u;
  uint32_t word = 0;
  int sum = 0;
  for (int i = 0; i < net2; i += 32) {
    uint32_t pl[P];
#pragma unroll
    for (int p = 0; p < P; p++) pl[p] = __ldg(planes + (i >> 5) * P + p);
    const int lim = min(32, net2 - i);
    for (int j = 0; j < lim; j++) {
      uint32_t c = 0;
#pragma unroll
      for (int p = 0; p < P; p++) c |= ((pl[p] >> j) & 1u) << p;
      word = ((word << bits) | c) & mask;
      if (i + j >= w - 1) sum += (list[word >> 5] >> (word & 31)) & 1u;
    }
  }
  return sum;
}

// Composition sum of candidate c against the representative counts rc[].
template <int A>
__device__ __forceinline__ int base_sum(const uint32_t *__restrict__ cnt, int c, const uint32_t *rc) {
  int sum = 0;
  if (A == 4) {
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(cnt) + c);
    sum = (int)(min(q.x, rc[0]) + min(q.y, rc[1]) + min(q.z, rc[2]) + min(q.w, rc[3]));
  } else {
    const uint4 *q4 = reinterpret_cast<const uint4 *>(cnt + (int64_t)c * 28);
#pragma unroll
    for (int k = 0; k < 7; k++) {
      const uint4 q = __ldg(q4 + k);
      sum += (int)(min(q.x, rc[4 * k]) + min(q.y, rc[4 * k + 1]) + min(q.z, rc[4 * k + 2]) + min(q.w, rc[4 * k + 3]));
    }
  }
  return sum;
}

}  // namespace ngia
