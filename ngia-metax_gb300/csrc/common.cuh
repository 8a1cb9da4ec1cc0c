// common.cuh — device-side definitions shared by the loader, filter,
// alignment and driver kernels: the device database view, the run state,
// the work-queue classes, and the PTX wrappers for bulk (TMA) copies and
// bounded mbarrier waits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ngia {

constexpr unsigned kFullMask = 0xFFFFFFFFu;
constexpr int kMaxLenDev = 65536;              // makeDB keeps records <= 65,536
constexpr int kMaxBlocks = kMaxLenDev / 32;    // 2048 plane blocks
constexpr int kListWords = 2048;               // rep k-mer presence bitset (65,536 bits)
constexpr int kRefGridThreads = 128 * 128;     // BLOCK*WARP of the reference launch

// Alignment work classes.  Pairs are queued by the width A of their active
// band window (rep blocks touched by one query block, min(2B+1, nb1)).  The
// register-window classes hold the whole window in registers (capacity WC);
// the tiled classes keep up to 64 or 128 window rows per pair in a
// shared-memory ring and stream them through 16-slot register tiles; the last
// class of each type (any width) runs the tiled kernel on a global-memory
// ring.
constexpr int kNumClasses = 7;
constexpr int kRingBlocks = 128;  // largest ring (the tiled classes use 64 and 128)
__host__ __device__ inline int class_cap(int type, int c) {
  // DNA: 8,16,24,32 | tiled 64, 128 | any;  protein: 8,16 | tiled 64, 128 | any
  if (type == 0) {
    const int caps[7] = {8, 16, 24, 32, 64, 128, 0};
    return caps[c];
  }
  const int caps[7] = {8, 16, 64, 128, 0, 0, 0};
  return caps[c];
}
__host__ __device__ inline int num_classes(int type) { return type == 0 ? 7 : 5; }
__host__ __device__ inline int generic_class(int type) { return num_classes(type) - 1; }
__host__ __device__ inline bool is_tiled_class(int type, int c) {
  return c == generic_class(type) - 1 || c == generic_class(type) - 2;
}
// DNA register-window classes in use (caps 8, 16, 24, 32 blocks, in that
// order); windows above the last one in use go to the 64-block tiled class.
// Two: windows of 17-64 blocks share the tiled class's persistent launch,
// where their pairs fill the launch's tail instead of running as separate
// latency-bound launches beside it.  Measured on GB300 (1M DNA s=0.85,
// graph driver): 4, 3, 2 and 0 classes gave 136.1M, 137.6M, 138.0M and
// 138.0M candidate seqs/s.
#ifndef NGIA_DNA_WIN_CLASSES
#define NGIA_DNA_WIN_CLASSES 2
#endif
__host__ __device__ inline int class_of(int type, int A) {
  const int g = generic_class(type);
  for (int c = 0; c < g; c++) {
    if (type == 0 && c < 4 && c >= NGIA_DNA_WIN_CLASSES) continue;
    if (A <= class_cap(type, c)) return c;
  }
  return g;
}

// Device copy of the makeDB database plus per-sequence header arrays.
struct DevDB {
  const uint32_t *words;  // records, contiguous (makeDB layout)
  const int64_t *off;     // word offset of record i
  const int32_t *len;     // raw length (record word 0)
  const int32_t *net;     // net length (record word 1)
  const uint32_t *cnt;    // residue counts, 4 (DNA) or 28 (protein) per sequence
  const uint32_t *codes;  // protein: each record's residue codes as a bit stream
                          // (5 words per 32-residue block, at the planes'
                          // offsets); null for DNA
  int32_t n, type;
  int32_t hw, P, A;       // header words, planes, count words
  int32_t max_nb;         // max plane blocks over all records
  int32_t has_short;      // some record has net length < 16
};

// Device-resident run state of the greedy driver.
struct RunState {
  int32_t rep;            // current representative (sorted index)
  int32_t done;           // no unclustered sequence left
  int32_t err;            // device error code (0 = ok)
  int32_t err_where;      // kernel id that set err
  int64_t iter;           // representatives taken so far
  int64_t iter_limit;     // graph loop stops when iter reaches it
  uint32_t qcount[kNumClasses];  // pairs queued per class this iteration
  uint32_t qhead[kNumClasses];   // pairs claimed per class
  uint32_t long_count;    // candidates left for k_filter_long this iteration
  int32_t word_first;     // 1: short-word filter before alignment
  int32_t word_active;    // 1: short-word filter applies this iteration
  int32_t rep_nb;         // plane blocks of the representative (net)
  int32_t rep_len, rep_net;
  // statistics (device-accumulated)
  unsigned long long st_candidates, st_base_pass, st_align_pairs, st_members;
  unsigned long long st_band_cells, st_filter_bytes, st_word_checks, st_word_pass;
  unsigned long long st_done_cells;  // in-band cells actually computed
  unsigned long long st_class_pairs[kNumClasses];
  unsigned long long st_class_done[kNumClasses];    // in-band cells computed per class
  unsigned long long st_class_qwords[kNumClasses];  // query plane words of the pairs per class
};

// Polls of an mbarrier wait before a kernel gives up (each poll blocks for a
// hardware-defined interval; a staging copy lands within a few polls).
constexpr uint32_t kWaitPolls = 1u << 20;

// Run parameters (constant during one clustering).
struct RunParams {
  float s;
  int32_t w;
  int32_t precise;
  int32_t word_order;     // 0 auto, 1 word first, 2 alignment first
  int32_t refill;         // tiled alignment: idle lanes a warp waits for before it claims new pairs
  uint32_t wait_polls = kWaitPolls;  // poll limit of the alignment kernels' staging wait
};

// Order of the two cheap-to-expensive tests.  Both orders give the same
// members (a candidate joins iff all three tests pass); the short-word filter
// goes first when it is expected to reject most candidates.
__host__ __device__ inline int word_first_of(int type, const RunParams &prm) {
  if (prm.word_order == 1) return 1;
  if (prm.word_order == 2) return 0;
  return type == 0 ? (prm.s >= 0.93f) : 1;
}

// Device buffers of one clustering run.
struct RunBufs {
  RunState *st;
  int32_t *cluster;       // cluster[i] = representative of i, -1 = none yet
  int32_t *ident;         // banded-LCS score against the representative
  uint32_t *alive;        // bit i = sequence i not yet clustered
  int32_t *queue[kNumClasses];
  uint32_t *rep_rec;      // 16-byte aligned copy of the representative record
  uint32_t *rep_list;     // representative k-mer presence bitset
  // exact short-word path (databases with net length < 16 records)
  uint8_t *flags;         // per-sequence stage flags
  int32_t *pos;           // position of a base survivor in the job list
  int32_t *first_short;   // per reference thread: first job with net < 16
  uint32_t *scan_part;    // scan partials
  int32_t *long_list;     // candidates whose short-word count k_filter_long takes (one warp each)
  uint32_t *scratch;      // per-lane band rows of the widest class (global ring)
  int64_t scratch_words;
  int32_t generic_lanes;
  uint32_t ring_mask;     // global ring size - 1 (power of two >= the widest record)
  // filter counters, 32 stripes x kFilterStats (one 64-byte line each),
  // added per CTA and folded into the run state by k_next
  unsigned long long *fstats;
  // pair-score mode
  const int32_t *score_cands;
  int32_t *score_out;
};

constexpr int kFilterStats = 8;     // counters per stripe (5 used)
constexpr int kFilterStripes = 32;

#define NGIA_ERR_MBAR_TIMEOUT 1
#define NGIA_ERR_SCRATCH 2
#define NGIA_ERR_RANGE 3

__device__ __forceinline__ void set_error(RunState *st, int code, int where) {
  if (atomicCAS(&st->err, 0, code) == 0) st->err_where = where;
}

// ---- PTX wrappers ---------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// 1-D bulk copy global -> shared (the TMA unit, non-tensor form).  Both
// addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` polls (each poll itself blocks for a
// hardware-defined interval) and returns false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t limit) {
  for (uint32_t i = 0; i < limit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Stages `words` uint32 from global `src` (16-byte aligned) into shared `dst`
// with one bulk copy issued by thread 0; every thread waits on the barrier.
// Returns false (after recording an error) if the copy did not land.
__device__ __forceinline__ bool stage_to_smem(uint32_t *dst, const uint32_t *src, uint32_t words,
                                              uint64_t *bar, RunState *st, int where) {
  const uint32_t bytes = (words * 4u + 15u) & ~15u;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    if (bytes) {
      mbar_expect_tx(bar, bytes);
      bulk_g2s(dst, src, bytes, bar);
    } else {
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
    }
  }
  __syncthreads();
  bool ok = mbar_wait_bounded(bar, 0, 1u << 20);
  if (!ok) {
    set_error(st, NGIA_ERR_MBAR_TIMEOUT, where);
    mbar_wait_bounded(bar, 0, 1u << 20);  // let the copy in flight land
  }
  return __syncthreads_and(ok);
}

// Block-band parameters of one (rep, query) pair, func.cu:469-470: the shift
// is ceil of one fused multiply-add (nvcc contracts (float)L1-(float)L2*s).
__device__ __forceinline__ int band_blocks(int L1, int L2, float s) {
  int shift = (int)ceilf(__fmaf_rn(-(float)L2, s, (float)L1));
  return (shift + 31) / 32;
}
// ceil((float)L2*s), func.cu:334, 515.
__device__ __forceinline__ int cutoff_of(int L2, float s) { return (int)ceilf(__fmul_rn((float)L2, s)); }
// Short-word threshold, func.cu:393-395.
__device__ __forceinline__ int word_min(int L2, int w, float s) {
  int length = (int)ceilf(__fmul_rn((float)L2, __fsub_rn(1.0f, s)));
  return (L2 - w + 1) - length * w;
}

// Window width (rep blocks per query block) of a pair.
__host__ __device__ __forceinline__ int window_of(int B, int nb1) {
  if (B < 0 || nb1 <= 0) return 0;
  int a = 2 * B + 1;
  return a < nb1 ? a : nb1;
}

// Reference band cells of one pair: sum over query blocks of
// (jend - jstart + 1) * 32 * cols (func.cu:473-484).
__device__ __forceinline__ long long band_cells(int B, int nb1, int net2) {
  const int nq = (net2 + 31) / 32;
  long long c = 0;
  for (int i = 0; i < nq; i++) {
    int js = max(i - B, 0), je = min(i + B, nb1 - 1);
    if (je >= js) {
      int cols = ((i + 1) * 32 > net2) ? (net2 & 31) : 32;
      c += (long long)(je - js + 1) * 32 * cols;
    }
  }
  return c;
}

}  // namespace ngia
