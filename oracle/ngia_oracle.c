/*
 * ngia_oracle.c — line-faithful CPU restatement of nGIA's single-node
 * clustering, CUDA/signalNode/src/func.cu (same algorithm in
 * OneAPI/SignalNode/src/func.cpp).  TEST INFRASTRUCTURE: it gives the
 * results the parity tests compare against and the timed CPU baseline; the
 * product library never links, loads or calls it.
 *
 * Parity pins: the database format is pinned against the reference makeDB
 * tool built from its own source (oracle/build_oracle.py); the clustering is
 * pinned by the reference's own CUDA program, built from its sources and run
 * on a GB300 (oracle/ref_cluster.py), whose outputs for 4 fixtures x 15
 * parameter sets are committed under tests/golden/ref/ and reproduced byte
 * for byte (tests/test_host_cpu.py::test_oracle_matches_reference_golden),
 * and by known-answer cases in tests/test_host_cpu.py (exact LCS when the
 * band covers the matrix, the fused-multiply-add band case).
 *
 * Compiled with -ffp-contract=off: the only fused multiply-add is the
 * explicit fmaf() of the band shift, which nvcc contracts in the reference
 * kernels (func.cu:469, 540); every other threshold is a plain product.
 *
 * The reference launches every kernel as <<<128,128>>> with a grid-stride
 * loop (func.h:8-9); the short-word kernel returns a whole thread when it
 * meets a query with net length < 16 (func.cu:375, 420), which leaves every
 * later job of that thread passing.  ora_cluster reproduces that with the
 * 16,384-thread job-to-thread map.
 */
#define _GNU_SOURCE
#include "ngia_oracle.h"

#include <limits.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define REF_GRID_THREADS (128 * 128) /* BLOCK * WARP, func.h:8-9 */

static inline unsigned umin_(unsigned a, unsigned b) { return a < b ? a : b; }
static inline int imax_(int a, int b) { return a > b ? a : b; }
static inline int imin_(int a, int b) { return a < b ? a : b; }
static inline int hdr_words(int type) { return type ? 30 : 6; }
static inline int planes(int type) { return type ? 5 : 2; }

/* readIndex parameter clamps, func.cu:57-75. */
void ora_clamp(int type, float *s, int *w, int *precise) {
  float sim = *s;
  if (!(sim >= 0.1f)) sim = 0.1f;
  if (sim > 1.0f) sim = 1.0f;
  int p = *precise;
  if (p < 0) p = 0;
  if (p > 1) p = 1;
  int wl = *w;
  if (type == 0) {
    if (sim < 0.75f) p = 1;
    wl = imax_(4, wl);
    wl = imin_(8, wl);
    if (sim < 0.88f) wl = imin_(7, wl);
    if (sim < 0.86f) wl = imin_(6, wl);
    if (sim < 0.84f) wl = imin_(5, wl);
    if (sim < 0.81f) wl = imin_(4, wl);
  } else {
    if (sim < 0.5f) p = 1;
    wl = imax_(2, wl);
    wl = imin_(3, wl);
    if (sim < 0.7f) wl = imin_(2, wl);
  }
  *s = sim;
  *w = wl;
  *precise = p;
}

/* kernel_baseFilterGen/Pro job body, func.cu:328-335, 345-352. */
static int base_sum(const uint32_t *q, const uint32_t *r, int type) {
  int sum = 0;
  for (int i = 0; i < (type ? 28 : 4); i++) sum += (int)umin_(q[2 + i], r[2 + i]);
  return sum;
}
static int base_pass(const uint32_t *q, const uint32_t *r, int type, float s) {
  int length2 = (int)q[0];
  int length = (int)ceilf((float)length2 * s);
  return !(base_sum(q, r, type) < length);
}

/* generateListGen/Pro, func.cu:241-302: presence bits of every w-mer of the
 * representative's net sequence, first residue in the high bits. */
static void gen_list(const uint32_t *rep, int type, int w, uint32_t *list) {
  memset(list, 0, sizeof(uint32_t) * 2048);
  const int net = (int)rep[1], P = planes(type), bits = type ? 5 : 2;
  const uint32_t *packed = rep + hdr_words(type);
  const unsigned mask = (1u << (w * bits)) - 1;
  if (net < 16) return;
  unsigned word = 0;
  for (int i = 0; i < w - 1; i++) {
    word <<= bits;
    for (int p = 0; p < P; p++) word += ((packed[p] >> i) & 1u) << p;
  }
  for (int i = w - 1, k = w - 1; i < net; i++, k++) {
    word <<= bits;
    for (int p = 0; p < P; p++) word += ((packed[p] >> k) & 1u) << p;
    word &= mask;
    list[word / 32] |= 1u << (word % 32);
    if (k == 31) {
      k = -1;
      packed += P;
    }
  }
}

/* kernel_wordFilterGen/Pro job body, func.cu:376-391, 421-439: number of
 * net positions p >= w-1 whose w-mer is in the representative's set. */
static int word_sum(const uint32_t *q, int type, int w, const uint32_t *list) {
  const int net2 = (int)q[1], P = planes(type), bits = type ? 5 : 2;
  const uint32_t *packed2 = q + hdr_words(type);
  const unsigned mask = (1u << (w * bits)) - 1;
  int sum = 0;
  unsigned word = 0;
  for (int i = 0; i < net2; i += 32, packed2 += P) {
    for (int j = 0; j < 32; j++) {
      if (i + j == net2) break;
      word <<= bits;
      for (int p = 0; p < P; p++) word += ((packed2[p] >> j) & 1u) << p;
      word &= mask;
      if (i + j > w - 2) sum += (list[word / 32] & (1u << (word % 32))) > 0;
    }
  }
  return sum;
}
/* func.cu:393-396 */
static int word_pass_thr(int sum, int length2, int w, float s) {
  int len = length2 - w + 1;
  int length = (int)ceilf((float)length2 * (1.0f - s));
  int minLen = len - length * w;
  return !(sum < minLen);
}

/* kernel_dynamicGen/Pro job body, func.cu:453-515 / 524-601. */
int ora_dp_sum(const uint32_t *rep, const uint32_t *query, int type, float s, int *band,
               int64_t *cells) {
  const int P = planes(type), hw = hdr_words(type);
  const int length1 = (int)rep[0], netLength1 = (int)rep[1];
  const int netLen321 = (netLength1 + 31) / 32;
  const uint32_t *packed1 = rep + hw;
  const int length2 = (int)query[0], netLength2 = (int)query[1];
  const int netLen322 = (netLength2 + 31) / 32;
  const uint32_t *packed2 = query + hw;
  uint32_t line[2048];
  memset(line, 0xFF, sizeof(uint32_t) * (size_t)(netLen321 > 0 ? netLen321 : 1));
  /* nvcc contracts (float)L1 - (float)L2 * s into one fused multiply-add;
   * ORA_BAND_NOFMA builds the separately rounded variant, used only to find
   * inputs on which the two differ (tests/golden/make_golden.py). */
#ifdef ORA_BAND_NOFMA
  volatile float prod = (float)length2 * s;
  int shift = (int)ceilf((float)length1 - prod);
#else
  int shift = (int)ceilf(fmaf(-(float)length2, s, (float)length1));
#endif
  shift = (shift + 31) / 32;
  if (band) *band = shift;
  int64_t ncell = 0;
  int cols = 32;
  for (int i = 0; i < netLen322; i++) {
    if ((i + 1) * 32 > netLength2) cols = netLength2 % 32;
    uint32_t column[32] = {0};
    uint32_t Col[5];
    for (int p = 0; p < P; p++) Col[p] = packed2[i * P + p];
    int jstart = imax_(i - shift, 0);
    int jend = imin_(i + shift, netLen321 - 1);
    for (int j = jstart; j <= jend; j++) {
      uint32_t Row[5];
      for (int p = 0; p < P; p++) Row[p] = packed1[j * P + p];
      uint32_t row = line[j];
      for (int k = 0; k < cols; k++) {
        uint32_t match = 0xFFFFFFFFu;
        for (int p = 0; p < P; p++) {
          uint32_t colp = ((Col[p] >> k) & 1u) ? 0xFFFFFFFFu : 0u;
          match &= ~(Row[p] ^ colp);
        }
        uint32_t unmatch = ~match;
        uint32_t temp3 = row & match;
        uint32_t temp4 = row & unmatch;
        uint32_t carry = column[k];
        uint32_t temp5 = row + carry;
        uint32_t carry1 = temp5 < row;
        temp5 += temp3;
        uint32_t carry2 = temp5 < temp3;
        carry = carry1 | carry2;
        row = temp5 | temp4;
        column[k] = carry;
      }
      line[j] = row;
    }
    if (jend >= jstart) ncell += (int64_t)(jend - jstart + 1) * 32 * cols;
  }
  int sum = 0, rows = 32;
  for (int i = 0; i < netLen321; i++) {
    if ((i + 1) * 32 > netLength1) rows = netLength1 % 32;
    uint32_t row = line[i];
    for (int j = 0; j < rows; j++) sum += ((row >> j) & 1u) ^ 1u;
  }
  if (cells) *cells = ncell;
  return sum;
}

static int dp_pass(int sum, int length2, float s) {
  int cutoff = (int)ceilf((float)length2 * s);
  return !(sum < cutoff);
}

void ora_pair(const uint32_t *buf, const int64_t *offsets, int type, float s, int w, int rep,
              int cand, int32_t *out) {
  const uint32_t *r = buf + offsets[rep], *q = buf + offsets[cand];
  uint32_t list[2048];
  gen_list(r, type, w, list);
  out[0] = base_sum(q, r, type);
  out[4] = base_pass(q, r, type, s);
  if ((int)r[1] < 16 || (int)q[1] < 16) {
    out[1] = -1;
    out[5] = 1;
  } else {
    out[1] = word_sum(q, type, w, list);
    out[5] = word_pass_thr(out[1], (int)q[0], w, s);
  }
  int band = 0;
  int64_t cells = 0;
  out[2] = ora_dp_sum(r, q, type, s, &band, &cells);
  out[3] = band;
  out[6] = dp_pass(out[2], (int)q[0], s);
  out[7] = (int32_t)cells;
}

/* clustering(), func.cu:607-677 with updateRepresent (186-238) and
 * updateJobs (305-320): jobs are (index, result) pairs, result 0 = still
 * passing, -1 = rejected; each stage runs over the compacted survivors of
 * the previous one, in ascending sequence order. */
int64_t ora_cluster(const uint32_t *buf, const int64_t *offsets, int n, int type, float s,
                    int w, int precise, int nthreads, int64_t max_iters, int32_t *cluster,
                    int32_t *identity, int64_t *stats) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  const int A = type ? 28 : 4, P = planes(type);
  int *remains = (int *)malloc(sizeof(int) * (size_t)n);
  int *jobs = (int *)malloc(sizeof(int) * 2 * (size_t)n);
  int *sums = (int *)malloc(sizeof(int) * (size_t)n);
  int *first_short = (int *)malloc(sizeof(int) * REF_GRID_THREADS);
  uint32_t *list = (uint32_t *)malloc(sizeof(uint32_t) * 2048);
  int64_t st[ORA_NSTATS];
  memset(st, 0, sizeof(st));
  for (int i = 0; i < n; i++) {
    remains[i] = i;
    jobs[2 * i] = i;
    jobs[2 * i + 1] = -1;
    cluster[i] = -1;
    if (identity) identity[i] = -1;
    sums[i] = -1;
  }
  int remainCount = n, jobCount = n, top = -1;
  int64_t iters = 0;
  while (1) {
    /* updateRepresent: members of the previous representative */
    for (int i = 0; i < jobCount; i++)
      if (jobs[2 * i + 1] == 0) {
        cluster[jobs[2 * i]] = top;
        if (identity) identity[jobs[2 * i]] = sums[i];
      }
    int count = 0;
    for (int i = 0; i < remainCount; i++) {
      int idx = remains[i];
      if (cluster[idx] == -1) {
        remains[count] = idx;
        jobs[2 * count] = idx;
        jobs[2 * count + 1] = 0;
        count++;
      }
    }
    remainCount = jobCount = count;
    if (remainCount == 0) break;
    if (max_iters > 0 && iters >= max_iters) break;
    top = remains[0];
    cluster[top] = top;
    iters++;
    const uint32_t *rep = buf + offsets[top];
    gen_list(rep, type, w, list);
    st[ORA_CAND] += jobCount;
    st[ORA_FILTER_BYTES] += (int64_t)jobCount * 4 * (2 + A);
    /* base filter over all remaining sequences (func.cu:630-644) */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < jobCount; i++)
      if (!base_pass(buf + offsets[jobs[2 * i]], rep, type, s)) jobs[2 * i + 1] = -1;
    count = 0;
    for (int i = 0; i < jobCount; i++)
      if (jobs[2 * i + 1] == 0) {
        jobs[2 * count] = jobs[2 * i];
        jobs[2 * count + 1] = 0;
        count++;
      }
    jobCount = count;
    st[ORA_BASE_PASS] += jobCount;
    if (!precise) { /* short-word filter (func.cu:645-659) */
      if ((int)rep[1] >= 16) {
        /* thread t of the 16,384 handles jobs t, t+16384, ... and returns
         * at its first job whose net length is < 16 */
        for (int t = 0; t < REF_GRID_THREADS; t++) first_short[t] = INT_MAX;
        for (int i = 0; i < jobCount; i++) {
          int t = i % REF_GRID_THREADS;
          if (first_short[t] == INT_MAX && (int)buf[offsets[jobs[2 * i]] + 1] < 16) first_short[t] = i;
        }
        int64_t evals = 0, pbytes = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : evals, pbytes)
        for (int i = 0; i < jobCount; i++) {
          if (i >= first_short[i % REF_GRID_THREADS]) continue;
          const uint32_t *q = buf + offsets[jobs[2 * i]];
          int sum = word_sum(q, type, w, list);
          evals++;
          pbytes += (int64_t)4 * P * (((int)q[1] + 31) / 32);
          if (!word_pass_thr(sum, (int)q[0], w, s)) jobs[2 * i + 1] = -1;
        }
        st[ORA_WORD_EVAL] += evals;
        st[ORA_FILTER_BYTES] += pbytes;
      }
      count = 0;
      for (int i = 0; i < jobCount; i++)
        if (jobs[2 * i + 1] == 0) {
          jobs[2 * count] = jobs[2 * i];
          jobs[2 * count + 1] = 0;
          count++;
        }
      jobCount = count;
    }
    st[ORA_WORD_PASS] += jobCount;
    /* banded bit-parallel alignment (func.cu:660-674) */
    int64_t cells = 0, members = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : cells, members)
    for (int i = 0; i < jobCount; i++) {
      const uint32_t *q = buf + offsets[jobs[2 * i]];
      int64_t c = 0;
      int sum = ora_dp_sum(rep, q, type, s, NULL, &c);
      cells += c;
      sums[i] = sum;
      if (!dp_pass(sum, (int)q[0], s))
        jobs[2 * i + 1] = -1;
      else
        members++;
    }
    st[ORA_CELLS] += cells;
    st[ORA_MEMBERS] += members;
  }
  st[ORA_ITER] = iters;
  if (stats) memcpy(stats, st, sizeof(st));
  free(remains);
  free(jobs);
  free(sums);
  free(first_short);
  free(list);
  return iters;
}

/* readIndex + readData, func.cu:42-154 (single process: rank 0 of 1). */
int64_t ora_assign(const uint32_t *rbuf, const int64_t *roff, int nrep, const uint32_t *qbuf,
                   const int64_t *qoff, int nq, int type, float s, int w, int precise, int nthreads,
                   int32_t *rep_out, int32_t *ident_out) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  uint32_t *lists = (uint32_t *)malloc(sizeof(uint32_t) * 2048 * (size_t)(nrep > 0 ? nrep : 1));
#pragma omp parallel for schedule(dynamic, 16)
  for (int r = 0; r < nrep; r++) gen_list(rbuf + roff[r], type, w, lists + (size_t)2048 * r);
#pragma omp parallel for schedule(dynamic, 4)
  for (int q = 0; q < nq; q++) {
    const uint32_t *qr = qbuf + qoff[q];
    rep_out[q] = INT32_MIN;
    ident_out[q] = -1;
    for (int r = 0; r < nrep; r++) {
      const uint32_t *rr = rbuf + roff[r];
      if (!base_pass(qr, rr, type, s)) continue;
      if (!precise && (int)rr[1] >= 16 && (int)qr[1] >= 16 &&
          !word_pass_thr(word_sum(qr, type, w, lists + (size_t)2048 * r), (int)qr[0], w, s))
        continue;
      int band = 0;
      int64_t cells = 0;
      const int sum = ora_dp_sum(rr, qr, type, s, &band, &cells);
      if (!dp_pass(sum, (int)qr[0], s)) continue;
      rep_out[q] = r;
      ident_out[q] = sum;
      break;
    }
  }
  free(lists);
  int nleft = 0;
  int64_t *loff = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nq > 0 ? nq : 1));
  int *lidx = (int *)malloc(sizeof(int) * (size_t)(nq > 0 ? nq : 1));
  for (int q = 0; q < nq; q++)
    if (rep_out[q] == INT32_MIN) {
      loff[nleft] = qoff[q];
      lidx[nleft++] = q;
    }
  int64_t clusters = 0;
  if (nleft) {
    int32_t *lc = (int32_t *)malloc(sizeof(int32_t) * (size_t)nleft);
    int32_t *li = (int32_t *)malloc(sizeof(int32_t) * (size_t)nleft);
    ora_cluster(qbuf, loff, nleft, type, s, w, precise, nthreads, 0, lc, li, NULL);
    for (int k = 0; k < nleft; k++) {
      rep_out[lidx[k]] = -1 - lidx[lc[k]];
      ident_out[lidx[k]] = li[k];
      if (lc[k] == k) clusters++;
    }
    free(lc);
    free(li);
  }
  free(loff);
  free(lidx);
  return clusters;
}

/* ---- makeDB packing (makeDB/src/makeDB.cpp) ---------------------------------
 * Residue code of one character, -1 for a character the record skips
 * (counted in the raw length, not in the net length): DNA a c g t/u -> 0..3
 * (makeDataGen, makeDB.cpp:108-151); protein a..z -> 0..25, '*' -> 26,
 * '-' -> 27 for lower case and A..Z -> 0..25 for upper case (makeDataPro,
 * makeDB.cpp:153-252: '*' and '-' appear only in its lower-case branch, and
 * the upper-case branch has no code for them, so both cases map the same). */
static int res_code(int type, unsigned char c) {
  if (type == 0) {
    switch (c) {
      case 'a': case 'A': return 0;
      case 'c': case 'C': return 1;
      case 'g': case 'G': return 2;
      case 't': case 'T': case 'u': case 'U': return 3;
      default: return -1;
    }
  }
  if (c >= 'a' && c <= 'z') return c - 'a';
  if (c >= 'A' && c <= 'Z') return c - 'A';
  if (c == '*') return 26;
  if (c == '-') return 27;
  return -1;
}

/* One record: [len, net, counts, planes]; residue k of each 32-residue
 * block of the net sequence sits at bit k of the block's planes (makeDB
 * shifts each new residue in from the top and shifts a partial last block
 * down to bit 0). */
static void pack_record(int type, const unsigned char *r, int64_t len, uint32_t *out) {
  const int A = type ? 28 : 4, P = planes(type), hw = hdr_words(type);
  const int64_t nb = (len + 31) / 32;
  memset(out, 0, sizeof(uint32_t) * (size_t)(hw + nb * P));
  int64_t net = 0;
  for (int64_t i = 0; i < len; i++) {
    const int c = res_code(type, r[i]);
    if (c < 0) continue;
    out[2 + c] += 1;
    uint32_t *blk = out + hw + (net / 32) * P;
    for (int p = 0; p < P; p++) blk[p] |= (uint32_t)((c >> p) & 1) << (net % 32);
    net++;
  }
  (void)A;
  out[0] = (uint32_t)len;
  out[1] = (uint32_t)net;
}

int64_t ora_pack(int type, const char *seq, const int64_t *off, int64_t n, uint32_t *words,
                 int64_t *rec_off, int64_t *n_words) {
  /* stable counting sort by raw length, longest first */
  int64_t *cnt = (int64_t *)calloc(65537 + 1, sizeof(int64_t));
  int64_t kept = 0, total = 0;
  for (int64_t i = 0; i < n; i++) {
    const int64_t len = off[i + 1] - off[i];
    if (len > 65536) continue;
    cnt[65536 - len]++;
    kept++;
    total += hdr_words(type) + (len + 31) / 32 * planes(type);
  }
  if (n_words) *n_words = total;
  if (!words || !rec_off) {
    free(cnt);
    return kept;
  }
  int64_t *start = (int64_t *)calloc(65537 + 1, sizeof(int64_t));
  for (int k = 1; k <= 65537; k++) start[k] = start[k - 1] + cnt[k - 1];
  int64_t *order = (int64_t *)malloc(sizeof(int64_t) * (size_t)(kept ? kept : 1));
  for (int64_t i = 0; i < n; i++) {
    const int64_t len = off[i + 1] - off[i];
    if (len > 65536) continue;
    order[start[65536 - len]++] = i;
  }
  int64_t w = 0;
  for (int64_t k = 0; k < kept; k++) {
    rec_off[k] = w;
    w += hdr_words(type) + (off[order[k] + 1] - off[order[k]] + 31) / 32 * planes(type);
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t k = 0; k < kept; k++) {
    const int64_t i = order[k];
    pack_record(type, (const unsigned char *)seq + off[i], off[i + 1] - off[i], words + rec_off[k]);
  }
  free(order);
  free(start);
  free(cnt);
  return kept;
}

int ora_load(const char *dir, ora_db *db) {
  memset(db, 0, sizeof(*db));
  char path[4096];
  snprintf(path, sizeof(path), "%s/data.bin", dir);
  FILE *f = fopen(path, "rb");
  if (!f) return -1;
  int32_t h[4];
  if (fread(h, 4, 4, f) != 4 || h[0] <= 0 || (h[3] != 0 && h[3] != 1)) {
    fclose(f);
    return -2;
  }
  const int n = h[0];
  db->n = n;
  db->longest = h[1];
  db->shortest = h[2];
  db->type = h[3];
  db->name_len = (int32_t *)malloc(4 * (size_t)n);
  db->read_len = (int32_t *)malloc(4 * (size_t)n);
  db->fasta_off = (int64_t *)malloc(8 * (size_t)n);
  db->pack_off = (int64_t *)malloc(8 * (size_t)n);
  db->offsets = (int64_t *)malloc(8 * (size_t)n);
  if (fread(db->name_len, 4, (size_t)n, f) != (size_t)n || fread(db->read_len, 4, (size_t)n, f) != (size_t)n ||
      fread(db->fasta_off, 8, (size_t)n, f) != (size_t)n || fread(db->pack_off, 8, (size_t)n, f) != (size_t)n) {
    fclose(f);
    ora_free(db);
    return -3;
  }
  int64_t len = 0;
  for (int i = 0; i < n; i++) {
    db->offsets[i] = len;
    len += hdr_words(db->type) + (int64_t)(db->read_len[i] + 31) / 32 * planes(db->type);
  }
  db->buf_words = len;
  db->buf = (uint32_t *)calloc((size_t)len + 1, 4);
  for (int i = 0; i < n; i++) {
    int64_t words = hdr_words(db->type) + (int64_t)(db->read_len[i] + 31) / 32 * planes(db->type);
    if (fseek(f, (long)db->pack_off[i], SEEK_SET) != 0 ||
        fread(db->buf + db->offsets[i], 4, (size_t)words, f) != (size_t)words) {
      fclose(f);
      ora_free(db);
      return -4;
    }
  }
  fclose(f);
  return 0;
}

void ora_free(ora_db *db) {
  free(db->name_len);
  free(db->read_len);
  free(db->fasta_off);
  free(db->pack_off);
  free(db->offsets);
  free(db->buf);
  memset(db, 0, sizeof(*db));
}

/* getline + '\r' strip of saveResult (func.cu:734-741). */
static long read_line(FILE *f, char **line, size_t *cap) {
  ssize_t k = getline(line, cap, f);
  if (k < 0) return -1;
  if (k > 0 && (*line)[k - 1] == '\n') (*line)[--k] = 0;
  if (k > 0 && (*line)[k - 1] == '\r') (*line)[--k] = 0;
  return (long)k;
}

/* saveResult, func.cu:680-764: members grouped by representative, file
 * offsets precomputed from the index lengths, every record read from
 * data.fasta and written at its offset with a seek. */
int ora_save(const char *dbdir, const char *outdir, const ora_db *db, const int32_t *cluster,
             int32_t *n_clusters) {
  const int n = db->n;
  int *cnt = (int *)calloc((size_t)n, sizeof(int));
  int *first = (int *)malloc(sizeof(int) * (size_t)n);
  for (int i = 0; i < n; i++) first[i] = -1;
  for (int i = 0; i < n; i++) {
    if (cluster[i] < 0 || cluster[i] >= n) {
      free(cnt);
      free(first);
      return -1;
    }
    if (first[cluster[i]] < 0) first[cluster[i]] = i;
    cnt[cluster[i]]++;
  }
  int32_t count = 0;
  for (int i = 0; i < n; i++) count += cnt[i] > 0;
  /* offsets (func.cu:708-724): iterate clusters in rep order, members ascending */
  int64_t *clusOff = (int64_t *)malloc(8 * (size_t)n), *reprOff = (int64_t *)malloc(8 * (size_t)n);
  int *is_rep = (int *)calloc((size_t)n, sizeof(int));
  int **members = (int **)calloc((size_t)n, sizeof(int *));
  int *fill = (int *)calloc((size_t)n, sizeof(int));
  for (int i = 0; i < n; i++)
    if (cnt[i]) members[i] = (int *)malloc(sizeof(int) * (size_t)cnt[i]);
  for (int i = 0; i < n; i++) members[cluster[i]][fill[cluster[i]]++] = i;
  int64_t clusOffset = 0, reprOffset = 0;
  for (int i = 0; i < n; i++)
    for (int j = 0; j < cnt[i]; j++) {
      int idx = members[i][j];
      clusOff[idx] = clusOffset;
      clusOffset += db->name_len[idx] + 3;
      if (j == 0) {
        is_rep[idx] = 1;
        reprOff[idx] = reprOffset;
        reprOffset += db->name_len[idx] + db->read_len[idx] + 2;
        clusOffset -= 2;
      }
    }
  char path[4096];
  snprintf(path, sizeof(path), "%s/data.fasta", dbdir);
  FILE *in = fopen(path, "rb");
  snprintf(path, sizeof(path), "%s/cluster.txt", outdir);
  FILE *cf = fopen(path, "wb");
  snprintf(path, sizeof(path), "%s/represent.fasta", outdir);
  FILE *rf = fopen(path, "wb");
  int rc = (in && cf && rf) ? 0 : -2;
  char *line = NULL, *name = NULL, *read = NULL;
  size_t cap = 0, rcap = 0;
  for (int i = 0; i < n && rc == 0; i++) {
    fseek(in, (long)db->fasta_off[i], SEEK_SET);
    long k = read_line(in, &line, &cap);
    free(name);
    name = strdup(k >= 0 ? line : "");
    size_t rlen = 0;
    if (!read) {
      rcap = 1024;
      read = (char *)malloc(rcap);
    }
    read[0] = 0;
    for (;;) {
      int c = fgetc(in);
      if (c == EOF) break;
      ungetc(c, in);
      if (c == '>') break;
      k = read_line(in, &line, &cap);
      if (k < 0) break;
      if (rlen + (size_t)k + 1 > rcap) {
        while (rlen + (size_t)k + 1 > rcap) rcap *= 2;
        read = (char *)realloc(read, rcap);
      }
      memcpy(read + rlen, line, (size_t)k);
      rlen += (size_t)k;
      read[rlen] = 0;
    }
    fseek(cf, (long)clusOff[i], SEEK_SET);
    if (is_rep[i]) {
      fprintf(cf, "%s\n", name);
      fseek(rf, (long)reprOff[i], SEEK_SET);
      fprintf(rf, "%s\n%s\n", name, read);
    } else {
      fprintf(cf, "  %s\n", name);
    }
  }
  if (in) fclose(in);
  if (cf) fclose(cf);
  if (rf) fclose(rf);
  free(line);
  free(name);
  free(read);
  for (int i = 0; i < n; i++) free(members[i]);
  free(members);
  free(fill);
  free(is_rep);
  free(clusOff);
  free(reprOff);
  free(cnt);
  free(first);
  if (n_clusters) *n_clusters = count;
  return rc;
}
