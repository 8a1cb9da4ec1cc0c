// checkpoint.cu — saving and resuming a clustering run (no counterpart in
// the reference, whose runs cannot be interrupted).  A checkpoint holds the
// run's whole device state after the last completed step: the run state
// (representative, iteration, counters), the unclustered-set bitmap, the
// assignment and score arrays, and the parameters.  It names its database by
// record count, word count and a hash of the records computed on the device,
// and ends with a checksum of everything before it; resume refuses files that
// do not match the loaded database or are damaged (NGIA_E_FORMAT).
#include <cstdio>
#include <cstring>
#include <vector>

#include "../host/host_common.h"
#include "ctx.h"

using ngia::fail;

namespace {

constexpr char kMagic[8] = {'N', 'G', 'I', 'A', 'C', 'K', 'P', '1'};
constexpr uint32_t kVersion = 2;  // 2: run state with the long-candidate count

struct CkptHeader {
  char magic[8];
  uint32_t version;
  int32_t type, n;
  int32_t state_bytes;
  int64_t n_words;
  uint64_t db_hash;
  float similarity;
  int32_t word_length, precise, word_order, refill;
  int32_t reserved;
};

// Order-independent 64-bit hash of the records: the sum over words of an odd
// multiplier times (word, index) mixed.
__global__ void k_db_hash(const uint32_t *__restrict__ words, int64_t n_words, unsigned long long *out) {
  unsigned long long h = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_words; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long x = ((unsigned long long)i << 32) ^ words[i];
    x ^= x >> 31;
    x *= 0x9E3779B97F4A7C15ull;
    x ^= x >> 29;
    h += x;
  }
  for (int o = 16; o; o >>= 1) h += __shfl_down_sync(0xFFFFFFFFu, h, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, h);
}

int db_hash(ngia_ctx *c, uint64_t *out) {
  unsigned long long *d = nullptr;
  cudaError_t e = cudaMalloc((void **)&d, sizeof(*d));
  if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, sizeof(*d), c->stream);
  if (e == cudaSuccess) {
    k_db_hash<<<c->num_sms * 4, 256, 0, c->stream>>>(c->d_words, c->n_words, d);
    e = cudaGetLastError();
  }
  unsigned long long h = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  cudaFree(d);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "checkpoint: database hash: %s", cudaGetErrorString(e));
  *out = h;
  return NGIA_OK;
}

// FNV-1a over a byte range, continuing from h.
uint64_t fnv(uint64_t h, const void *p, size_t n) {
  const unsigned char *b = static_cast<const unsigned char *>(p);
  for (size_t i = 0; i < n; i++) {
    h ^= b[i];
    h *= 0x100000001B3ull;
  }
  return h;
}

}  // namespace

extern "C" int ngia_cluster_save(ngia_ctx *c, const char *path) {
  ngia::clear_error();
  if (!c || !path) return fail(NGIA_E_ARG, "ngia_cluster_save: null argument");
  if (!c->begun) return fail(NGIA_E_STATE, "ngia_cluster_save before ngia_cluster_begin");
  int rc = ngia::drv::pull_state(c);
  if (rc) return rc;
  const size_t n = (size_t)c->db.n, nbw = (n + 31) / 32;
  CkptHeader h{};
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.type = c->db.type;
  h.n = c->db.n;
  h.state_bytes = (int32_t)sizeof(ngia::RunState);
  h.n_words = c->n_words;
  rc = db_hash(c, &h.db_hash);
  if (rc) return rc;
  h.similarity = c->prm.s;
  h.word_length = c->prm.w;
  h.precise = c->prm.precise;
  h.word_order = c->prm.word_order;
  h.refill = c->prm.refill;
  std::vector<uint32_t> alive(nbw);
  std::vector<int32_t> cl(n), id(n);
  cudaError_t e = cudaMemcpyAsync(alive.data(), c->rb.alive, 4 * nbw, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(cl.data(), c->rb.cluster, 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(id.data(), c->rb.ident, 4 * n, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "ngia_cluster_save: %s", cudaGetErrorString(e));
  ngia::RunState st = *c->h_state;
  uint64_t sum = 0xCBF29CE484222325ull;
  sum = fnv(sum, &h, sizeof(h));
  sum = fnv(sum, &st, sizeof(st));
  sum = fnv(sum, alive.data(), 4 * nbw);
  sum = fnv(sum, cl.data(), 4 * n);
  sum = fnv(sum, id.data(), 4 * n);
  const std::string tmp = std::string(path) + ".part";
  FILE *f = fopen(tmp.c_str(), "wb");
  if (!f) return fail(NGIA_E_IO, "ngia_cluster_save: cannot write %s", tmp.c_str());
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(&st, sizeof(st), 1, f) == 1 &&
            fwrite(alive.data(), 4, nbw, f) == nbw && fwrite(cl.data(), 4, n, f) == n &&
            fwrite(id.data(), 4, n, f) == n && fwrite(&sum, sizeof(sum), 1, f) == 1;
  ok = (fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(NGIA_E_IO, "ngia_cluster_save: writing %s failed", path);
  }
  return NGIA_OK;
}

extern "C" int ngia_cluster_resume(ngia_ctx *c, const char *path, int32_t mode) {
  ngia::clear_error();
  if (!c || !path) return fail(NGIA_E_ARG, "ngia_cluster_resume: null argument");
  if (mode != NGIA_MODE_PLAIN && mode != NGIA_MODE_GRAPH && mode != NGIA_MODE_SPEC)
    return fail(NGIA_E_ARG, "unknown mode %d", mode);
  FILE *f = fopen(path, "rb");
  if (!f) return fail(NGIA_E_IO, "ngia_cluster_resume: cannot open %s", path);
  CkptHeader h{};
  const size_t n = (size_t)c->db.n, nbw = (n + 31) / 32;
  ngia::RunState st{};
  std::vector<uint32_t> alive(nbw);
  std::vector<int32_t> cl(n), id(n);
  uint64_t sum_file = 0;
  bool ok = fread(&h, sizeof(h), 1, f) == 1;
  const bool same_db = ok && std::memcmp(h.magic, kMagic, 8) == 0 && h.version == kVersion &&
                       h.type == c->db.type && h.n == c->db.n && h.n_words == c->n_words &&
                       h.state_bytes == (int32_t)sizeof(ngia::RunState);
  if (same_db)
    ok = fread(&st, sizeof(st), 1, f) == 1 && fread(alive.data(), 4, nbw, f) == nbw && fread(cl.data(), 4, n, f) == n &&
         fread(id.data(), 4, n, f) == n && fread(&sum_file, sizeof(sum_file), 1, f) == 1;
  fclose(f);
  if (!same_db) return fail(NGIA_E_FORMAT, "ngia_cluster_resume: %s is not a checkpoint of this database", path);
  if (!ok) return fail(NGIA_E_FORMAT, "ngia_cluster_resume: %s is truncated", path);
  uint64_t sum = 0xCBF29CE484222325ull;
  sum = fnv(sum, &h, sizeof(h));
  sum = fnv(sum, &st, sizeof(st));
  sum = fnv(sum, alive.data(), 4 * nbw);
  sum = fnv(sum, cl.data(), 4 * n);
  sum = fnv(sum, id.data(), 4 * n);
  if (sum != sum_file) return fail(NGIA_E_FORMAT, "ngia_cluster_resume: %s is damaged (checksum)", path);
  uint64_t hash = 0;
  int rc = db_hash(c, &hash);
  if (rc) return rc;
  if (hash != h.db_hash) return fail(NGIA_E_FORMAT, "ngia_cluster_resume: %s belongs to another database", path);
  const ngia_params p = {h.similarity, h.word_length, h.precise};
  rc = ngia::drv::validate_params(c->db.type, &p);
  if (rc) return rc;
  // the same ranges ngia_set_tuning accepts: the checksum only catches
  // accidental damage, not a well-formed file with settings out of range
  if (h.word_order < 0 || h.word_order > 2 || h.refill < 1 || h.refill > 32)
    return fail(NGIA_E_FORMAT, "ngia_cluster_resume: %s holds tuning settings out of range", path);
  // from the first device write on, the context holds no run that can be
  // stepped until the driver of the resumed run is ready
  c->begun = false;
  c->prm.s = h.similarity;
  c->prm.w = h.word_length;
  c->prm.precise = h.precise;
  c->prm.word_order = h.word_order;
  c->prm.refill = h.refill;
  st.iter_limit = INT64_MAX;
  *c->h_state = st;
  cudaError_t e = cudaMemcpyAsync(c->rb.st, c->h_state, sizeof(st), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->rb.alive, alive.data(), 4 * nbw, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->rb.cluster, cl.data(), 4 * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->rb.ident, id.data(), 4 * n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "ngia_cluster_resume: %s", cudaGetErrorString(e));
  c->mode = mode;
  c->ms_filter = c->ms_align = 0.0;
  for (double &m : c->ms_class) m = 0.0;
  if (mode == NGIA_MODE_GRAPH) {
    ngia::drv::destroy_graph(c);
    rc = ngia::drv::build_graph(c);
    if (rc) return rc;
  }
  if (mode == NGIA_MODE_SPEC) {
    rc = ngia::drv::spec_prepare(c);
    if (rc) return rc;
  }
  c->begun = true;
  return NGIA_OK;
}
