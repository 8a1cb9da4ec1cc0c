// noalloc.cu — banded-LCS scores of one representative against a batch of
// queries, for callers that cannot allocate device memory.
//
// Who needs this: host applications whose CUDA memory is owned by someone
// else — a framework or pool allocator that has reserved the device memory and
// hands out sub-buffers, or a latency-bound service loop that must not call
// cudaMalloc/cudaFree (they can synchronise the device and take milliseconds).
// Such a caller already holds its inputs and outputs in device memory; this
// entry point uses them as given and allocates nothing.
//
// The alignment needs per-thread working rows (one 32-bit word per 32
// representative residues).  Here they live in a fixed file-scope device
// array, g_noalloc_rows, of kNoAllocWords words (4 MiB).  Every GPU that loads
// this library keeps that array until the process exits.  Its size caps the
// representative at 65,536 residues (2,048 words per thread row); the grid is
// sized so that every thread's row fits.
//
// Host code must not use the array's name as a device address: the first call
// on each device looks its address up with cudaGetSymbolAddress (with that
// device current) and caches it; make that first call before any stream
// capture.  The cached address belongs to the module loaded in the device's
// primary context: after a cudaDeviceReset it would be stale, so the entry
// point is not for use across a device reset.  Each call copies the
// representative's two header words to the host to size its grid, which
// waits for `stream` to reach that copy.  All calls share the array, so calls
// whose kernels overlap on the GPU (different streams, or concurrent host
// threads) race on it; serialise them.  Nothing in the array has to start at
// zero: each thread initialises its row for every pair it scores.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../host/host_common.h"
#include "common.cuh"

namespace {

constexpr int kNoAllocWords = 1 << 20;  // 4 MiB of per-thread rows
constexpr int kThreads = 128;

__device__ __align__(256) uint32_t g_noalloc_rows[kNoAllocWords];

uint32_t *g_rows_addr[64] = {nullptr};  // per-device address of g_noalloc_rows
std::mutex g_rows_mu;

// Generic (any band width) banded bit-parallel LCS of the representative
// staged in shared memory against one query record, in the reference's
// (query block i, rep block j, residue k) loop order (func.cu:473-514); the
// 32 column carries of a block are packed into one word.  line[j * stride]
// is this thread's working row j.
template <int P>
__device__ int banded_lcs(const uint32_t *s_pl, int nb1, int net1, int L1, const uint32_t *q, int hw, float s,
                          uint32_t *line, int64_t stride) {
  const int L2 = (int)q[0], net2 = (int)q[1];
  const int nq = (net2 + 31) >> 5;
  const int B = ngia::band_blocks(L1, L2, s);
  const uint32_t *qpl = q + hw;
  const uint32_t vlast = (net1 & 31) ? ((1u << (net1 & 31)) - 1u) : 0xFFFFFFFFu;
  for (int j = 0; j < nb1; j++) line[j * stride] = 0xFFFFFFFFu;
  for (int i = 0; i < nq; i++) {
    const int cols = ((i + 1) * 32 > net2) ? (net2 & 31) : 32;
    uint32_t col[P];
#pragma unroll
    for (int p = 0; p < P; p++) col[p] = qpl[i * P + p];
    const int jstart = max(i - B, 0), jend = min(i + B, nb1 - 1);
    uint32_t cw = 0;
    for (int j = jstart; j <= jend; j++) {
      uint32_t R[P];
#pragma unroll
      for (int p = 0; p < P; p++) R[p] = s_pl[j * P + p];
      uint32_t row = line[j * stride], ncw = 0;
      for (int k = 0; k < cols; k++) {
        uint32_t x = row;
#pragma unroll
        for (int p = 0; p < P; p++) x &= ~(R[p] ^ (0u - ((col[p] >> k) & 1u)));
        const unsigned long long t = (unsigned long long)row + x + ((cw >> k) & 1u);
        ncw |= (uint32_t)(t >> 32) << k;
        row = (uint32_t)t | (row ^ x);
      }
      line[j * stride] = row;
      cw = ncw;
    }
  }
  int sum = 0;
  for (int j = 0; j < nb1; j++) sum += __popc(~line[j * stride] & (j == nb1 - 1 ? vlast : 0xFFFFFFFFu));
  return sum;
}

template <int P>
__global__ void __launch_bounds__(kThreads) k_noalloc_scores(const uint32_t *__restrict__ words, int64_t rep_off,
                                                             const int64_t *__restrict__ query_off, int n, float s,
                                                             int *__restrict__ scores, uint32_t *rows,
                                                             int64_t lanes, int cap_blocks) {
  extern __shared__ uint32_t s_pl[];
  constexpr int hw = P == 2 ? 6 : 30;
  const uint32_t *rep = words + rep_off;
  const int L1 = (int)rep[0], net1 = (int)rep[1];
  const int nb1 = (net1 + 31) / 32;
  if (nb1 > cap_blocks) return;  // the host checked this; never index past the rows
  for (int t = threadIdx.x; t < nb1 * P; t += blockDim.x) s_pl[t] = rep[hw + t];
  __syncthreads();
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t *line = rows + g;
  for (int64_t k = g; k < n; k += lanes) {
    const uint32_t *q = words + query_off[k];
    const uint32_t L2 = q[0], net2 = q[1];
    if (L2 > (uint32_t)ngia::kMaxLenDev || net2 > L2) {
      scores[k] = -1;  // not a makeDB record
      continue;
    }
    scores[k] = banded_lcs<P>(s_pl, nb1, net1, L1, q, hw, s, line, lanes);
  }
}

// Address of g_noalloc_rows on the current device, looked up once per device.
int rows_address(uint32_t **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return ngia::fail(NGIA_E_CUDA, "ngia_rep_scores_noalloc: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= 64) return ngia::fail(NGIA_E_LIMIT, "ngia_rep_scores_noalloc: device %d >= 64", dev);
  std::lock_guard<std::mutex> lock(g_rows_mu);
  if (!g_rows_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_rows);
    if (e != cudaSuccess || !p)
      return ngia::fail(NGIA_E_CUDA, "ngia_rep_scores_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_rows_addr[dev] = (uint32_t *)p;
  }
  *out = g_rows_addr[dev];
  return NGIA_OK;
}

}  // namespace

extern "C" int ngia_rep_scores_noalloc(const uint32_t *d_words, int64_t rep_off, const int64_t *d_query_off,
                                       int32_t n, int32_t type, float similarity, int32_t *d_scores,
                                       void *stream) {
  if (!d_words || (n > 0 && (!d_query_off || !d_scores)) || n < 0 || rep_off < 0)
    return ngia::fail(NGIA_E_ARG, "ngia_rep_scores_noalloc: bad argument");
  if (type != 0 && type != 1) return ngia::fail(NGIA_E_ARG, "ngia_rep_scores_noalloc: type %d not 0/1", type);
  if (!(similarity >= 0.1f && similarity <= 1.0f))
    return ngia::fail(NGIA_E_ARG, "ngia_rep_scores_noalloc: similarity outside [0.1, 1.0]");
  uint32_t *rows = nullptr;
  int rc = rows_address(&rows);
  if (rc) return rc;
  if (n == 0) return NGIA_OK;
  cudaStream_t st = (cudaStream_t)stream;
  uint32_t hdr[2] = {0, 0};  // representative raw and net length
  cudaError_t e = cudaMemcpyAsync(hdr, d_words + rep_off, sizeof(hdr), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return ngia::fail(NGIA_E_CUDA, "ngia_rep_scores_noalloc: %s", cudaGetErrorString(e));
  if (hdr[0] > (uint32_t)ngia::kMaxLenDev || hdr[1] > hdr[0])
    return ngia::fail(NGIA_E_LIMIT,
                      "ngia_rep_scores_noalloc: representative of %u residues (net %u); the fixed working "
                      "rows hold at most 65,536",
                      hdr[0], hdr[1]);
  const int nb1 = ((int)hdr[1] + 31) / 32;
  const int P = type == 0 ? 2 : 5;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // Every thread owns one row of nb1 words; the grid is as large as the
  // array allows (at least 4 CTAs: 2,048-word rows x 512 threads).
  const int64_t max_lanes = kNoAllocWords / (nb1 > 0 ? nb1 : 1);
  int grid = (int)std::min<int64_t>((int64_t)std::max(sms, 1) * 4, max_lanes / kThreads);
  grid = std::max(1, std::min(grid, (n + kThreads - 1) / kThreads));
  const int64_t lanes = (int64_t)grid * kThreads;
  const int cap_blocks = (int)(kNoAllocWords / lanes);
  const size_t smem = sizeof(uint32_t) * (size_t)std::max(1, nb1 * P);
  if (type == 0)
    k_noalloc_scores<2><<<grid, kThreads, smem, st>>>(d_words, rep_off, d_query_off, n, similarity, d_scores, rows,
                                                      lanes, cap_blocks);
  else
    k_noalloc_scores<5><<<grid, kThreads, smem, st>>>(d_words, rep_off, d_query_off, n, similarity, d_scores, rows,
                                                      lanes, cap_blocks);
  e = cudaGetLastError();
  if (e != cudaSuccess) return ngia::fail(NGIA_E_CUDA, "ngia_rep_scores_noalloc: %s", cudaGetErrorString(e));
  return NGIA_OK;
}
