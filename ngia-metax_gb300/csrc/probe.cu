// probe.cu — INT32 issue-rate probe for the roofline of the alignment
// kernels.  The probe runs, per thread, eight independent copies of the
// alignment inner-loop mix: two LOP3 building the match word, one 32-bit add,
// one LOP3 merging the row (the same C expressions as dp_column, minus the
// carry chain, so the hardware can overlap them).  Lane-operations per second
// are the denominator the alignment kernels' achieved rate is reported
// against.
#include <cuda_runtime.h>

#include "../host/host_common.h"

namespace {

__global__ void k_int_probe(uint32_t *out, int iters, uint32_t seed) {
  uint32_t r[8], p0[8], p1[8];
#pragma unroll
  for (int u = 0; u < 8; u++) {
    r[u] = seed * (threadIdx.x + 17u * u + 1u);
    p0[u] = r[u] ^ 0x9E3779B9u;
    p1[u] = r[u] * 0x85EBCA6Bu;
  }
  // residue masks come from rotating words, as the kernels derive them from
  // the query planes (two operations per plane per residue)
  uint32_t q0 = seed * 0x27D4EB2Fu + blockIdx.x, q1 = q0 * 0x165667B1u;
  for (int i = 0; i < iters; i++) {
    const uint32_t m0 = (uint32_t)((int)q0 >> 31), m1 = (uint32_t)((int)q1 >> 31);
    q0 = __funnelshift_l(q0, q0, 1);
    q1 = __funnelshift_l(q1, q1, 1);
#pragma unroll
    for (int u = 0; u < 8; u++) {
      uint32_t x = r[u] & ~(p0[u] ^ m0) & ~(p1[u] ^ m1);
      uint32_t t = r[u] + x;
      r[u] = t | (r[u] ^ x);
    }
  }
  uint32_t acc = 0;
#pragma unroll
  for (int u = 0; u < 8; u++) acc ^= r[u];
  if (acc == 0x12345678u) out[blockIdx.x * blockDim.x + threadIdx.x] = acc;  // keeps the loop live
}

}  // namespace

extern "C" int ngia_measure_int_peak(double *gops) {
  if (!gops) return ngia::fail(NGIA_E_ARG, "ngia_measure_int_peak: null argument");
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return ngia::fail(NGIA_E_CUDA, "ngia_measure_int_peak: no device");
  const int threads = 256, blocks = sms * 8, iters = 20000;
  uint32_t *out = nullptr;
  cudaEvent_t a, b;
  if (cudaMalloc(&out, sizeof(uint32_t) * (size_t)threads * blocks) != cudaSuccess)
    return ngia::fail(NGIA_E_NOMEM, "ngia_measure_int_peak: allocation failed");
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_int_probe<<<blocks, threads>>>(out, iters / 10, 3u);  // warm-up
  cudaEventRecord(a);
  k_int_probe<<<blocks, threads>>>(out, iters, 5u);
  cudaEventRecord(b);
  cudaError_t e = cudaEventSynchronize(b);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) return ngia::fail(NGIA_E_CUDA, "ngia_measure_int_peak: %s", cudaGetErrorString(e));
  // per iteration: 8 x (2 LOP3 + IADD3 + LOP3) + 4 mask operations
  const double ops = 36.0 * (double)iters * threads * blocks;
  *gops = ops / (ms * 1e-3) / 1e9;
  return NGIA_OK;
}
