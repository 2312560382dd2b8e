// Measured ceiling of the histogram kernel's own bound: the rate at which this
// GPU retires conflict-free shared-memory atomic adds.  The histogram kernel
// does one such add per (sample, candidate) evaluation (each lane increments
// its own column of a [class][rank][lane] tile, so the 32 lanes of a warp hit
// 32 different banks); this kernel issues the same instruction in the same
// layout, with eight independent adds in flight per thread, at several
// occupancies, and reports the best rate.
#include <algorithm>
#include <cstring>

#include "pd_common.cuh"

namespace pd {

constexpr int kPeakThreads = 256;
constexpr int kPeakRows = 128;  // [row][lane] words: 16 KiB per CTA
constexpr int kPeakInflight = 8;

__global__ void __launch_bounds__(kPeakThreads) k_smem_atomic_peak(uint32_t iters, uint32_t *__restrict__ sink) {
  __shared__ uint32_t tile[kPeakRows * 32];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t i = threadIdx.x; i < kPeakRows * 32; i += blockDim.x) tile[i] = 0;
  __syncthreads();
  uint32_t row = (warp * 17u + blockIdx.x) & (kPeakRows - 1);
  for (uint32_t it = 0; it < iters; it++) {
#pragma unroll
    for (int j = 0; j < kPeakInflight; j++) {
      // rows differ between the adds in flight (no dependence through one word)
      atomicAdd(&tile[((row + 13u * j) & (kPeakRows - 1)) * 32 + lane], 1u + (uint32_t)(j & 1) * 65535u);
    }
    row = (row * 5u + 3u) & (kPeakRows - 1);
  }
  __syncthreads();
  uint32_t s = 0;
  for (uint32_t r = warp; r < kPeakRows; r += blockDim.x / 32) s += tile[r * 32 + lane];
  if (s == 0xFFFFFFFFu) sink[blockIdx.x] = s;  // keeps the adds observable
}

}  // namespace pd

using namespace pd;

extern "C" int pd_measure_smem_atomics(int device, double *adds_per_s, int32_t *best_ctas_per_sm) {
  PD_CHECK(adds_per_s, PD_ERR_INVALID, "null argument");
  PD_CUDA(cudaSetDevice(device));
  int sms = 0;
  PD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  uint32_t *sink = nullptr;
  PD_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
  PD_CUDA(cudaEventCreate(&e0));
  PD_CUDA(cudaEventCreate(&e1));
  cudaError_t err = cudaMalloc(&sink, (size_t)sms * 8 * sizeof(uint32_t));
  double best = 0.0;
  int best_ctas = 0;
  const uint32_t iters = 4096;
  for (int ctas : {2, 4, 8}) {
    if (err != cudaSuccess) break;
    const unsigned grid = (unsigned)(sms * ctas);
    for (int rep = 0; rep < 3 && err == cudaSuccess; rep++) {
      err = cudaEventRecord(e0, st);
      k_smem_atomic_peak<<<grid, kPeakThreads, 0, st>>>(iters, sink);
      if (err == cudaSuccess) err = cudaGetLastError();
      if (err == cudaSuccess) err = cudaEventRecord(e1, st);
      if (err == cudaSuccess) err = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
      if (err == cudaSuccess && rep > 0 && ms > 0.f) {  // the first launch warms up
        const double adds = (double)grid * kPeakThreads * iters * kPeakInflight;
        const double rate = adds / (ms * 1e-3);
        if (rate > best) {
          best = rate;
          best_ctas = ctas;
        }
      }
    }
  }
  cudaFree(sink);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(st);
  PD_CHECK(err == cudaSuccess, PD_ERR_CUDA, "shared-memory atomic measurement failed: %s", cudaGetErrorString(err));
  *adds_per_s = best;
  if (best_ctas_per_sm) *best_ctas_per_sm = best_ctas;
  return PD_OK;
}
