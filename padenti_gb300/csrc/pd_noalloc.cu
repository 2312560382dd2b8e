// pd_split_noalloc: the best-split computation for callers that cannot
// allocate device memory.
//
// Some callers cannot call cudaMalloc at all: a host that hands out only memory
// it pre-allocated from its own pool, or an embedding runtime whose allocator
// must not be bypassed (allocating behind its back would break its accounting or
// its memory limit).  This entry point takes device pointers for its inputs and
// outputs from the caller and does all its intermediate work in one fixed,
// file-scope device array, kSplitScratchBytes (32 MiB) in size, which every GPU
// that loads this library holds until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the
// device address of the array with cudaGetSymbolAddress and fills the part of it
// that holds the exact log2 table; it synchronises the stream it is given.  Make
// that first call before any stream capture begins.  The address is kept per
// device for the life of the process, so cudaDeviceReset on a device after its
// first call is not supported (the array would be reloaded without the table).
//
// Limits: every node must hold fewer than 2^20 samples (the log2 table of the
// array has 2^20 entries), and the per-call working set must fit the array.
//
// The array is shared by every call: each call clears the parts that must start
// at zero, and two calls whose work overlaps on the GPU (for example on two
// streams, or from two threads) race on it and give wrong results.  Serialise
// them.  Each call reads its error flag back and synchronises its stream before
// returning.
#include <cstring>
#include <mutex>

#include "pd_ctx.cuh"
#include "pd_train_kernels.cuh"

namespace pd {

constexpr size_t kSplitScratchBytes = 32ull << 20;
constexpr uint32_t kNoallocLog2Len = 1u << 20;  // nodes of fewer than 2^20 samples
constexpr size_t kNoallocLog2Bytes = (size_t)kNoallocLog2Len * sizeof(double);

static __device__ __align__(256) unsigned char g_split_scratch[kSplitScratchBytes];

static std::mutex g_setup_mutex;
static unsigned char *g_scratch_ptr[256] = {};  // device address per device ordinal

__global__ void k_noalloc_error(const uint32_t *__restrict__ class_tot, uint32_t n, uint32_t K, uint32_t limit,
                                unsigned *__restrict__ err) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t N = 0;
  for (uint32_t l = 0; l < K; l++) N += class_tot[(size_t)i * K + l];
  if (N >= limit) atomicMax(err, 1u);
}

__global__ void k_noalloc_out(const SplitOut *__restrict__ so, uint32_t n, int32_t *__restrict__ t,
                              int32_t *__restrict__ f, double *__restrict__ g) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  t[i] = so[i].t;
  f[i] = so[i].f;
  g[i] = so[i].gain;
}

static int noalloc_setup(int dev, cudaStream_t st, unsigned char **out) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  PD_CHECK(dev >= 0 && dev < 256, PD_ERR_UNSUPPORTED, "device ordinal %d", dev);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    PD_CUDA(cudaGetSymbolAddress(&p, g_split_scratch));
    unsigned char *base = static_cast<unsigned char *>(p);
    k_log2_table<<<(kNoallocLog2Len + 255) / 256, 256, 0, st>>>(reinterpret_cast<double *>(base), kNoallocLog2Len,
                                                                 dd_inv_ln2());
    PD_CUDA(cudaGetLastError());
    PD_CUDA(cudaStreamSynchronize(st));
    g_scratch_ptr[dev] = base;
  }
  *out = g_scratch_ptr[dev];
  return PD_OK;
}

}  // namespace pd

using namespace pd;

extern "C" int pd_split_noalloc(const pd_train_params *params, uint32_t n_classes, const uint32_t *hist_device,
                                const uint32_t *class_tot_device, uint32_t n_nodes, int32_t *out_t_device,
                                int32_t *out_f_device, double *out_gain_device, void *stream) {
  PD_CHECK(params && hist_device && class_tot_device && out_t_device && out_f_device && out_gain_device,
           PD_ERR_INVALID, "null argument");
  PD_CHECK(n_classes >= 1 && n_classes <= PD_MAX_CLASSES, PD_ERR_UNSUPPORTED, "nClasses %u outside [1,%d]",
           n_classes, PD_MAX_CLASSES);
  PD_CHECK(params->n_features >= 1 && params->n_thresholds >= 1 && params->n_thresholds <= PD_MAX_THRESHOLDS,
           PD_ERR_INVALID, "n_features and n_thresholds must be in [1,...] and n_thresholds <= %d",
           PD_MAX_THRESHOLDS);
  if (n_nodes == 0) return PD_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint32_t F = params->n_features, T = params->n_thresholds, K = n_classes;
  const uint32_t max_parts = (F + kSplitCols - 1) / kSplitCols;
  uint32_t parts = std::min<uint32_t>(max_parts, std::max<uint32_t>(1, (4 * 152 + n_nodes - 1) / n_nodes));
  uint32_t cols = (F + parts - 1) / parts;
  cols = (cols + 31) / 32 * 32;
  parts = (F + cols - 1) / cols;
  // scratch layout after the log2 table, each region 256-byte aligned
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t b_g32 = up((size_t)n_nodes * T * F * sizeof(float));
  const size_t b_max = up((size_t)n_nodes * 8 + 16);  // node_max, done, error flag, recheck counter
  const size_t b_parts = up((size_t)n_nodes * parts * sizeof(SplitPart));
  const size_t b_out = up((size_t)n_nodes * sizeof(SplitOut));
  const size_t b_cl = up((size_t)n_nodes * K * 4);
  const size_t need = kNoallocLog2Bytes + b_g32 + b_max + b_parts + b_out + b_cl + 256;
  PD_CHECK(need <= kSplitScratchBytes, PD_ERR_UNSUPPORTED,
           "pd_split_noalloc: %u nodes of %u thresholds x %u features need %zu bytes of working memory; the "
           "fixed array holds %zu (call with fewer nodes)",
           n_nodes, T, F, need, kSplitScratchBytes);
  int dev = 0;
  PD_CUDA(cudaGetDevice(&dev));
  unsigned char *base = nullptr;
  PD_TRY(noalloc_setup(dev, st, &base));
  unsigned char *p = base + kNoallocLog2Bytes;
  float *g32 = reinterpret_cast<float *>(p);
  p += b_g32;
  unsigned *node_max = reinterpret_cast<unsigned *>(p);
  unsigned *done = node_max + n_nodes;
  unsigned *err = done + n_nodes;
  unsigned long long *rechecked = reinterpret_cast<unsigned long long *>(p + (((size_t)n_nodes * 8 + 4 + 7) / 8 * 8));
  p += b_max;
  SplitPart *part_best = reinterpret_cast<SplitPart *>(p);
  p += b_parts;
  SplitOut *so = reinterpret_cast<SplitOut *>(p);
  p += b_out;
  uint32_t *out_cl = reinterpret_cast<uint32_t *>(p);
  // what must start at zero: node maxima, finished-part counters, error flag, counter
  PD_CUDA(cudaMemsetAsync(node_max, 0, b_max, st));
  k_noalloc_error<<<(n_nodes + 255) / 256, 256, 0, st>>>(class_tot_device, n_nodes, K, kNoallocLog2Len, err);
  PD_CUDA(cudaGetLastError());
  SplitArgs a;
  memset(&a, 0, sizeof(a));
  a.hist = hist_device;
  a.perm = nullptr;
  a.class_tot = class_tot_device;
  a.g32 = g32;
  a.L = reinterpret_cast<const double *>(base);
  a.L_len = kNoallocLog2Len;
  a.F = F;
  a.T = T;
  a.K = K;
  a.delta = recheck_delta(K);
  a.cols = cols;
  a.parts = parts;
  a.node_max = node_max;
  a.done = done;
  a.part_best = part_best;
  a.out = so;
  a.out_cl = out_cl;
  a.rechecked = rechecked;
  a.slot_list = nullptr;
  const dim3 grid(parts, n_nodes);
  auto run = [&]<int KM>() -> int {
    k_split_g32<KM, true><<<grid, kSplitCols, 0, st>>>(a);
    k_split_pick<KM, true><<<grid, kSplitCols, 0, st>>>(a);
    PD_CUDA(cudaGetLastError());
    return PD_OK;
  };
  if (K <= 3) PD_TRY(run.template operator()<3>());
  else if (K <= 4) PD_TRY(run.template operator()<4>());
  else if (K <= 8) PD_TRY(run.template operator()<8>());
  else if (K <= 9) PD_TRY(run.template operator()<9>());
  else if (K <= 16) PD_TRY(run.template operator()<16>());
  else if (K <= 21) PD_TRY(run.template operator()<21>());
  else if (K <= 32) PD_TRY(run.template operator()<32>());
  else PD_TRY(run.template operator()<64>());
  k_noalloc_out<<<(n_nodes + 255) / 256, 256, 0, st>>>(so, n_nodes, out_t_device, out_f_device, out_gain_device);
  PD_CUDA(cudaGetLastError());
  unsigned h_err = 0;
  PD_CUDA(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, st));
  PD_CUDA(cudaStreamSynchronize(st));
  PD_CHECK(h_err == 0, PD_ERR_UNSUPPORTED,
           "pd_split_noalloc: a node holds %u (2^20) or more samples; nodes must hold fewer (the fixed log2 table "
           "of the working memory has %u entries)",
           kNoallocLog2Len, kNoallocLog2Len);
  return PD_OK;
}
