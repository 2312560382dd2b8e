// The colour-to-class step of the reference's label loader (CVRGBLabelsLoader,
// _rgb2label at cv_image_loader_impl.hpp:233-266) on the GPU: every pixel of an
// RGB or RGBA label image becomes 1 + the first class whose colour it has, or 0.
// The reference searches the colour list per pixel; here the host builds an
// open-addressing table from colour to first class (512 entries, in shared
// memory) and each thread maps 16 pixels with 16-byte loads and one 16-byte store.
#include <algorithm>
#include <cstring>
#include <thread>
#include <vector>

#include "pd_ctx.cuh"

namespace pd {
namespace {

constexpr uint32_t kLabThreads = 256;
constexpr uint32_t kColourSlots = 512;  // power of two >= 2 * 255 classes

PD_HD uint32_t colour_hash(uint32_t rgb) { return (rgb * 0x9E3779B1u) >> 23; }  // 9 bits

// Table entry: rgb | (class + 1) << 24; 0 = empty.
PD_D uint32_t colour_class(const uint32_t *tab, uint32_t rgb) {
  uint32_t h = colour_hash(rgb);
  for (uint32_t i = 0; i < kColourSlots; i++) {
    const uint32_t e = tab[h];
    if (e == 0) return 0;
    if ((e & 0xFFFFFFu) == rgb) return e >> 24;
    h = (h + 1) & (kColourSlots - 1);
  }
  return 0;
}

PD_D uint32_t byte_of(const uint32_t *w, uint32_t i) { return (w[i >> 2] >> (8 * (i & 3))) & 0xFFu; }

// n pixels of CH (3 or 4) bytes at src (16-byte aligned) -> n labels at dst.
template <uint32_t CH>
__global__ void __launch_bounds__(kLabThreads) k_rgb_to_labels(const uint8_t *__restrict__ src, uint64_t n,
                                                               const uint32_t *__restrict__ table,
                                                               uint8_t *__restrict__ dst) {
  constexpr uint32_t channels = CH;
  __shared__ uint32_t tab[kColourSlots];
  for (uint32_t i = threadIdx.x; i < kColourSlots; i += kLabThreads) tab[i] = table[i];
  __syncthreads();
  const uint64_t groups = (n + 15) / 16;
  for (uint64_t g = blockIdx.x * (uint64_t)kLabThreads + threadIdx.x; g < groups;
       g += (uint64_t)gridDim.x * kLabThreads) {
    const uint64_t p0 = g * 16;
    uint32_t out[4] = {0, 0, 0, 0};
    if (p0 + 16 <= n) {
      uint32_t w[16];
      const uint4 *s = reinterpret_cast<const uint4 *>(src + p0 * channels);
#pragma unroll
      for (uint32_t v = 0; v < 4; v++) {
        if (v < channels) {
          const uint4 q = __ldg(s + v);
          w[4 * v] = q.x;
          w[4 * v + 1] = q.y;
          w[4 * v + 2] = q.z;
          w[4 * v + 3] = q.w;
        }
      }
#pragma unroll
      for (uint32_t i = 0; i < 16; i++) {
        const uint32_t b = i * channels;
        const uint32_t rgb = byte_of(w, b) | byte_of(w, b + 1) << 8 | byte_of(w, b + 2) << 16;
        out[i >> 2] |= colour_class(tab, rgb) << (8 * (i & 3));
      }
      *reinterpret_cast<uint4 *>(dst + p0) = make_uint4(out[0], out[1], out[2], out[3]);
    } else {
      for (uint64_t p = p0; p < n; p++) {
        const uint8_t *q = src + p * channels;
        dst[p] = (uint8_t)colour_class(tab, q[0] | (uint32_t)q[1] << 8 | (uint32_t)q[2] << 16);
      }
    }
  }
}

int colour_table(const uint8_t *map, uint32_t n_classes, std::vector<uint32_t> *tab) {
  PD_CHECK(map, PD_ERR_INVALID, "null colour map");
  PD_CHECK(n_classes >= 1 && n_classes <= 255, PD_ERR_INVALID, "nClasses %u outside [1,255]", n_classes);
  tab->assign(kColourSlots, 0u);
  for (uint32_t k = 0; k < n_classes; k++) {
    const uint32_t rgb = map[3 * k] | (uint32_t)map[3 * k + 1] << 8 | (uint32_t)map[3 * k + 2] << 16;
    uint32_t h = colour_hash(rgb);
    while ((*tab)[h] != 0 && ((*tab)[h] & 0xFFFFFFu) != rgb) h = (h + 1) & (kColourSlots - 1);
    if ((*tab)[h] == 0) (*tab)[h] = rgb | (k + 1) << 24;  // an earlier class with this colour wins
  }
  return PD_OK;
}

int launch_rgb(pd_ctx *ctx, const uint8_t *src, uint64_t n, uint32_t channels, const std::vector<uint32_t> &tab,
               uint8_t *dst) {
  PD_TRY(ctx->lab_tab.ensure(kColourSlots * 4));
  PD_CUDA(h2d(ctx, ctx->lab_tab.ptr, tab.data(), kColourSlots * 4));
  int sms = 0;
  PD_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const uint64_t groups = (n + 15) / 16;
  const uint32_t grid =
      (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((groups + kLabThreads - 1) / kLabThreads, (uint64_t)sms * 8));
  PD_CUDA(cudaEventRecord(ctx->ev[0], ctx->stream));
  if (channels == 3)
    k_rgb_to_labels<3><<<grid, kLabThreads, 0, ctx->stream>>>(src, n, ctx->lab_tab.as<uint32_t>(), dst);
  else
    k_rgb_to_labels<4><<<grid, kLabThreads, 0, ctx->stream>>>(src, n, ctx->lab_tab.as<uint32_t>(), dst);
  PD_CUDA(cudaGetLastError());
  PD_CUDA(cudaEventRecord(ctx->ev[1], ctx->stream));
  ctx->launches++;
  return PD_OK;
}

}  // namespace
}  // namespace pd

using namespace pd;

extern "C" int pd_rgb_to_labels(pd_ctx *ctx, uint32_t n_images, const uint8_t *const *images, const uint32_t *widths,
                                const uint32_t *heights, uint32_t channels, const uint8_t *map, uint32_t n_classes,
                                uint8_t *const *out) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  PD_CHECK(channels == 3 || channels == 4, PD_ERR_INVALID, "label images have 3 or 4 channels (got %u)", channels);
  std::vector<uint32_t> tab;
  PD_TRY(colour_table(map, n_classes, &tab));
  if (n_images == 0) return PD_OK;
  PD_CHECK(images && widths && heights && out, PD_ERR_INVALID, "null argument");
  std::vector<uint64_t> off(n_images + 1, 0);
  for (uint32_t i = 0; i < n_images; i++) {
    PD_CHECK(images[i] && out[i], PD_ERR_INVALID, "image %u has a null buffer", i);
    off[i + 1] = off[i] + (uint64_t)widths[i] * heights[i];
  }
  const uint64_t n = off[n_images];
  if (n == 0) return PD_OK;
  PD_CUDA(cudaSetDevice(ctx->device));
  // pixels of all images back to back (the mapping is per pixel), padded to 16 pixels
  const uint64_t in_bytes = (n + 16) * channels, out_bytes = n + 16;
  PD_TRY(ctx->h_lab.ensure(in_bytes + out_bytes));
  uint8_t *hs = ctx->h_lab.as<uint8_t>(), *ho = hs + in_bytes;
  const unsigned nt = std::max(1u, std::min({16u, std::thread::hardware_concurrency(), n_images}));
  auto stage = [&](unsigned th) {
    for (uint32_t i = th; i < n_images; i += nt) std::memcpy(hs + off[i] * channels, images[i], (off[i + 1] - off[i]) * channels);
  };
  {
    std::vector<std::thread> th;
    for (unsigned k = 1; k < nt; k++) th.emplace_back(stage, k);
    stage(0);
    for (auto &x : th) x.join();
  }
  PD_TRY(ctx->lab_src.ensure(in_bytes));
  PD_TRY(ctx->lab_dst.ensure(out_bytes));
  PD_CUDA(h2d(ctx, ctx->lab_src.ptr, hs, n * channels));
  PD_TRY(launch_rgb(ctx, ctx->lab_src.as<uint8_t>(), n, channels, tab, ctx->lab_dst.as<uint8_t>()));
  PD_CUDA(d2h(ctx, ho, ctx->lab_dst.ptr, n));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  for (uint32_t i = 0; i < n_images; i++) std::memcpy(out[i], ho + off[i], off[i + 1] - off[i]);
  return PD_OK;
}

extern "C" int pd_rgb_to_labels_device(pd_ctx *ctx, uint64_t n_pixels, const uint8_t *src_device, uint32_t channels,
                                       const uint8_t *map, uint32_t n_classes, uint8_t *dst_device, float *ms) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  PD_CHECK(channels == 3 || channels == 4, PD_ERR_INVALID, "label images have 3 or 4 channels (got %u)", channels);
  std::vector<uint32_t> tab;
  PD_TRY(colour_table(map, n_classes, &tab));
  if (n_pixels == 0) return PD_OK;
  PD_CHECK(src_device && dst_device, PD_ERR_INVALID, "null argument");
  PD_CHECK(((uintptr_t)src_device % 16) == 0 && ((uintptr_t)dst_device % 16) == 0, PD_ERR_UNSUPPORTED,
           "device buffers must be 16-byte aligned");
  PD_CUDA(cudaSetDevice(ctx->device));
  PD_TRY(launch_rgb(ctx, src_device, n_pixels, channels, tab, dst_device));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  if (ms) PD_CUDA(cudaEventElapsedTime(ms, ctx->ev[0], ctx->ev[1]));
  return PD_OK;
}
