// Forest prediction kernels: one thread per pixel walks every tree of the
// forest (cl_classifier_impl.hpp:478-552, predict.cl:36-117).  A header so that
// the kernels also compile, through NVRTC, for a user feature plugin.
#pragma once

#include "pd_plugins.cuh"

namespace pd {

struct TreeMeta {
  unsigned long long off;  // first node of the tree in the forest arrays
  uint32_t depth, pad;
};

constexpr int kPredX = 32, kPredY = 8, kPredThreads = kPredX * kPredY;

template <class P>
PD_D int32_t walk(const typename P::Prep &prep, const int32_t *__restrict__ lc,
                  const typename P::feat_t *__restrict__ feat, const typename P::feat_t *__restrict__ thr,
                  uint32_t depth) {
  using FeatT = typename P::feat_t;
  constexpr int D = P::kFeatDim;
  int32_t node = 0;
  for (uint32_t d = 1; d < depth; d++) {
    const int32_t c = ldg(lc + node);
    if (c < 0) break;  // leaf (-1); an untrained root (-2) also stops
    FeatT fv[D];
#pragma unroll
    for (int k = 0; k < D; k++) fv[k] = ldg(feat + (size_t)node * D + k);
    const FeatT r = P::eval(prep, fv);
    node = c + (r <= ldg(thr + node) ? 0 : 1);
  }
  return node;
}

// grid (ceil(W/32), ceil(H/8), n_images); dynamic smem n_trees*256 int32.
template <class P>
__global__ void __launch_bounds__(kPredThreads) k_predict_posterior(
    const uint8_t *__restrict__ images, uint64_t img_bytes, uint32_t W, uint32_t H,
    const uint8_t *__restrict__ masks, float *__restrict__ out, const int32_t *__restrict__ lc,
    const typename P::feat_t *__restrict__ feat, const typename P::feat_t *__restrict__ thr,
    const float *__restrict__ post, const TreeMeta *__restrict__ meta, uint32_t n_trees, uint32_t K,
    const uint32_t *__restrict__ magic) {
  using ImgT = typename P::img_t;
  constexpr int D = P::kFeatDim;
  extern __shared__ int32_t leaf_s[];
  const uint32_t tid = threadIdx.y * kPredX + threadIdx.x;
  const uint32_t x = blockIdx.x * kPredX + threadIdx.x, y = blockIdx.y * kPredY + threadIdx.y, z = blockIdx.z;
  if (x >= W || y >= H) return;
  const size_t P_ = (size_t)W * H, pix = (size_t)y * W + x;
  float *o = out + (size_t)z * K * P_ + pix;
  if (masks && !masks[(size_t)z * P_ + pix]) {
    for (uint32_t l = 0; l < K; l++) o[l * P_] = 0.0f;
    return;
  }
  ImageRef<ImgT> im;
  im.data = reinterpret_cast<const ImgT *>(images + (size_t)z * img_bytes);
  im.w = (int32_t)W;
  im.h = (int32_t)H;
  im.magic = magic;
  const auto prep = P::prepare(im, (int32_t)x, (int32_t)y);
  for (uint32_t t = 0; t < n_trees; t++) {
    const size_t off = meta[t].off;
    leaf_s[t * kPredThreads + tid] = walk<P>(prep, lc + off, feat + off * D, thr + off, meta[t].depth);
  }
  const float nt = (float)n_trees;
  for (uint32_t l = 0; l < K; l++) {
    float acc = 0.0f;
    for (uint32_t t = 0; t < n_trees; t++)
      acc = acc + ldg(post + (meta[t].off + (size_t)leaf_s[t * kPredThreads + tid]) * K + l);
    o[l * P_] = fdiv(acc, nt);
  }
}

template <class P>
__global__ void __launch_bounds__(kPredThreads) k_predict_leaf(const uint8_t *__restrict__ image, uint32_t W,
                                                               uint32_t H, const uint8_t *__restrict__ mask,
                                                               int32_t *__restrict__ out,
                                                               const int32_t *__restrict__ lc,
                                                               const typename P::feat_t *__restrict__ feat,
                                                               const typename P::feat_t *__restrict__ thr,
                                                               uint32_t depth, const uint32_t *__restrict__ magic) {
  using ImgT = typename P::img_t;
  const uint32_t x = blockIdx.x * kPredX + threadIdx.x, y = blockIdx.y * kPredY + threadIdx.y;
  if (x >= W || y >= H) return;
  const size_t pix = (size_t)y * W + x;
  if (mask && !mask[pix]) {
    out[pix] = 0;
    return;
  }
  ImageRef<ImgT> im;
  im.data = reinterpret_cast<const ImgT *>(image);
  im.w = (int32_t)W;
  im.h = (int32_t)H;
  im.magic = magic;
  out[pix] = walk<P>(P::prepare(im, (int32_t)x, (int32_t)y), lc, feat, thr, depth);
}

}  // namespace pd
