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

// One forest node as the prediction kernels read it: the plugin's candidate
// record (P::candidate of its features, built once per forest upload), its
// threshold and its left child, together in one 16-byte-aligned record -- one
// visit fetches one or two 32-byte sectors instead of three arrays.
template <class P>
struct __align__(16) NodeRec {
  typename P::Cand c;
  typename P::feat_t thr;
  int32_t lc;
};

constexpr int kPredX = 32, kPredY = 8, kPredThreads = kPredX * kPredY;
// Tree walks interleaved per pixel.  On the 3-tree, depth-16 forest of 640x480
// depth maps, 1 measures fastest (7.07e9 pixels/s; 2: 6.91e9, 3: 7.08e9): the
// wider walks cost registers and occupancy.
#ifndef PD_PRED_GROUP
#define PD_PRED_GROUP 1
#endif
constexpr int kPredGroup = PD_PRED_GROUP;

// Leaf reached by one tree from the root (nodes: the tree's records).
// AF: every node of the forest takes the plugin's fast path (P::fast, checked
// once per forest upload), so the walk carries no per-visit test or slow path.
template <class P, bool AF = false>
PD_D int32_t walk(const typename P::Prep &prep, const NodeRec<P> *__restrict__ nodes, uint32_t depth) {
  using FeatT = typename P::feat_t;
  int32_t node = 0;
  for (uint32_t d = 1; d < depth; d++) {
    const NodeRec<P> nr = nodes[node];
    if (nr.lc < 0) break;  // leaf (-1); an untrained root (-2) also stops
    const FeatT r = (AF || P::fast(nr.c)) ? P::template eval<true>(prep, nr.c) : P::template eval<false>(prep, nr.c);
    node = nr.lc + (r <= nr.thr ? 0 : 1);
  }
  return node;
}

// The record of every forest node, for the prediction kernels.
template <class P>
__global__ void k_forest_nodes(const typename P::feat_t *__restrict__ feat, const typename P::feat_t *__restrict__ thr,
                               const int32_t *__restrict__ lc, unsigned long long n_nodes,
                               NodeRec<P> *__restrict__ out) {
  const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (i < n_nodes) {
    NodeRec<P> r;
    r.c = P::candidate(feat + i * P::kFeatDim);
    r.thr = thr[i];
    r.lc = lc[i];
    out[i] = r;
  }
}

// Clears *all_fast when a node of the forest needs the plugin's slow path.
template <class P>
__global__ void k_forest_fast(const NodeRec<P> *__restrict__ nodes, unsigned long long n_nodes,
                              int *__restrict__ all_fast) {
  const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  if (i < n_nodes && !P::fast(nodes[i].c)) *all_fast = 0;
}

// The leaves of trees t0 .. t0+G-1 (those below n_trees) for one pixel, the G
// walks interleaved level by level so that their loads overlap; each walk is
// the one walk() does.
template <class P, int G, bool AF = false>
PD_D void walk_group(const typename P::Prep &prep, const NodeRec<P> *__restrict__ nodes,
                     const TreeMeta *__restrict__ meta, uint32_t t0, uint32_t n_trees, int32_t *leaf_s,
                     uint32_t tid) {
  using FeatT = typename P::feat_t;
  int32_t node[G];
  size_t off[G];
  uint32_t depth[G];
#pragma unroll
  for (int g = 0; g < G; g++) {
    node[g] = 0;
    const bool have = t0 + g < n_trees;
    off[g] = have ? meta[t0 + g].off : 0;
    depth[g] = have ? meta[t0 + g].depth : 0;  // depth 0: no step
  }
  uint32_t live = 0;
#pragma unroll
  for (int g = 0; g < G; g++) live |= (depth[g] > 1 ? 1u : 0u) << g;
  for (uint32_t d = 1; live; d++) {
#pragma unroll
    for (int g = 0; g < G; g++) {
      if (!((live >> g) & 1u)) continue;
      const NodeRec<P> nr = nodes[off[g] + node[g]];
      if (nr.lc < 0) {  // leaf (-1); an untrained root (-2) also stops
        live &= ~(1u << g);
        continue;
      }
      const FeatT r = (AF || P::fast(nr.c)) ? P::template eval<true>(prep, nr.c) : P::template eval<false>(prep, nr.c);
      node[g] = nr.lc + (r <= nr.thr ? 0 : 1);
      if (d + 1 >= depth[g]) live &= ~(1u << g);
    }
  }
#pragma unroll
  for (int g = 0; g < G; g++)
    if (t0 + g < n_trees) leaf_s[(t0 + g) * kPredThreads + tid] = node[g];
}

// The forest posterior of pixel (x, y): the leaf of every tree (kept in the
// CTA's leaf_s, [tree][thread]), then the leaf posteriors summed in tree order
// and divided by the tree count, written planar with stride plane.
template <class P, bool AF = false>
PD_D void predict_pixel(const ImageRef<typename P::img_t> &im, uint32_t x, uint32_t y, bool masked_out, float *o,
                        size_t plane, const NodeRec<P> *__restrict__ nodes, const float *__restrict__ post,
                        const TreeMeta *__restrict__ meta, uint32_t n_trees, uint32_t K, int32_t *leaf_s,
                        uint32_t tid) {
  if (masked_out) {
    for (uint32_t l = 0; l < K; l++) o[l * plane] = 0.0f;
    return;
  }
  const auto prep = P::prepare(im, (int32_t)x, (int32_t)y);
  for (uint32_t t = 0; t < n_trees; t += kPredGroup)
    walk_group<P, kPredGroup, AF>(prep, nodes, meta, t, n_trees, leaf_s, tid);
  const float nt = (float)n_trees;
  for (uint32_t l = 0; l < K; l++) {
    float acc = 0.0f;
    for (uint32_t t = 0; t < n_trees; t++)
      acc = acc + ldg(post + (meta[t].off + (size_t)leaf_s[t * kPredThreads + tid]) * K + l);
    o[l * plane] = fdiv(acc, nt);
  }
}

// grid (ceil(W/32), ceil(H/8), n_images); dynamic smem n_trees*256 int32.
template <class P, bool AF = false>
__global__ void __launch_bounds__(kPredThreads) k_predict_posterior(
    const uint8_t *__restrict__ images, uint64_t img_bytes, uint32_t W, uint32_t H,
    const uint8_t *__restrict__ masks, float *__restrict__ out, const NodeRec<P> *__restrict__ nodes,
    const float *__restrict__ post, const TreeMeta *__restrict__ meta, uint32_t n_trees, uint32_t K,
    const uint32_t *__restrict__ magic) {
  using ImgT = typename P::img_t;
  extern __shared__ int32_t leaf_s[];
  const uint32_t tid = threadIdx.y * kPredX + threadIdx.x;
  const uint32_t x = blockIdx.x * kPredX + threadIdx.x, y = blockIdx.y * kPredY + threadIdx.y, z = blockIdx.z;
  if (x >= W || y >= H) return;
  const size_t P_ = (size_t)W * H, pix = (size_t)y * W + x;
  ImageRef<ImgT> im;
  im.data = reinterpret_cast<const ImgT *>(images + (size_t)z * img_bytes);
  im.w = (int32_t)W;
  im.h = (int32_t)H;
  im.magic = magic;
  predict_pixel<P, AF>(im, x, y, masks && !masks[(size_t)z * P_ + pix], out + (size_t)z * K * P_ + pix, P_, nodes,
                       post, meta, n_trees, K, leaf_s, tid);
}

// One image of a mixed-size batch: byte offsets of its pixels, mask and
// posterior planes in the batch buffers, its size and its first tile.
struct BatchImage {
  unsigned long long img_off, mask_off, out_off;
  uint32_t w, h, tiles_x, tile0;
  uint32_t has_mask, pad;
};

// A mixed-size batch in one launch: CTA b serves tile b of the concatenated
// tile lists (32x8 pixels; its image found by binary search over tile0).
template <class P, bool AF = false>
__global__ void __launch_bounds__(kPredThreads) k_predict_batch(
    const uint8_t *__restrict__ images, const uint8_t *__restrict__ masks, uint8_t *__restrict__ out,
    const BatchImage *__restrict__ batch, uint32_t n, const NodeRec<P> *__restrict__ nodes,
    const float *__restrict__ post, const TreeMeta *__restrict__ meta, uint32_t n_trees, uint32_t K,
    const uint32_t *__restrict__ magic) {
  using ImgT = typename P::img_t;
  extern __shared__ int32_t leaf_s[];
  uint32_t lo = 0, hi = n;  // the last image whose first tile is <= blockIdx.x
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (batch[mid].tile0 <= blockIdx.x) lo = mid;
    else hi = mid;
  }
  const BatchImage b = batch[lo];
  const uint32_t t = blockIdx.x - b.tile0;
  const uint32_t x = (t % b.tiles_x) * kPredX + threadIdx.x, y = (t / b.tiles_x) * kPredY + threadIdx.y;
  if (x >= b.w || y >= b.h) return;
  const uint32_t tid = threadIdx.y * kPredX + threadIdx.x;
  const size_t P_ = (size_t)b.w * b.h, pix = (size_t)y * b.w + x;
  ImageRef<ImgT> im;
  im.data = reinterpret_cast<const ImgT *>(images + b.img_off);
  im.w = (int32_t)b.w;
  im.h = (int32_t)b.h;
  im.magic = magic;
  const bool masked_out = b.has_mask && !masks[b.mask_off + pix];
  predict_pixel<P, AF>(im, x, y, masked_out, reinterpret_cast<float *>(out + b.out_off) + pix, P_, nodes, post, meta,
                       n_trees, K, leaf_s, tid);
}

template <class P, bool AF = false>
__global__ void __launch_bounds__(kPredThreads) k_predict_leaf(const uint8_t *__restrict__ image, uint32_t W,
                                                               uint32_t H, const uint8_t *__restrict__ mask,
                                                               int32_t *__restrict__ out,
                                                               const NodeRec<P> *__restrict__ nodes,
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
  out[pix] = walk<P, AF>(P::prepare(im, (int32_t)x, (int32_t)y), nodes, depth);
}

// One step of the per-pixel node map of features that read the tree
// (kernels/predict.cl:36-85, launched once per level by
// cl_tree_trainer_impl_traverse_ts.hpp:215-232 and cl_classifier_impl.hpp:478-520):
// a pixel inside the mask whose node has children moves to the child its
// feature selects -- the feature reading the map before the step and the tree
// as seen from that map's level -- and every other pixel keeps its node.  Pixel q of the concatenated images
// (image i starts at map_off[i]; n_images + 1 offsets).
struct NodeMapStep {
  const uint8_t *pixels;
  const uint64_t *img_off;   // byte offset of each image
  const uint32_t *img_wh;    // w | h << 16
  const uint64_t *map_off;
  uint32_t n_images;
  uint64_t n_pix;
  const uint8_t *mask;       // per pixel (nonzero: inside); null: every pixel
  const int32_t *map_in;
  int32_t *map_out;
  const int32_t *lc;
  const void *feat, *thr;    // feat_t [node][D], [node]
  const float *post;
  uint32_t n_classes;
  int32_t level, n_nodes;    // the level of map_in (root 0), the tree's node count
  const uint32_t *magic;
};

template <class P>
__global__ void __launch_bounds__(256) k_node_map_step(NodeMapStep a) {
  using FeatT = typename P::feat_t;
  using ImgT = typename P::img_t;
  constexpr int D = P::kFeatDim;
  const uint64_t q = (uint64_t)blockIdx.x * 256u + threadIdx.x;
  if (q >= a.n_pix) return;
  const int32_t n = a.map_in[q];
  int32_t out = n;
  const int32_t c = (a.mask && !a.mask[q]) ? -1 : a.lc[n];
  if (c >= 0) {
    uint32_t lo = 0, hi = a.n_images;  // the last image starting at or before q
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (a.map_off[mid] <= q) lo = mid;
      else hi = mid;
    }
    const uint32_t wh = a.img_wh[lo], w = wh & 0xffffu;
    const uint64_t pix = q - a.map_off[lo];
    ImageRef<ImgT> im;
    im.data = reinterpret_cast<const ImgT *>(a.pixels + a.img_off[lo]);
    im.w = (int32_t)w;
    im.h = (int32_t)(wh >> 16);
    im.magic = a.magic;
    im.nodes = a.map_in + a.map_off[lo];
    im.tree_lc = a.lc;
    im.tree_post = a.post;
    im.n_classes = a.n_classes;
    im.tree_level = a.level;
    im.tree_nodes = a.n_nodes;
    const FeatT *fp = static_cast<const FeatT *>(a.feat) + (size_t)n * D;
    FeatT fv[D];
#pragma unroll
    for (int d = 0; d < D; d++) fv[d] = fp[d];
    const auto prep = P::prepare(im, (int32_t)(pix % w), (int32_t)(pix / w));
    const FeatT resp = P::eval(prep, fv);
    out = c + (resp > static_cast<const FeatT *>(a.thr)[n] ? 1 : 0);
  }
  a.map_out[q] = out;
}

}  // namespace pd
