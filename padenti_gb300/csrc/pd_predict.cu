// Forest container and prediction: CLClassifier (cl_classifier_impl.hpp).
// The reference launches `predict` (depth-1) times per tree with an image copy
// between levels, then `computePosterior`, reads the [K][H][W] buffer back and
// sums on the host (cl_classifier_impl.hpp:478-552).  Here one kernel walks the
// whole forest per pixel, keeps the leaf ids of all trees, sums the leaf
// posteriors in tree order and divides by the tree count, writing the planar
// posterior once, coalesced.  A user feature that reads the tree and the node
// map (auto-context) needs every pixel's node of the level before it, so its
// prediction keeps the reference's level-synchronous steps (node_map_predict).
#include <algorithm>
#include <cstring>
#include <vector>

#include "pd_ctx.cuh"
#include "pd_plugins.cuh"
#include "pd_predict_kernels.cuh"
#include "pd_rtc.cuh"

namespace pd {

static int upload_forest(pd_ctx *ctx) {
  if (!ctx->forest_dirty) return PD_OK;
  const size_t nodes = ctx->h_lc.size();
  const uint32_t nt = (uint32_t)ctx->tree_depth.size();
  std::vector<TreeMeta> meta(nt);
  for (uint32_t t = 0; t < nt; t++) {
    meta[t].off = ctx->tree_off[t];
    meta[t].depth = ctx->tree_depth[t];
    meta[t].pad = 0;
  }
  PD_TRY(ctx->f_lc.ensure(nodes * 4 + 4));
  PD_TRY(ctx->f_feat.ensure(ctx->h_feat.size() + 4));
  PD_TRY(ctx->f_thr.ensure(ctx->h_thr.size() + 4));
  PD_TRY(ctx->f_post.ensure(ctx->h_post.size() * 4 + 4));
  PD_TRY(ctx->f_meta.ensure(nt * sizeof(TreeMeta) + 16));
  if (nodes) {
    PD_CUDA(h2d(ctx, ctx->f_lc.ptr, ctx->h_lc.data(), nodes * 4));
    PD_CUDA(h2d(ctx, ctx->f_feat.ptr, ctx->h_feat.data(), ctx->h_feat.size()));
    PD_CUDA(h2d(ctx, ctx->f_thr.ptr, ctx->h_thr.data(), ctx->h_thr.size()));
    PD_CUDA(h2d(ctx, ctx->f_post.ptr, ctx->h_post.data(), ctx->h_post.size() * 4));
    PD_CUDA(h2d(ctx, ctx->f_meta.ptr, meta.data(), nt * sizeof(TreeMeta)));
  }
  ctx->forest_dirty = false;
  ctx->forest_version++;
  return PD_OK;
}

// Bytes of one node's record: NodeRec<P>, or for a user feature the
// NodeRec<UserPlugin> compiled at run time (its size read from the module).
template <class P>
static int node_record(pd_ctx *ctx, size_t *bytes) {
  if (is_user_plugin(ctx)) {
    const RtcKernels *rk = nullptr;
    PD_TRY(rtc_kernels(ctx, &rk));
    *bytes = (size_t)rk->node_rec_bytes;
    return PD_OK;
  }
  if constexpr (!P::kRtcOnly) *bytes = sizeof(NodeRec<P>);
  return PD_OK;
}

// The record of every forest node (k_forest_nodes), rebuilt when the forest
// changes, so that a tree walk loads each node in one record.
template <class P>
static int ensure_forest_nodes(pd_ctx *ctx) {
  if (ctx->cand_version == ctx->forest_version) return PD_OK;
  using FeatT = typename P::feat_t;
  unsigned long long nodes = ctx->h_lc.size();
  size_t rec = 0;
  PD_TRY(node_record<P>(ctx, &rec));
  PD_CHECK(rec >= 16 && rec % 16 == 0, PD_ERR_STATE, "node record of %zu bytes", rec);
  PD_TRY(ctx->f_cand.ensure(nodes * rec + 16));
  const FeatT *ft = ctx->f_feat.as<FeatT>(), *th = ctx->f_thr.as<FeatT>();
  const int32_t *lc = ctx->f_lc.as<int32_t>();
  const dim3 grid((unsigned)((nodes + 255) / 256 + (nodes == 0)));
  if (is_user_plugin(ctx)) {
    const RtcKernels *rk = nullptr;
    PD_TRY(rtc_kernels(ctx, &rk));
    void *out = ctx->f_cand.ptr;
    void *args[] = {&ft, &th, &lc, &nodes, &out};
    PD_TRY(rtc_launch(ctx, rk->forest_nodes, grid, dim3(256), 0, args));
  } else if constexpr (!P::kRtcOnly) {
    k_forest_nodes<P><<<grid, 256, 0, ctx->stream>>>(ft, th, lc, nodes, ctx->f_cand.as<NodeRec<P>>());
    PD_CUDA(cudaGetLastError());
    // whether every node takes the fast path: the prediction kernels then carry no slow path
    PD_TRY(ctx->f_fast.ensure(16));
    int all = 1;
    PD_CUDA(h2d(ctx, ctx->f_fast.ptr, &all, 4));
    k_forest_fast<P><<<grid, 256, 0, ctx->stream>>>(ctx->f_cand.as<NodeRec<P>>(), nodes, ctx->f_fast.as<int>());
    PD_CUDA(cudaGetLastError());
    PD_CUDA(d2h(ctx, &all, ctx->f_fast.ptr, 4));
    PD_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->forest_fast = all != 0;
    ctx->launches += 2;
  }
  ctx->cand_version = ctx->forest_version;
  return PD_OK;
}

template <class P>
static int launch_posterior(pd_ctx *ctx, uint32_t n, const void *images, uint32_t W, uint32_t H,
                            const uint8_t *masks, float *out) {
  using FeatT = typename P::feat_t;
  const uint32_t nt = (uint32_t)ctx->tree_depth.size();
  const size_t smem = (size_t)nt * kPredThreads * 4;
  dim3 grid((W + kPredX - 1) / kPredX, (H + kPredY - 1) / kPredY, n);
  const uint64_t img_bytes = (uint64_t)W * H * ctx->cfg.n_channels * img_size(ctx->cfg.img_type);
  PD_TRY(ensure_forest_nodes<P>(ctx));
  if (is_user_plugin(ctx)) {
    const RtcKernels *rk = nullptr;
    PD_TRY(rtc_kernels(ctx, &rk));
    PD_TRY(rtc_set_smem(ctx, rk->predict_posterior, smem));
    const uint8_t *im = static_cast<const uint8_t *>(images);
    uint64_t ib = img_bytes;
    uint32_t w_ = W, h_ = H, nt_ = nt, k_ = (uint32_t)ctx->cfg.n_classes;
    const void *nd = ctx->f_cand.ptr;
    const float *po = ctx->f_post.as<float>();
    const TreeMeta *me = ctx->f_meta.as<TreeMeta>();
    const uint32_t *mg = ctx->magic_tab.as<uint32_t>();
    void *args[] = {&im, &ib, &w_, &h_, &masks, &out, &nd, &po, &me, &nt_, &k_, &mg};
    return rtc_launch(ctx, rk->predict_posterior, grid, dim3(kPredX, kPredY), smem, args);
  }
  if constexpr (!P::kRtcOnly) {
    auto kern = ctx->forest_fast ? k_predict_posterior<P, true> : k_predict_posterior<P, false>;
    PD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, dim3(kPredX, kPredY), smem, ctx->stream>>>(
        static_cast<const uint8_t *>(images), img_bytes, W, H, masks, out, ctx->f_cand.as<NodeRec<P>>(),
        ctx->f_post.as<float>(), ctx->f_meta.as<TreeMeta>(), nt, (uint32_t)ctx->cfg.n_classes,
        ctx->magic_tab.as<uint32_t>());
    PD_CUDA(cudaGetLastError());
    ctx->launches++;
  }
  return PD_OK;
}

// The forest posterior of features that read the tree, one tree at a time
// (computePosterior, kernels/predict.cl:88-117): each pixel adds its node's
// posterior to the planes in tree order and the last tree divides by the tree
// count -- the sums and the division of k_predict_posterior; masked-out pixels 0.
static __global__ void __launch_bounds__(256) k_node_map_posterior(const int32_t *__restrict__ map,
                                                                   const uint8_t *__restrict__ masks,
                                                                   const float *__restrict__ post, uint32_t K,
                                                                   float *__restrict__ out, uint64_t plane,
                                                                   uint64_t n_pix, int first, int last, float nt) {
  const uint64_t q = (uint64_t)blockIdx.x * 256u + threadIdx.x;
  if (q >= n_pix) return;
  float *o = out + (q / plane) * K * plane + q % plane;
  if (masks && !masks[q]) {
    if (first)
      for (uint32_t l = 0; l < K; l++) o[l * plane] = 0.0f;
    return;
  }
  const float *pn = post + (size_t)map[q] * K;
  for (uint32_t l = 0; l < K; l++) {
    float acc = (first ? 0.0f : o[l * plane]) + pn[l];
    if (last) acc = fdiv(acc, nt);
    o[l * plane] = acc;
  }
}

// Prediction of n same-size images (device buffers) for a feature that reads
// the tree: per tree, the node map from the root (all pixels at node 0) through
// depth - 1 synchronous steps (cl_classifier_impl.hpp:478-520), then either the
// posterior accumulation (leaf_tree < 0) or the map itself as the leaf ids of
// tree leaf_tree.
static int node_map_predict(pd_ctx *ctx, uint32_t n, const void *images, uint32_t W, uint32_t H, const uint8_t *masks,
                            float *post_out, int64_t leaf_tree, int32_t *leaf_out) {
  PD_CHECK(W < 65536 && H < 65536, PD_ERR_UNSUPPORTED, "image %ux%u: a feature that reads the tree needs sides < 65536",
           W, H);
  const RtcKernels *rk = nullptr;
  PD_TRY(rtc_kernels(ctx, &rk));
  const uint64_t P_ = (uint64_t)W * H, NP = P_ * n;
  const uint64_t img_bytes = P_ * ctx->cfg.n_channels * img_size(ctx->cfg.img_type);
  const uint32_t K = (uint32_t)ctx->cfg.n_classes, D = (uint32_t)ctx->cfg.feat_dim;
  const size_t fs = feat_size(ctx->cfg.feat_type);
  cudaStream_t st = ctx->stream;
  PD_TRY(ctx->np_map[0].ensure(NP * 4));
  PD_TRY(ctx->np_map[1].ensure(NP * 4));
  // descriptors: map offsets [n + 1], image byte offsets [n], sizes [n]
  std::vector<uint64_t> desc(2 * (size_t)n + 1 + ((size_t)n + 1) / 2, 0);
  uint32_t *wh = reinterpret_cast<uint32_t *>(desc.data() + 2 * (size_t)n + 1);
  for (uint32_t z = 0; z <= n; z++) desc[z] = (uint64_t)z * P_;
  for (uint32_t z = 0; z < n; z++) {
    desc[n + 1 + z] = (uint64_t)z * img_bytes;
    wh[z] = W | (H << 16);
  }
  PD_TRY(ctx->np_desc.ensure(desc.size() * 8));
  PD_CUDA(h2d(ctx, ctx->np_desc.ptr, desc.data(), desc.size() * 8));
  const uint64_t *dd = ctx->np_desc.as<uint64_t>();
  const uint32_t nt = (uint32_t)ctx->tree_depth.size();
  const uint32_t t0 = leaf_tree < 0 ? 0u : (uint32_t)leaf_tree, t1 = leaf_tree < 0 ? nt : t0 + 1;
  const dim3 grid((unsigned)((NP + 255) / 256));
  for (uint32_t t = t0; t < t1; t++) {
    const uint64_t off = ctx->tree_off[t];
    int cur = 0;
    PD_CUDA(cudaMemsetAsync(ctx->np_map[0].ptr, 0, NP * 4, st));
    for (uint32_t d = 1; d < ctx->tree_depth[t]; d++) {
      NodeMapStep a;
      a.pixels = static_cast<const uint8_t *>(images);
      a.img_off = dd + n + 1;
      a.img_wh = reinterpret_cast<const uint32_t *>(dd + 2 * (size_t)n + 1);
      a.map_off = dd;
      a.n_images = n;
      a.n_pix = NP;
      a.mask = masks;
      a.map_in = ctx->np_map[cur].as<int32_t>();
      a.map_out = ctx->np_map[1 - cur].as<int32_t>();
      a.lc = ctx->f_lc.as<int32_t>() + off;
      a.feat = ctx->f_feat.as<uint8_t>() + off * D * fs;
      a.thr = ctx->f_thr.as<uint8_t>() + off * fs;
      a.post = ctx->f_post.as<float>() + off * K;
      a.n_classes = K;
      a.level = (int32_t)d - 1;
      a.n_nodes = (int32_t)((1u << ctx->tree_depth[t]) - 1u);
      a.magic = ctx->magic_tab.as<uint32_t>();
      void *args[] = {&a};
      PD_TRY(rtc_launch(ctx, rk->node_map_step, grid, dim3(256), 0, args));
      cur = 1 - cur;
    }
    if (leaf_tree >= 0) {
      PD_CUDA(cudaMemcpyAsync(leaf_out, ctx->np_map[cur].ptr, NP * 4, cudaMemcpyDeviceToDevice, st));
    } else {
      k_node_map_posterior<<<grid, 256, 0, st>>>(ctx->np_map[cur].as<int32_t>(), masks,
                                                 ctx->f_post.as<float>() + off * K, K, post_out, P_, NP, t == 0,
                                                 t + 1 == nt, (float)nt);
      PD_CUDA(cudaGetLastError());
      ctx->launches++;
    }
  }
  return PD_OK;
}

}  // namespace pd

using namespace pd;

extern "C" int pd_forest_clear(pd_ctx *ctx) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  ctx->tree_depth.clear();
  ctx->tree_off.clear();
  ctx->h_lc.clear();
  ctx->h_feat.clear();
  ctx->h_thr.clear();
  ctx->h_post.clear();
  ctx->forest_dirty = true;
  return PD_OK;
}

extern "C" int pd_forest_add_tree(pd_ctx *ctx, uint32_t depth, const int32_t *left_child, const void *features,
                                  const void *thresholds, const float *posteriors) {
  PD_CHECK(ctx && left_child && features && thresholds && posteriors, PD_ERR_INVALID, "null argument");
  PD_CHECK(depth >= 1 && depth <= 24, PD_ERR_UNSUPPORTED, "tree depth %u outside [1,24]", depth);
  PD_CHECK(ctx->tree_depth.size() < PD_MAX_TREES, PD_ERR_UNSUPPORTED, "forest already holds %d trees", PD_MAX_TREES);
  const uint64_t nodes = (1ull << depth) - 1ull;
  const size_t fs = feat_size(ctx->cfg.feat_type), D = ctx->cfg.feat_dim, K = ctx->cfg.n_classes;
  // Every split node must point to an existing child pair.
  for (uint64_t i = 0; i < nodes; i++) {
    const int32_t c = left_child[i];
    PD_CHECK(c == -1 || c == -2 || (c >= 1 && (uint64_t)c + 1 < nodes), PD_ERR_INVALID,
             "node %llu has left child %d outside the tree", (unsigned long long)i, c);
  }
  ctx->tree_off.push_back(ctx->h_lc.size());
  ctx->tree_depth.push_back(depth);
  ctx->h_lc.insert(ctx->h_lc.end(), left_child, left_child + nodes);
  const uint8_t *fb = static_cast<const uint8_t *>(features), *tb = static_cast<const uint8_t *>(thresholds);
  ctx->h_feat.insert(ctx->h_feat.end(), fb, fb + nodes * D * fs);
  ctx->h_thr.insert(ctx->h_thr.end(), tb, tb + nodes * fs);
  ctx->h_post.insert(ctx->h_post.end(), posteriors, posteriors + nodes * K);
  ctx->forest_dirty = true;
  return PD_OK;
}

extern "C" int pd_forest_size(pd_ctx *ctx, uint32_t *n_trees) {
  PD_CHECK(ctx && n_trees, PD_ERR_INVALID, "null argument");
  *n_trees = (uint32_t)ctx->tree_depth.size();
  return PD_OK;
}

extern "C" int pd_predict_posterior_device(pd_ctx *ctx, uint32_t n_images, const void *images_device, uint32_t width,
                                           uint32_t height, const uint8_t *masks_device, float *out_device) {
  PD_CHECK(ctx && images_device && out_device, PD_ERR_INVALID, "null argument");
  PD_CHECK(!ctx->tree_depth.empty(), PD_ERR_STATE, "empty forest");
  PD_CHECK(width >= 1 && height >= 1 && n_images >= 1 && n_images <= 65535, PD_ERR_INVALID, "bad image batch");
  PD_CUDA(cudaSetDevice(ctx->device));
  PD_TRY(upload_forest(ctx));
  if (ctx->tree_feature)
    return node_map_predict(ctx, n_images, images_device, width, height, masks_device, out_device, -1, nullptr);
  return dispatch_config(ctx->cfg, [&]<class P>() {
    return launch_posterior<P>(ctx, n_images, images_device, width, height, masks_device, out_device);
  });
}

extern "C" int pd_predict_posterior(pd_ctx *ctx, const void *image, uint32_t width, uint32_t height,
                                    const uint8_t *mask, float *out) {
  PD_CHECK(ctx && image && out, PD_ERR_INVALID, "null argument");
  PD_CHECK(!ctx->tree_depth.empty(), PD_ERR_STATE, "empty forest");
  PD_CHECK(width >= 1 && height >= 1, PD_ERR_INVALID, "empty image");
  PD_CUDA(cudaSetDevice(ctx->device));
  const size_t P_ = (size_t)width * height;
  const size_t ib = P_ * ctx->cfg.n_channels * img_size(ctx->cfg.img_type);
  const size_t ob = P_ * ctx->cfg.n_classes * 4;
  PD_TRY(ctx->p_img.ensure(ib));
  PD_TRY(ctx->p_out.ensure(ob));
  if (mask) PD_TRY(ctx->p_mask.ensure(P_));
  cudaStream_t st = ctx->stream;
  PD_CUDA(h2d(ctx, ctx->p_img.ptr, image, ib));
  if (mask) PD_CUDA(h2d(ctx, ctx->p_mask.ptr, mask, P_));
  PD_TRY(pd_predict_posterior_device(ctx, 1, ctx->p_img.ptr, width, height, mask ? ctx->p_mask.as<uint8_t>() : nullptr,
                                     ctx->p_out.as<float>()));
  PD_CUDA(d2h(ctx, out, ctx->p_out.ptr, ob));
  PD_CUDA(cudaStreamSynchronize(st));
  return PD_OK;
}

// A serving batch: images of mixed sizes in one launch of
// k_predict_batch (one CTA per 32x8 tile of any image), captured in a CUDA graph
// that is replayed while the batch layout (sizes, masks) and the forest stay the
// same.  Inputs and outputs are the caller's host buffers, copied per image.
extern "C" int pd_predict_posterior_batch(pd_ctx *ctx, uint32_t n, const void *const *images,
                                          const uint32_t *widths, const uint32_t *heights,
                                          const uint8_t *const *masks, float *const *outs) {
  PD_CHECK(ctx && images && widths && heights && outs, PD_ERR_INVALID, "null argument");
  PD_CHECK(n >= 1, PD_ERR_INVALID, "empty batch");
  PD_CHECK(!ctx->tree_depth.empty(), PD_ERR_STATE, "empty forest");
  PD_CUDA(cudaSetDevice(ctx->device));
  if (ctx->tree_feature) {
    // a feature that reads the tree: the node-map steps of each image in turn
    for (uint32_t i = 0; i < n; i++) {
      PD_CHECK(images[i] && outs[i], PD_ERR_INVALID, "batch image %u: null buffer", i);
      PD_TRY(pd_predict_posterior(ctx, images[i], widths[i], heights[i], masks ? masks[i] : nullptr, outs[i]));
    }
    return PD_OK;
  }
  PD_TRY(upload_forest(ctx));
  const uint32_t K = (uint32_t)ctx->cfg.n_classes, nt = (uint32_t)ctx->tree_depth.size();
  const size_t px = (size_t)ctx->cfg.n_channels * img_size(ctx->cfg.img_type);
  auto up16 = [](uint64_t v) { return (v + 15) / 16 * 16; };
  std::vector<BatchImage> desc(n);
  std::vector<uint64_t> key{(uint64_t)n, ctx->forest_version};
  uint64_t ib = 0, mb = 0, ob = 0, tiles = 0;
  for (uint32_t i = 0; i < n; i++) {
    PD_CHECK(images[i] && outs[i] && widths[i] >= 1 && heights[i] >= 1 && widths[i] < 65536 && heights[i] < 65536,
             PD_ERR_INVALID, "batch image %u: null buffer or size %ux%u", i, widths[i], heights[i]);
    const uint64_t P_ = (uint64_t)widths[i] * heights[i];
    BatchImage &d = desc[i];
    d.w = widths[i];
    d.h = heights[i];
    d.tiles_x = (d.w + kPredX - 1) / kPredX;
    d.tile0 = (uint32_t)tiles;
    d.has_mask = masks && masks[i] ? 1u : 0u;
    d.pad = 0;
    d.img_off = ib;
    d.mask_off = mb;
    d.out_off = ob;
    ib += up16(P_ * px);
    if (d.has_mask) mb += up16(P_);
    ob += up16(P_ * K * 4);
    tiles += (uint64_t)d.tiles_x * ((d.h + kPredY - 1) / kPredY);
    key.push_back(d.w | ((uint64_t)d.h << 16) | ((uint64_t)d.has_mask << 32));
  }
  PD_CHECK(tiles < (1ull << 31), PD_ERR_UNSUPPORTED, "batch of %llu tiles", (unsigned long long)tiles);
  cudaStream_t st = ctx->stream;
  if (key != ctx->batch_key || !ctx->batch_graph) {
    // a new layout: buffers, descriptor table and the graph of the kernel
    if (ctx->batch_graph) cudaGraphExecDestroy(ctx->batch_graph);
    ctx->batch_graph = nullptr;
    ctx->batch_key.clear();
    PD_TRY(ctx->b_img.ensure(ib));
    PD_TRY(ctx->b_mask.ensure(std::max<uint64_t>(16, mb)));
    PD_TRY(ctx->b_out.ensure(ob));
    PD_TRY(ctx->b_desc.ensure(n * sizeof(BatchImage)));
    PD_CUDA(h2d(ctx, ctx->b_desc.ptr, desc.data(), n * sizeof(BatchImage)));
    PD_CUDA(cudaStreamSynchronize(st));
    const size_t smem = (size_t)nt * kPredThreads * 4;
    const int rc = dispatch_config(ctx->cfg, [&]<class P>() -> int {
      PD_TRY(ensure_forest_nodes<P>(ctx));
      PD_CUDA(cudaStreamSynchronize(st));
      const uint8_t *im = ctx->b_img.as<uint8_t>(), *mk = ctx->b_mask.as<uint8_t>();
      uint8_t *o = ctx->b_out.as<uint8_t>();
      const BatchImage *bd = ctx->b_desc.as<BatchImage>();
      uint32_t n_ = n, nt_ = nt, k_ = K;
      const void *nd = ctx->f_cand.ptr;
      const float *po = ctx->f_post.as<float>();
      const TreeMeta *me = ctx->f_meta.as<TreeMeta>();
      const uint32_t *mg = ctx->magic_tab.as<uint32_t>();
      void *args[] = {&im, &mk, &o, &bd, &n_, &nd, &po, &me, &nt_, &k_, &mg};
      const void *fn = nullptr;
      if (is_user_plugin(ctx)) {
        const RtcKernels *rk = nullptr;
        PD_TRY(rtc_kernels(ctx, &rk));
        PD_TRY(rtc_set_smem(ctx, rk->predict_batch, smem));
        fn = (const void *)rk->predict_batch;
      } else if constexpr (!P::kRtcOnly) {
        auto kern = ctx->forest_fast ? k_predict_batch<P, true> : k_predict_batch<P, false>;
        fn = (const void *)kern;
        PD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      }
      cudaGraph_t g = nullptr;
      PD_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const cudaError_t le = cudaLaunchKernel(fn, dim3((unsigned)tiles), dim3(kPredX, kPredY), args, smem, st);
      const cudaError_t ce = cudaStreamEndCapture(st, &g);
      PD_CUDA(le);
      PD_CUDA(ce);
      const cudaError_t ie = cudaGraphInstantiate(&ctx->batch_graph, g, 0);
      cudaGraphDestroy(g);
      PD_CUDA(ie);
      return PD_OK;
    });
    PD_TRY(rc);
    ctx->batch_key = key;
  }
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t P_ = (uint64_t)desc[i].w * desc[i].h;
    PD_CUDA(h2d(ctx, ctx->b_img.as<uint8_t>() + desc[i].img_off, images[i], P_ * px));
    if (desc[i].has_mask) PD_CUDA(h2d(ctx, ctx->b_mask.as<uint8_t>() + desc[i].mask_off, masks[i], P_));
  }
  PD_CUDA(cudaGraphLaunch(ctx->batch_graph, st));
  ctx->launches++;
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t P_ = (uint64_t)desc[i].w * desc[i].h;
    PD_CUDA(d2h(ctx, outs[i], ctx->b_out.as<uint8_t>() + desc[i].out_off, P_ * K * 4));
  }
  PD_CUDA(cudaStreamSynchronize(st));
  return PD_OK;
}

extern "C" int pd_predict_leaf(pd_ctx *ctx, uint32_t tree, const void *image, uint32_t width, uint32_t height,
                               const uint8_t *mask, int32_t *out) {
  PD_CHECK(ctx && image && out, PD_ERR_INVALID, "null argument");
  PD_CHECK(tree < ctx->tree_depth.size(), PD_ERR_INVALID, "tree %u not in the forest", tree);
  PD_CHECK(width >= 1 && height >= 1, PD_ERR_INVALID, "empty image");
  PD_CUDA(cudaSetDevice(ctx->device));
  PD_TRY(upload_forest(ctx));
  const size_t P_ = (size_t)width * height;
  const size_t ib = P_ * ctx->cfg.n_channels * img_size(ctx->cfg.img_type);
  PD_TRY(ctx->p_img.ensure(ib));
  PD_TRY(ctx->p_out.ensure(P_ * 4));
  if (mask) PD_TRY(ctx->p_mask.ensure(P_));
  cudaStream_t st = ctx->stream;
  PD_CUDA(h2d(ctx, ctx->p_img.ptr, image, ib));
  if (mask) PD_CUDA(h2d(ctx, ctx->p_mask.ptr, mask, P_));
  const size_t off = ctx->tree_off[tree];
  const uint32_t depth = ctx->tree_depth[tree];
  if (ctx->tree_feature) {
    PD_TRY(node_map_predict(ctx, 1, ctx->p_img.ptr, width, height, mask ? ctx->p_mask.as<uint8_t>() : nullptr, nullptr,
                            tree, ctx->p_out.as<int32_t>()));
    PD_CUDA(d2h(ctx, out, ctx->p_out.ptr, P_ * 4));
    PD_CUDA(cudaStreamSynchronize(st));
    return PD_OK;
  }
  PD_TRY(dispatch_config(ctx->cfg, [&]<class P>() {
    dim3 grid((width + kPredX - 1) / kPredX, (height + kPredY - 1) / kPredY, 1);
    PD_TRY(ensure_forest_nodes<P>(ctx));
    size_t rec = 0;
    PD_TRY(node_record<P>(ctx, &rec));
    if (is_user_plugin(ctx)) {
      const RtcKernels *rk = nullptr;
      PD_TRY(rtc_kernels(ctx, &rk));
      const uint8_t *im = ctx->p_img.as<uint8_t>(), *mk = mask ? ctx->p_mask.as<uint8_t>() : nullptr;
      uint32_t w_ = width, h_ = height, dp = depth;
      int32_t *o = ctx->p_out.as<int32_t>();
      const void *nd = ctx->f_cand.as<uint8_t>() + off * rec;
      const uint32_t *mg = ctx->magic_tab.as<uint32_t>();
      void *args[] = {&im, &w_, &h_, &mk, &o, &nd, &dp, &mg};
      return rtc_launch(ctx, rk->predict_leaf, grid, dim3(kPredX, kPredY), 0, args);
    }
    if constexpr (!P::kRtcOnly) {
      auto kern = ctx->forest_fast ? k_predict_leaf<P, true> : k_predict_leaf<P, false>;
      kern<<<grid, dim3(kPredX, kPredY), 0, st>>>(
          ctx->p_img.as<uint8_t>(), width, height, mask ? ctx->p_mask.as<uint8_t>() : nullptr,
          ctx->p_out.as<int32_t>(), ctx->f_cand.as<NodeRec<P>>() + off, depth, ctx->magic_tab.as<uint32_t>());
      PD_CUDA(cudaGetLastError());
    }
    return PD_OK;
  }));
  PD_CUDA(d2h(ctx, out, ctx->p_out.ptr, P_ * 4));
  PD_CUDA(cudaStreamSynchronize(st));
  return PD_OK;
}
