// Host orchestration of the training pass: CLTreeTrainer::train
// (cl_tree_trainer_impl.hpp:203-255) re-designed for one GPU with the whole
// training set resident in HBM.  Per depth: candidate table, histogram work
// list over all frontier nodes (one launch per histogram slice), best split on
// the device, finalize on the host (it is O(frontier)), device tree update,
// reassignment and stable regrouping of the active samples.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <vector>

#include "pd_ctx.cuh"
#include "pd_hist_grid.cuh"
#include "pd_rtc.cuh"
#include "pd_predict_kernels.cuh"
#include "pd_train_kernels.cuh"

namespace pd {

// Threshold rows padded to the next power of two above T, so the branch-free
// search needs no bounds test.
static uint32_t padded_rows(uint32_t T) {
  uint32_t p = 1;
  while (p < T + 1) p <<= 1;
  return p;
}

// Shared memory of a histogram launch: packed tile histogram, threshold table
// and, when the launch has fused-split items, the larger of the table and the
// fused scratch (gains + packed left totals) that overlays it.
static size_t hist_smem(const pd_ctx *ctx, uint32_t T, bool fused = true) {
  const size_t hist = (size_t)ctx->cfg.n_classes * (T + 1) * 32 * 4;  // rank T rows are never read
  const size_t thr = (size_t)padded_rows(T) * kTileF * feat_size(ctx->cfg.feat_type);
  const size_t scratch = (size_t)T * kTileF * 4 + (size_t)T * 32 * 4;
  return hist + (fused ? std::max(thr, scratch) : thr);
}

static DevSet devset(const pd_ctx *ctx) {
  DevSet d;
  d.magic = ctx->magic_tab.as<uint32_t>();
  d.pixels = ctx->pixels.as<uint8_t>();
  d.img_off = ctx->img_off.as<uint64_t>();
  d.img_wh = ctx->img_wh.as<uint32_t>();
  d.s_xy = ctx->s_xy.as<uint32_t>();
  d.s_img = ctx->s_img.as<uint32_t>();
  d.s_label = ctx->s_label.as<uint8_t>();
  const bool tf = ctx->tree_feature && ctx->nm_pixels;
  d.nodes = tf ? ctx->nm_map[ctx->nm_cur].as<int32_t>() : nullptr;
  d.map_off = tf ? ctx->nm_off.as<uint64_t>() : nullptr;
  d.tree_lc = ctx->t_lc.as<int32_t>();
  d.tree_post = ctx->t_post.as<float>();
  d.n_classes = (uint32_t)ctx->cfg.n_classes;
  d.tree_level = ctx->nm_level;
  d.tree_nodes = ctx->nm_nodes;
  return d;
}

int ensure_log2_table(pd_ctx *ctx, uint64_t n) {
  if (n <= ctx->log2_len) return PD_OK;
  PD_CHECK(n <= (1ull << 32), PD_ERR_UNSUPPORTED, "log2 table of %llu entries", (unsigned long long)n);
  PD_TRY(ctx->log2_tab.ensure(n * sizeof(double)));
  const DD inv = dd_inv_ln2();
  k_log2_table<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>(ctx->log2_tab.as<double>(), n, inv);
  PD_CUDA(cudaGetLastError());
  const uint32_t m = (uint32_t)std::min<uint64_t>(n, kXlog2Len);
  PD_TRY(ctx->xlog2_tab.ensure((size_t)kXlog2Len * sizeof(float)));
  k_xlog2_table<<<(m + 255) / 256, 256, 0, ctx->stream>>>(ctx->xlog2_tab.as<float>(), ctx->log2_tab.as<double>(), m);
  PD_CUDA(cudaGetLastError());
  ctx->log2_len = n;
  return PD_OK;
}

int map_training_pixels(pd_ctx *ctx, uint64_t bytes) {
  return dispatch_config(ctx->cfg, [&]<class P>() -> int {
    if constexpr (P::kTrainMapsZero) {
      static_assert(sizeof(typename P::img_t) == 2, "zero mapping of 16-bit images");
      const uint64_t n = is_user_plugin(ctx) ? 0 : bytes / 2;  // a user feature reads the images as given
      if (n) {
        k_zero_to_background<<<4 * 152, 256, 0, ctx->stream>>>(ctx->pixels.as<uint16_t>(), n);
        PD_CUDA(cudaGetLastError());
      }
    }
    return PD_OK;
  });
}

int build_sample_records(pd_ctx *ctx, uint64_t S) {
  PD_TRY(ctx->s_rec.ensure(S * sizeof(SampleRec) + sizeof(SampleRec)));
  if (!S) return PD_OK;
  return dispatch_config(ctx->cfg, [&]<class P>() -> int {
    const dim3 grid((unsigned)((S + 255) / 256));
    if (is_user_plugin(ctx)) {
      const RtcKernels *rk = nullptr;
      PD_TRY(rtc_kernels(ctx, &rk));
      DevSet ds = devset(ctx);
      uint32_t n = (uint32_t)S;
      SampleRec *rec = ctx->s_rec.as<SampleRec>();
      void *args[] = {&ds, &n, &rec};
      return rtc_launch(ctx, rk->build_rec, grid, dim3(256), 0, args);
    }
    if constexpr (!P::kRtcOnly) {
      k_build_rec<P><<<grid, 256, 0, ctx->stream>>>(devset(ctx), (uint32_t)S, ctx->s_rec.as<SampleRec>());
      PD_CUDA(cudaGetLastError());
    }
    return PD_OK;
  });
}

int init_tables(pd_ctx *ctx) {
  PD_TRY(ctx->magic_tab.ensure(65536 * 4));
  k_magic_table<<<256, 256, 0, ctx->stream>>>(ctx->magic_tab.as<uint32_t>());
  PD_CUDA(cudaGetLastError());
  return PD_OK;
}

static CandBounds bounds(const pd_train_params *p, int D, uint32_t f_base = 0) {
  CandBounds b;
  memset(&b, 0, sizeof(b));
  b.f_base = f_base;
  for (int d = 0; d < D; d++) {
    b.low[d] = p->feat_low[d];
    b.up[d] = p->feat_up[d];
  }
  b.thr_lo = p->thr_low;
  b.thr_hi = p->thr_up;
  return b;
}

static int check_params(const pd_ctx *ctx, const pd_train_params *p) {
  PD_CHECK(p, PD_ERR_INVALID, "null params");
  PD_CHECK(p->n_features >= 1 && p->n_thresholds >= 1, PD_ERR_INVALID, "n_features and n_thresholds must be >= 1");
  PD_CHECK(p->n_thresholds <= PD_MAX_THRESHOLDS, PD_ERR_UNSUPPORTED, "n_thresholds %u > %d",
           p->n_thresholds, PD_MAX_THRESHOLDS);
  const size_t smem = hist_smem(ctx, p->n_thresholds);
  PD_CHECK(smem <= 227 * 1024, PD_ERR_UNSUPPORTED,
           "nClasses*nThresholds too large for one shared-memory histogram tile (%zu bytes)", smem);
  return PD_OK;
}

// Scratch sized for `slots` frontier nodes.
static int ensure_slice(pd_ctx *ctx, const pd_train_params *p, uint32_t slots) {
  const uint64_t F = p->n_features, T = p->n_thresholds, K = ctx->cfg.n_classes;
  const size_t fs = feat_size(ctx->cfg.feat_type);
  PD_TRY(ctx->cand_feat.ensure(slots * ctx->cfg.feat_dim * F * fs));
  PD_TRY(ctx->cand_thr.ensure(slots * T * F * fs));
  PD_TRY(ctx->cand_perm.ensure(slots * T * F));
  PD_TRY(ctx->cand_ord.ensure(slots * F * 4));
  PD_TRY(ctx->hist.ensure(slots * K * T * F * 4));
  PD_TRY(ctx->g32.ensure(slots * T * F * 4));
  PD_TRY(ctx->split_out.ensure(slots * sizeof(SplitOut)));
  PD_TRY(ctx->split_par.ensure(slots * (ctx->cfg.feat_dim + 1) * fs));
  PD_TRY(ctx->split_cl.ensure(slots * K * 4));
  PD_TRY(ctx->recheck.ensure(sizeof(unsigned long long) + slots * K * 4 + slots * 4));
  return PD_OK;
}

static uint64_t slot_bytes(const pd_ctx *ctx, const pd_train_params *p) {
  const uint64_t F = p->n_features, T = p->n_thresholds, K = ctx->cfg.n_classes;
  const uint64_t fs = feat_size(ctx->cfg.feat_type);
  return K * T * F * 4 + T * F * 4 + T * F * (fs + 1) + ctx->cfg.feat_dim * F * fs + F * 4;
}

// ----------------------------------------------------------- launches ----
// Candidate tables of n slots.  With `ordered` (and F <= kOrderMaxF) the
// columns of each slot are sorted by first-probe offset and *ord_out receives
// the column -> original index map; otherwise column f is candidate f and
// *ord_out is null.
template <class P>
static int launch_candidates(pd_ctx *ctx, const pd_train_params *p, uint32_t tree, const int32_t *d_nodes,
                             uint32_t n, bool ordered = false, const uint32_t **ord_out = nullptr,
                             const PropSrc *prop = nullptr, uint32_t f_base = 0) {
  using FeatT = typename P::feat_t;
  const uint32_t F = p->n_features;
  const uint64_t total = (uint64_t)n * F;
  const uint32_t *ord = nullptr;
  if (ord_out) *ord_out = nullptr;
  if (!total) return PD_OK;
  const CandBounds b = bounds(p, P::kFeatDim, f_base);
  if (ordered && F <= kOrderMaxF) {
    uint32_t N = 1;
    while (N < F) N <<= 1;
    const size_t osmem = (size_t)N * 8;
    if (is_user_plugin(ctx)) {
      const RtcKernels *rk = nullptr;
      PD_TRY(rtc_kernels(ctx, &rk));
      PD_TRY(rtc_set_smem(ctx, rk->cand_order, osmem));
      uint32_t tr = tree, f_ = F;
      CandBounds bb = b;
      uint32_t *o = ctx->cand_ord.as<uint32_t>();
      PropSrc ps = prop ? *prop : PropSrc{};
      void *args[] = {&d_nodes, &tr, &f_, &bb, &o, &ps};
      PD_TRY(rtc_launch(ctx, rk->cand_order, dim3(n), dim3(kOrderThreads), osmem, args));
    } else if constexpr (!P::kRtcOnly) {
      PD_CUDA(cudaFuncSetAttribute(k_cand_order<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)osmem));
      k_cand_order<P><<<n, kOrderThreads, osmem, ctx->stream>>>(d_nodes, tree, F, b, ctx->cand_ord.as<uint32_t>(),
                                                                prop ? *prop : PropSrc{});
      PD_CUDA(cudaGetLastError());
      ctx->launches++;
    }
    ord = ctx->cand_ord.as<uint32_t>();
  }
  // draws lie in [lo, hi] (no narrowing wrap) and their offsets fit 24 bits:
  // value and index sort as one word
  const int64_t span = (int64_t)p->thr_up - p->thr_low;
  const bool packed = span >= 0 && span < (1 << 24) && (sizeof(FeatT) == 4 || span <= 32767);
  const unsigned grid = (unsigned)((total + kCandThreads - 1) / kCandThreads);
  const uint32_t T = p->n_thresholds;
  if (packed && T <= 64 && ctx->cand_regs) {
    // keys sorted in registers
    auto rk = T <= 16 ? k_candidates_reg<FeatT, 16> : (T <= 32 ? k_candidates_reg<FeatT, 32> : k_candidates_reg<FeatT, 64>);
    rk<<<grid, kCandThreads, 0, ctx->stream>>>(d_nodes, n, tree, F, T, P::kFeatDim, b, ord, ctx->cand_feat.as<FeatT>(),
                                               ctx->cand_thr.as<FeatT>(), ctx->cand_perm.as<uint8_t>(),
                                               prop ? *prop : PropSrc{});
    PD_CUDA(cudaGetLastError());
    ctx->launches++;
    if (ord_out) *ord_out = ord;
    return PD_OK;
  }
  const size_t smem = (size_t)p->n_thresholds * kCandThreads * (packed ? 4 : sizeof(FeatT) + 1);
  auto kern = packed ? k_candidates<FeatT, true> : k_candidates<FeatT, false>;
  PD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, kCandThreads, smem, ctx->stream>>>(
      d_nodes, n, tree, F, p->n_thresholds, P::kFeatDim, b, ord, ctx->cand_feat.as<FeatT>(),
      ctx->cand_thr.as<FeatT>(), ctx->cand_perm.as<uint8_t>(), prop ? *prop : PropSrc{});
  PD_CUDA(cudaGetLastError());
  ctx->launches++;
  if (ord_out) *ord_out = ord;
  return PD_OK;
}

// Builds the work list of slots [0, n) whose samples are act[off[i], off[i+1])
// and launches the histogram kernel.
template <class P>
// With `split_slots` non-null, nodes whose samples fit one work item get their
// split fused into the histogram kernel (multi = 2, rows never written) and the
// other slots are returned for the split kernels.
static int launch_hist(pd_ctx *ctx, const pd_train_params *p, const uint64_t *off, uint32_t n,
                       const SampleRec *d_rec, uint64_t *n_items_out, cudaEvent_t ev_before = nullptr,
                       cudaEvent_t ev_after = nullptr, std::vector<uint32_t> *split_slots = nullptr,
                       const uint32_t *d_class_tot = nullptr, const uint32_t *d_ord = nullptr) {
  using FeatT = typename P::feat_t;
  const uint32_t F = p->n_features, T = p->n_thresholds, K = ctx->cfg.n_classes;
  const uint32_t tiles = (F + kTileF - 1) / kTileF;
  PD_CHECK(ctx->chunk >= 1 && ctx->chunk <= kMaxChunk, PD_ERR_INVALID, "chunk %u outside [1,%u]", ctx->chunk, kMaxChunk);
  // the work list is written straight into pinned staging (sized by a first
  // pass); for a persistent launch it is ordered largest item first (by the
  // power of two of its sample count, stable), so the last items to start are
  // the short ones
  const bool persist = ctx->persist;
  auto bucket = [](uint64_t cnt) { return cnt ? 63 - __builtin_clzll(cnt) : 0; };  // floor(log2), <= 15
  uint64_t n_items = 0, pos[17] = {};
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t cnt = off[i + 1] - off[i];
    const uint64_t chunks = (cnt + ctx->chunk - 1) / ctx->chunk;
    n_items += chunks * tiles;
    for (uint64_t c = 0; persist && c < chunks; c++)
      pos[bucket(std::min<uint64_t>(cnt - c * ctx->chunk, ctx->chunk))] += tiles;
  }
  uint64_t acc = 0;
  for (int b = 15; persist && b >= 0; b--) {  // start of each bucket, largest first
    const uint64_t c = pos[b];
    pos[b] = acc;
    acc += c;
  }
  PD_TRY(ctx->h_items.ensure(std::max<uint64_t>(1, n_items) * sizeof(WorkItem)));
  WorkItem *items = ctx->h_items.as<WorkItem>();
  uint64_t ni = 0;
  std::vector<uint32_t> zero;
  for (uint32_t i = 0; i < n; i++) {
    const uint64_t b = off[i], e = off[i + 1];
    const uint64_t cnt = e - b;
    if (!cnt) {
      zero.push_back(i);
      if (split_slots) split_slots->push_back(i);
      continue;
    }
    const uint64_t chunks = (cnt + ctx->chunk - 1) / ctx->chunk;
    if (chunks > 1) zero.push_back(i);
    const bool fused = split_slots && chunks == 1 && cnt <= ctx->fuse_max;
    if (split_slots && !fused) split_slots->push_back(i);
    for (uint64_t c = 0; c < chunks; c++) {
      const uint32_t cb = (uint32_t)(b + c * ctx->chunk);
      const uint32_t ce = (uint32_t)std::min<uint64_t>(e, b + (c + 1) * ctx->chunk);
      for (uint32_t t = 0; t < tiles; t++) {
        WorkItem w;
        memset(&w, 0, sizeof(w));
        w.slot = i;
        w.tile = t;
        w.begin = cb;
        w.end = ce;
        w.multi = chunks > 1 ? 1u : (fused ? 2u : 0u);
        items[persist ? pos[bucket(ce - cb)]++ : ni] = w;
        ni++;
      }
    }
  }
  *n_items_out = ni;
  PD_TRY(ctx->items.ensure(std::max<size_t>(1, ni) * sizeof(WorkItem)));
  PD_TRY(ctx->zero_slots.ensure(std::max<size_t>(1, zero.size()) * 4));
  const uint64_t per_slot = (uint64_t)K * T * F;
  if (!zero.empty()) {
    PD_CUDA(h2d(ctx, ctx->zero_slots.ptr, zero.data(), zero.size() * 4));
    k_zero_slots<<<1216, 256, 0, ctx->stream>>>(ctx->hist.as<uint32_t>(), ctx->zero_slots.as<uint32_t>(),
                                                (uint32_t)zero.size(), per_slot);
    PD_CUDA(cudaGetLastError());
  }
  if (!zero.empty()) ctx->launches++;
  if (!ni) {
    if (ev_before) PD_CUDA(cudaEventRecord(ev_before, ctx->stream));
    if (ev_after) PD_CUDA(cudaEventRecord(ev_after, ctx->stream));
    return PD_OK;
  }
  PD_CUDA(h2d(ctx, ctx->items.ptr, items, ni * sizeof(WorkItem)));
  bool any_fused = false;
  for (uint64_t k = 0; k < ni; k++) any_fused |= items[k].multi == 2;
  const size_t smem = hist_smem(ctx, T, any_fused);
  FusedSplit fs;
  memset(&fs, 0, sizeof(fs));
  if (split_slots) {
    PD_TRY(ctx->fused_scratch.ensure((size_t)n * 4 + (size_t)n * tiles * (sizeof(SplitPart) + 4 * K) + 64));
    fs.done = ctx->fused_scratch.as<unsigned>();
    fs.part_best = reinterpret_cast<SplitPart *>(ctx->fused_scratch.as<uint8_t>() + ((size_t)n * 4 + 15) / 16 * 16);
    fs.part_cl = reinterpret_cast<uint32_t *>(fs.part_best + (size_t)n * tiles);
    PD_CUDA(cudaMemsetAsync(fs.done, 0, (size_t)n * 4, ctx->stream));
    fs.class_tot = d_class_tot;
    fs.perm = ctx->cand_perm.as<uint8_t>();
    fs.L = ctx->log2_tab.as<double>();
    fs.L_len = ctx->log2_len;
    fs.xlog2 = ctx->xlog2_tab.as<float>();
    PD_TRY(ctx->parent.ensure((size_t)n * sizeof(double)));
    k_parent_term<<<(n + 127) / 128, 128, 0, ctx->stream>>>(d_class_tot, n, K, fs.L, fs.L_len,
                                                            ctx->parent.as<double>());
    PD_CUDA(cudaGetLastError());
    ctx->launches++;
    fs.parent = ctx->parent.as<double>();
    fs.tiles = tiles;
    fs.out = ctx->split_out.as<SplitOut>();
    fs.out_cl = ctx->split_cl.as<uint32_t>();
    fs.rechecked = ctx->recheck.as<unsigned long long>();
    fs.ord = d_ord;
  }
  HistGrid g;
  g.ds = devset(ctx);
  g.rec = d_rec;
  g.items = ctx->items.as<WorkItem>();
  g.n_items = ni;
  g.cand_feat = ctx->cand_feat.ptr;
  g.cand_thr = ctx->cand_thr.ptr;
  g.hist = ctx->hist.as<uint32_t>();
  g.F = F;
  g.T = T;
  g.K = K;
  g.TP = padded_rows(T);
  g.smem = smem;
  g.fs = fs;
  g.ev_before = ev_before;
  g.queue = nullptr;
  if (persist && ni < 0x7fffffffull) {
    PD_TRY(ctx->hist_queue.ensure(16));
    g.queue = ctx->hist_queue.as<unsigned>();
  }
  if constexpr (P::kRtcOnly) {
    PD_TRY(launch_hist_grid_rtc(ctx, g));
  } else {
    PD_TRY(launch_hist_grid<P>(ctx, g));
  }
  if (ev_after) PD_CUDA(cudaEventRecord(ev_after, ctx->stream));
  return PD_OK;
}

// Algorithmic HBM bytes of one histogram launch: the training-set images read
// once, 16 bytes per active sample (its SampleRec), the
// candidate table of every slot read once, and the K*T*F uint32 histogram
// written once for each slot whose split is not fused into the kernel.
static uint64_t hist_algorithmic_bytes(const pd_ctx *ctx, const pd_train_params *p, uint64_t n_samples,
                                       uint32_t n_slots, uint32_t n_written, uint64_t image_bytes) {
  const uint64_t F = p->n_features, T = p->n_thresholds, K = ctx->cfg.n_classes;
  const uint64_t fs = feat_size(ctx->cfg.feat_type);
  return image_bytes + (uint64_t)sizeof(SampleRec) * n_samples + (uint64_t)n_slots * (T * F * fs + ctx->cfg.feat_dim * F * fs) +
         (uint64_t)n_written * K * T * F * 4;
}

// Split kernels over n slots: slots[0..n) of the slice, or 0..n-1 when
// d_slot_list is null.
template <bool CUM>
static int launch_split(pd_ctx *ctx, const pd_train_params *p, uint32_t n, const uint32_t *d_hist,
                        const uint8_t *d_perm, const uint32_t *d_class_tot,
                        const uint32_t *d_slot_list = nullptr, uint32_t slice_slots = 0,
                        const uint32_t *d_ord = nullptr) {
  if (!n) return PD_OK;
  const uint32_t all = d_slot_list ? slice_slots : n;
  const uint32_t F = p->n_features;
  // Parts per node: enough CTAs to fill the GPU when the frontier is small.
  const uint32_t max_parts = (F + kSplitCols - 1) / kSplitCols;
  uint32_t parts = std::min<uint32_t>(max_parts, std::max<uint32_t>(1, (4 * 152 + n - 1) / n));
  uint32_t cols = (F + parts - 1) / parts;
  cols = (cols + 31) / 32 * 32;
  parts = (F + cols - 1) / cols;
  PD_TRY(ctx->split_scratch.ensure((size_t)all * 8 + (size_t)all * parts * sizeof(SplitPart) + 16));
  unsigned *node_max = ctx->split_scratch.as<unsigned>();
  PD_CUDA(cudaMemsetAsync(node_max, 0, (size_t)all * 8, ctx->stream));
  SplitArgs a;
  a.hist = d_hist;
  a.perm = d_perm;
  a.class_tot = d_class_tot;
  a.g32 = ctx->g32.as<float>();
  a.L = ctx->log2_tab.as<double>();
  a.L_len = ctx->log2_len;
  a.F = F;
  a.T = p->n_thresholds;
  a.K = ctx->cfg.n_classes;
  a.delta = recheck_delta(ctx->cfg.n_classes);
  a.cols = cols;
  a.parts = parts;
  a.node_max = node_max;
  a.done = node_max + all;
  a.part_best = reinterpret_cast<SplitPart *>(ctx->split_scratch.as<uint8_t>() + (size_t)all * 8);
  a.slot_list = d_slot_list;
  a.ord = d_ord;
  a.out = ctx->split_out.as<SplitOut>();
  a.out_cl = ctx->split_cl.as<uint32_t>();
  a.rechecked = ctx->recheck.as<unsigned long long>();
  const dim3 grid(parts, n);
  auto run = [&]<int KM>() -> int {
    k_split_g32<KM, CUM><<<grid, kSplitCols, 0, ctx->stream>>>(a);
    k_split_pick<KM, CUM><<<grid, kSplitCols, 0, ctx->stream>>>(a);
    PD_CUDA(cudaGetLastError());
    ctx->launches += 2;
    return PD_OK;
  };
  // class loops are unrolled to KM >= K; the common class counts get exact KM
  const int K = ctx->cfg.n_classes;
  if (K <= 3) return run.template operator()<3>();
  if (K <= 4) return run.template operator()<4>();
  if (K <= 8) return run.template operator()<8>();
  if (K <= 9) return run.template operator()<9>();
  if (K <= 16) return run.template operator()<16>();
  if (K <= 21) return run.template operator()<21>();
  if (K <= 32) return run.template operator()<32>();
  return run.template operator()<64>();
}

static float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// ------------------------------------------------------------- one tree ----
// A rank of candidate-sharded training: it evaluates candidates
// [f_base, f_base + params->n_features) of F_total, and `exchange` turns the
// ranks' best splits of a slice into the global ones.
struct Shard {
  uint32_t f_base, F_total;
  pd_exchange_fn exchange;
  void *user;
};

// Order key of a double (the device's gain_order_key).
static int64_t gain_key_host(double g) {
  int64_t b;
  memcpy(&b, &g, 8);
  return b < 0 ? (INT64_MIN - b - 1) : b;
}

// With `prop`, candidates f < n_prop of every node come from the proposal
// network (learned proposals); with ctx->collect_records, one pd_record per
// split node is kept; with `shard`, this rank's candidates are a range of the
// node's and each slice's winners are exchanged with the other ranks.
// One level of the training images' node map (k_node_map_step over every
// pixel, labelled pixels advancing) with the device tree being trained.
static int launch_node_map_step(pd_ctx *ctx, const int32_t *in, int32_t *out) {
  const RtcKernels *rk = nullptr;
  PD_TRY(rtc_kernels(ctx, &rk));
  NodeMapStep a;
  a.pixels = ctx->pixels.as<uint8_t>();
  a.img_off = ctx->img_off.as<uint64_t>();
  a.img_wh = ctx->img_wh.as<uint32_t>();
  a.map_off = ctx->nm_off.as<uint64_t>();
  a.n_images = ctx->n_images;
  a.n_pix = ctx->nm_pixels;
  a.mask = ctx->nm_label.as<uint8_t>();
  a.map_in = in;
  a.map_out = out;
  a.lc = ctx->t_lc.as<int32_t>();
  a.feat = ctx->t_feat.ptr;
  a.thr = ctx->t_thr.ptr;
  a.post = ctx->t_post.as<float>();
  a.n_classes = (uint32_t)ctx->cfg.n_classes;
  a.level = ctx->nm_level;
  a.n_nodes = ctx->nm_nodes;
  a.magic = ctx->magic_tab.as<uint32_t>();
  void *args[] = {&a};
  return rtc_launch(ctx, rk->node_map_step, dim3((unsigned)((a.n_pix + 255) / 256)), dim3(256), 0, args);
}

template <class P>
static int train_tree_impl(pd_ctx *ctx, const pd_train_params *p, uint32_t tree_id, uint32_t end_depth,
                           const float *root_prior, int32_t *lc, typename P::feat_t *feats,
                           typename P::feat_t *thrs, float *posts, pd_proposer *prop = nullptr,
                           uint32_t n_prop = 0, const Shard *shard = nullptr) {
  using FeatT = typename P::feat_t;
  constexpr int D = P::kFeatDim;
  const auto t_start = std::chrono::steady_clock::now();
  const uint32_t F = p->n_features, K = ctx->cfg.n_classes;
  const uint64_t n_nodes = (1ull << end_depth) - 1ull;
  const uint64_t S = ctx->n_samples;
  cudaStream_t st = ctx->stream;
  pd_train_stats stats;
  memset(&stats, 0, sizeof(stats));
  const uint64_t h2d0 = ctx->bytes_h2d, d2h0 = ctx->bytes_d2h, launches0 = ctx->launches;
  const uint64_t image_bytes = ctx->pixels_bytes;
  ctx->records.clear();

  PD_TRY(ensure_log2_table(ctx, S + 2));
  PD_TRY(ctx->t_lc.ensure(n_nodes * 4));
  PD_TRY(ctx->t_feat.ensure(n_nodes * D * sizeof(FeatT)));
  PD_TRY(ctx->t_thr.ensure(n_nodes * sizeof(FeatT)));
  PD_TRY(ctx->t_post.ensure(n_nodes * K * 4));
  memcpy(posts, root_prior, sizeof(float) * K);
  // The tree as the caller holds it goes to the device (init:33-50).
  PD_CUDA(h2d(ctx, ctx->t_lc.ptr, lc, n_nodes * 4));
  PD_CUDA(h2d(ctx, ctx->t_feat.ptr, feats, n_nodes * D * sizeof(FeatT)));
  PD_CUDA(h2d(ctx, ctx->t_thr.ptr, thrs, n_nodes * sizeof(FeatT)));
  PD_CUDA(h2d(ctx, ctx->t_post.ptr, posts, n_nodes * K * 4));

  PD_TRY(ctx->snode.ensure(S * 4 + 4));
  for (int b = 0; b < 2; b++) {
    PD_TRY(ctx->act[b].ensure(S * 4 + 4));
    PD_TRY(ctx->act_slot[b].ensure(S * 4 + 4));
    PD_TRY(ctx->act_rec[b].ensure(S * sizeof(SampleRec) + sizeof(SampleRec)));
  }
  PD_TRY(ctx->flags.ensure(S + 16));
  PD_TRY(ctx->scan_blocks.ensure((S / kScanItems + 2) * 8 + 16));
  PD_TRY(ctx->scatter_err.ensure(16));
  PD_CUDA(cudaMemsetAsync(ctx->snode.ptr, 0, S * 4, st));
  if (ctx->tree_feature) {
    // every pixel starts at the root (traverse_ts.hpp:146-163 fills the node image with 0)
    PD_CHECK(ctx->nm_pixels, PD_ERR_STATE, "the training set was uploaded before the plugin was compiled");
    ctx->nm_cur = 0;
    ctx->nm_nodes = (int32_t)n_nodes;
    PD_CUDA(cudaMemsetAsync(ctx->nm_map[0].ptr, 0, ctx->nm_pixels * 4, st));
  }
  if (S) {
    k_iota<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(ctx->act[0].as<uint32_t>(), ctx->act_slot[0].as<uint32_t>(), (uint32_t)S);
    k_gather_rec<<<(unsigned)((S + 255) / 256), 256, 0, st>>>(ctx->act[0].as<uint32_t>(), (uint32_t)S,
                                                               ctx->s_rec.as<SampleRec>(), ctx->act_rec[0].as<SampleRec>());
    ctx->launches += 2;
  }
  PD_CUDA(cudaGetLastError());

  std::vector<uint32_t> node_tot(n_nodes, 0u), class_tot(n_nodes * K, 0u);
  node_tot[0] = (uint32_t)S;
  std::vector<int32_t> frontier{0};
  std::vector<uint64_t> cur_off{0, S};
  int cur = 0;
  uint64_t n_act = S;
  // slices are sized for all F_total candidates when sharded, so every rank cuts the same slices
  pd_train_params p_all = *p;
  if (shard) p_all.n_features = shard->F_total;
  const uint64_t per_slot = slot_bytes(ctx, &p_all);
  const uint32_t max_slots = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(ctx->hist_budget / per_slot, 1u << 30));
  DevBuf d_nodes, d_ctot, d_next, d_split_list;
  std::vector<SplitOut> h_out;
  std::vector<uint32_t> h_cl;
  std::vector<FeatT> h_par;
  std::vector<uint32_t> cl(K), cr(K);
  cudaEvent_t *ev = ctx->ev;

  for (uint32_t depth = 1; depth < end_depth; depth++) {
    if (depth == 1) {
      for (uint32_t l = 0; l < K; l++) class_tot[l] = ctx->root_class_tot[l];
    }
    ctx->nm_level = (int32_t)depth - 1;  // the node map's level: the frontier's
    const uint32_t nf = (uint32_t)frontier.size();
    if (nf == 0) break;
    for (uint32_t i = 0; i < nf; i++) stats.evals += (uint64_t)node_tot[frontier[i]] * F;
    stats.nodes_trained += nf;
    const uint32_t cap = std::min(nf, max_slots);
    PD_TRY(ensure_slice(ctx, p, cap));
    PD_TRY(d_nodes.ensure((size_t)cap * 4));
    PD_TRY(d_ctot.ensure((size_t)cap * K * 4));
    PD_TRY(d_split_list.ensure((size_t)cap * 4));
    std::vector<uint8_t> split_now(nf, 0);

    for (uint32_t s0 = 0; s0 < nf; s0 += cap) {
      const uint32_t ns = std::min(cap, nf - s0);
      std::vector<uint32_t> ctot((size_t)ns * K);
      for (uint32_t i = 0; i < ns; i++)
        memcpy(&ctot[(size_t)i * K], &class_tot[(size_t)frontier[s0 + i] * K], K * 4);
      PD_CUDA(h2d(ctx, d_nodes.ptr, &frontier[s0], (size_t)ns * 4));
      PD_CUDA(h2d(ctx, d_ctot.ptr, ctot.data(), (size_t)ns * K * 4));
      PD_CUDA(cudaMemsetAsync(ctx->recheck.ptr, 0, sizeof(unsigned long long), st));
      std::vector<uint64_t> off(cur_off.begin() + s0, cur_off.begin() + s0 + ns + 1);
      PD_CUDA(cudaEventRecord(ev[0], st));
      const uint32_t *d_ord = nullptr;
      if (prop) {
        // the network's mixture for every node of the slice, then the table drawn from it
        PropSrc src;
        PD_TRY(proposer_infer(prop, d_ctot.as<uint32_t>(), ns, depth, n_prop, &src));
        PD_TRY(launch_candidates<P>(ctx, p, tree_id, d_nodes.as<int32_t>(), ns, ctx->cand_order, &d_ord, &src));
      } else {
        PD_TRY(launch_candidates<P>(ctx, p, tree_id, d_nodes.as<int32_t>(), ns, ctx->cand_order, &d_ord, nullptr,
                                    shard ? shard->f_base : 0u));
      }
      PD_CUDA(cudaEventRecord(ev[1], st));
      uint64_t n_items = 0;
      std::vector<uint32_t> split_slots;
      PD_TRY(launch_hist<P>(ctx, p, off.data(), ns, ctx->act_rec[cur].as<SampleRec>(), &n_items, ev[6], ev[2],
                            &split_slots, d_ctot.as<uint32_t>(), d_ord));
      stats.hist_launches++;
      stats.hist_bytes += hist_algorithmic_bytes(ctx, p, off.back() - off.front(), ns, (uint32_t)split_slots.size(),
                                                 image_bytes);
      if (!split_slots.empty())
        PD_CUDA(h2d(ctx, d_split_list.ptr, split_slots.data(), split_slots.size() * 4));
      PD_TRY(launch_split<false>(ctx, p, (uint32_t)split_slots.size(), ctx->hist.as<uint32_t>(),
                                 ctx->cand_perm.as<uint8_t>(), d_ctot.as<uint32_t>(), d_split_list.as<uint32_t>(),
                                 ns, d_ord));
      // the winners' feature values and thresholds, from the candidate tables
      k_split_params<FeatT><<<(ns + 127) / 128, 128, 0, st>>>(
          ctx->split_out.as<SplitOut>(), ns, ctx->cand_feat.as<FeatT>(), ctx->cand_thr.as<FeatT>(),
          ctx->cand_perm.as<uint8_t>(), p->n_features, p->n_thresholds, D, ctx->split_par.as<FeatT>());
      PD_CUDA(cudaGetLastError());
      ctx->launches++;
      PD_CUDA(cudaEventRecord(ev[3], st));
      h_out.resize(ns);
      h_cl.resize((size_t)ns * K);
      h_par.resize((size_t)ns * (D + 1));
      unsigned long long rechecked = 0;
      PD_CUDA(d2h(ctx, h_out.data(), ctx->split_out.ptr, ns * sizeof(SplitOut)));
      PD_CUDA(d2h(ctx, h_cl.data(), ctx->split_cl.ptr, (size_t)ns * K * 4));
      PD_CUDA(d2h(ctx, h_par.data(), ctx->split_par.ptr, (size_t)ns * (D + 1) * sizeof(FeatT)));
      PD_CUDA(d2h(ctx, &rechecked, ctx->recheck.ptr, 8));
      PD_CUDA(cudaStreamSynchronize(st));
      stats.ms_candidates += elapsed(ev[0], ev[1]);
      stats.ms_hist += elapsed(ev[6], ev[2]);
      stats.ms_split += elapsed(ev[2], ev[3]);
      stats.split_rechecked += rechecked;

      if (shard) {
        // the ranks' best splits -> the global ones: largest exact gain, ties to the lowest t * F + f
        std::vector<int64_t> key(ns), idx(ns);
        for (uint32_t i = 0; i < ns; i++) {
          const SplitOut &o = h_out[i];
          key[i] = o.t < 0 ? INT64_MIN : gain_key_host(o.gain);
          idx[i] = o.t < 0 ? -1 : (int64_t)o.t * shard->F_total + (int64_t)(shard->f_base + (uint32_t)o.f);
          if (o.t < 0) memset(&h_cl[(size_t)i * K], 0, K * 4);
        }
        PD_CHECK(shard->exchange(shard->user, ns, K, key.data(), idx.data(), h_cl.data()) == 0, PD_ERR_STATE,
                 "the exchange of the ranks' best splits failed at depth %u", depth);
        for (uint32_t i = 0; i < ns; i++) {
          SplitOut &o = h_out[i];
          if (idx[i] < 0) {
            o.t = -1;
            continue;
          }
          const uint32_t t_g = (uint32_t)(idx[i] / shard->F_total), f_g = (uint32_t)(idx[i] % shard->F_total);
          const bool mine = o.t >= 0 && (uint32_t)o.t == t_g && shard->f_base + (uint32_t)o.f == f_g;
          o.t = (int32_t)t_g;
          o.gain = 0.0;
          if (!mine) {
            // the winner lives on another rank: its values from its seeds (hist_update.cl:62-184)
            const uint32_t node = (uint32_t)frontier[s0 + i];
            FeatT fv[PD_MAX_FEAT_DIM];
            candidate_feature<FeatT>(tree_id, node, f_g, D, p->feat_low, p->feat_up, fv);
            for (int d = 0; d < D; d++) h_par[(size_t)i * (D + 1) + d] = fv[d];
            h_par[(size_t)i * (D + 1) + D] = candidate_threshold<FeatT>(tree_id, node, f_g, t_g, p->thr_low, p->thr_up);
          }
        }
      }

      // finalize (learn_best_featthr.hpp:117-243)
      for (uint32_t i = 0; i < ns; i++) {
        const SplitOut &o = h_out[i];
        if (o.t < 0) continue;
        const uint32_t n = (uint32_t)frontier[s0 + i];
        uint32_t lsum = 0, rsum = 0;
        for (uint32_t l = 0; l < K; l++) {
          cl[l] = h_cl[(size_t)i * K + l];
          cr[l] = class_tot[(size_t)n * K + l] - cl[l];
          lsum += cl[l];
          rsum += cr[l];
        }
        if (!lsum || !rsum) continue;
        const uint64_t L = 2ull * n + 1, R = 2ull * n + 2;
        node_tot[L] = lsum;
        node_tot[R] = rsum;
        for (uint32_t l = 0; l < K; l++) {
          class_tot[L * K + l] = cl[l];
          class_tot[R * K + l] = cr[l];
          posts[L * K + l] = (float)cl[l] / (float)lsum;
          posts[R * K + l] = (float)cr[l] / (float)rsum;
        }
        lc[L] = -1;
        lc[R] = -1;
        // = candidate_feature / candidate_threshold of (o.f, o.t), read from the tables
        for (int d = 0; d < D; d++) feats[(size_t)n * D + d] = h_par[(size_t)i * (D + 1) + d];
        thrs[n] = h_par[(size_t)i * (D + 1) + D];
        lc[n] = (int32_t)L;
        split_now[s0 + i] = 1;
        stats.nodes_split++;
        if (ctx->collect_records) {
          pd_record r;
          memset(&r, 0, sizeof(r));
          r.depth = depth;
          r.count = node_tot[n];
          r.node = n;
          r.tree = tree_id;
          r.gain = o.gain;
          for (int d = 0; d < D; d++) r.feat[d] = (int32_t)feats[(size_t)n * D + d];
          r.thr = (int32_t)thrs[n];
          for (uint32_t l = 0; l < K; l++) r.class_count[l] = class_tot[(size_t)n * K + l];
          ctx->records.push_back(r);
        }
      }
    }

    // device tree update for the frontier nodes and their children
    const uint64_t nmin = (uint64_t)frontier.front(), nmax = (uint64_t)frontier.back();
    const uint64_t cmax = std::min<uint64_t>(n_nodes - 1, 2 * nmax + 2);
    PD_CUDA(h2d(ctx, ctx->t_lc.as<int32_t>() + nmin, lc + nmin, (cmax - nmin + 1) * 4));
    PD_CUDA(h2d(ctx, ctx->t_feat.as<FeatT>() + nmin * D, feats + nmin * D, (nmax - nmin + 1) * D * sizeof(FeatT)));
    PD_CUDA(h2d(ctx, ctx->t_thr.as<FeatT>() + nmin, thrs + nmin, (nmax - nmin + 1) * sizeof(FeatT)));
    if (2 * nmin + 1 < n_nodes)
      PD_CUDA(h2d(ctx, ctx->t_post.as<float>() + (2 * nmin + 1) * K, posts + (2 * nmin + 1) * K,
                              (cmax - (2 * nmin + 1) + 1) * K * 4));

    // next frontier (init:333-365: leaf children with more than perLeafSamplesThr samples)
    std::vector<int32_t> next;
    std::vector<uint64_t> next_off{0};
    std::vector<SlotNext> sn(nf);
    long long base_l = 0, base_r = 0;
    const bool more = depth + 1 < end_depth;
    for (uint32_t i = 0; i < nf; i++) {
      sn[i].k_l = sn[i].k_r = -1;
      sn[i].adj_l = sn[i].adj_r = 0;
      if (!split_now[i]) continue;
      const uint64_t n = (uint64_t)frontier[i];
      const uint64_t L = 2 * n + 1, R = 2 * n + 2;
      if (more && node_tot[L] > p->per_leaf_samples_thr) {
        sn[i].k_l = (int32_t)next.size();
        sn[i].adj_l = (long long)next_off.back() - base_l;
        base_l += node_tot[L];
        next.push_back((int32_t)L);
        next_off.push_back(next_off.back() + node_tot[L]);
      }
      if (more && node_tot[R] > p->per_leaf_samples_thr) {
        sn[i].k_r = (int32_t)next.size();
        sn[i].adj_r = (long long)next_off.back() - base_r;
        base_r += node_tot[R];
        next.push_back((int32_t)R);
        next_off.push_back(next_off.back() + node_tot[R]);
      }
    }
    PD_TRY(d_next.ensure((size_t)nf * sizeof(SlotNext)));
    PD_CUDA(h2d(ctx, d_next.ptr, sn.data(), (size_t)nf * sizeof(SlotNext)));
    PD_CUDA(cudaEventRecord(ev[4], st));
    if (n_act && is_user_plugin(ctx)) {
      const RtcKernels *rk = nullptr;
      PD_TRY(rtc_kernels(ctx, &rk));
      DevSet ds = devset(ctx);
      const uint32_t *a_ = ctx->act[cur].as<uint32_t>(), *as_ = ctx->act_slot[cur].as<uint32_t>();
      const SampleRec *r_ = ctx->act_rec[cur].as<SampleRec>();
      uint32_t na = (uint32_t)n_act;
      int32_t *sn_ = ctx->snode.as<int32_t>();
      const int32_t *lc_ = ctx->t_lc.as<int32_t>();
      const FeatT *tf = ctx->t_feat.as<FeatT>(), *tt = ctx->t_thr.as<FeatT>();
      const SlotNext *nx = d_next.as<SlotNext>();
      uint8_t *fl = ctx->flags.as<uint8_t>();
      void *args[] = {&ds, &a_, &r_, &as_, &na, &sn_, &lc_, &tf, &tt, &nx, &fl};
      PD_TRY(rtc_launch(ctx, rk->reassign, dim3((unsigned)((n_act + 255) / 256)), dim3(256), 0, args));
    } else if constexpr (!P::kRtcOnly) {
      if (n_act) {
        k_reassign<P><<<(unsigned)((n_act + 255) / 256), 256, 0, st>>>(
            devset(ctx), ctx->act[cur].as<uint32_t>(), ctx->act_rec[cur].as<SampleRec>(),
            ctx->act_slot[cur].as<uint32_t>(), (uint32_t)n_act,
            ctx->snode.as<int32_t>(), ctx->t_lc.as<int32_t>(), ctx->t_feat.as<FeatT>(), ctx->t_thr.as<FeatT>(),
            d_next.as<SlotNext>(), ctx->flags.as<uint8_t>());
        PD_CUDA(cudaGetLastError());
        ctx->launches++;
      }
    }
    if (ctx->tree_feature && !next.empty()) {
      // the node map of the next depth, from this depth's map and the tree as it now stands
      PD_TRY(launch_node_map_step(ctx, ctx->nm_map[ctx->nm_cur].as<int32_t>(),
                                  ctx->nm_map[1 - ctx->nm_cur].as<int32_t>()));
      ctx->nm_cur = 1 - ctx->nm_cur;
    }
    const uint64_t n_next = next_off.back();
    if (!next.empty() && n_act) {
      const uint32_t nb = (uint32_t)((n_act + kScanItems - 1) / kScanItems);
      unsigned long long *bs = ctx->scan_blocks.as<unsigned long long>();
      PD_CUDA(cudaMemsetAsync(ctx->scatter_err.ptr, 0, 4, st));
      k_scan_reduce<<<nb, 256, 0, st>>>(ctx->flags.as<uint8_t>(), (uint32_t)n_act, bs);
      k_scan_blocks<<<1, 1024, 0, st>>>(bs, nb, bs + nb);
      k_scatter<<<nb, 256, 0, st>>>(ctx->flags.as<uint8_t>(), (uint32_t)n_act, bs, ctx->act[cur].as<uint32_t>(),
                                    ctx->act_slot[cur].as<uint32_t>(), d_next.as<SlotNext>(), (uint32_t)n_next,
                                    ctx->act[1 - cur].as<uint32_t>(), ctx->act_slot[1 - cur].as<uint32_t>(),
                                    ctx->act_rec[cur].as<SampleRec>(), ctx->act_rec[1 - cur].as<SampleRec>(),
                                    ctx->scatter_err.as<uint32_t>());
      PD_CUDA(cudaGetLastError());
      ctx->launches += 3;
      unsigned long long total = 0;
      uint32_t err = 0;
      PD_CUDA(d2h(ctx, &total, bs + nb, 8));
      PD_CUDA(d2h(ctx, &err, ctx->scatter_err.ptr, 4));
      PD_CUDA(cudaEventRecord(ev[5], st));
      PD_CUDA(cudaStreamSynchronize(st));
      const uint64_t got = (total & 0xffffffffull) + (total >> 32);
      PD_CHECK(err == 0 && got == n_next, PD_ERR_STATE,
               "reassignment disagrees with the split counts at depth %u (%llu vs %llu samples, %u misplaced)",
               depth, (unsigned long long)got, (unsigned long long)n_next, err);
      cur = 1 - cur;
    } else {
      PD_CUDA(cudaEventRecord(ev[5], st));
      PD_CUDA(cudaStreamSynchronize(st));
    }
    stats.ms_reassign += elapsed(ev[4], ev[5]);
    n_act = n_next;
    frontier.swap(next);
    cur_off.swap(next_off);
  }
  PD_CUDA(cudaStreamSynchronize(st));
  stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
  stats.h2d_bytes = ctx->bytes_h2d - h2d0;
  stats.d2h_bytes = ctx->bytes_d2h - d2h0;
  stats.kernel_launches = ctx->launches - launches0;
  ctx->stats = stats;
  return PD_OK;
}

}  // namespace pd

using namespace pd;

extern "C" int pd_train_tree(pd_ctx *ctx, const pd_train_params *params, uint32_t tree_id, uint32_t start_depth,
                             uint32_t end_depth, const float *root_prior, int32_t *left_child, void *features,
                             void *thresholds, float *posteriors) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  PD_CHECK(ctx->have_dataset, PD_ERR_STATE, "no dataset uploaded");
  PD_CHECK(start_depth == 1, PD_ERR_INVALID, "Starting depth must be equal to 1");
  PD_CHECK(end_depth >= 1 && end_depth <= 24, PD_ERR_UNSUPPORTED, "end_depth %u outside [1,24]", end_depth);
  PD_CHECK(root_prior && left_child && features && thresholds && posteriors, PD_ERR_INVALID, "null tree array");
  PD_TRY(check_params(ctx, params));
  PD_CUDA(cudaSetDevice(ctx->device));
  return dispatch_config(ctx->cfg, [&]<class P>() {
    using FeatT = typename P::feat_t;
    return train_tree_impl<P>(ctx, params, tree_id, end_depth, root_prior, left_child,
                              static_cast<FeatT *>(features), static_cast<FeatT *>(thresholds), posteriors);
  });
}

extern "C" int pd_train_tree_proposed(pd_ctx *ctx, pd_proposer *prop, const pd_train_params *params,
                                      uint32_t n_proposed, uint32_t tree_id, uint32_t start_depth, uint32_t end_depth,
                                      const float *root_prior, int32_t *left_child, void *features, void *thresholds,
                                      float *posteriors) {
  PD_CHECK(ctx && prop, PD_ERR_INVALID, "null context or proposer");
  PD_CHECK(ctx->have_dataset, PD_ERR_STATE, "no dataset uploaded");
  PD_CHECK(start_depth == 1, PD_ERR_INVALID, "Starting depth must be equal to 1");
  PD_CHECK(end_depth >= 1 && end_depth <= 24, PD_ERR_UNSUPPORTED, "end_depth %u outside [1,24]", end_depth);
  PD_CHECK(root_prior && left_child && features && thresholds && posteriors, PD_ERR_INVALID, "null tree array");
  PD_TRY(check_params(ctx, params));
  PD_CHECK(n_proposed <= params->n_features, PD_ERR_INVALID, "n_proposed %u above n_features %u", n_proposed,
           params->n_features);
  PD_CUDA(cudaSetDevice(ctx->device));
  return dispatch_config(ctx->cfg, [&]<class P>() {
    using FeatT = typename P::feat_t;
    return train_tree_impl<P>(ctx, params, tree_id, end_depth, root_prior, left_child,
                              static_cast<FeatT *>(features), static_cast<FeatT *>(thresholds), posteriors, prop,
                              n_proposed);
  });
}

extern "C" int pd_train_tree_sharded(pd_ctx *ctx, const pd_train_params *params, uint32_t f_begin, uint32_t f_end,
                                     pd_exchange_fn exchange, void *user, uint32_t tree_id, uint32_t start_depth,
                                     uint32_t end_depth, const float *root_prior, int32_t *left_child, void *features,
                                     void *thresholds, float *posteriors) {
  PD_CHECK(ctx && exchange, PD_ERR_INVALID, "null context or exchange function");
  PD_CHECK(ctx->have_dataset, PD_ERR_STATE, "no dataset uploaded");
  PD_CHECK(start_depth == 1, PD_ERR_INVALID, "Starting depth must be equal to 1");
  PD_CHECK(end_depth >= 1 && end_depth <= 24, PD_ERR_UNSUPPORTED, "end_depth %u outside [1,24]", end_depth);
  PD_CHECK(root_prior && left_child && features && thresholds && posteriors, PD_ERR_INVALID, "null tree array");
  PD_TRY(check_params(ctx, params));
  PD_CHECK(f_begin < f_end && f_end <= params->n_features, PD_ERR_INVALID,
           "candidate range [%u, %u) outside [0, %u)", f_begin, f_end, params->n_features);
  PD_CUDA(cudaSetDevice(ctx->device));
  pd_train_params local = *params;
  local.n_features = f_end - f_begin;
  const Shard shard{f_begin, params->n_features, exchange, user};
  return dispatch_config(ctx->cfg, [&]<class P>() {
    using FeatT = typename P::feat_t;
    return train_tree_impl<P>(ctx, &local, tree_id, end_depth, root_prior, left_child, static_cast<FeatT *>(features),
                              static_cast<FeatT *>(thresholds), posteriors, nullptr, 0, &shard);
  });
}

extern "C" int pd_train_records(pd_ctx *ctx, pd_record *out, uint64_t cap, uint64_t *n) {
  PD_CHECK(ctx && n, PD_ERR_INVALID, "null argument");
  *n = ctx->records.size();
  if (out) memcpy(out, ctx->records.data(), std::min<uint64_t>(cap, ctx->records.size()) * sizeof(pd_record));
  return PD_OK;
}

extern "C" int pd_train_get_stats(pd_ctx *ctx, pd_train_stats *out) {
  PD_CHECK(ctx && out, PD_ERR_INVALID, "null argument");
  *out = ctx->stats;
  return PD_OK;
}

extern "C" int pd_train_sample_nodes(pd_ctx *ctx, int32_t *out) {
  PD_CHECK(ctx && out, PD_ERR_INVALID, "null argument");
  PD_CHECK(ctx->have_dataset && ctx->snode.cap >= ctx->n_samples * 4, PD_ERR_STATE, "no training run");
  PD_CUDA(cudaSetDevice(ctx->device));
  PD_CUDA(d2h(ctx, out, ctx->snode.ptr, ctx->n_samples * 4));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  return PD_OK;
}

// ------------------------------------------------------ stage entry points ----
extern "C" int pd_candidates(pd_ctx *ctx, const pd_train_params *params, uint32_t tree_id, const int32_t *nodes,
                             uint32_t n_nodes, void *features_out, void *thresholds_out) {
  PD_CHECK(ctx && nodes && features_out && thresholds_out, PD_ERR_INVALID, "null argument");
  PD_TRY(check_params(ctx, params));
  PD_CUDA(cudaSetDevice(ctx->device));
  return dispatch_config(ctx->cfg, [&]<class P>() {
    using FeatT = typename P::feat_t;
    constexpr int D = P::kFeatDim;
    const uint32_t F = params->n_features, T = params->n_thresholds;
    PD_TRY(ensure_slice(ctx, params, n_nodes));
    DevBuf dn;
    PD_TRY(dn.ensure((size_t)n_nodes * 4));
    PD_CUDA(h2d(ctx, dn.ptr, nodes, (size_t)n_nodes * 4));
    PD_TRY(launch_candidates<P>(ctx, params, tree_id, dn.as<int32_t>(), n_nodes));
    std::vector<FeatT> f((size_t)n_nodes * D * F), t((size_t)n_nodes * T * F);
    std::vector<uint8_t> perm((size_t)n_nodes * T * F);
    PD_CUDA(d2h(ctx, f.data(), ctx->cand_feat.ptr, f.size() * sizeof(FeatT)));
    PD_CUDA(d2h(ctx, t.data(), ctx->cand_thr.ptr, t.size() * sizeof(FeatT)));
    PD_CUDA(d2h(ctx, perm.data(), ctx->cand_perm.ptr, perm.size()));
    PD_CUDA(cudaStreamSynchronize(ctx->stream));
    dn.release();
    FeatT *fo = static_cast<FeatT *>(features_out), *to = static_cast<FeatT *>(thresholds_out);
    for (uint32_t n = 0; n < n_nodes; n++)
      for (uint32_t ff = 0; ff < F; ff++) {
        for (int d = 0; d < D; d++) fo[((size_t)n * F + ff) * D + d] = f[((size_t)n * D + d) * F + ff];
        for (uint32_t j = 0; j < T; j++) {
          const size_t src = ((size_t)n * T + j) * F + ff;
          to[((size_t)n * F + ff) * T + perm[src]] = t[src];
        }
      }
    return PD_OK;
  });
}

extern "C" int pd_hist(pd_ctx *ctx, const pd_train_params *params, uint32_t tree_id, const int32_t *sample_node,
                       const int32_t *nodes, uint32_t n_nodes, uint32_t *hist_out) {
  PD_CHECK(ctx && sample_node && nodes && hist_out, PD_ERR_INVALID, "null argument");
  PD_CHECK(ctx->have_dataset, PD_ERR_STATE, "no dataset uploaded");
  PD_CHECK(!ctx->tree_feature, PD_ERR_UNSUPPORTED,
           "the feature reads the tree and the node map, which only pd_train_tree keeps: no stage call");
  PD_TRY(check_params(ctx, params));
  PD_CUDA(cudaSetDevice(ctx->device));
  const uint64_t S = ctx->n_samples;
  const uint32_t F = params->n_features, T = params->n_thresholds, K = ctx->cfg.n_classes;
  // group samples by slot (stable)
  std::vector<std::pair<int32_t, uint32_t>> map(n_nodes);
  for (uint32_t i = 0; i < n_nodes; i++) map[i] = {nodes[i], i};
  std::sort(map.begin(), map.end());
  std::vector<uint64_t> cnt(n_nodes + 1, 0);
  std::vector<int64_t> slot_of(S, -1);
  for (uint64_t s = 0; s < S; s++) {
    auto it = std::lower_bound(map.begin(), map.end(), std::make_pair(sample_node[s], 0u));
    if (it != map.end() && it->first == sample_node[s]) {
      slot_of[s] = it->second;
      cnt[it->second + 1]++;
    }
  }
  for (uint32_t i = 0; i < n_nodes; i++) cnt[i + 1] += cnt[i];
  std::vector<uint32_t> act(cnt[n_nodes]);
  std::vector<uint64_t> pos(cnt.begin(), cnt.end() - 1);
  for (uint64_t s = 0; s < S; s++)
    if (slot_of[s] >= 0) act[pos[slot_of[s]]++] = (uint32_t)s;
  return dispatch_config(ctx->cfg, [&]<class P>() {
    PD_TRY(ensure_slice(ctx, params, n_nodes));
    DevBuf dn, da, drec, dref;
    PD_TRY(dn.ensure((size_t)n_nodes * 4));
    PD_TRY(da.ensure(act.size() * 4 + 4));
    PD_TRY(drec.ensure(act.size() * sizeof(SampleRec) + sizeof(SampleRec)));
    PD_TRY(dref.ensure((size_t)n_nodes * K * T * F * 4 + 4));
    PD_CUDA(h2d(ctx, dn.ptr, nodes, (size_t)n_nodes * 4));
    if (!act.empty()) {
      PD_CUDA(h2d(ctx, da.ptr, act.data(), act.size() * 4));
      k_gather_rec<<<(unsigned)((act.size() + 255) / 256), 256, 0, ctx->stream>>>(
          da.as<uint32_t>(), (uint32_t)act.size(), ctx->s_rec.as<SampleRec>(), drec.as<SampleRec>());
      PD_CUDA(cudaGetLastError());
      ctx->launches++;
    }
    PD_TRY(launch_candidates<P>(ctx, params, tree_id, dn.as<int32_t>(), n_nodes));
    uint64_t n_items = 0;
    PD_TRY(launch_hist<P>(ctx, params, cnt.data(), n_nodes, drec.as<SampleRec>(), &n_items));
    const uint64_t total = (uint64_t)n_nodes * K * F;
    if (total) {
      k_hist_to_ref<<<(unsigned)((total + 255) / 256), 256, 0, ctx->stream>>>(
          ctx->hist.as<uint32_t>(), ctx->cand_perm.as<uint8_t>(), dref.as<uint32_t>(), n_nodes, K, T, F);
      PD_CUDA(cudaGetLastError());
    }
    PD_CUDA(d2h(ctx, hist_out, dref.ptr, (size_t)n_nodes * K * T * F * 4));
    PD_CUDA(cudaStreamSynchronize(ctx->stream));
    return PD_OK;
  });
}

extern "C" int pd_split(pd_ctx *ctx, const pd_train_params *params, const uint32_t *hist, const uint32_t *class_tot,
                        uint32_t n_nodes, int32_t *out_t, int32_t *out_f, double *out_gain) {
  PD_CHECK(ctx && hist && class_tot && out_t && out_f && out_gain, PD_ERR_INVALID, "null argument");
  PD_TRY(check_params(ctx, params));
  PD_CUDA(cudaSetDevice(ctx->device));
  const uint32_t F = params->n_features, T = params->n_thresholds, K = ctx->cfg.n_classes;
  uint64_t maxn = 2;
  for (uint32_t i = 0; i < n_nodes; i++) {
    uint64_t N = 0;
    for (uint32_t l = 0; l < K; l++) N += class_tot[(size_t)i * K + l];
    maxn = std::max(maxn, N + 2);
  }
  PD_TRY(ensure_log2_table(ctx, maxn));
  PD_TRY(ensure_slice(ctx, params, n_nodes));
  DevBuf dh, dc;
  PD_TRY(dh.ensure((size_t)n_nodes * K * T * F * 4 + 4));
  PD_TRY(dc.ensure((size_t)n_nodes * K * 4 + 4));
  PD_CUDA(h2d(ctx, dh.ptr, hist, (size_t)n_nodes * K * T * F * 4));
  PD_CUDA(h2d(ctx, dc.ptr, class_tot, (size_t)n_nodes * K * 4));
  PD_CUDA(cudaMemsetAsync(ctx->recheck.ptr, 0, 8, ctx->stream));
  PD_TRY(launch_split<true>(ctx, params, n_nodes, dh.as<uint32_t>(), nullptr, dc.as<uint32_t>()));
  std::vector<SplitOut> o(n_nodes);
  PD_CUDA(d2h(ctx, o.data(), ctx->split_out.ptr, n_nodes * sizeof(SplitOut)));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  for (uint32_t i = 0; i < n_nodes; i++) {
    out_t[i] = o[i].t;
    out_f[i] = o[i].f;
    out_gain[i] = o[i].gain;
  }
  return PD_OK;
}

extern "C" int pd_log2_table(pd_ctx *ctx, uint32_t n, double *out) {
  PD_CHECK(ctx && out, PD_ERR_INVALID, "null argument");
  PD_CUDA(cudaSetDevice(ctx->device));
  PD_TRY(ensure_log2_table(ctx, n));
  PD_CUDA(d2h(ctx, out, ctx->log2_tab.ptr, (size_t)n * 8));
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  return PD_OK;
}
