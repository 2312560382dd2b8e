// Context, error reporting and training-set upload of libpadenti_gb300.
#include <algorithm>
#include <cstring>
#include <string>
#include <chrono>
#include <thread>
#include <vector>

#include "pd_ctx.cuh"
#include "pd_plugins.cuh"
#include "pd_rtc.cuh"

namespace pd {

static thread_local std::string g_last_error;

int set_error(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}
const char *last_error() { return g_last_error.c_str(); }

// Checks a pd_config against the plugin's compiled types.
static int check_config(const pd_config *c) {
  PD_CHECK(c, PD_ERR_INVALID, "null config");
  PD_CHECK(c->n_classes >= 1 && c->n_classes <= PD_MAX_CLASSES, PD_ERR_UNSUPPORTED, "nClasses %d outside [1,%d]",
           c->n_classes, PD_MAX_CLASSES);
  if (c->plugin == PD_PLUGIN_USER) {
    // a run-time compiled feature: any FeatDim 1..8, int16 / int32 features, and
    // uint8 / uint16 / int16 / int32 / float images of 1..4 channels
    PD_CHECK(c->feat_dim >= 1 && c->feat_dim <= PD_MAX_FEAT_DIM, PD_ERR_UNSUPPORTED, "FeatDim %d outside [1,%d]",
             c->feat_dim, PD_MAX_FEAT_DIM);
    PD_CHECK(c->feat_type == PD_FEAT_I16 || c->feat_type == PD_FEAT_I32, PD_ERR_UNSUPPORTED,
             "feat_type %d (supported: PD_FEAT_I16, PD_FEAT_I32)", c->feat_type);
    PD_CHECK(c->img_type >= PD_IMG_U8 && c->img_type <= PD_IMG_F32, PD_ERR_UNSUPPORTED, "img_type %d", c->img_type);
    PD_CHECK(c->n_channels >= 1 && c->n_channels <= 4, PD_ERR_UNSUPPORTED, "%d channels outside [1,4]",
             c->n_channels);
    return PD_OK;
  }
  return dispatch_config(*c, [&]<class P>() {
    const int img = sizeof(typename P::img_t) == 1 ? PD_IMG_U8 : PD_IMG_U16;
    const int ft = sizeof(typename P::feat_t) == 2 ? PD_FEAT_I16 : PD_FEAT_I32;
    PD_CHECK(c->img_type == img && c->n_channels == P::kChannels && c->feat_type == ft &&
                 c->feat_dim == P::kFeatDim,
             PD_ERR_INVALID,
             "plugin %d needs img_type %d, %d channel(s), feat_type %d, FeatDim %d (got %d, %d, %d, %d)", c->plugin,
             img, P::kChannels, ft, P::kFeatDim, c->img_type, c->n_channels, c->feat_type, c->feat_dim);
    return PD_OK;
  });
}

}  // namespace pd

using namespace pd;

extern "C" const char *pd_last_error(void) { return last_error(); }
extern "C" int pd_version(void) { return 10000; }

extern "C" int pd_ctx_create(const pd_config *cfg, int device, pd_ctx **out) {
  PD_CHECK(out, PD_ERR_INVALID, "null output");
  *out = nullptr;
  PD_TRY(check_config(cfg));
  int n = 0;
  PD_CUDA(cudaGetDeviceCount(&n));
  PD_CHECK(device >= 0 && device < n, PD_ERR_INVALID, "device %d not present (%d devices)", device, n);
  PD_CUDA(cudaSetDevice(device));
  pd_ctx *c = new pd_ctx();
  c->cfg = *cfg;
  c->device = device;
  cudaDeviceGetAttribute(&c->n_sms, cudaDevAttrMultiProcessorCount, device);
  if (c->n_sms <= 0) c->n_sms = 1;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return set_error(PD_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
  }
  for (auto &ev : c->ev) cudaEventCreate(&ev);
  const int rc = init_tables(c);
  if (rc != PD_OK) {
    pd_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return PD_OK;
}

extern "C" int pd_ctx_destroy(pd_ctx *ctx) {
  if (!ctx) return PD_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  DevBuf *bufs[] = {&ctx->pixels, &ctx->img_off, &ctx->img_wh, &ctx->s_xy, &ctx->s_img, &ctx->s_label,
                    &ctx->log2_tab, &ctx->magic_tab, &ctx->snode, &ctx->act[0], &ctx->act[1], &ctx->act_rec[0], &ctx->act_rec[1], &ctx->s_rec, &ctx->act_slot[0],
                    &ctx->act_slot[1], &ctx->flags, &ctx->scan_blocks, &ctx->slot_adj, &ctx->scatter_err,
                    &ctx->cand_feat, &ctx->cand_thr, &ctx->cand_perm, &ctx->cand_ord, &ctx->parent, &ctx->xlog2_tab, &ctx->split_par, &ctx->hist, &ctx->g32, &ctx->items, &ctx->hist_queue,
                    &ctx->zero_slots, &ctx->split_out, &ctx->split_cl, &ctx->recheck, &ctx->split_scratch, &ctx->fused_scratch, &ctx->t_lc,
                    &ctx->t_feat, &ctx->t_thr, &ctx->t_post, &ctx->f_lc, &ctx->f_feat, &ctx->f_thr,
                    &ctx->f_post, &ctx->f_meta, &ctx->f_cand, &ctx->p_img, &ctx->p_mask, &ctx->p_out,
                    &ctx->nm_map[0], &ctx->nm_map[1], &ctx->nm_off, &ctx->nm_label, &ctx->np_map[0],
                    &ctx->np_map[1], &ctx->np_desc, &ctx->f_fast};
  for (DevBuf *b : bufs) b->release();
  if (ctx->batch_graph) cudaGraphExecDestroy(ctx->batch_graph);
  ctx->b_img.release();
  ctx->b_mask.release();
  ctx->b_out.release();
  ctx->b_desc.release();
  rtc_release(ctx);
  ctx->sm_data.release();
  ctx->sm_lab.release();
  ctx->sm_desc.release();
  ctx->sm_out.release();
  ctx->h_sm.release();
  ctx->h_sm_desc.release();
  for (auto &sl : ctx->samp) {
    sl.h_data.release();
    sl.h_desc.release();
    sl.h_out.release();
    sl.d_data.release();
    sl.d_desc.release();
    sl.d_out.release();
    for (cudaEvent_t &e : sl.ev)
      if (e) cudaEventDestroy(e);
  }
  ctx->lab_tab.release();
  ctx->lab_src.release();
  ctx->lab_dst.release();
  ctx->h_lab.release();
  ctx->h_stage.release();
  ctx->h_items.release();
  for (auto &ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return PD_OK;
}

extern "C" int pd_ctx_set_hist_budget(pd_ctx *ctx, uint64_t bytes) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  PD_CHECK(bytes >= (1ull << 20), PD_ERR_INVALID, "histogram budget below 1 MiB");
  ctx->hist_budget = bytes;
  return PD_OK;
}

namespace pd {

// Copy of n16 16-byte words from pinned, device-mapped host memory by the SMs
// (each thread keeps four loads in flight over the host link) -- the
// alternative to the copy engine for the training images.
static __global__ void __launch_bounds__(256) k_copy_from_host(const uint4 *__restrict__ src, uint4 *__restrict__ dst,
                                                               uint64_t n16) {
  const uint64_t stride = (uint64_t)gridDim.x * 256u;
  uint64_t i = (uint64_t)blockIdx.x * 256u + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n16; i += stride) dst[i] = src[i];
}

}  // namespace pd

// Host -> device copy of bulk inputs (training images, staged sampler batches):
// by the SMs when the source is pinned host memory the device can address and
// both ends are 16-byte aligned (upload_copy = 1), else by the copy engine.  On
// GB300 the copy engine's first large copy after the host link has been idle
// for a few hundred milliseconds runs at ~30 GB/s instead of ~210 GB/s; the SM
// copy does not slow down.
int pd::upload_bytes(pd_ctx *ctx, void *dst, const void *src, size_t n) {
  if (ctx->upload_copy == 1 && n >= 16) {
    cudaPointerAttributes a;
    memset(&a, 0, sizeof(a));
    if (cudaPointerGetAttributes(&a, src) == cudaSuccess && a.type == cudaMemoryTypeHost && a.devicePointer &&
        ((uintptr_t)a.devicePointer % 16) == 0 && ((uintptr_t)dst % 16) == 0) {
      const uint64_t n16 = n / 16;
      const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n16 + 255) / 256, (uint64_t)ctx->n_sms * 8));
      k_copy_from_host<<<grid, 256, 0, ctx->stream>>>(static_cast<const uint4 *>(a.devicePointer),
                                                      static_cast<uint4 *>(dst), n16);
      PD_CUDA(cudaGetLastError());
      ctx->launches++;
      ctx->bytes_h2d += n16 * 16;
      if (n % 16)
        PD_CUDA(h2d(ctx, static_cast<uint8_t *>(dst) + n16 * 16, static_cast<const uint8_t *>(src) + n16 * 16, n % 16));
      return PD_OK;
    }
    cudaGetLastError();  // a pointer the runtime does not know reports an error: clear it
  }
  PD_CUDA(h2d(ctx, dst, src, n));
  return PD_OK;
}

extern "C" int pd_ctx_set_tuning(pd_ctx *ctx, const char *name, int64_t value) {
  PD_CHECK(ctx && name, PD_ERR_INVALID, "null argument");
  const std::string n(name);
  if (n == "chunk") {
    PD_CHECK(value >= 256 && value <= 65535, PD_ERR_INVALID, "chunk %lld outside [256,65535]", (long long)value);
    ctx->chunk = (uint32_t)value;
  } else if (n == "hist_spi") {
    PD_CHECK(valid_hist_spi((uint32_t)value), PD_ERR_INVALID, "hist_spi must be 2, 4 or 8");
    ctx->hist_spi = (uint32_t)value;
  } else if (n == "fuse_max") {
    PD_CHECK(value >= 0 && value <= 65535, PD_ERR_INVALID, "fuse_max %lld outside [0,65535]", (long long)value);
    ctx->fuse_max = (uint32_t)value;
  } else if (n == "cand_order") {
    PD_CHECK(value == 0 || value == 1, PD_ERR_INVALID, "cand_order must be 0 or 1");
    ctx->cand_order = value != 0;
  } else if (n == "sample_group") {
    PD_CHECK(value >= 4096, PD_ERR_INVALID, "sample_group %lld below 4096 bytes", (long long)value);
    ctx->sample_group = (uint64_t)value;
  } else if (n == "persist") {
    PD_CHECK(value == 0 || value == 1, PD_ERR_INVALID, "persist must be 0 or 1");
    ctx->persist = value != 0;
  } else if (n == "records") {
    PD_CHECK(value == 0 || value == 1, PD_ERR_INVALID, "records must be 0 or 1");
    ctx->collect_records = value != 0;
  } else if (n == "cand_regs") {
    PD_CHECK(value == 0 || value == 1, PD_ERR_INVALID, "cand_regs must be 0 or 1");
    ctx->cand_regs = value != 0;
  } else if (n == "upload_copy") {
    PD_CHECK(value == 0 || value == 1, PD_ERR_INVALID, "upload_copy must be 0 (copy engine) or 1 (SM copy)");
    ctx->upload_copy = (int)value;
  } else {
    return set_error(PD_ERR_INVALID, "unknown tuning knob '%s'", name);
  }
  return PD_OK;
}

extern "C" int pd_ctx_sync(pd_ctx *ctx) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  PD_CUDA(cudaStreamSynchronize(ctx->stream));
  return PD_OK;
}

extern "C" void *pd_ctx_stream(pd_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

extern "C" int pd_ctx_transfer_bytes(pd_ctx *ctx, uint64_t *h2d_bytes, uint64_t *d2h_bytes) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  if (h2d_bytes) *h2d_bytes = ctx->bytes_h2d;
  if (d2h_bytes) *d2h_bytes = ctx->bytes_d2h;
  return PD_OK;
}

extern "C" int pd_dataset_upload(pd_ctx *ctx, const pd_dataset_desc *ds) {
  const auto t_start = std::chrono::steady_clock::now();
  PD_CHECK(ctx && ds, PD_ERR_INVALID, "null argument");
  PD_CHECK(ds->n_images >= 1, PD_ERR_INVALID, "empty training set");
  PD_CHECK(ds->pixels && ds->pix_off && ds->width && ds->height && ds->labels && ds->lab_off && ds->samples &&
               ds->samp_off,
           PD_ERR_INVALID, "null dataset array");
  PD_CUDA(cudaSetDevice(ctx->device));
  if (is_user_plugin(ctx)) {
    const RtcKernels *rk = nullptr;
    PD_TRY(rtc_kernels(ctx, &rk));  // the sample records need the plugin
  }
  const uint32_t n = ds->n_images;
  const size_t px = img_size(ctx->cfg.img_type) * ctx->cfg.n_channels;
  const uint64_t S = ds->samp_off[n];
  PD_CHECK(n < (1u << 24), PD_ERR_UNSUPPORTED, "%u images (max 2^24-1)", n);
  PD_CHECK(S < (1ull << 31), PD_ERR_UNSUPPORTED, "%llu samples (max 2^31-1)", (unsigned long long)S);
  uint64_t bytes = 0;
  std::vector<uint64_t> off(n);
  std::vector<uint32_t> wh(n);
  for (uint32_t i = 0; i < n; i++) {
    PD_CHECK(ds->width[i] >= 1 && ds->height[i] >= 1 && ds->width[i] < 65536 && ds->height[i] < 65536,
             PD_ERR_UNSUPPORTED, "image %u is %ux%u (sides must be in [1,65535])", i, ds->width[i], ds->height[i]);
    PD_CHECK(ds->samp_off[i + 1] >= ds->samp_off[i], PD_ERR_INVALID, "sample offsets not monotone at image %u", i);
    PD_CHECK(ds->pix_off[i] % img_size(ctx->cfg.img_type) == 0, PD_ERR_INVALID,
             "image %u starts at byte %llu, not a multiple of the pixel type size", i,
             (unsigned long long)ds->pix_off[i]);
    off[i] = ds->pix_off[i];
    wh[i] = ds->width[i] | (ds->height[i] << 16);
    bytes = std::max<uint64_t>(bytes, ds->pix_off[i] + (uint64_t)ds->width[i] * ds->height[i] * px);
  }
  // per-sample position, image and class: host threads over interleaved images,
  // into pinned staging, with per-thread class totals; each thread keeps its
  // first bad sample and the lowest one is reported (the one a sequential pass
  // meets first).  Nothing reaches the device before every sample is checked, so
  // a failed upload keeps the training set uploaded before.
  PD_TRY(ctx->h_stage.ensure(S * 9 + 16));
  uint32_t *xy = ctx->h_stage.as<uint32_t>(), *im = xy + S;
  uint8_t *lab = reinterpret_cast<uint8_t *>(im + S);
  const unsigned nt = std::max(1u, std::min({16u, std::thread::hardware_concurrency(), n}));
  struct Bad {
    uint64_t k = UINT64_MAX;
    uint32_t image = 0;
    int label = -1;  // -1: the sample lies outside the image
  };
  std::vector<Bad> bad(nt);
  struct alignas(64) ClassCount {  // one cache line set per thread
    uint32_t c[PD_MAX_CLASSES];
  };
  std::vector<ClassCount> cls(nt);
  auto work = [&](unsigned t) {
    uint32_t ct[PD_MAX_CLASSES] = {};
    for (uint32_t i = t; i < n; i += nt) {
      const uint32_t w = ds->width[i], h = ds->height[i];
      for (uint64_t k = ds->samp_off[i]; k < ds->samp_off[i + 1]; k++) {
        const uint32_t p = ds->samples[k];
        if ((uint64_t)p >= (uint64_t)w * h) {
          if (k < bad[t].k) bad[t] = {k, i, -1};
          continue;
        }
        const uint8_t l = ds->labels[ds->lab_off[i] + p];
        if (l < 1 || l > ctx->cfg.n_classes) {
          if (k < bad[t].k) bad[t] = {k, i, (int)l};
          continue;
        }
        xy[k] = (p % w) | ((p / w) << 16);
        im[k] = i;
        lab[k] = (uint8_t)(l - 1);
        ct[l - 1]++;
      }
    }
    memcpy(cls[t].c, ct, sizeof(ct));
  };
  {
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; t++) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
  }
  const auto t_samples = std::chrono::steady_clock::now();
  Bad first;
  for (const Bad &b : bad)
    if (b.k < first.k) first = b;
  if (first.k != UINT64_MAX) {
    if (first.label < 0)
      return set_error(PD_ERR_INVALID, "sample %llu of image %u outside the image", (unsigned long long)first.k,
                       first.image);
    return set_error(PD_ERR_INVALID, "sample %llu of image %u has label %d (sampled pixels need a label in [1,%d])",
                     (unsigned long long)first.k, first.image, first.label, ctx->cfg.n_classes);
  }
  cudaStream_t st = ctx->stream;
  ctx->have_dataset = false;  // until the new set is in place
  PD_TRY(ctx->pixels.ensure(bytes));
  PD_TRY(ctx->img_off.ensure(n * 8));
  PD_TRY(ctx->img_wh.ensure(n * 4));
  PD_TRY(ctx->s_xy.ensure(S * 4 + 4));
  PD_TRY(ctx->s_img.ensure(S * 4 + 4));
  PD_TRY(ctx->s_label.ensure(S + 4));
  PD_TRY(upload_bytes(ctx, ctx->pixels.ptr, ds->pixels, bytes));
  PD_TRY(map_training_pixels(ctx, bytes));
  PD_CUDA(h2d(ctx, ctx->img_off.ptr, off.data(), n * 8));
  PD_CUDA(h2d(ctx, ctx->img_wh.ptr, wh.data(), n * 4));
  if (S) {
    PD_CUDA(h2d(ctx, ctx->s_xy.ptr, xy, S * 4));
    PD_CUDA(h2d(ctx, ctx->s_img.ptr, im, S * 4));
    PD_CUDA(h2d(ctx, ctx->s_label.ptr, lab, S));
  }
  PD_TRY(build_sample_records(ctx, S));
  ctx->root_class_tot.assign(ctx->cfg.n_classes, 0u);
  for (const auto &c : cls)
    for (int l = 0; l < ctx->cfg.n_classes; l++) ctx->root_class_tot[l] += c.c[l];
  if (ctx->tree_feature) {
    // the node map's layout and every pixel's label: the map advances on labelled pixels
    // (cl_tree_trainer_impl_traverse_ts.hpp:215-232 passes the label image as the mask)
    std::vector<uint64_t> moff(n + 1, 0);
    for (uint32_t i = 0; i < n; i++) moff[i + 1] = moff[i] + (uint64_t)ds->width[i] * ds->height[i];
    const uint64_t np = moff[n];
    PD_TRY(ctx->nm_off.ensure((n + 1) * 8));
    PD_TRY(ctx->nm_label.ensure(np));
    PD_TRY(ctx->nm_map[0].ensure(np * 4));
    PD_TRY(ctx->nm_map[1].ensure(np * 4));
    PD_CUDA(h2d(ctx, ctx->nm_off.ptr, moff.data(), (n + 1) * 8));
    for (uint32_t i = 0; i < n; i++)
      PD_CUDA(h2d(ctx, ctx->nm_label.as<uint8_t>() + moff[i], ds->labels + ds->lab_off[i], moff[i + 1] - moff[i]));
    ctx->nm_pixels = np;
  } else {
    ctx->nm_pixels = 0;
  }
  PD_CUDA(cudaStreamSynchronize(st));
  ctx->pixels_bytes = bytes;
  ctx->n_images = n;
  ctx->n_samples = S;
  ctx->have_dataset = true;
  PD_TRY(ensure_log2_table(ctx, S + 2));
  PD_CUDA(cudaStreamSynchronize(st));
  const auto t_end = std::chrono::steady_clock::now();
  ctx->upload_stats.ms_samples = std::chrono::duration<double, std::milli>(t_samples - t_start).count();
  ctx->upload_stats.ms_device = std::chrono::duration<double, std::milli>(t_end - t_samples).count();
  ctx->upload_stats.ms_total = std::chrono::duration<double, std::milli>(t_end - t_start).count();
  return PD_OK;
}

extern "C" int pd_dataset_upload_stats(pd_ctx *ctx, pd_upload_stats *out) {
  PD_CHECK(ctx && out, PD_ERR_INVALID, "null argument");
  *out = ctx->upload_stats;
  return PD_OK;
}

extern "C" int pd_dataset_info(pd_ctx *ctx, uint64_t *n_samples, uint32_t *n_images) {
  PD_CHECK(ctx, PD_ERR_INVALID, "null context");
  if (n_samples) *n_samples = ctx->n_samples;
  if (n_images) *n_images = ctx->n_images;
  return PD_OK;
}
