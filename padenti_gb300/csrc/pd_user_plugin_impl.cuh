// UserPlugin: the user's computeFeature behind the kernels' plugin interface
// (no per-pixel preload; a candidate is its feature vector).  Included after the
// user source.
#pragma once

namespace pd {

struct UserPlugin {
  using img_t = ::img_t;
  using feat_t = ::feat_t;
  static constexpr int kFeatDim = PD_FEAT_DIM;
  static constexpr int kChannels = PD_CHANNELS;
  static constexpr int kId = PD_PLUGIN_USER;
  static constexpr int kOrderDim = 0;            // columns ordered by feature dims 0 and 1
  static constexpr bool kTrainMapsZero = false;  // the images as given
  static constexpr int kPreWords = 1;
  struct Prep {
    ImageView im;
    int32_t x, y;
  };
  struct __align__(16) Cand {  // one 16-byte-aligned record per tree node in prediction
    feat_t f[kFeatDim];
  };
  static PD_D void preload(const ImageRef<img_t> &, int32_t, int32_t, uint32_t *pre) { pre[0] = 0u; }
  static PD_D Prep prepare(const ImageRef<img_t> &im, int32_t x, int32_t y, const uint32_t *) {
    Prep p;
    p.im.data = im.data;
    p.im.w = im.w;
    p.im.h = im.h;
    p.im.c = kChannels;
    p.x = x;
    p.y = y;
    return p;
  }
  static PD_D Prep prepare(const ImageRef<img_t> &im, int32_t x, int32_t y) { return prepare(im, x, y, nullptr); }
  static PD_D Cand candidate(const feat_t *f) {
    Cand c;
#pragma unroll
    for (int k = 0; k < kFeatDim; k++) c.f[k] = f[k];
    return c;
  }
  static PD_D bool fast(const Cand &) { return true; }
  template <bool FAST = false>
  static PD_D feat_t eval(const Prep &p, const Cand &c) {
    return computeFeature(p.im, make_int2(p.x, p.y), c.f, (unsigned)kFeatDim);
  }
  template <bool FAST = false>
  static PD_D feat_t eval_train(const Prep &p, const Cand &c) { return eval<FAST>(p, c); }
  static PD_D feat_t eval(const Prep &p, const feat_t *f) {
    return computeFeature(p.im, make_int2(p.x, p.y), f, (unsigned)kFeatDim);
  }
};

}  // namespace pd
