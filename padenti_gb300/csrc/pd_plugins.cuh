// Built-in per-pixel feature plugins.  The reference compiles a user OpenCL C
// computeFeature() into its kernels (kernels/hist_update.cl:33,
// kernels/predict.cl:32; prototype in padenti.hpp.in:169-187).  Here a plugin is
// a device functor in steps:
//   preload(im, x, y, pre)   loads what depends only on the pixel into kPreWords
//                            words (a warp preloads 32 pixels at once, in parallel);
//   prepare(im, x, y, pre)   builds the per-pixel state from those words;
//   candidate(f)             per-candidate constants, computed once per tile;
//   eval(prep, cand)         the response of one candidate at one pixel;
//   eval_train(prep, cand)   the same on the trainer's copy of the images, which
//                            kTrainMapsZero plugins store with 0 replaced by the
//                            background depth (equal responses, one test fewer);
// and kOrderDim, the feature dims (kOrderDim, kOrderDim + 1) of its first probe
// offset, by which the trainer orders a node's candidates.
// eval(prep, f) runs all of it for a single evaluation.
#pragma once

#include "pd_common.cuh"

namespace pd {

constexpr int32_t kBgDepth = 10000;  // out-of-image / zero-depth reading

template <typename ImgT>
struct ImageRef {
  const ImgT *data;        // interleaved [H][W][C]
  int32_t w, h;
  const uint32_t *magic;   // RoundDiv multipliers by depth (65536 entries)
  // for features that read the tree (kUsesTree plugins): this image's per-pixel
  // node map (null when none is kept), the tree being trained or evaluated, the
  // map's level and the tree's node count
  const int32_t *nodes = nullptr;
  const int32_t *tree_lc = nullptr;
  const float *tree_post = nullptr;
  uint32_t n_classes = 0;
  int32_t tree_level = 0, tree_nodes = 0;
};

template <typename T>
PD_D T ldg(const T *p) {
#if defined(__CUDA_ARCH__)
  return __ldg(p);
#else
  return *p;
#endif
}

// Exact rounded quotients round_half_away(u / d) for integers u and d > 0.
//
// The plugins compute an offset as (int)roundf((float)u / (float)d), the round
// half away from zero of the correctly rounded float quotient.  For |u| < 2^23
// that quotient lies within 2^-24 |u/d| < 1/(2d) of u/d, and u/d is either a
// half-integer (then the quotient is exact) or at least 1/(2d) away from every
// half-integer, so the float rounding never crosses a rounding boundary and the
// result is the exact rational rounding
//     sign(u) * floor((2|u| + d) / (2d)).
// The floor is a division by the per-pixel invariant M = 2d, done as a
// multiply-high by a magic number (Granlund & Montgomery, "Division by
// invariant integers using multiplication", 1994): with s = floor(log2 M) and
// m = floor(2^(31+s) / M) + 1 < 2^32, m*M - 2^(31+s) lies in (0, M] and M <=
// 2^(8+s), so floor(N*m / 2^(31+s)) = floor(N/M) for every N < 2^23.  Offsets
// with |u| > 2^21 (so that N >= 2^23 is possible) take the float path.
struct RoundDiv {
  uint32_t m, sh;  // multiplier and shift for M = 2d
  int32_t d;
  uint64_t dm;     // d * m: (n2 + d) * m is then one wide multiply-add
  static PD_HD uint32_t multiplier(uint32_t d) {
    const uint32_t M = 2u * d;
    uint32_t s = 31;
    while (!((M >> s) & 1u)) s--;
    return (uint32_t)((1ull << (31 + s)) / M + 1ull);
  }
  // d in [1, 65535]; magic[d] = multiplier(d)
  static PD_D RoundDiv make(int32_t d, const uint32_t *magic) {
    RoundDiv r;
    r.d = d;
    r.m = ldg(magic + d);
    r.sh = 31u - (uint32_t)__clz(d);  // floor(log2 2d) - 1 = floor(log2 d)
    r.dm = (uint64_t)(uint32_t)d * r.m;
    return r;
  }
  // From the depth d and its multiplier m (magic[d]).
  static PD_D RoundDiv of(uint32_t d, uint32_t m) {
    RoundDiv r;
    r.d = (int32_t)d;
    r.m = m;
    r.sh = 31u - (uint32_t)__clz((int)d);
    r.dm = (uint64_t)d * m;
    return r;
  }
  // n2 = 2|u| (|u| <= 2^21): floor((2|u| + d) / (2d)), the high word of
  // (n2 + d) * m = n2 * m + dm (< 2^55) shifted right by sh
  PD_D uint32_t q(uint32_t n2) const { return (uint32_t)(((uint64_t)n2 * m + dm) >> 32) >> sh; }
};

// Per-candidate constants of an offset: 2|u| and the sign, or the raw u when
// |u| > 2^21 (float path).
struct OffsetConst {
  uint32_t n2;  // 2|u|, or (uint32_t)u on the float path
  int32_t sg;   // +1 / -1, or 0 on the float path
  static PD_D OffsetConst make(int32_t u) {
    OffsetConst o;
    const int64_t a = u < 0 ? -(int64_t)u : (int64_t)u;
    if (a > (1 << 21)) {
      o.n2 = (uint32_t)u;
      o.sg = 0;
    } else {
      o.n2 = (uint32_t)(2 * a);
      o.sg = u < 0 ? -1 : 1;
    }
    return o;
  }
  PD_D bool fast() const { return sg != 0; }
  // round_half_away(u / d), identical to (int)roundf((float)u / (float)d);
  // FAST assumes fast() (|u| <= 2^21).
  template <bool FAST = false>
  PD_D int32_t apply(const RoundDiv &r) const {
    if (!FAST && sg == 0) return (int32_t)roundf(fdiv((float)(int32_t)n2, (float)r.d));
    return (int32_t)r.q(n2) * sg;
  }
};

// I(x+u/d(x)) - I(x+v/d(x)); u,v in pixel*mm, d(x) the centre depth in mm.
// Probes outside the image or on zero depth read 10000; a zero centre depth
// scales as 10000.  Offsets are (int)roundf((float)u / (float)d), computed
// exactly by OffsetConst::apply.
struct DepthDiff2 {
  using img_t = uint16_t;
  using feat_t = int32_t;
  static constexpr int kFeatDim = 4;
  static constexpr int kChannels = 1;
  static constexpr int kId = PD_PLUGIN_DEPTH_DIFF2;
  static constexpr int kOrderDim = 0;  // feature dims (0, 1): the first probe offset
  static constexpr bool kTrainMapsZero = true;  // 0 and 10000 read alike everywhere
  static constexpr bool kRtcOnly = false;     // kernels compiled into the library
  static constexpr bool kUsesTree = false;    // reads neither the tree nor a node map
  struct Prep {
    const uint16_t *im;
    uint32_t w, h;
    int32_t x, y;
    RoundDiv div;
  };
  struct __align__(16) Cand {  // one 16-byte-aligned record per tree node in prediction
    OffsetConst o[4];
  };
  static constexpr int kPreWords = 2;  // centre depth, its RoundDiv multiplier
  static PD_D void preload(const ImageRef<uint16_t> &im, int32_t x, int32_t y, uint32_t *pre) {
    const uint16_t c = ldg(im.data + (size_t)y * im.w + x);
    pre[0] = c ? (uint32_t)c : (uint32_t)kBgDepth;
    pre[1] = ldg(im.magic + pre[0]);
  }
  static PD_D Prep prepare(const ImageRef<uint16_t> &im, int32_t x, int32_t y, const uint32_t *pre) {
    Prep p;
    p.im = im.data;
    p.w = (uint32_t)im.w;
    p.h = (uint32_t)im.h;
    p.x = x;
    p.y = y;
    p.div = RoundDiv::of(pre[0], pre[1]);
    return p;
  }
  static PD_D Prep prepare(const ImageRef<uint16_t> &im, int32_t x, int32_t y) {
    uint32_t pre[kPreWords];
    preload(im, x, y, pre);
    return prepare(im, x, y, pre);
  }
  static PD_D Cand candidate(const int32_t *f) {
    Cand c;
#pragma unroll
    for (int k = 0; k < 4; k++) c.o[k] = OffsetConst::make(f[k]);
    return c;
  }
  static PD_D bool fast(const Cand &c) {
    return c.o[0].fast() && c.o[1].fast() && c.o[2].fast() && c.o[3].fast();
  }
  // A predicated load: an outside probe loads nothing and reads as 0, then
  // 10000.  Sides are below 2^16, so an inside index y*w + x fits 32 bits.
  static PD_D int32_t probe(const Prep &p, int32_t x, int32_t y) {
    uint32_t v = 0u;
    if ((uint32_t)x < p.w && (uint32_t)y < p.h) v = ldg(p.im + ((uint32_t)y * p.w + (uint32_t)x));
    return v ? (int32_t)v : kBgDepth;
  }
  // On the trainer's copy (zeros stored as 10000): one predicated load, 10000
  // outside the image.
  static PD_D int32_t probe_train(const Prep &p, int32_t x, int32_t y) {
    uint32_t v = (uint32_t)kBgDepth;
    if ((uint32_t)x < p.w && (uint32_t)y < p.h) v = ldg(p.im + ((uint32_t)y * p.w + (uint32_t)x));
    return (int32_t)v;
  }
  template <bool FAST = false, bool TRAIN = false>
  static PD_D int32_t eval(const Prep &p, const Cand &c) {
    const int32_t x1 = p.x + c.o[0].template apply<FAST>(p.div);
    const int32_t y1 = p.y + c.o[1].template apply<FAST>(p.div);
    const int32_t x2 = p.x + c.o[2].template apply<FAST>(p.div);
    const int32_t y2 = p.y + c.o[3].template apply<FAST>(p.div);
    if (TRAIN) return probe_train(p, x1, y1) - probe_train(p, x2, y2);
    return probe(p, x1, y1) - probe(p, x2, y2);
  }
  template <bool FAST = false>
  static PD_D int32_t eval_train(const Prep &p, const Cand &c) { return eval<FAST, true>(p, c); }
  static PD_D int32_t eval(const Prep &p, const int32_t *f) { return eval(p, candidate(f)); }
};

// The reference example plugin test/feature.cl:29-64 with feat_t = short:
// D(x) - D(x + round(u*500/D(x))), out-of-image or zero probe = 10000.  A zero
// centre depth (a division by zero in the reference) reads the probe as 10000.
// (float)u*500 is exact for short u, so the offset is the exact rounded
// quotient of 500u by D(x) (OffsetConst::apply) for a positive depth.
struct DepthDiff1 {
  using img_t = uint16_t;
  using feat_t = int16_t;
  static constexpr int kFeatDim = 2;
  static constexpr int kChannels = 1;
  static constexpr int kId = PD_PLUGIN_DEPTH_DIFF1;
  static constexpr int kOrderDim = 0;  // feature dims (0, 1): the probe offset
  static constexpr bool kTrainMapsZero = false;  // the centre depth is used as read
  static constexpr bool kRtcOnly = false;     // kernels compiled into the library
  static constexpr bool kUsesTree = false;    // reads neither the tree nor a node map
  struct Prep {
    const uint16_t *im;
    uint32_t w, h;
    int32_t x, y;
    int16_t depth;
    RoundDiv div;
  };
  struct __align__(16) Cand {  // one 16-byte-aligned record per tree node in prediction
    OffsetConst o[2];
    int16_t f[2];
  };
  static constexpr int kPreWords = 2;  // centre depth as short, multiplier of max(depth,1)
  static PD_D void preload(const ImageRef<uint16_t> &im, int32_t x, int32_t y, uint32_t *pre) {
    const int16_t depth = (int16_t)ldg(im.data + (size_t)y * im.w + x);
    pre[0] = (uint32_t)(int32_t)depth;
    pre[1] = ldg(im.magic + (depth > 0 ? depth : 1));
  }
  static PD_D Prep prepare(const ImageRef<uint16_t> &im, int32_t x, int32_t y, const uint32_t *pre) {
    Prep p;
    p.im = im.data;
    p.w = (uint32_t)im.w;
    p.h = (uint32_t)im.h;
    p.x = x;
    p.y = y;
    p.depth = (int16_t)(int32_t)pre[0];
    p.div = RoundDiv::of(p.depth > 0 ? (uint32_t)p.depth : 1u, pre[1]);
    return p;
  }
  static PD_D Prep prepare(const ImageRef<uint16_t> &im, int32_t x, int32_t y) {
    uint32_t pre[kPreWords];
    preload(im, x, y, pre);
    return prepare(im, x, y, pre);
  }
  static PD_D Cand candidate(const int16_t *f) {
    Cand c;
    c.o[0] = OffsetConst::make(500 * (int32_t)f[0]);
    c.o[1] = OffsetConst::make(500 * (int32_t)f[1]);
    c.f[0] = f[0];
    c.f[1] = f[1];
    return c;
  }
  static PD_D bool fast(const Cand &c) { return c.o[0].fast() && c.o[1].fast(); }
  template <bool FAST = false>
  static PD_D int16_t eval(const Prep &p, const Cand &c) {
    int32_t probe = kBgDepth;
    if (p.depth != 0) {
      int32_t ox, oy;
      if (p.depth > 0) {
        ox = p.x + c.o[0].template apply<FAST>(p.div);
        oy = p.y + c.o[1].template apply<FAST>(p.div);
      } else {
        const float dd = (float)p.depth;
        ox = p.x + (int32_t)roundf(fdiv(fmul((float)c.f[0], 500.0f), dd));
        oy = p.y + (int32_t)roundf(fdiv(fmul((float)c.f[1], 500.0f), dd));
      }
      int16_t v = 0;
      if ((uint32_t)ox < p.w && (uint32_t)oy < p.h) v = (int16_t)ldg(p.im + ((uint32_t)oy * p.w + (uint32_t)ox));
      probe = v ? v : kBgDepth;
    }
    return (int16_t)((int32_t)p.depth - probe);
  }
  template <bool FAST = false>
  static PD_D int16_t eval_train(const Prep &p, const Cand &c) { return eval<FAST>(p, c); }
  static PD_D int16_t eval(const Prep &p, const int16_t *f) { return eval(p, candidate(f)); }
};

// I_c1(x+u) - I_c2(x+v) on an RGB uint8 image; channels clamped to [0,2]
// (channel bounds [0,3) can draw 3 after float rounding); outside reads 0.
struct ChannelDiff {
  using img_t = uint8_t;
  using feat_t = int32_t;
  static constexpr int kFeatDim = 6;
  static constexpr int kChannels = 3;
  static constexpr int kId = PD_PLUGIN_CHANNEL_DIFF;
  static constexpr int kOrderDim = 2;  // feature dims (2, 3): the first probe offset
  static constexpr bool kTrainMapsZero = false;
  static constexpr bool kRtcOnly = false;     // kernels compiled into the library
  static constexpr bool kUsesTree = false;    // reads neither the tree nor a node map
  struct Prep {
    const uint8_t *im;
    uint32_t w, h;
    int32_t x, y;
  };
  struct __align__(16) Cand {  // one 16-byte-aligned record per tree node in prediction
    int32_t c1, c2, ux, uy, vx, vy;
  };
  static constexpr int kPreWords = 1;
  static PD_D void preload(const ImageRef<uint8_t> &, int32_t, int32_t, uint32_t *pre) { pre[0] = 0u; }
  static PD_D Prep prepare(const ImageRef<uint8_t> &im, int32_t x, int32_t y, const uint32_t *) {
    Prep p;
    p.im = im.data;
    p.w = (uint32_t)im.w;
    p.h = (uint32_t)im.h;
    p.x = x;
    p.y = y;
    return p;
  }
  static PD_D Prep prepare(const ImageRef<uint8_t> &im, int32_t x, int32_t y) { return prepare(im, x, y, nullptr); }
  static PD_D Cand candidate(const int32_t *f) {
    Cand c;
    c.c1 = f[0] < 0 ? 0 : (f[0] > 2 ? 2 : f[0]);
    c.c2 = f[1] < 0 ? 0 : (f[1] > 2 ? 2 : f[1]);
    c.ux = f[2];
    c.uy = f[3];
    c.vx = f[4];
    c.vy = f[5];
    return c;
  }
  static PD_D bool fast(const Cand &) { return true; }
  static PD_D int32_t read(const Prep &p, int32_t x, int32_t y, int32_t c) {
    int32_t v = 0;
    if ((uint32_t)x < p.w && (uint32_t)y < p.h)
      v = ldg(p.im + ((uint64_t)((uint32_t)y * p.w + (uint32_t)x) * 3u + (uint32_t)c));
    return v;
  }
  template <bool FAST = false>
  static PD_D int32_t eval(const Prep &p, const Cand &c) {
    return read(p, p.x + c.ux, p.y + c.uy, c.c1) - read(p, p.x + c.vx, p.y + c.vy, c.c2);
  }
  template <bool FAST = false>
  static PD_D int32_t eval_train(const Prep &p, const Cand &c) { return eval<FAST>(p, c); }
  static PD_D int32_t eval(const Prep &p, const int32_t *f) { return eval(p, candidate(f)); }
};

// Calls fn.template operator()<Plugin>() for the plugin id; returns
// PD_ERR_UNSUPPORTED for an unknown id.
template <typename Fn>
int dispatch_plugin(int plugin, Fn &&fn) {
  switch (plugin) {
    case PD_PLUGIN_DEPTH_DIFF2: return fn.template operator()<DepthDiff2>();
    case PD_PLUGIN_DEPTH_DIFF1: return fn.template operator()<DepthDiff1>();
    case PD_PLUGIN_CHANNEL_DIFF: return fn.template operator()<ChannelDiff>();
    default: return set_error(PD_ERR_UNSUPPORTED, "unknown plugin id %d", plugin);
  }
}

#if !defined(__CUDACC_RTC__)
// The host-side stand-in of a feature compiled at run time (PD_PLUGIN_USER):
// the feature type and dimension the host paths need.  Every kernel of such a
// context is the run-time compiled one (the compiled-in kernels are never
// instantiated for it); image sizes come from the configuration.
template <typename FeatT, int D>
struct UserHost {
  using feat_t = FeatT;
  using img_t = uint8_t;  // unused: sizes come from the configuration
  static constexpr int kFeatDim = D;
  static constexpr int kChannels = 0;
  static constexpr int kId = PD_PLUGIN_USER;
  static constexpr bool kTrainMapsZero = false;
  static constexpr bool kRtcOnly = true;
  static constexpr bool kUsesTree = false;  // known at run time: pd_ctx::tree_feature
  struct __align__(16) Cand {
    FeatT f[D];
  };
};

template <typename FeatT, typename Fn>
int dispatch_user_dim(int D, Fn &&fn) {
  switch (D) {
    case 1: return fn.template operator()<UserHost<FeatT, 1>>();
    case 2: return fn.template operator()<UserHost<FeatT, 2>>();
    case 3: return fn.template operator()<UserHost<FeatT, 3>>();
    case 4: return fn.template operator()<UserHost<FeatT, 4>>();
    case 5: return fn.template operator()<UserHost<FeatT, 5>>();
    case 6: return fn.template operator()<UserHost<FeatT, 6>>();
    case 7: return fn.template operator()<UserHost<FeatT, 7>>();
    case 8: return fn.template operator()<UserHost<FeatT, 8>>();
    default: return set_error(PD_ERR_UNSUPPORTED, "FeatDim %d outside [1,%d]", D, PD_MAX_FEAT_DIM);
  }
}

// The plugin whose host paths serve a configuration: the built-in plugin, or
// for PD_PLUGIN_USER the stand-in of its feature type and dimension.
template <typename Fn>
int dispatch_config(const pd_config &c, Fn &&fn) {
  if (c.plugin != PD_PLUGIN_USER) return dispatch_plugin(c.plugin, fn);
  if (c.feat_type == PD_FEAT_I16) return dispatch_user_dim<int16_t>(c.feat_dim, fn);
  if (c.feat_type == PD_FEAT_I32) return dispatch_user_dim<int32_t>(c.feat_dim, fn);
  return set_error(PD_ERR_UNSUPPORTED, "feat_type %d (supported: PD_FEAT_I16, PD_FEAT_I32)", c.feat_type);
}
#endif

}  // namespace pd
