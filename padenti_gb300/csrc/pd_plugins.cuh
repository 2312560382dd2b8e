// Built-in per-pixel feature plugins.  The reference compiles a user OpenCL C
// computeFeature() into its kernels (kernels/hist_update.cl:33,
// kernels/predict.cl:32; prototype in padenti.hpp.in:169-187).  Here a plugin is
// a device functor in two steps: prepare() reads what depends only on the pixel
// (done once per pixel), eval() computes the response for one candidate
// feature vector (done once per candidate).
#pragma once

#include "pd_common.cuh"

namespace pd {

constexpr int32_t kBgDepth = 10000;  // out-of-image / zero-depth reading

template <typename ImgT>
struct ImageRef {
  const ImgT *data;  // interleaved [H][W][C]
  int32_t w, h;
};

template <typename T>
PD_D T ldg(const T *p) {
#if defined(__CUDA_ARCH__)
  return __ldg(p);
#else
  return *p;
#endif
}

// (int)roundf((float)u / (float)d) -- round half away from zero of the
// correctly rounded float quotient -- for an integer offset u and a depth
// 1 <= d <= 65535, given rcp ~= 1/d.
//
// For |u| < 2^23 the float quotient lies within 2^-24 |u/d| < 1/(2d) of u/d,
// and u/d is either a half-integer (then the quotient is exact) or at least
// 1/(2d) away from every half-integer, so the float rounding never crosses a
// rounding boundary: the result is the exact rational rounding
// sign(u) * floor((2|u| + d) / (2d)).  That is computed here with an estimate
// from rcp and one integer correction step (the estimate is within 1 for
// |u| <= 2^21); larger |u| take the float path.
PD_D int32_t round_div(int32_t u, int32_t d, float rcp) {
  const int32_t a = u < 0 ? -u : u;
  if (a > (1 << 21)) return (int32_t)roundf(fdiv((float)u, (float)d));
#if defined(__CUDA_ARCH__)
  int32_t q = __float2int_rz(__fmaf_rn((float)a, rcp, 0.5f));
#else
  int32_t q = (int32_t)((float)a * rcp + 0.5f);
#endif
  const int32_t r = 2 * a + d - 2 * d * q;  // (2a + d) - 2d*q, in [-2d, 4d)
  q += (r >= 2 * d ? 1 : 0) - (r < 0 ? 1 : 0);
  return u < 0 ? -q : q;
}

// I(x+u/d(x)) - I(x+v/d(x)); u,v in pixel*mm, d(x) the centre depth in mm.
// Probes outside the image or on zero depth read 10000; a zero centre depth
// scales as 10000.  Offsets are round-half-away of the IEEE float quotient
// (round_div, bit-identical to roundf(u/d)).
struct DepthDiff2 {
  using img_t = uint16_t;
  using feat_t = int32_t;
  static constexpr int kFeatDim = 4;
  static constexpr int kChannels = 1;
  static constexpr int kId = PD_PLUGIN_DEPTH_DIFF2;
  struct Prep {
    const uint16_t *im;
    int32_t w, h, x, y, d;
    float rcp;
  };
  static PD_D Prep prepare(const ImageRef<uint16_t> &im, int32_t x, int32_t y) {
    Prep p;
    p.im = im.data;
    p.w = im.w;
    p.h = im.h;
    p.x = x;
    p.y = y;
    const uint16_t c = ldg(im.data + (size_t)y * im.w + x);
    p.d = c ? (int32_t)c : kBgDepth;
    p.rcp = 1.0f / (float)p.d;
    return p;
  }
  static PD_D int32_t probe(const Prep &p, int32_t x, int32_t y) {
    if ((uint32_t)x >= (uint32_t)p.w || (uint32_t)y >= (uint32_t)p.h) return kBgDepth;
    const uint16_t v = ldg(p.im + (size_t)y * p.w + x);
    return v ? (int32_t)v : kBgDepth;
  }
  static PD_D int32_t eval(const Prep &p, const int32_t *f) {
    const int32_t x1 = p.x + round_div(f[0], p.d, p.rcp);
    const int32_t y1 = p.y + round_div(f[1], p.d, p.rcp);
    const int32_t x2 = p.x + round_div(f[2], p.d, p.rcp);
    const int32_t y2 = p.y + round_div(f[3], p.d, p.rcp);
    return probe(p, x1, y1) - probe(p, x2, y2);
  }
};

// The reference example plugin test/feature.cl:29-64 with feat_t = short:
// D(x) - D(x + round(u*500/D(x))), out-of-image or zero probe = 10000.  A zero
// centre depth (a division by zero in the reference) reads the probe as 10000.
struct DepthDiff1 {
  using img_t = uint16_t;
  using feat_t = int16_t;
  static constexpr int kFeatDim = 2;
  static constexpr int kChannels = 1;
  static constexpr int kId = PD_PLUGIN_DEPTH_DIFF1;
  struct Prep {
    const uint16_t *im;
    int32_t w, h, x, y;
    int16_t depth;
  };
  static PD_D Prep prepare(const ImageRef<uint16_t> &im, int32_t x, int32_t y) {
    Prep p;
    p.im = im.data;
    p.w = im.w;
    p.h = im.h;
    p.x = x;
    p.y = y;
    p.depth = (int16_t)ldg(im.data + (size_t)y * im.w + x);
    return p;
  }
  static PD_D int16_t eval(const Prep &p, const int16_t *f) {
    int32_t probe = kBgDepth;
    if (p.depth != 0) {
      const float dd = (float)p.depth;
      const int32_t ox = p.x + (int32_t)roundf(fdiv(fmul((float)f[0], 500.0f), dd));
      const int32_t oy = p.y + (int32_t)roundf(fdiv(fmul((float)f[1], 500.0f), dd));
      const bool out = ox < 0 || oy < 0 || ox >= p.w || oy >= p.h;
      const int16_t v = out ? (int16_t)kBgDepth : (int16_t)ldg(p.im + (size_t)oy * p.w + ox);
      probe = v ? v : kBgDepth;
    }
    return (int16_t)((int32_t)p.depth - probe);
  }
};

// I_c1(x+u) - I_c2(x+v) on an RGB uint8 image; channels clamped to [0,2]
// (channel bounds [0,3) can draw 3 after float rounding); outside reads 0.
struct ChannelDiff {
  using img_t = uint8_t;
  using feat_t = int32_t;
  static constexpr int kFeatDim = 6;
  static constexpr int kChannels = 3;
  static constexpr int kId = PD_PLUGIN_CHANNEL_DIFF;
  struct Prep {
    const uint8_t *im;
    int32_t w, h, x, y;
  };
  static PD_D Prep prepare(const ImageRef<uint8_t> &im, int32_t x, int32_t y) {
    Prep p;
    p.im = im.data;
    p.w = im.w;
    p.h = im.h;
    p.x = x;
    p.y = y;
    return p;
  }
  static PD_D int32_t read(const Prep &p, int32_t x, int32_t y, int32_t c) {
    if (x < 0 || y < 0 || x >= p.w || y >= p.h) return 0;
    return ldg(p.im + ((size_t)y * p.w + x) * 3 + c);
  }
  static PD_D int32_t eval(const Prep &p, const int32_t *f) {
    const int32_t c1 = f[0] < 0 ? 0 : (f[0] > 2 ? 2 : f[0]);
    const int32_t c2 = f[1] < 0 ? 0 : (f[1] > 2 ? 2 : f[1]);
    return read(p, p.x + f[2], p.y + f[3], c1) - read(p, p.x + f[4], p.y + f[5], c2);
  }
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

}  // namespace pd
