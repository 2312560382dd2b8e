// Exposes the reference's own pixel samplers (src/padenti/uniform_image_sampler_impl.hpp:34-63,
// src/padenti/classweighted_image_sampler_impl.hpp:25-120), compiled from the
// reference source tree over the Boost stand-ins in ref_shim/boost (libstdc++'s
// mt19937, zlib's CRC-32, the two distributions restated), to the oracle tests
// through C symbols.  Test infrastructure only.
#include <padenti/image_sampler.hpp>
#include <padenti/uniform_image_sampler.hpp>
#include <padenti/classweighted_image_sampler.hpp>

#include <cstdint>

namespace {
template <typename T, unsigned C>
unsigned uniform(const void *data, const uint8_t *labels, unsigned w, unsigned h, unsigned n_samples,
                 unsigned seed, unsigned *out) {
  UniformImageSampler<T, C> s(n_samples, seed);
  return s.sample(static_cast<const T *>(data), labels, w, h, out);
}
template <typename T, unsigned C>
unsigned class_weighted(const void *data, const uint8_t *labels, unsigned w, unsigned h, unsigned n_samples,
                        unsigned n_classes, const float *weights, unsigned seed, unsigned *out) {
  if (weights) {
    ClassWeightedImageSampler<T, C> s(n_samples, n_classes, weights, seed);
    return s.sample(static_cast<const T *>(data), labels, w, h, out);
  }
  ClassWeightedImageSampler<T, C> s(n_samples, n_classes, seed);
  return s.sample(static_cast<const T *>(data), labels, w, h, out);
}
}  // namespace

// img: 2 = uint16 x 1 channel, 1 = uint8 x 3 channels (the two image types of the tests)
extern "C" unsigned ref_sample_uniform(int img, const void *data, const uint8_t *labels, unsigned w, unsigned h,
                                       unsigned n_samples, unsigned seed, unsigned *out) {
  return img == 2 ? uniform<unsigned short, 1>(data, labels, w, h, n_samples, seed, out)
                  : uniform<unsigned char, 3>(data, labels, w, h, n_samples, seed, out);
}

extern "C" unsigned ref_sample_class_weighted(int img, const void *data, const uint8_t *labels, unsigned w,
                                              unsigned h, unsigned n_samples, unsigned n_classes,
                                              const float *weights, unsigned seed, unsigned *out) {
  return img == 2 ? class_weighted<unsigned short, 1>(data, labels, w, h, n_samples, n_classes, weights, seed, out)
                  : class_weighted<unsigned char, 3>(data, labels, w, h, n_samples, n_classes, weights, seed, out);
}
