// ImageSampler and its two implementations, the reference's pixel samplers
// (image_sampler.hpp:31-73, uniform_image_sampler_impl.hpp:34-63,
// classweighted_image_sampler_impl.hpp:25-120), sampling on the GPU through
// pd_sample: CUDAUniformImageSampler and CUDAClassWeightedImageSampler return the
// samples the reference's samplers return (same CRC-32 ^ seed seeding of
// MT19937, same draws, sorted).  sample() takes one image, as the reference's
// TrainingSet constructor calls it (training_set_impl.hpp:106); sampleBatch()
// takes many images of any sizes in one call.  Errors throw std::runtime_error.
#ifndef PADENTI_GB300_IMAGE_SAMPLER_HPP
#define PADENTI_GB300_IMAGE_SAMPLER_HPP

#include <padenti/training_set.hpp>
#include <padenti_gb300.h>

#include <stdexcept>
#include <string>
#include <vector>

template <typename type, unsigned int nChannels>
class ImageSampler {
 protected:
  unsigned int m_nSamples;
  unsigned int m_seed;

 public:
  ImageSampler(unsigned int nSamples, unsigned int seed = 0) : m_nSamples(nSamples), m_seed(seed) {}
  virtual ~ImageSampler() {}
  virtual unsigned int sample(const type *data, const unsigned char *labels, unsigned int width,
                              unsigned int height, unsigned int *samples) const = 0;
};

namespace padenti_gb300 {

// The sampler's GPU side: a context of its own and the pd_sampler arguments.
template <typename type, unsigned int nChannels>
class GpuSampler {
  pd_ctx *m_ctx = nullptr;
  pd_sampler m_s{};
  std::vector<float> m_weights;

  static void check(int rc) {
    if (rc != PD_OK) throw std::runtime_error(std::string("padenti_gb300: ") + pd_last_error());
  }

 public:
  GpuSampler(int kind, unsigned int nSamples, unsigned int seed, unsigned int nClasses, const float *weights,
             int device) {
    if (weights) m_weights.assign(weights, weights + nClasses);
    m_s.kind = kind;
    m_s.n_samples = nSamples;
    m_s.seed = seed;
    m_s.n_classes = nClasses;
    m_s.weights = weights ? m_weights.data() : nullptr;
    m_s.pixel_bytes = (uint32_t)(sizeof(type) * nChannels);
    const pd_config cfg{PD_PLUGIN_DEPTH_DIFF2, PD_IMG_U16, 1, PD_FEAT_I32, 4, 2};  // any valid configuration
    check(pd_ctx_create(&cfg, device, &m_ctx));
  }
  GpuSampler(const GpuSampler &) = delete;
  GpuSampler &operator=(const GpuSampler &) = delete;
  ~GpuSampler() { pd_ctx_destroy(m_ctx); }

  unsigned int stride() const {
    uint32_t s = 0;
    check(pd_sampler_stride(&m_s, &s));
    return s;
  }
  // samples of image i at samples + i * stride(); returns the counts
  std::vector<unsigned int> sampleBatch(const std::vector<const type *> &data,
                                        const std::vector<const unsigned char *> &labels,
                                        const std::vector<unsigned int> &widths,
                                        const std::vector<unsigned int> &heights, unsigned int *samples) const {
    const uint32_t n = (uint32_t)data.size();
    if (labels.size() != n || widths.size() != n || heights.size() != n)
      throw std::runtime_error("padenti_gb300: sampleBatch needs one label image and size per image");
    std::vector<const void *> im(data.begin(), data.end());
    std::vector<uint32_t> w(widths.begin(), widths.end()), h(heights.begin(), heights.end()), c(n);
    check(pd_sample(m_ctx, &m_s, n, im.data(), labels.data(), w.data(), h.data(), stride(), samples, c.data()));
    return std::vector<unsigned int>(c.begin(), c.end());
  }
  unsigned int sampleOne(const type *data, const unsigned char *labels, unsigned int width, unsigned int height,
                         unsigned int *samples) const {
    return sampleBatch({data}, {labels}, {width}, {height}, samples)[0];
  }
};

}  // namespace padenti_gb300

template <typename type, unsigned int nChannels>
class CUDAUniformImageSampler : public ImageSampler<type, nChannels> {
  padenti_gb300::GpuSampler<type, nChannels> m_gpu;

 public:
  CUDAUniformImageSampler(unsigned int nSamples, unsigned int seed = 0, int device = 0)
      : ImageSampler<type, nChannels>(nSamples, seed), m_gpu(PD_SAMPLER_UNIFORM, nSamples, seed, 0, nullptr, device) {}
  unsigned int sample(const type *data, const unsigned char *labels, unsigned int width, unsigned int height,
                      unsigned int *samples) const override {
    return m_gpu.sampleOne(data, labels, width, height, samples);
  }
  const padenti_gb300::GpuSampler<type, nChannels> &gpu() const { return m_gpu; }
};

template <typename type, unsigned int nChannels>
class CUDAClassWeightedImageSampler : public ImageSampler<type, nChannels> {
  padenti_gb300::GpuSampler<type, nChannels> m_gpu;

 public:
  CUDAClassWeightedImageSampler(unsigned int nSamples, unsigned int nClasses, unsigned int seed = 0, int device = 0)
      : ImageSampler<type, nChannels>(nSamples, seed),
        m_gpu(PD_SAMPLER_CLASS_WEIGHTED, nSamples, seed, nClasses, nullptr, device) {}
  CUDAClassWeightedImageSampler(unsigned int nSamples, unsigned int nClasses, const float *weights,
                                unsigned int seed = 0, int device = 0)
      : ImageSampler<type, nChannels>(nSamples, seed),
        m_gpu(PD_SAMPLER_CLASS_WEIGHTED, nSamples, seed, nClasses, weights, device) {}
  // samples buffers must hold gpu().stride() entries (the sum of the class buckets)
  unsigned int sample(const type *data, const unsigned char *labels, unsigned int width, unsigned int height,
                      unsigned int *samples) const override {
    return m_gpu.sampleOne(data, labels, width, height, samples);
  }
  const padenti_gb300::GpuSampler<type, nChannels> &gpu() const { return m_gpu; }
};

// The TrainingSet constructor over a directory (training_set_impl.hpp:40-112)
// without the image loaders: images and labels in memory, every image sampled
// by `sampler`; pairs of different sizes are skipped, as the reference skips them.
template <typename type, unsigned int nChannels>
TrainingSet<type, nChannels> sampledTrainingSet(unsigned int nClasses,
                                                const std::vector<Image<type, nChannels>> &images,
                                                const std::vector<Image<unsigned char, 1>> &labels,
                                                const ImageSampler<type, nChannels> &sampler,
                                                unsigned int maxSamples) {
  std::vector<TrainingSetImage<type, nChannels>> out;
  std::vector<unsigned int> buf(maxSamples);
  for (size_t i = 0; i < images.size() && i < labels.size(); i++) {
    if (images[i].getWidth() != labels[i].getWidth() || images[i].getHeight() != labels[i].getHeight()) continue;
    const unsigned int n = sampler.sample(images[i].getData(), labels[i].getData(), images[i].getWidth(),
                                          images[i].getHeight(), buf.data());
    out.emplace_back(images[i].getData(), images[i].getWidth(), images[i].getHeight(), labels[i].getData(), nClasses,
                     buf.data(), n);
  }
  return TrainingSet<type, nChannels>(nClasses, out);
}

#endif
