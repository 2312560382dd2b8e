// TrainingSetImage and TrainingSet -- the reference's training-set containers
// (training_set_image.hpp:38-110, training_set.hpp:39-112) with the same
// conventions: labels are one byte per pixel, 0 = unlabelled and class k stored
// as k+1; samples are pixel indices y*W+x (a multiset); per-image priors are the
// class frequencies of the labelled samples (training_set_image_impl.hpp:38-52).
// The set prior is the mean of the image priors when the set is built from a
// list of images (training_set_impl.hpp:116-133), and is updated incrementally
// by operator<< (training_set_impl.hpp:157-170).
#ifndef PADENTI_GB300_TRAINING_SET_HPP
#define PADENTI_GB300_TRAINING_SET_HPP

#include <padenti/image.hpp>

#include <cstdint>
#include <vector>

template <typename type, unsigned int nChannels>
class TrainingSetImage : public Image<type, nChannels> {
  std::vector<unsigned char> m_labels;
  std::vector<unsigned int> m_samples;
  std::vector<float> m_priors;

 public:
  TrainingSetImage(const type *data, unsigned int width, unsigned int height, const unsigned char *labels,
                   unsigned int nClasses, const unsigned int *samples, unsigned int nSamples)
      : Image<type, nChannels>(data, width, height),
        m_labels(labels, labels + (size_t)width * height),
        m_samples(samples, samples + nSamples),
        m_priors(nClasses, 0.0f) {
    std::vector<unsigned int> count(nClasses, 0u);
    unsigned int labelled = 0;
    for (unsigned int s : m_samples) {
      const unsigned char l = m_labels[s];
      if (l) {
        count[l - 1]++;
        labelled++;
      }
    }
    for (unsigned int c = 0; c < nClasses; c++) m_priors[c] = (float)count[c] / (float)labelled;
  }
  const unsigned char *getLabels() const { return m_labels.data(); }
  const unsigned int *getSamples() const { return m_samples.data(); }
  unsigned int getNSamples() const { return (unsigned int)m_samples.size(); }
  const float *getPriors() const { return m_priors.data(); }
};

template <typename type, unsigned int nChannels>
class TrainingSet {
  unsigned int m_nClasses;
  std::vector<TrainingSetImage<type, nChannels>> m_images;
  std::vector<float> m_priors;

 public:
  explicit TrainingSet(unsigned int nClasses) : m_nClasses(nClasses), m_priors(nClasses, 0.0f) {}
  // A set built at once from its images: priors = mean of the image priors.
  TrainingSet(unsigned int nClasses, const std::vector<TrainingSetImage<type, nChannels>> &images)
      : m_nClasses(nClasses), m_images(images), m_priors(nClasses, 0.0f) {
    std::vector<double> acc(nClasses, 0.0);
    for (const auto &im : m_images)
      for (unsigned int c = 0; c < nClasses; c++) acc[c] += (double)im.getPriors()[c];
    for (unsigned int c = 0; c < nClasses; c++) m_priors[c] = (float)(acc[c] / (double)m_images.size());
  }
  TrainingSet &operator<<(const TrainingSetImage<type, nChannels> &image) {
    const double n = (double)m_images.size();
    for (unsigned int c = 0; c < m_nClasses; c++)
      m_priors[c] = (float)((double)m_priors[c] * n / (n + 1.0) + (double)image.getPriors()[c] / (n + 1.0));
    m_images.push_back(image);
    return *this;
  }
  const std::vector<TrainingSetImage<type, nChannels>> &getImages() const { return m_images; }
  unsigned int getNImages() const { return (unsigned int)m_images.size(); }
  const float *getPriors() const { return m_priors.data(); }
  unsigned int getNClasses() const { return m_nClasses; }
};

#endif
