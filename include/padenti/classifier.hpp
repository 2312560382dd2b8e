// The Classifier interface, as the reference defines it (classifier.hpp:52-93).
#ifndef PADENTI_GB300_CLASSIFIER_HPP
#define PADENTI_GB300_CLASSIFIER_HPP

#include <padenti/image.hpp>
#include <padenti/tree.hpp>

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
class Classifier {
 public:
  virtual void predict(unsigned int id, const Image<ImgType, nChannels> &image, Image<int, 1> &prediction) = 0;
  virtual void predict(unsigned int id, const Image<ImgType, nChannels> &image, Image<int, 1> &prediction,
                       Image<unsigned char, 1> &mask) = 0;
  virtual void predict(const Image<ImgType, nChannels> &image, Image<float, nClasses> &prediction) = 0;
  virtual void predict(const Image<ImgType, nChannels> &image, Image<float, nClasses> &prediction,
                       Image<unsigned char, 1> &mask) = 0;
  virtual ~Classifier() {}
};

#endif
