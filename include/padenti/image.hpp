// Image<type, nChannels>: an owned, contiguous pixel buffer -- the reference's
// image container (image.hpp:34-111): interleaved row-major [H][W][C] for
// inputs; the classifier's float posterior image is planar [C][H][W]
// (cl_classifier_impl.hpp:533-552).
#ifndef PADENTI_GB300_IMAGE_HPP
#define PADENTI_GB300_IMAGE_HPP

#include <algorithm>
#include <cstddef>
#include <vector>

template <typename type, unsigned int nChannels>
class Image {
 protected:
  std::vector<type> m_buf;
  unsigned int m_width = 0;
  unsigned int m_height = 0;

 public:
  Image() = default;
  Image(unsigned int width, unsigned int height)
      : m_buf((size_t)width * height * nChannels), m_width(width), m_height(height) {}
  Image(const type *data, unsigned int width, unsigned int height) : Image(width, height) {
    std::copy(data, data + m_buf.size(), m_buf.begin());
  }
  type *getData() const { return const_cast<type *>(m_buf.data()); }
  unsigned int getWidth() const { return m_width; }
  unsigned int getHeight() const { return m_height; }
};

#endif
