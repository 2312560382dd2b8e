// ImageLoader and the label loader, the reference's image loaders
// (image_loader.hpp:35-59, cv_image_loader.hpp:28-52) without OpenCV: images are
// binary netpbm files (PGM: 8- or 16-bit grey, PPM: 8-bit RGB) in place of the
// PNG files cv::imread reads, and the colour-to-class step of
// CVRGBLabelsLoader (_rgb2label, cv_image_loader_impl.hpp:233-266) runs on the
// GPU (pd_rgb_to_labels).  The ROI loaders crop to the largest bounding
// rectangle of the components of the pixels > 0 (pd_image_roi).  loadTrainingSet()
// is the TrainingSet constructor over a directory (training_set_impl.hpp:40-112).
// Errors throw std::runtime_error.
#ifndef PADENTI_GB300_IMAGE_LOADER_HPP
#define PADENTI_GB300_IMAGE_LOADER_HPP

#include <padenti/image_sampler.hpp>
#include <padenti/training_set.hpp>
#include <padenti_gb300.h>

#include <algorithm>
#include <cctype>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

template <typename type, unsigned int nChannels>
class ImageLoader {
 public:
  virtual ~ImageLoader() {}
  virtual void load(const std::string &imagePath, type *data, unsigned int *width, unsigned int *height) = 0;
  virtual Image<type, nChannels> load(const std::string &imagePath) = 0;
};

namespace padenti_gb300 {

// A binary netpbm file: its size, channel count (1 for P5, 3 for P6), bytes per
// sample (1, or 2 stored big-endian) and samples.
struct Pnm {
  unsigned int width = 0, height = 0, channels = 0, bytes = 0;
  std::vector<unsigned char> raw;
};

inline Pnm read_pnm(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw std::runtime_error("padenti_gb300: cannot read " + path);
  std::string magic;
  f >> magic;
  unsigned long v[3];
  for (unsigned long &x : v) {
    while (f >> std::ws && f.peek() == '#') f.ignore(1 << 20, '\n');
    f >> x;
  }
  f.get();
  if ((magic != "P5" && magic != "P6") || !f) throw std::runtime_error("padenti_gb300: " + path + " is not a binary PGM/PPM");
  Pnm p;
  p.width = (unsigned int)v[0];
  p.height = (unsigned int)v[1];
  p.channels = magic == "P5" ? 1 : 3;
  p.bytes = v[2] < 256 ? 1 : 2;
  p.raw.resize((size_t)p.width * p.height * p.channels * p.bytes);
  f.read(reinterpret_cast<char *>(p.raw.data()), (std::streamsize)p.raw.size());
  if (!f) throw std::runtime_error("padenti_gb300: " + path + " is truncated");
  return p;
}

}  // namespace padenti_gb300

// CVImageLoader (cv_image_loader_impl.hpp:37-73) for PGM/PPM files.
template <typename type, unsigned int nChannels>
class PNMImageLoader : public ImageLoader<type, nChannels> {
 public:
  void load(const std::string &imagePath, type *data, unsigned int *width, unsigned int *height) override {
    const padenti_gb300::Pnm p = padenti_gb300::read_pnm(imagePath);
    if (p.channels != nChannels || p.bytes != sizeof(type)) throw "Image type different from expected one";
    *width = p.width;
    *height = p.height;
    const size_t n = (size_t)p.width * p.height * nChannels;
    for (size_t i = 0; i < n; i++)
      data[i] = p.bytes == 1 ? (type)p.raw[i] : (type)((p.raw[2 * i] << 8) | p.raw[2 * i + 1]);
  }
  Image<type, nChannels> load(const std::string &imagePath) override {
    const padenti_gb300::Pnm p = padenti_gb300::read_pnm(imagePath);
    Image<type, nChannels> img(p.width, p.height);
    unsigned int w, h;
    PNMImageLoader::load(imagePath, img.getData(), &w, &h);  // this class's, not an override's
    return img;
  }
};

// CVRGBLabelsLoader (cv_image_loader.hpp:37-52) for PPM label images; the
// colour-to-class mapping runs on the GPU.
class CUDARGBLabelsLoader : public ImageLoader<unsigned char, 1> {
  std::vector<unsigned char> m_map;
  pd_ctx *m_ctx = nullptr;

  static void check(int rc) {
    if (rc != PD_OK) throw std::runtime_error(std::string("padenti_gb300: ") + pd_last_error());
  }

 public:
  CUDARGBLabelsLoader(const unsigned char (*rgb2labelMap)[3], unsigned int nClasses, int device = 0)
      : m_map(&rgb2labelMap[0][0], &rgb2labelMap[0][0] + 3 * nClasses) {
    const pd_config cfg{PD_PLUGIN_DEPTH_DIFF2, PD_IMG_U16, 1, PD_FEAT_I32, 4, 2};  // any valid configuration
    check(pd_ctx_create(&cfg, device, &m_ctx));
  }
  CUDARGBLabelsLoader(const CUDARGBLabelsLoader &) = delete;
  CUDARGBLabelsLoader &operator=(const CUDARGBLabelsLoader &) = delete;
  ~CUDARGBLabelsLoader() override { pd_ctx_destroy(m_ctx); }

  // labels of an RGB (channels 3) or RGBA (4) image in memory
  void convert(const unsigned char *rgb, unsigned int width, unsigned int height, unsigned int channels,
               unsigned char *labels) const {
    uint8_t *out[1] = {labels};
    const uint8_t *in[1] = {rgb};
    check(pd_rgb_to_labels(m_ctx, 1, in, &width, &height, channels, m_map.data(), (uint32_t)(m_map.size() / 3), out));
  }
  void load(const std::string &imagePath, unsigned char *data, unsigned int *width, unsigned int *height) override {
    const padenti_gb300::Pnm p = padenti_gb300::read_pnm(imagePath);
    if (p.channels != 3 || p.bytes != 1) throw "Labels image type must be 8-bit RGB";
    *width = p.width;
    *height = p.height;
    convert(p.raw.data(), p.width, p.height, 3, data);
  }
  Image<unsigned char, 1> load(const std::string &imagePath) override {
    const padenti_gb300::Pnm p = padenti_gb300::read_pnm(imagePath);
    Image<unsigned char, 1> img(p.width, p.height);
    unsigned int w, h;
    CUDARGBLabelsLoader::load(imagePath, img.getData(), &w, &h);  // this class's, not an override's
    return img;
  }
};

namespace padenti_gb300 {
// Crops data (width x height pixels of `channels` values) in place to the ROI
// of its pixels > 0 (pd_image_roi); returns {x, y, width, height}.
template <typename type>
constexpr int32_t roi_img_type() {
  if constexpr (std::is_same_v<type, unsigned char>) return PD_IMG_U8;
  else if constexpr (std::is_same_v<type, unsigned short>) return PD_IMG_U16;
  else if constexpr (std::is_same_v<type, short>) return PD_IMG_I16;
  else if constexpr (std::is_same_v<type, int>) return PD_IMG_I32;
  else {
    static_assert(std::is_same_v<type, float>, "ROI loaders take uint8, uint16, int16, int32 or float images");
    return PD_IMG_F32;
  }
}

template <typename type>
std::vector<unsigned int> crop_to_roi(type *data, unsigned int *width, unsigned int *height, unsigned int channels) {
  uint32_t roi[4];
  const int rc = pd_image_roi(data, *width, *height, roi_img_type<type>(), channels, roi);
  if (rc != PD_OK) throw std::runtime_error(std::string("padenti_gb300: ") + pd_last_error());
  const size_t row = (size_t)roi[2] * channels;
  for (unsigned int y = 0; y < roi[3]; y++)
    std::memmove(data + y * row, data + ((size_t)(roi[1] + y) * *width + roi[0]) * channels, row * sizeof(type));
  *width = roi[2];
  *height = roi[3];
  return {roi[0], roi[1], roi[2], roi[3]};
}
}  // namespace padenti_gb300

// CVImageROILoader (cv_image_loader.hpp:52-65): the image cropped to the ROI of
// its pixels > 0.
template <typename type, unsigned int nChannels>
class PNMImageROILoader : public PNMImageLoader<type, nChannels> {
  unsigned int m_roiX = 0, m_roiY = 0;

 public:
  void load(const std::string &imagePath, type *data, unsigned int *width, unsigned int *height) override {
    PNMImageLoader<type, nChannels>::load(imagePath, data, width, height);
    const std::vector<unsigned int> r = padenti_gb300::crop_to_roi(data, width, height, nChannels);
    m_roiX = r[0];
    m_roiY = r[1];
  }
  Image<type, nChannels> load(const std::string &imagePath) override {
    Image<type, nChannels> full = PNMImageLoader<type, nChannels>::load(imagePath);
    unsigned int w = full.getWidth(), h = full.getHeight();
    const std::vector<unsigned int> r = padenti_gb300::crop_to_roi(full.getData(), &w, &h, nChannels);
    m_roiX = r[0];
    m_roiY = r[1];
    return Image<type, nChannels>(full.getData(), w, h);
  }
  unsigned int getRoiX() const { return m_roiX; }
  unsigned int getRoiY() const { return m_roiY; }
};

// CVRGBLabelsROILoader (cv_image_loader.hpp:69-82): the labels cropped to the ROI
// of the labelled pixels.
class CUDARGBLabelsROILoader : public CUDARGBLabelsLoader {
  unsigned int m_roiX = 0, m_roiY = 0;

 public:
  using CUDARGBLabelsLoader::CUDARGBLabelsLoader;
  void load(const std::string &imagePath, unsigned char *data, unsigned int *width, unsigned int *height) override {
    CUDARGBLabelsLoader::load(imagePath, data, width, height);
    const std::vector<unsigned int> r = padenti_gb300::crop_to_roi(data, width, height, 1u);
    m_roiX = r[0];
    m_roiY = r[1];
  }
  Image<unsigned char, 1> load(const std::string &imagePath) override {
    Image<unsigned char, 1> full = CUDARGBLabelsLoader::load(imagePath);
    unsigned int w = full.getWidth(), h = full.getHeight();
    const std::vector<unsigned int> r = padenti_gb300::crop_to_roi(full.getData(), &w, &h, 1u);
    m_roiX = r[0];
    m_roiY = r[1];
    return Image<unsigned char, 1>(full.getData(), w, h);
  }
  unsigned int getRoiX() const { return m_roiX; }
  unsigned int getRoiY() const { return m_roiY; }
};

// TrainingSet(tsPath, dataSuffix, labelsSuffix, nClasses, dataLoader,
// labelsLoader, sampler) (training_set_impl.hpp:40-112): files in name order
// (the reference takes the directory's order), pairs of different sizes skipped.
template <typename type, unsigned int nChannels>
TrainingSet<type, nChannels> loadTrainingSet(const std::string &tsPath, const std::string &dataSuffix,
                                             const std::string &labelsSuffix, unsigned int nClasses,
                                             ImageLoader<type, nChannels> &dataLoader,
                                             ImageLoader<unsigned char, 1> &labelsLoader,
                                             const ImageSampler<type, nChannels> &sampler, unsigned int maxSamples) {
  namespace fs = std::filesystem;
  std::vector<std::string> names;
  for (const auto &e : fs::directory_iterator(tsPath)) {
    const std::string n = e.path().filename().string();
    if (!e.is_directory() && n.size() >= dataSuffix.size() &&
        n.compare(n.size() - dataSuffix.size(), dataSuffix.size(), dataSuffix) == 0)
      names.push_back(n);
  }
  std::sort(names.begin(), names.end());
  std::vector<Image<type, nChannels>> images;
  std::vector<Image<unsigned char, 1>> labels;
  for (const std::string &n : names) {
    const std::string lp = tsPath + "/" + n.substr(0, n.size() - dataSuffix.size()) + labelsSuffix;
    if (!fs::exists(lp)) continue;
    images.push_back(dataLoader.load(tsPath + "/" + n));
    labels.push_back(labelsLoader.load(lp));
  }
  return sampledTrainingSet(nClasses, images, labels, sampler, maxSamples);
}

#endif
