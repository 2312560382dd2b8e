// CUDATreeTrainer and CUDAClassifier: the GB300 counterparts of CLTreeTrainer
// (cl_tree_trainer.hpp:115-120) and CLClassifier (cl_classifier.hpp:81-94),
// forwarding to the C ABI of libpadenti_gb300 (padenti_gb300.h).  Like the
// OpenCL classes, they take the user's feature: the path of a feature.cu (or of
// the directory holding it) whose computeFeature is compiled at run time for
// the template parameters' types (pd_plugin_compile).  They also take one of the
// plugins compiled into the library (PD_PLUGIN_*), whose types the template
// parameters must match (pd_ctx_create checks them).  Errors throw
// std::runtime_error with the library's message (the reference throws
// cl::Error / std::string).
#ifndef PADENTI_GB300_CUDA_TREE_TRAINER_HPP
#define PADENTI_GB300_CUDA_TREE_TRAINER_HPP

#include <padenti/classifier.hpp>
#include <padenti/tree_trainer.hpp>
#include <padenti_gb300.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

namespace padenti_gb300 {

inline void check(int rc) {
  if (rc != PD_OK) throw std::runtime_error(std::string("padenti_gb300: ") + pd_last_error());
}

// ImgType / FeatType -> the library's type codes.  Types the library has no
// kernels for do not compile (the reference's type traits throw at run time,
// cl_img_fmt_traits.hpp:25-280, cl_feat_fmt_traits.hpp:25-109).
template <typename ImgType>
constexpr int32_t img_type_code() {
  if constexpr (std::is_same_v<ImgType, unsigned char>) return PD_IMG_U8;
  else if constexpr (std::is_same_v<ImgType, unsigned short>) return PD_IMG_U16;
  else if constexpr (std::is_same_v<ImgType, short>) return PD_IMG_I16;
  else if constexpr (std::is_same_v<ImgType, int>) return PD_IMG_I32;
  else {
    static_assert(std::is_same_v<ImgType, float>,
                  "padenti_gb300: ImgType must be unsigned char, unsigned short, short, int or float");
    return PD_IMG_F32;
  }
}
template <typename FeatType>
constexpr int32_t feat_type_code() {
  if constexpr (std::is_same_v<FeatType, short>) return PD_FEAT_I16;
  else {
    static_assert(std::is_same_v<FeatType, int>, "padenti_gb300: FeatType must be short or int");
    return PD_FEAT_I32;
  }
}

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
pd_ctx *make_context(int plugin, int device) {
  pd_config cfg;
  cfg.plugin = plugin;
  cfg.img_type = img_type_code<ImgType>();
  cfg.n_channels = (int)nChannels;
  cfg.feat_type = feat_type_code<FeatType>();
  cfg.feat_dim = (int)FeatDim;
  cfg.n_classes = (int)nClasses;
  pd_ctx *ctx = nullptr;
  check(pd_ctx_create(&cfg, device, &ctx));
  return ctx;
}

// The source of a user feature: the file itself, or feature.cu in a directory
// (the reference takes the directory of feature.cl).
inline std::string read_feature_source(const std::string &path) {
  std::ifstream f(path + "/feature.cu");
  if (!f) f.open(path);
  if (!f) throw std::runtime_error("padenti_gb300: cannot read the feature source " + path);
  std::stringstream s;
  s << f.rdbuf();
  return s.str();
}

// The reference's useCPU flag (cl_tree_trainer.hpp:115, cl_classifier.hpp:81)
// picks an OpenCL CPU device; this library has no CPU path, so useCPU = true is
// refused and useCPU = false means GPU 0.
inline int device_of(bool useCPU) {
  if (useCPU) throw std::runtime_error("padenti_gb300: useCPU=true: this library runs on CUDA GPUs only");
  return 0;
}

// Content fingerprint of a range of bytes (64-bit multiply-xorshift over 8-byte
// words, on several threads for large ranges): the trainer re-uploads a training
// set whose images, labels or samples changed in place.
inline uint64_t fingerprint(const void *data, size_t n) {
  const unsigned char *p = static_cast<const unsigned char *>(data);
  auto part = [p](size_t b, size_t e) {
    uint64_t h = 0x9e3779b97f4a7c15ull ^ (e - b);
    size_t i = b;
    for (; i + 8 <= e; i += 8) {
      uint64_t w;
      std::memcpy(&w, p + i, 8);
      h = (h ^ w) * 0xff51afd7ed558ccdull;
      h ^= h >> 32;
    }
    for (; i < e; i++) h = (h ^ p[i]) * 0xc4ceb9fe1a85ec53ull;
    return h;
  };
  const unsigned nt = n < (64u << 20) ? 1u : std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  std::vector<uint64_t> hs(nt);
  std::vector<std::thread> th;
  const size_t step = (n / nt + 7) / 8 * 8;
  for (unsigned t = 0; t < nt; t++) {
    const size_t b = std::min(n, t * step), e = t + 1 == nt ? n : std::min(n, (t + 1) * step);
    if (t + 1 == nt) hs[t] = part(b, e);
    else th.emplace_back([&, t, b, e] { hs[t] = part(b, e); });
  }
  for (auto &x : th) x.join();
  uint64_t h = n;
  for (uint64_t x : hs) h = (h ^ x) * 0x9e3779b97f4a7c15ull + (h >> 29);
  return h;
}

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
pd_ctx *make_user_context(const std::string &feature_path, int device) {
  pd_ctx *ctx = make_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(PD_PLUGIN_USER, device);
  const int rc = pd_plugin_compile(ctx, read_feature_source(feature_path).c_str());
  if (rc != PD_OK) {
    const std::string msg = pd_last_error();
    pd_ctx_destroy(ctx);
    throw std::runtime_error("padenti_gb300: " + msg);
  }
  return ctx;
}

}  // namespace padenti_gb300

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
class CUDATreeTrainer : public TreeTrainer<ImgType, nChannels, FeatType, FeatDim, nClasses> {
  pd_ctx *m_ctx;
  bool m_have_upload = false;
  std::vector<uint64_t> m_uploaded;  // content key of the training set in device memory

  static std::vector<uint64_t> content_key(const TrainingSet<ImgType, nChannels> &ts) {
    std::vector<uint64_t> k;
    for (const auto &im : ts.getImages()) {
      const size_t n = (size_t)im.getWidth() * im.getHeight();
      k.push_back((uint64_t)im.getWidth() | ((uint64_t)im.getHeight() << 32));
      k.push_back(im.getNSamples());
      k.push_back(padenti_gb300::fingerprint(im.getData(), n * nChannels * sizeof(ImgType)));
      k.push_back(padenti_gb300::fingerprint(im.getLabels(), n));
      k.push_back(padenti_gb300::fingerprint(im.getSamples(), (size_t)im.getNSamples() * sizeof(unsigned int)));
    }
    return k;
  }

 public:
  explicit CUDATreeTrainer(int plugin, int device = 0)
      : m_ctx(padenti_gb300::make_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(plugin, device)) {}
  // CLTreeTrainer(featureKernelPath): a user feature compiled at run time.
  explicit CUDATreeTrainer(const std::string &featurePath, int device = 0)
      : m_ctx(padenti_gb300::make_user_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(featurePath, device)) {}
  // CLTreeTrainer(featureKernelPath, useCPU) (cl_tree_trainer.hpp:115).
  CUDATreeTrainer(const std::string &featurePath, bool useCPU)
      : CUDATreeTrainer(featurePath, padenti_gb300::device_of(useCPU)) {}
  CUDATreeTrainer(const CUDATreeTrainer &) = delete;
  CUDATreeTrainer &operator=(const CUDATreeTrainer &) = delete;
  ~CUDATreeTrainer() { pd_ctx_destroy(m_ctx); }
  pd_ctx *context() const { return m_ctx; }

  // Copies the training set into device memory (train() does it when the set's
  // content differs from the one uploaded last).
  void upload(const TrainingSet<ImgType, nChannels> &ts) { upload(ts, content_key(ts)); }

 private:
  void upload(const TrainingSet<ImgType, nChannels> &ts, std::vector<uint64_t> key) {
    const auto &imgs = ts.getImages();
    std::vector<uint64_t> pix_off, lab_off, samp_off(1, 0);
    std::vector<uint32_t> w, h, samples;
    std::vector<ImgType> pixels;
    std::vector<uint8_t> labels;
    for (const auto &im : imgs) {
      const size_t n = (size_t)im.getWidth() * im.getHeight();
      pix_off.push_back(pixels.size() * sizeof(ImgType));
      lab_off.push_back(labels.size());
      w.push_back(im.getWidth());
      h.push_back(im.getHeight());
      pixels.insert(pixels.end(), im.getData(), im.getData() + n * nChannels);
      labels.insert(labels.end(), im.getLabels(), im.getLabels() + n);
      samples.insert(samples.end(), im.getSamples(), im.getSamples() + im.getNSamples());
      samp_off.push_back(samples.size());
    }
    pd_dataset_desc d;
    d.n_images = (uint32_t)imgs.size();
    d.pixels = pixels.data();
    d.pix_off = pix_off.data();
    d.width = w.data();
    d.height = h.data();
    d.labels = labels.data();
    d.lab_off = lab_off.data();
    d.samples = samples.data();
    d.samp_off = samp_off.data();
    m_have_upload = false;
    padenti_gb300::check(pd_dataset_upload(m_ctx, &d));
    m_uploaded = std::move(key);
    m_have_upload = true;
  }

 public:

  void train(Tree<FeatType, FeatDim, nClasses> &tree, const TrainingSet<ImgType, nChannels> &ts,
             const TreeTrainerParameters<FeatType, FeatDim> &p, unsigned int startDepth,
             unsigned int endDepth) override {
    std::vector<uint64_t> key = content_key(ts);
    if (!m_have_upload || key != m_uploaded) upload(ts, std::move(key));
    pd_train_params q = {};
    q.n_features = p.nFeatures;
    q.n_thresholds = p.nThresholds;
    for (unsigned int i = 0; i < FeatDim; i++) {
      q.feat_low[i] = (int32_t)p.featLowBounds[i];
      q.feat_up[i] = (int32_t)p.featUpBounds[i];
    }
    q.thr_low = (int32_t)p.thrLowBound;
    q.thr_up = (int32_t)p.thrUpBound;
    q.per_leaf_samples_thr = p.perLeafSamplesThr;
    padenti_gb300::check(pd_train_tree(m_ctx, &q, tree.getID(), startDepth, endDepth, ts.getPriors(),
                                       tree.getLeftChildren(), tree.getFeatures(), tree.getThresholds(),
                                       tree.getPosteriors()));
  }

  pd_train_stats stats() const {
    pd_train_stats s;
    padenti_gb300::check(pd_train_get_stats(m_ctx, &s));
    return s;
  }
};

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
class CUDAClassifier : public Classifier<ImgType, nChannels, FeatType, FeatDim, nClasses> {
  pd_ctx *m_ctx;

 public:
  explicit CUDAClassifier(int plugin, int device = 0)
      : m_ctx(padenti_gb300::make_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(plugin, device)) {}
  // CLClassifier(featureKernelPath): a user feature compiled at run time.
  explicit CUDAClassifier(const std::string &featurePath, int device = 0)
      : m_ctx(padenti_gb300::make_user_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(featurePath, device)) {}
  // CLClassifier(featureKernelPath, useCPU) (cl_classifier.hpp:81).
  CUDAClassifier(const std::string &featurePath, bool useCPU)
      : CUDAClassifier(featurePath, padenti_gb300::device_of(useCPU)) {}
  CUDAClassifier(const CUDAClassifier &) = delete;
  CUDAClassifier &operator=(const CUDAClassifier &) = delete;
  ~CUDAClassifier() { pd_ctx_destroy(m_ctx); }

  CUDAClassifier &operator<<(const Tree<FeatType, FeatDim, nClasses> &tree) {
    padenti_gb300::check(pd_forest_add_tree(m_ctx, tree.getDepth(), tree.getLeftChildren(), tree.getFeatures(),
                                            tree.getThresholds(), tree.getPosteriors()));
    return *this;
  }
  void predict(unsigned int id, const Image<ImgType, nChannels> &image, Image<int, 1> &prediction) override {
    padenti_gb300::check(pd_predict_leaf(m_ctx, id, image.getData(), image.getWidth(), image.getHeight(), nullptr,
                                         prediction.getData()));
  }
  void predict(unsigned int id, const Image<ImgType, nChannels> &image, Image<int, 1> &prediction,
               Image<unsigned char, 1> &mask) override {
    padenti_gb300::check(pd_predict_leaf(m_ctx, id, image.getData(), image.getWidth(), image.getHeight(),
                                         mask.getData(), prediction.getData()));
  }
  void predict(const Image<ImgType, nChannels> &image, Image<float, nClasses> &prediction) override {
    padenti_gb300::check(pd_predict_posterior(m_ctx, image.getData(), image.getWidth(), image.getHeight(), nullptr,
                                              prediction.getData()));
  }
  void predict(const Image<ImgType, nChannels> &image, Image<float, nClasses> &prediction,
               Image<unsigned char, 1> &mask) override {
    padenti_gb300::check(pd_predict_posterior(m_ctx, image.getData(), image.getWidth(), image.getHeight(),
                                              mask.getData(), prediction.getData()));
  }
};

#endif
