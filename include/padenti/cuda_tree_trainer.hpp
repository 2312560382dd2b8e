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

#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace padenti_gb300 {

inline void check(int rc) {
  if (rc != PD_OK) throw std::runtime_error(std::string("padenti_gb300: ") + pd_last_error());
}

template <typename ImgType, unsigned int nChannels, typename FeatType, unsigned int FeatDim, unsigned int nClasses>
pd_ctx *make_context(int plugin, int device) {
  pd_config cfg;
  cfg.plugin = plugin;
  cfg.img_type = sizeof(ImgType) == 1 ? PD_IMG_U8 : PD_IMG_U16;
  cfg.n_channels = (int)nChannels;
  cfg.feat_type = sizeof(FeatType) == 2 ? PD_FEAT_I16 : PD_FEAT_I32;
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
  const void *m_uploaded = nullptr;  // the training set currently in device memory
  size_t m_uploaded_images = 0;

 public:
  explicit CUDATreeTrainer(int plugin, int device = 0)
      : m_ctx(padenti_gb300::make_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(plugin, device)) {}
  // CLTreeTrainer(featureKernelPath): a user feature compiled at run time.
  explicit CUDATreeTrainer(const std::string &featurePath, int device = 0)
      : m_ctx(padenti_gb300::make_user_context<ImgType, nChannels, FeatType, FeatDim, nClasses>(featurePath, device)) {}
  CUDATreeTrainer(const CUDATreeTrainer &) = delete;
  CUDATreeTrainer &operator=(const CUDATreeTrainer &) = delete;
  ~CUDATreeTrainer() { pd_ctx_destroy(m_ctx); }
  pd_ctx *context() const { return m_ctx; }

  // Copies the training set into device memory (train() does it on first use).
  void upload(const TrainingSet<ImgType, nChannels> &ts) {
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
    padenti_gb300::check(pd_dataset_upload(m_ctx, &d));
    m_uploaded = &ts;
    m_uploaded_images = imgs.size();
  }

  void train(Tree<FeatType, FeatDim, nClasses> &tree, const TrainingSet<ImgType, nChannels> &ts,
             const TreeTrainerParameters<FeatType, FeatDim> &p, unsigned int startDepth,
             unsigned int endDepth) override {
    if (m_uploaded != &ts || m_uploaded_images != ts.getImages().size()) upload(ts);
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
