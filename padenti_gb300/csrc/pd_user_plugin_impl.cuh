// UserPlugin: the user's computeFeature behind the kernels' plugin interface
// (no per-pixel preload; a candidate is its feature vector).  Included after the
// user source.
#pragma once

namespace pd {

// Whether the user's computeFeature is the tree-reading form (auto-context):
// it then receives the tree, and the library keeps the per-pixel node map.
template <class Im, class Tv>
inline constexpr bool kReadsTree = requires(const Im &im, const Tv &t, const feat_t *f) {
  computeFeature(im, make_int2(0, 0), t, f, 0u);
};
inline constexpr bool kUserReadsTree = kReadsTree<ImageView, TreeView>;

struct UserPlugin {
  using img_t = ::img_t;
  using feat_t = ::feat_t;
  static constexpr int kFeatDim = PD_FEAT_DIM;
  static constexpr int kChannels = PD_CHANNELS;
  static constexpr int kId = PD_PLUGIN_USER;
  static constexpr int kOrderDim = 0;            // columns ordered by feature dims 0 and 1
  static constexpr bool kTrainMapsZero = false;  // the images as given
  static constexpr bool kRtcOnly = false;
  static constexpr bool kUsesTree = kUserReadsTree;
  static constexpr int kPreWords = 1;
  struct Prep {
    ImageView im;
    TreeView tree;
    int32_t x, y;
  };
  struct __align__(16) Cand {  // one 16-byte-aligned record per tree node in prediction
    feat_t f[kFeatDim];
  };
  static PD_D void preload(const ImageRef<img_t> &, int32_t, int32_t, uint32_t *pre) { pre[0] = 0u; }
  static PD_D Prep prepare(const ImageRef<img_t> &im, int32_t x, int32_t y, const uint32_t *) {
    Prep p;
    p.im.data = im.data;
    p.im.w = im.w;
    p.im.h = im.h;
    p.im.c = kChannels;
    p.im.nodes = im.nodes;
    p.tree.lc_ = im.tree_lc;
    p.tree.post_ = im.tree_post;
    p.tree.nClasses = im.n_classes;
    p.tree.level = im.tree_level;
    p.tree.nNodes = im.tree_nodes;
    p.x = x;
    p.y = y;
    return p;
  }
  static PD_D Prep prepare(const ImageRef<img_t> &im, int32_t x, int32_t y) { return prepare(im, x, y, nullptr); }
  static PD_D Cand candidate(const feat_t *f) {
    Cand c;
#pragma unroll
    for (int k = 0; k < kFeatDim; k++) c.f[k] = f[k];
    return c;
  }
  static PD_D bool fast(const Cand &) { return true; }
  // the user's form: with the tree (auto-context) or without
  template <class Pr>
  static PD_D feat_t call(const Pr &p, const feat_t *f) {
    if constexpr (kReadsTree<decltype(p.im), decltype(p.tree)>)
      return computeFeature(p.im, make_int2(p.x, p.y), p.tree, f, (unsigned)kFeatDim);
    else
      return computeFeature(p.im, make_int2(p.x, p.y), f, (unsigned)kFeatDim);
  }
  template <bool FAST = false>
  static PD_D feat_t eval(const Prep &p, const Cand &c) {
    return call(p, c.f);
  }
  template <bool FAST = false>
  static PD_D feat_t eval_train(const Prep &p, const Cand &c) { return eval<FAST>(p, c); }
  static PD_D feat_t eval(const Prep &p, const feat_t *f) { return call(p, f); }
};

}  // namespace pd

// Read by the host after loading the module (pd_plugin_compile).
extern "C" __device__ const int pd_user_reads_tree = pd::kUserReadsTree ? 1 : 0;
extern "C" __device__ const int pd_node_rec_bytes = (int)sizeof(pd::NodeRec<pd::UserPlugin>);
