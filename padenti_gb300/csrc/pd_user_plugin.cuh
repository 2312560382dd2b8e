// A user feature plugin compiled at run time (NVRTC): the CUDA counterpart of
// Padenti's feature.cl, whose computeFeature the reference compiles into its
// kernels (padenti.hpp.in:169-187, kernels/hist_update.cl:33).  The user source
// defines
//   __device__ feat_t computeFeature(const pd::ImageView &img, int2 coords,
//                                    const feat_t *features, unsigned featDim);
// or, to read the tree (auto-context features),
//   __device__ feat_t computeFeature(const pd::ImageView &img, int2 coords, const pd::TreeView &tree,
//                                    const feat_t *features, unsigned featDim);
// with img_t, feat_t, PD_FEAT_DIM and PD_CHANNELS defined before it from the
// context's configuration (as the reference generates feat_type.cl).  UserPlugin
// adapts it to the kernels' plugin interface.
#pragma once

#include "pd_plugins.cuh"

namespace pd {

// The image a feature reads: interleaved [H][W][C]; read() returns 0 outside
// the W x H pixels (the reference reads through CLK_ADDRESS_CLAMP).  nodeID(x, y)
// is the node that pixel (x, y) occupies in the tree being trained or evaluated
// (the reference's imageNodesID), kept for features that define PD_NODE_MAP;
// 0 outside the image or when no map is kept.
struct ImageView {
  const img_t *data;
  int32_t w, h, c;
  const int32_t *nodes;
  __device__ __forceinline__ img_t read(int x, int y, int ch) const {
    if ((uint32_t)x >= (uint32_t)w || (uint32_t)y >= (uint32_t)h) return (img_t)0;
    return ldg(data + ((size_t)((uint32_t)y * (uint32_t)w + (uint32_t)x)) * (uint32_t)c + ch);
  }
  __device__ __forceinline__ int nodeID(int x, int y) const {
    if (!nodes || (uint32_t)x >= (uint32_t)w || (uint32_t)y >= (uint32_t)h) return 0;
    return ldg(nodes + (size_t)((uint32_t)y * (uint32_t)w + (uint32_t)x));
  }
};

// The tree being trained or evaluated, as a feature sees it at the level of
// the node map (the root's level is 0): the splits of the nodes above that
// level and the posteriors ([node][nClasses]) of the nodes down to it -- the
// part of the tree that is the same while it is trained and when it predicts.
// (The reference passes its raw treeLeftChildren / treePosteriors buffers, whose
// entries at and below the level being trained differ between the two.)
struct TreeView {
  const int32_t *lc_;
  const float *post_;
  unsigned nClasses;
  int level;    // of the node map
  int nNodes;   // 2^depth - 1
  __device__ __forceinline__ static int nodeLevel(int node) { return 31 - __clz(node + 1); }
  // left child (the right one is left + 1); -1 for a leaf, a node at or below
  // the map's level, or a node outside the tree
  __device__ __forceinline__ int leftChild(int node) const {
    if (node < 0 || node >= nNodes || nodeLevel(node) >= level) return -1;
    return ldg(lc_ + node);
  }
  // posterior of class k at node; 0 below the map's level or outside the tree
  __device__ __forceinline__ float posterior(int node, int k) const {
    if (node < 0 || node >= nNodes || nodeLevel(node) > level || k < 0 || (unsigned)k >= nClasses) return 0.0f;
    return ldg(post_ + (size_t)node * nClasses + k);
  }
};

}  // namespace pd
