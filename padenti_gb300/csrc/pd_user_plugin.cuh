// A user feature plugin compiled at run time (NVRTC): the CUDA counterpart of
// Padenti's feature.cl, whose computeFeature the reference compiles into its
// kernels (padenti.hpp.in:169-187, kernels/hist_update.cl:33).  The user source
// defines
//   __device__ feat_t computeFeature(const pd::ImageView &img, int2 coords,
//                                    const feat_t *features, unsigned featDim);
// with img_t, feat_t, PD_FEAT_DIM and PD_CHANNELS defined before it from the
// context's configuration (as the reference generates feat_type.cl).  UserPlugin
// adapts it to the kernels' plugin interface.
#pragma once

#include "pd_plugins.cuh"

namespace pd {

// The image a feature reads: interleaved [H][W][C]; read() returns 0 outside
// the W x H pixels (the reference reads through CLK_ADDRESS_CLAMP).
struct ImageView {
  const img_t *data;
  int32_t w, h, c;
  __device__ __forceinline__ img_t read(int x, int y, int ch) const {
    if ((uint32_t)x >= (uint32_t)w || (uint32_t)y >= (uint32_t)h) return (img_t)0;
    return ldg(data + ((size_t)((uint32_t)y * (uint32_t)w + (uint32_t)x)) * (uint32_t)c + ch);
  }
};

}  // namespace pd
