// Learned candidate proposals: what the candidate-table kernel needs to draw a
// node's candidates from the proposal network's output, and the network's
// input encoding of a node.  No reference counterpart: the reference draws
// every candidate uniformly (kernels/hist_update.cl:62-184); here a node's
// first n_prop candidates come from a 16-component Gaussian mixture over the
// normalised (feature, threshold) space that a small MLP predicts from the
// node's statistics, and the rest are the reference's uniform MD5 candidates.
// Every candidate is still scored by the exact histogram and split kernels.
#pragma once

#include "pd_common.cuh"

namespace pd {

constexpr int kPropG = 16;    // mixture components
constexpr int kPropH = 256;   // hidden width
constexpr int kPropLayers = 3;
constexpr float kPropSMin = -6.0f, kPropSMax = 3.0f;  // clamp of the log standard deviations

PD_HD uint32_t prop_round16(uint32_t x) { return (x + 15u) / 16u * 16u; }
// Network input width for K classes: depth, log-count, the K class frequencies, zero padding.
PD_HD uint32_t prop_in_dim(uint32_t K) { return prop_round16(2u + K); }
// Output width for DY = FeatDim + 1 drawn dimensions: G logits, G x DY means, G x DY log-sds.
PD_HD uint32_t prop_out_dim(uint32_t DY) { return prop_round16((uint32_t)kPropG * (1u + 2u * DY)); }

// Input row of a node: depth / 24, log2(count + 1) / 24, class frequencies.
PD_HD float prop_input(uint32_t j, uint32_t depth, uint32_t count, const uint32_t *counts, uint32_t K) {
  if (j == 0) return (float)depth * (1.0f / 24.0f);
  if (j == 1) return log2f((float)count + 1.0f) * (1.0f / 24.0f);
  if (j - 2 < K && count) return (float)counts[j - 2] / (float)count;
  return 0.0f;
}

PD_HD uint64_t prop_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// Uniform in (0, 1) from 24 hash bits.
PD_HD float prop_unit(uint64_t h) { return ((float)(uint32_t)(h >> 40) + 0.5f) * (1.0f / 16777216.0f); }

// Where a node's proposals come from: the network output rows of the slice
// (row = slot), the mixture layout, the first n_prop candidates of a node that
// are drawn from it, and the normalisation of the drawn dimensions.
struct PropSrc {
  const float *out;  // [slots][ldo]
  uint32_t ldo, DY, n_prop;
  uint64_t seed;
  float lo[PD_MAX_FEAT_DIM + 1], span[PD_MAX_FEAT_DIM + 1];  // value = lo + (y + 1) / 2 * span
};

// The mixture component of candidate c of slot s (categorical draw on the
// softmax of the logits) and the hash stream of its draws.
PD_D uint32_t prop_component(const PropSrc &p, uint32_t slot, uint64_t stream) {
  const float *o = p.out + (size_t)slot * p.ldo;
  float m = o[0];
  for (int g = 1; g < kPropG; g++) m = fmaxf(m, o[g]);
  float tot = 0.0f;
  for (int g = 0; g < kPropG; g++) tot += __expf(o[g] - m);
  const float u = prop_unit(prop_mix(stream)) * tot;
  float acc = 0.0f;
  uint32_t pick = kPropG - 1;
  for (int g = 0; g < kPropG; g++) {
    acc += __expf(o[g] - m);
    if (u < acc) {
      pick = (uint32_t)g;
      break;
    }
  }
  return pick;
}

// Draw k of dimension d of component g, mapped back to the value range,
// rounded to the nearest integer and clamped.  The standard normal variate is
// an Irwin-Hall sum of four 16-bit uniforms of one hash, scaled to unit
// variance (support +-3.46 sd): no transcendental function per draw, and the
// same value on every device.
PD_D int32_t prop_draw(const PropSrc &p, uint32_t slot, uint32_t g, uint32_t d, uint64_t stream, uint32_t k) {
  const float *o = p.out + (size_t)slot * p.ldo;
  const float mu = o[kPropG + g * p.DY + d];
  const float s = fminf(fmaxf(o[kPropG + kPropG * p.DY + g * p.DY + d], kPropSMin), kPropSMax);
  const uint64_t h = prop_mix(stream ^ (0x51ED27ull + 2ull * k + 1ull) * 0x2545F4914F6CDD1Dull);
  const uint32_t u = (uint32_t)(h & 0xffffu) + (uint32_t)((h >> 16) & 0xffffu) + (uint32_t)((h >> 32) & 0xffffu) +
                     (uint32_t)(h >> 48);
  const float z = ((float)u - 131070.0f) * (1.7320508f / 65536.0f);
  const float y = mu + __expf(s) * z;
  float v = p.lo[d] + (y + 1.0f) * 0.5f * p.span[d];
  v = fminf(fmaxf(v, p.lo[d]), p.lo[d] + p.span[d]);
  return (int32_t)rintf(v);
}

PD_HD uint64_t prop_stream(uint64_t seed, uint32_t tree, uint32_t node, uint32_t c) {
  return prop_mix(seed ^ prop_mix(((uint64_t)tree << 40) ^ ((uint64_t)node << 12) ^ c));
}

}  // namespace pd
