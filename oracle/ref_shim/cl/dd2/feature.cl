// The two-offset depth-difference feature of the benchmark configurations,
// written as a Padenti feature.cl (prototype src/padenti/padenti.hpp.in:169-177)
// so that the reference's own kernels can evaluate it: I(x + u/d(x)) - I(x + v/d(x)),
// with d(x) the centre depth (10000 when it is 0), offsets rounded half away
// from zero, and probes outside the image or on a zero depth reading 10000.
// Test infrastructure only; the same definition as the oracle's DEPTH_DIFF2.

#define PD_BG_DEPTH 10000

feat_t computeFeature(__read_only image_t image,
                      uint nChannels, uint width, uint height, int2 coords,
                      __global int *treeLeftChildren,
                      __global float *treePosteriors,
                      __read_only image2d_t imageNodesID,
                      __local feat_t *features, uint featDim)
{
  const sampler_t sampler = CLK_NORMALIZED_COORDS_FALSE | CLK_ADDRESS_CLAMP | CLK_FILTER_NEAREST;
  uint c = read_imageui(image, sampler, coords).x;
  float d = (float)(c ? (int)c : PD_BG_DEPTH);
  int2 p, q;
  p.x = coords.x + (int)round((float)ACCESS_FEATURE(features, 0, featDim) / d);
  p.y = coords.y + (int)round((float)ACCESS_FEATURE(features, 1, featDim) / d);
  q.x = coords.x + (int)round((float)ACCESS_FEATURE(features, 2, featDim) / d);
  q.y = coords.y + (int)round((float)ACCESS_FEATURE(features, 3, featDim) / d);
  bool outP = p.x < 0 || p.y < 0 || p.x >= (int)width || p.y >= (int)height;
  bool outQ = q.x < 0 || q.y < 0 || q.x >= (int)width || q.y >= (int)height;
  uint a = outP ? 0u : read_imageui(image, sampler, p).x;
  uint b = outQ ? 0u : read_imageui(image, sampler, q).x;
  int da = a ? (int)a : PD_BG_DEPTH;
  int db = b ? (int)b : PD_BG_DEPTH;
  return (feat_t)(da - db);
}
