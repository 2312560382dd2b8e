// The channel-difference feature of the RGB configuration, written as a
// Padenti feature.cl (prototype src/padenti/padenti.hpp.in:169-177) so that
// the reference's own kernels can evaluate it: I_c1(x + u) - I_c2(x + v),
// features (c1, c2, ux, uy, vx, vy), channels clamped to [0, 2], probes outside
// the image reading 0.  Test infrastructure only; the same definition as the
// oracle's CHANNEL_DIFF.

feat_t computeFeature(__read_only image_t image,
                      uint nChannels, uint width, uint height, int2 coords,
                      __global int *treeLeftChildren,
                      __global float *treePosteriors,
                      __read_only image2d_t imageNodesID,
                      __local feat_t *features, uint featDim)
{
  const sampler_t sampler = CLK_NORMALIZED_COORDS_FALSE | CLK_ADDRESS_CLAMP | CLK_FILTER_NEAREST;
  int c1 = ACCESS_FEATURE(features, 0, featDim);
  int c2 = ACCESS_FEATURE(features, 1, featDim);
  c1 = c1 < 0 ? 0 : (c1 > 2 ? 2 : c1);
  c2 = c2 < 0 ? 0 : (c2 > 2 ? 2 : c2);
  int2 p, q;
  p.x = coords.x + ACCESS_FEATURE(features, 2, featDim);
  p.y = coords.y + ACCESS_FEATURE(features, 3, featDim);
  q.x = coords.x + ACCESS_FEATURE(features, 4, featDim);
  q.y = coords.y + ACCESS_FEATURE(features, 5, featDim);
  uint4 vp = read_imageui(image, sampler, p);  // outside the image: the border colour, 0 in x, y, z
  uint4 vq = read_imageui(image, sampler, q);
  int a = (int)(c1 == 0 ? vp.x : (c1 == 1 ? vp.y : vp.z));
  int b = (int)(c2 == 0 ? vq.x : (c2 == 1 ? vq.y : vq.z));
  return (feat_t)(a - b);
}
