// A feature that reads the tree (auto-context), written as a Padenti feature.cl
// (prototype src/padenti/padenti.hpp.in:169-177) so that the reference's own
// kernels evaluate it with their treeLeftChildren, treePosteriors and
// imageNodesID arguments.  With n1 the node of pixel (x+f0, y+f1) (0 outside:
// the sampler's border) and k = f2 mod nClasses:
//   (int)(posterior(n1, k) * 1000) + (leftChild(n1) >= 0 ? 2000 : 0)
//     + (I(x+f3, y) - I(x, y)) / 16 + n1 % 5,    I = 0 outside the image,
// where the tree is read as seen from the level L of the node map: leftChild is
// -1 for nodes at level >= L, posterior 0 for nodes below L.  Every pixel whose
// feature the kernels evaluate sits on an inner node of level L (the frontier
// while training, the level being advanced while predicting), so L is the level
// of the pixel's own node.  The reference's prototype carries no class count: a
// feature.cl fixes it (3, the tests' count).  Test infrastructure only; the
// same definition as the oracle's OR_PLUGIN_AUTO_CONTEXT.

#define PD_N_CLASSES 3

static int pd_node_level(int n)
{
  int l = 0;
  for (uint v = (uint)n + 1u; v > 1u; v >>= 1) l++;
  return l;
}

feat_t computeFeature(__read_only image_t image,
                      uint nChannels, uint width, uint height, int2 coords,
                      __global int *treeLeftChildren,
                      __global float *treePosteriors,
                      __read_only image2d_t imageNodesID,
                      __local feat_t *features, uint featDim)
{
  const sampler_t sampler = CLK_NORMALIZED_COORDS_FALSE | CLK_ADDRESS_CLAMP | CLK_FILTER_NEAREST;
  int level = pd_node_level(read_imagei(imageNodesID, sampler, coords).x);
  int2 p, q;
  p.x = coords.x + ACCESS_FEATURE(features, 0, featDim);
  p.y = coords.y + ACCESS_FEATURE(features, 1, featDim);
  int n1 = read_imagei(imageNodesID, sampler, p).x;
  int k = ((ACCESS_FEATURE(features, 2, featDim) % PD_N_CLASSES) + PD_N_CLASSES) % PD_N_CLASSES;
  int l1 = pd_node_level(n1);
  float pv = l1 <= level ? treePosteriors[n1 * PD_N_CLASSES + k] : 0.0f;
  int inner = (l1 < level && treeLeftChildren[n1] >= 0) ? 2000 : 0;
  q.x = coords.x + ACCESS_FEATURE(features, 3, featDim);
  q.y = coords.y;
  bool outQ = q.x < 0 || q.x >= (int)width;
  int a = outQ ? 0 : (int)read_imageui(image, sampler, q).x;
  int b = (int)read_imageui(image, sampler, coords).x;
  return (feat_t)((int)(pv * 1000.0f) + inner + (a - b) / 16 + n1 % 5);
}
