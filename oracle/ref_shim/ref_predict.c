/*
 * The reference's own traversal and posterior kernels
 * (src/padenti/kernels/predict.cl:36-85 predict, :88-117 computePosterior),
 * compiled as C through cl/cl_shim.h and executed over their NDRange on the
 * host.  TEST INFRASTRUCTURE ONLY.
 *
 * NDRange as both callers launch it (cl_tree_trainer_impl_traverse_ts.hpp:229-240,
 * cl_classifier_impl.hpp:498-516): the image padded up to multiples of 16 in each
 * direction, local (16, 16); featuresBuff holds 256 * featDim feat_t
 * (cl_tree_trainer_impl_init.hpp:247).  Neither kernel uses barriers or shares
 * local memory between work-items, so a loop over the work-items executes the
 * NDRange exactly.
 */
#include "cl_shim.h"

#define computeFeature ref_pred_compute_feature
#include <predict_c.cl>
#undef computeFeature

#include <stdlib.h>

#define RP_WG 16

static uint rp_padded(uint n) { return (n % RP_WG) ? n + RP_WG - n % RP_WG : n; }

/* One launch of `predict`: nodes_out[p] = the child of nodes_in[p] that pixel p
 * goes to (or nodes_in[p] at a leaf) for pixels with mask[p] != 0; other pixels
 * of nodes_out are left as they are.  Tree arrays as the reference stores them
 * (features [node][featDim]); feature values and thresholds given as int32 and
 * converted to feat_t. */
int ref_predict_step(int img_type, uint n_channels, const void *pixels, uint width, uint height,
                     const uint8_t *mask, const int32_t *left_child, const int32_t *features, uint feat_dim,
                     const int32_t *thresholds, uint n_nodes, const float *posteriors, const int32_t *nodes_in,
                     int32_t *nodes_out) {
  cl_shim_image img = {(void *)pixels, img_type == 1 ? CL_SHIM_U8 : CL_SHIM_U16, width, height, n_channels};
  cl_shim_image msk = {(void *)mask, CL_SHIM_U8, width, height, 1};
  cl_shim_image nin = {(void *)nodes_in, CL_SHIM_I32, width, height, 1};
  cl_shim_image nout = {(void *)nodes_out, CL_SHIM_I32, width, height, 1};
  feat_t *f = (feat_t *)malloc((size_t)n_nodes * feat_dim * sizeof(feat_t) + 1);
  feat_t *t = (feat_t *)malloc((size_t)n_nodes * sizeof(feat_t) + 1);
  feat_t *buf = (feat_t *)calloc((size_t)RP_WG * RP_WG * feat_dim + 1, sizeof(feat_t));
  if (!f || !t || !buf) {
    free(f), free(t), free(buf);
    return -3;
  }
  for (size_t i = 0; i < (size_t)n_nodes * feat_dim; i++) f[i] = (feat_t)features[i];
  for (size_t i = 0; i < n_nodes; i++) t[i] = (feat_t)thresholds[i];
  const uint gw = rp_padded(width), gh = rp_padded(height);
  cl_shim_lsize[0] = RP_WG;
  cl_shim_lsize[1] = RP_WG;
  cl_shim_gsize[0] = gw;
  cl_shim_gsize[1] = gh;
  for (uint y = 0; y < gh; y++)
    for (uint x = 0; x < gw; x++) {
      cl_shim_wi.gid[0] = x;
      cl_shim_wi.gid[1] = y;
      cl_shim_wi.lid[0] = x % RP_WG;
      cl_shim_wi.lid[1] = y % RP_WG;
      predict(&img, &msk, n_channels, width, height, (int *)left_child, f, feat_dim, t, (float *)posteriors, &nin,
              &nout, buf);
    }
  free(f), free(t), free(buf);
  return 0;
}

/* One launch of `computePosterior`: out[l][y][x] = posteriors[node(x,y)][l] for
 * masked pixels (others left as they are), planar [nClasses][H][W]. */
void ref_compute_posterior(const int32_t *nodes, uint width, uint height, uint n_classes, const float *posteriors,
                           const uint8_t *mask, float *out) {
  cl_shim_image nd = {(void *)nodes, CL_SHIM_I32, width, height, 1};
  cl_shim_image msk = {(void *)mask, CL_SHIM_U8, width, height, 1};
  const uint gw = rp_padded(width), gh = rp_padded(height);
  cl_shim_lsize[0] = RP_WG;
  cl_shim_lsize[1] = RP_WG;
  cl_shim_gsize[0] = gw;
  cl_shim_gsize[1] = gh;
  for (uint y = 0; y < gh; y++)
    for (uint x = 0; x < gw; x++) {
      cl_shim_wi.gid[0] = x;
      cl_shim_wi.gid[1] = y;
      cl_shim_wi.lid[0] = x % RP_WG;
      cl_shim_wi.lid[1] = y % RP_WG;
      computePosterior(&nd, width, height, n_classes, (float *)posteriors, &msk, out);
    }
}
