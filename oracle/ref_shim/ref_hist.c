/*
 * The reference's own per-image histogram kernel
 * (src/padenti/kernels/hist_update.cl:36-187, computePerImageHistogram),
 * compiled as C through cl/cl_shim.h and executed over its NDRange on the host,
 * so the oracle's histograms can be checked against the reference code.
 * TEST INFRASTRUCTURE ONLY.
 *
 * NDRange as the trainer launches it (cl_tree_trainer_impl_traverse_ts.hpp:265-275):
 * global (nSamples, nFeatures), local (1, 256) (WG_LHIST_UPDATE_HEIGHT/WIDTH,
 * cl_tree_trainer_impl.hpp:67-68), so nFeatures must be a multiple of 256.
 * Local buffers as cl_tree_trainer_impl_init.hpp:265-267: tmp of 8 feat_t,
 * featuresBuff of 256 * featDim feat_t.  The kernel synchronises its work-group
 * with barrier() around the shared feature bounds, so each work-group runs as
 * 256 coroutines switched at every barrier.
 */
#define CL_SHIM_BARRIERS
#include "cl_shim.h"

#define computeFeature ref_hist_compute_feature
#include <hist_update_c.cl>
#undef computeFeature

#include <stdlib.h>
#include <string.h>

#define RH_GROUP 256
#define RH_STACK (64 * 1024)

static struct {
  image2d_t image, labels, nodes;
  uint n_channels, width, height;
  uint *samples;
  uint n_samples, feat_dim;
  feat_t *low, *up;
  uint n_thresholds;
  feat_t thr_low, thr_up;
  uchar *hist;
  uint tree;
  int start_node, end_node;
  int *lc;
  float *post;
  feat_t *tmp, *buf;
} A;

/* The tree the kernel passes to computeFeature (treeLeftChildren,
 * treePosteriors): null unless set by ref_hist_tree. */
static int *rh_lc;
static float *rh_post;

void ref_hist_tree(const int32_t *lc, const float *post) {
  rh_lc = (int *)lc;
  rh_post = (float *)post;
}

static int rh_done[RH_GROUP];
static int rh_barriers[RH_GROUP];

static void rh_entry(void) {
  computePerImageHistogram(A.image, A.n_channels, A.width, A.height, A.labels, A.nodes, A.samples, A.n_samples,
                           A.feat_dim, A.low, A.up, A.n_thresholds, A.thr_low, A.thr_up, A.hist, A.tree,
                           A.start_node, A.end_node, A.lc, A.post, A.tmp, A.buf);
  rh_done[cl_shim_cur] = 1;
}

/* Per-image indicators out[s][t][f] = (response of sample s to candidate f <=
 * threshold t) for samples whose node (nodes_img at the sample pixel) is in
 * [start_node, end_node]; other rows are left as they are (the reference leaves
 * them unwritten).  img_type: 1 = uint8, 2 = uint16.  Returns 0, or -1 for a
 * feature count that is not a multiple of 256, -2 if the work-items of a group
 * passed different numbers of barriers, -3 if memory runs out. */
int ref_per_image_hist(int img_type, uint n_channels, const void *pixels, uint width, uint height,
                       const int32_t *nodes_img, const uint32_t *samples, uint n_samples, uint n_features,
                       uint feat_dim, const int32_t *low, const int32_t *up, uint n_thresholds, int32_t thr_low,
                       int32_t thr_up, uint tree, int start_node, int end_node, uint8_t *out) {
  if (n_features % RH_GROUP) return -1;
  cl_shim_image img = {(void *)pixels, img_type == 1 ? CL_SHIM_U8 : CL_SHIM_U16, width, height, n_channels};
  cl_shim_image nodes = {(void *)nodes_img, CL_SHIM_I32, width, height, 1};
  feat_t flo[8], fup[8];
  for (uint d = 0; d < feat_dim && d < 8; d++) {
    flo[d] = (feat_t)low[d];
    fup[d] = (feat_t)up[d];
  }
  feat_t tmp[8];
  feat_t *buf = (feat_t *)calloc((size_t)RH_GROUP * feat_dim, sizeof(feat_t));
  char *stacks = (char *)malloc((size_t)RH_GROUP * RH_STACK);
  ucontext_t *ctx = (ucontext_t *)calloc(RH_GROUP, sizeof(ucontext_t));
  cl_shim_item *items = (cl_shim_item *)calloc(RH_GROUP, sizeof(cl_shim_item));
  if (!buf || !stacks || !ctx || !items) {
    free(buf), free(stacks), free(ctx), free(items);
    return -3;
  }
  A.image = &img;
  A.labels = NULL;
  A.nodes = &nodes;
  A.n_channels = n_channels;
  A.width = width;
  A.height = height;
  A.samples = (uint *)samples;
  A.n_samples = n_samples;
  A.feat_dim = feat_dim;
  A.low = flo;
  A.up = fup;
  A.n_thresholds = n_thresholds;
  A.thr_low = (feat_t)thr_low;
  A.thr_up = (feat_t)thr_up;
  A.hist = out;
  A.tree = tree;
  A.start_node = start_node;
  A.end_node = end_node;
  A.lc = rh_lc;
  A.post = rh_post;
  A.tmp = tmp;
  A.buf = buf;
  cl_shim_lsize[0] = 1;
  cl_shim_lsize[1] = RH_GROUP;
  cl_shim_gsize[0] = n_samples;
  cl_shim_gsize[1] = n_features;
  cl_shim_ctx = ctx;
  int rc = 0;
  for (uint s = 0; s < n_samples && !rc; s++)
    for (uint g = 0; g < n_features / RH_GROUP && !rc; g++) {
      for (int k = 0; k < RH_GROUP; k++) {
        items[k].gid[0] = s;
        items[k].gid[1] = (size_t)g * RH_GROUP + k;
        items[k].lid[0] = 0;
        items[k].lid[1] = k;
        rh_done[k] = 0;
        rh_barriers[k] = 0;
        getcontext(&ctx[k]);
        ctx[k].uc_stack.ss_sp = stacks + (size_t)k * RH_STACK;
        ctx[k].uc_stack.ss_size = RH_STACK;
        ctx[k].uc_link = &cl_shim_main;
        makecontext(&ctx[k], rh_entry, 0);
      }
      for (;;) {
        int live = 0;
        for (int k = 0; k < RH_GROUP; k++) {
          if (rh_done[k]) continue;
          live++;
          cl_shim_cur = (size_t)k;
          cl_shim_wi = items[k];
          swapcontext(&cl_shim_main, &ctx[k]);
          if (!rh_done[k]) rh_barriers[k]++;
        }
        if (!live) break;
      }
      for (int k = 1; k < RH_GROUP; k++)
        if (rh_barriers[k] != rh_barriers[0]) rc = -2;
    }
  free(buf), free(stacks), free(ctx), free(items);
  return rc;
}
