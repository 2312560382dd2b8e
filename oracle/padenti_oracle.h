/*
 * padenti_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C CPU restatement of Padenti's random-forest training and
 * prediction hot path.  It is the checker for the CUDA library in
 * padenti_gb300/: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline (and its reference arm) may load it.  Nothing in the product
 * links, calls or falls back to it.
 *
 * Parity status (each pin compiles the reference's own source here and
 * compares on the same inputs; oracle/Makefile "ref", oracle/ref_shim):
 *   - MD5 counter RNG (candidate and threshold generation): RFC-1321 known
 *     answers (Python hashlib) and the reference's src/padenti/prng.hpp.
 *   - Histograms (indicator writes + host accumulation), traversal and
 *     reassignment, split finalize (stored split, child posteriors) and the
 *     forest posterior: the reference's kernels/hist_update.cl and
 *     kernels/predict.cl compiled as C through an OpenCL shim and run over
 *     their NDRanges, with the host steps around them restated from
 *     cl_tree_trainer_impl_traverse_ts.hpp and cl_classifier_impl.hpp, at
 *     every depth of trained trees for three features
 *     (tests/test_reference_kernels.py).
 *   - The split rule: the reference's learnBestFeature kernel
 *     (kernels/learn_best_feature.cl) compiled as C, on the same histograms;
 *     winners agree except at FP32 near-ties of the reference's float gains.
 *   - The single-offset depth plugin: the reference's test/feature.cl.
 *   - Arithmetic: IEEE single precision with correctly rounded division,
 *     where OpenCL allows a less accurate divide and log2.
 * tests/golden/ref_kernels.npz carries outputs of those reference kernels to
 * machines without the Padenti sources.
 */
#ifndef PADENTI_ORACLE_H
#define PADENTI_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { OR_FEAT_I16 = 1, OR_FEAT_I32 = 2 };
enum { OR_IMG_U8 = 1, OR_IMG_U16 = 2 };
/* Built-in feature plugins (same numbering as the CUDA library). */
enum {
  OR_PLUGIN_DEPTH_DIFF2 = 1,   /* I(x+u/d) - I(x+v/d), int32, D=4 */
  OR_PLUGIN_DEPTH_DIFF1 = 2,   /* test/feature.cl: D(x) - D(x+round(u*500/D(x))), int16, D=2 */
  OR_PLUGIN_CHANNEL_DIFF = 3,  /* I_c1(x+u) - I_c2(x+v), RGB u8, int32, D=6 */
  /* A feature that reads the tree (auto-context), for the tests of the plugin
   * arguments treeLeftChildren / treePosteriors / imageNodesID
   * (padenti.hpp.in:169-177); uint16 images, int32, D=4:
   *   n1 = node map at (x+f0, y+f1) (0 outside), k = f2 mod K,
   *   (int)(posterior(n1, k) * 1000) + (left_child(n1) >= 0 ? 2000 : 0)
   *     + (I(x+f3, y) - I(x, y)) / 16 + n1 % 5      (I = 0 outside),
   * with the tree seen from the node map's level L (root 0): left_child(n) is
   * -1 for nodes at level >= L, posterior(n, k) 0 for nodes below L.  Trees
   * and predictions of this plugin keep a per-pixel node map, advanced one
   * level at a time over the labelled (training) or masked-in pixels. */
  OR_PLUGIN_AUTO_CONTEXT = 16
};

#define OR_MAX_FEAT_DIM 8

typedef struct {
  int32_t plugin;
  int32_t feat_type;          /* OR_FEAT_* */
  int32_t feat_dim;           /* D */
  int32_t n_classes;          /* K */
  uint32_t n_features;        /* F */
  uint32_t n_thresholds;      /* T */
  int32_t feat_low[OR_MAX_FEAT_DIM];
  int32_t feat_up[OR_MAX_FEAT_DIM];
  int32_t thr_low;
  int32_t thr_up;
  uint32_t per_leaf_samples_thr;
} or_params;

/* A training set flattened into host arrays (images interleaved row-major). */
typedef struct {
  uint32_t n_images;
  uint32_t n_channels;
  uint32_t img_type;            /* OR_IMG_* */
  const uint8_t *pixels;        /* all images, concatenated */
  const uint64_t *pix_off;      /* byte offset of each image */
  const uint32_t *width;
  const uint32_t *height;
  const uint8_t *labels;        /* per-pixel labels, 0 = unlabelled, class k = k+1 */
  const uint64_t *lab_off;      /* label offset (pixels) of each image */
  const uint32_t *samples;      /* sampled pixel indices y*W+x, per image, concatenated */
  const uint64_t *samp_off;     /* n_images+1 offsets into samples */
} or_dataset;

typedef struct {
  uint64_t evals;               /* (sample, candidate) feature evaluations */
  uint64_t nodes_trained;       /* frontier nodes processed */
  uint64_t nodes_split;
  double seconds_hist;
  double seconds_split;
} or_stats;

/* a1: one MD5 compression of the 16-byte little-endian block (s0..s3). */
void or_md5(const uint32_t in[4], uint32_t out[4]);

/* a2+a3: candidate f of node `node` of tree `tree_id`. */
void or_candidate(const or_params *p, uint32_t tree_id, uint32_t node, uint32_t f,
                  int32_t *feat_out /*[D]*/, int32_t *thr_out /*[T]*/);

/* a4: built-in plugin response at pixel (x,y) of one image (a feature that
 * reads the tree sees node 0, no posteriors and no children here). */
int32_t or_feature(int32_t plugin, int32_t feat_type, const void *img, uint32_t w, uint32_t h,
                   uint32_t n_channels, int32_t x, int32_t y, const int32_t *feat);

/* Per-integer log2 table used by the exact gain: out[n] = log2(n), out[0] = 0. */
void or_log2_table(uint32_t n, double *out);

/* a5+a6: histograms hist[i][l][t][f] for frontier nodes nodes[i], given each
 * sample's current node.  reference_cost=1 regenerates the candidate with MD5
 * per (sample, candidate) exactly as the reference kernel does. */
int or_hist(const or_params *p, const or_dataset *ds, uint32_t tree_id,
            const int32_t *sample_node, const int32_t *nodes, uint32_t n_nodes,
            uint32_t *hist, int reference_cost, int n_threads);

/* or_hist for a feature that reads the tree: maps holds every image's node
 * map (concatenated in image order, [H][W] each) at `level`, lc / post the
 * tree (tree_nodes nodes). */
int or_hist_tree(const or_params *p, const or_dataset *ds, uint32_t tree_id, const int32_t *sample_node,
                 const int32_t *nodes, uint32_t n_nodes, uint32_t *hist, const int32_t *maps, const int32_t *lc,
                 const float *post, int32_t level, int32_t tree_nodes, int n_threads);

/* a7: exact best split per node.  out_t/out_f/out_gain receive the winner. */
int or_split(const or_params *p, const uint32_t *hist, const uint32_t *class_tot,
             uint32_t n_nodes, const double *log2_table, uint64_t table_len,
             int32_t *out_t, int32_t *out_f, double *out_gain,
             float *out_gain32_max /* nullable: FP32 reference-formula max gain */,
             double *out_max_abs_err /* nullable: max |gain32 - gain64| seen */);

/* Training-set priors: mean of per-image priors over labelled samples. */
void or_priors(const or_dataset *ds, uint32_t n_classes, float *out_priors);

/* a9..a12: train one tree of depth end_depth (levels 1..end_depth-1 are split).
 * Tree arrays have 2^end_depth - 1 nodes and must be initialised by the caller
 * as a fresh reference Tree (left_child -2, zeros).  sample_leaf (nullable)
 * receives each sample's node after training. */
int or_train_tree(const or_params *p, const or_dataset *ds, uint32_t tree_id, uint32_t end_depth,
                  const float *root_prior, int32_t *left_child, int32_t *features,
                  int32_t *thresholds, float *posteriors, int32_t *sample_leaf,
                  int reference_cost, int n_threads, or_stats *stats);

/* Candidate-sharded training (the library's pd_train_tree_sharded protocol):
 * this rank splits on candidates [f0, f1) of every node and, per frontier
 * slice, `exchange` receives its best splits -- gain_key (order key of the exact
 * gain, INT64_MIN for none), cand_index (t * F + f, -1 for none), left_counts
 * [n][K] -- and must leave the global winners in cand_index / left_counts. */
typedef int (*or_exchange_fn)(void *user, uint32_t n_nodes, uint32_t n_classes, int64_t *gain_key,
                              int64_t *cand_index, uint32_t *left_counts);
int or_train_tree_sharded(const or_params *p, const or_dataset *ds, uint32_t tree_id, uint32_t end_depth,
                          const float *root_prior, uint32_t f0, uint32_t f1, or_exchange_fn exchange, void *user,
                          int32_t *lc, int32_t *feats, int32_t *thrs, float *posts, int32_t *sample_leaf,
                          int n_threads);

/* a11: forest posterior, planar [K][H][W]; masked-out pixels are 0.
 * Trees are given as concatenated SoA arrays; tree t has 2^depth[t]-1 nodes
 * starting at node_off[t]. */
int or_predict_posterior(const or_params *p, const void *img, uint32_t w, uint32_t h,
                         uint32_t n_channels, const uint8_t *mask, uint32_t n_trees,
                         const uint32_t *depth, const uint64_t *node_off,
                         const int32_t *left_child, const int32_t *features,
                         const int32_t *thresholds, const float *posteriors,
                         float *out, int n_threads);

/* Leaf-ID prediction of one tree (unmasked pixels get 0). */
int or_predict_leaf(const or_params *p, const void *img, uint32_t w, uint32_t h,
                    uint32_t n_channels, const uint8_t *mask, uint32_t depth,
                    const int32_t *left_child, const int32_t *features,
                    const int32_t *thresholds, int32_t *out, int n_threads);

/* Leaf-ID prediction of one tree with its posteriors, for every plugin
 * (a feature that reads the tree needs them; or_predict_leaf refuses it). */
int or_predict_leaf_tree(const or_params *p, const void *img, uint32_t w, uint32_t h, uint32_t nch,
                         const uint8_t *mask, uint32_t depth, const int32_t *lc, const int32_t *feats,
                         const int32_t *thrs, const float *posts, int32_t *out, int n_threads);

/* Pixel samplers (image_sampler.c): UniformImageSampler and
 * ClassWeightedImageSampler with their Boost randomness restated. */
typedef struct {
  uint32_t x[624];
  int i;
} or_mt;
uint32_t or_crc32(const uint8_t *p, uint64_t n);
void or_mt_seed(or_mt *m, uint32_t s);
uint32_t or_mt_next(or_mt *m);
uint32_t or_uniform_int(or_mt *m, uint32_t range);
double or_uniform01(or_mt *m);
uint32_t or_bucket_sizes(uint32_t n_samples, uint32_t n_classes, const float *weights, uint32_t *sizes);
uint32_t or_sample_uniform(const void *data, uint64_t data_bytes, const uint8_t *labels, uint32_t n_pix,
                           uint32_t n_samples, uint32_t seed, uint32_t *out);
int64_t or_sample_class_weighted(const void *data, uint64_t data_bytes, const uint8_t *labels, uint32_t n_pix,
                                 uint32_t n_classes, const uint32_t *sizes, uint32_t seed, uint32_t *out);
void or_sample_batch(int kind, const void *images, uint64_t data_bytes, const uint8_t *labels, uint32_t n_pix,
                     uint32_t n_images, uint32_t n_samples, uint32_t n_classes, const uint32_t *sizes,
                     uint32_t seed, uint32_t stride, uint32_t *out, int64_t *counts);

/* The benchmark's seeded synthetic depth maps (synth.c): the same bytes as the
 * library's pd_synth_depth, for callers that must not load the library. */
int or_synth_depth(uint64_t seed, uint32_t first_image, uint32_t n_images, uint32_t width, uint32_t height,
                   uint32_t min_ellipses, uint32_t max_ellipses, uint32_t parts, uint32_t samples_per_image,
                   uint32_t bg_permille, uint16_t *pixels, uint8_t *labels, uint32_t *samples);

/* The proposal network of learned proposals (proposal.c): network outputs of
 * n rows, and the weighted-mean mixture loss with its gradient with respect to
 * the FP32 parameter vector (grad: double, one per parameter).  bf16 = 1
 * rounds to BF16 where the GPU stores BF16. */
int or_prop_forward(const float *params, uint32_t IN, uint32_t H, uint32_t OUT, const float *x, uint32_t n,
                    int bf16, float *out);
int or_prop_loss_grad(const float *params, uint32_t IN, uint32_t H, uint32_t OUT, uint32_t DY, const float *x,
                      const float *y, const float *w, uint32_t n, int bf16, double *loss, double *grad);

/* Label images (image_loader.c): _rgb2label. */
void or_rgb_to_labels(const uint8_t *src, uint64_t n_pix, uint32_t channels, const uint8_t *map, uint32_t n_classes,
                      uint8_t *dst);

#ifdef __cplusplus
}
#endif
#endif
