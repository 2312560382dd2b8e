/*
 * padenti_gb300.h -- C ABI of the GB300-native Padenti hot path.
 *
 * libpadenti_gb300.so runs Padenti's per-depth random-forest training pass
 * (candidate evaluation + class histograms, best split, pixel reassignment)
 * and forest prediction as sm_103a CUDA kernels.  The reference is a
 * header-only C++ template library with no FFI of its own; these entry points
 * are what its C++ classes bind in the header-only facade under
 * include/padenti/ (cuda_tree_trainer.hpp, cuda_classifier.hpp), and what the
 * Python package padenti_gb300 binds with ctypes.
 *
 * Conventions:
 *   - Every function returns PD_OK (0) or a negative PD_ERR_* code; the
 *     message of the last failure on the calling thread is pd_last_error().
 *   - Pointers are host pointers unless the name says _device.
 *   - One context = one GPU = one CUDA stream.  Calls on one context must be
 *     serialised by the caller; separate contexts may be used from separate
 *     threads.
 *   - The template parameters of the reference classes
 *     <ImgType, nChannels, FeatType, FeatDim, nClasses> are the pd_config
 *     given at context creation.
 */
#ifndef PADENTI_GB300_H
#define PADENTI_GB300_H

#if !defined(__CUDACC_RTC__)
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PD_OK 0
#define PD_ERR_INVALID (-1)      /* bad argument or inconsistent sizes */
#define PD_ERR_CUDA (-2)         /* CUDA runtime error (message has the call) */
#define PD_ERR_NOMEM (-3)        /* device or host allocation failed */
#define PD_ERR_UNSUPPORTED (-4)  /* configuration outside the built kernels */
#define PD_ERR_STATE (-5)        /* call out of order (e.g. no dataset uploaded) */

/* Image element types (ImgType). */
#define PD_IMG_U8 1
#define PD_IMG_U16 2
#define PD_IMG_I16 3
#define PD_IMG_I32 4
#define PD_IMG_F32 5

#define PD_FEAT_I16 1
#define PD_FEAT_I32 2

/* Built-in feature plugins.  The reference compiles a user OpenCL C
 * computeFeature() into its kernels (kernels/hist_update.cl:33,
 * kernels/predict.cl:32); here a plugin is a CUDA device functor compiled into
 * the kernels.
 *   DEPTH_DIFF2  uint16 x1, int32, D=4 (ux,uy,vx,vy):
 *                I(x+u/d(x)) - I(x+v/d(x)); out-of-image or zero probes = 10000.
 *   DEPTH_DIFF1  uint16 x1, int16, D=2: the reference test/feature.cl:29-64,
 *                D(x) - D(x + round(u*500/D(x))).
 *   CHANNEL_DIFF uint8 x3, int32, D=6 (c1,c2,ux,uy,vx,vy):
 *                I_c1(x+u) - I_c2(x+v), channels clamped to [0,2], outside = 0. */
#define PD_PLUGIN_DEPTH_DIFF2 1
#define PD_PLUGIN_DEPTH_DIFF1 2
#define PD_PLUGIN_CHANNEL_DIFF 3
/* A feature compiled at run time from CUDA source (pd_plugin_compile), the
 * counterpart of the reference's user feature.cl. */
#define PD_PLUGIN_USER 100

#define PD_MAX_FEAT_DIM 8
#define PD_MAX_CLASSES 64
#define PD_MAX_THRESHOLDS 256
#define PD_MAX_TREES 64

typedef struct pd_ctx pd_ctx;

/* The reference's class template parameters. */
typedef struct {
  int32_t plugin;       /* PD_PLUGIN_* */
  int32_t img_type;     /* PD_IMG_* (ImgType) */
  int32_t n_channels;   /* nChannels */
  int32_t feat_type;    /* PD_FEAT_* (FeatType) */
  int32_t feat_dim;     /* FeatDim */
  int32_t n_classes;    /* nClasses */
} pd_config;

/* TreeTrainerParameters (tree_trainer.hpp:35-51).  Bounds are given as int32
 * and converted to FeatType. */
typedef struct {
  uint32_t n_features;
  uint32_t n_thresholds;
  int32_t feat_low[PD_MAX_FEAT_DIM];
  int32_t feat_up[PD_MAX_FEAT_DIM];
  int32_t thr_low;
  int32_t thr_up;
  uint32_t per_leaf_samples_thr;
} pd_train_params;

/* A TrainingSet (training_set.hpp:39-112) flattened into host arrays.
 * Images are interleaved row-major [H][W][C]; labels are one byte per pixel
 * with 0 = unlabelled and class k stored as k+1 (training_set_image.hpp:29-33);
 * samples are pixel indices y*W+x (training_set_image.hpp:38-110). */
typedef struct {
  uint32_t n_images;
  const void *pixels;        /* all images concatenated */
  const uint64_t *pix_off;   /* byte offset of image i in pixels */
  const uint32_t *width;
  const uint32_t *height;
  const uint8_t *labels;     /* all label images concatenated */
  const uint64_t *lab_off;   /* offset of image i in labels (pixels) */
  const uint32_t *samples;   /* all sample lists concatenated */
  const uint64_t *samp_off;  /* n_images+1 offsets into samples */
} pd_dataset_desc;

/* Counters and CUDA-event times of the last pd_train_tree call. */
typedef struct {
  uint64_t evals;            /* (sample, candidate) evaluations, each with T comparisons */
  uint64_t nodes_trained;
  uint64_t nodes_split;
  uint64_t hist_launches;
  uint64_t split_rechecked;  /* candidates rechecked in FP64 */
  uint64_t kernel_launches;  /* kernels this library launched in the call */
  uint64_t hist_bytes;       /* algorithmic HBM bytes of all histogram launches */
  uint64_t h2d_bytes;        /* host->device bytes copied by the call */
  uint64_t d2h_bytes;        /* device->host bytes copied by the call */
  double ms_candidates;
  double ms_hist;            /* CUDA-event time of the histogram kernels alone */
  double ms_split;
  double ms_reassign;
  double ms_total;           /* wall time of the call */
} pd_train_stats;

const char *pd_last_error(void);
int pd_version(void);

/* Context ------------------------------------------------------------------ */
int pd_ctx_create(const pd_config *cfg, int device, pd_ctx **out);
int pd_ctx_destroy(pd_ctx *ctx);

/* User feature plugins -------------------------------------------------------
 * Replaces the reference's run-time compiled feature.cl (CLTreeTrainer and
 * CLClassifier build it into their OpenCL program: cl_tree_trainer_impl.hpp:73-198,
 * cl_classifier_impl.hpp:72-140; prototype padenti.hpp.in:169-187).  A context
 * created with plugin = PD_PLUGIN_USER compiles CUDA source that defines
 *
 *   __device__ feat_t computeFeature(const pd::ImageView &img, int2 coords,
 *                                    const feat_t *features, unsigned featDim);
 *
 * with NVRTC for the context's GPU.  img_t, feat_t, PD_FEAT_DIM and PD_CHANNELS
 * are defined before the source from the configuration (the reference generates
 * feat_type.cl the same way); img.read(x, y, c) returns 0 outside the image.
 * The configuration must have the types and dimensions of a built-in plugin:
 * (uint16, 1 channel, int32, 4), (uint16, 1, int16, 2) or (uint8, 3, int32, 6).
 * Compile before uploading a training set or adding trees; compiling again
 * replaces the plugin (the training set must then be uploaded again). */
int pd_plugin_compile(pd_ctx *ctx, const char *source);
/* Compiles only (no GPU needed): PD_OK, or PD_ERR_INVALID with the compiler's
 * log in log[0..log_size) (NUL-terminated; may be NULL). */
int pd_plugin_check(const pd_config *cfg, const char *source, char *log, size_t log_size);
/* Device memory the training pass may use for histograms (default 8 GiB);
 * frontiers whose histograms exceed it are processed in slices, as the
 * reference does with its 20 GiB host cap (cl_tree_trainer_impl.hpp:47-50). */
int pd_ctx_set_hist_budget(pd_ctx *ctx, uint64_t bytes);
/* Launch-shape knobs of the histogram kernel (results do not depend on them):
 *   "chunk"     samples per histogram work item, [256, 65535] (default 16384);
 *   "hist_spi"  samples evaluated together per warp iteration, 2, 4 or 8 (default 8);
 *   "fuse_max"  nodes with at most this many samples (and within one work item)
 *               get their split computed inside the histogram kernel, [0, 65535];
 *   "cand_order" 1 (default): each node's candidate table is laid out in the
 *               order of the candidates' first probe offsets (n_features <= 8192),
 *               so that neighbouring lanes probe neighbouring pixels; 0: index order;
 *   "sample_group" bytes of images and labels pd_sample stages per round trip,
 *               >= 4096 (default 512 MiB);
 *   "persist"   1: one persistent histogram grid per launch (a few CTAs per SM) pulling the work
 *               items from a device counter, largest first; 0 (default): one CTA per work item;
 *   "records"   1: training calls keep one pd_record per split node (pd_train_records); 0 (default): none;
 *   "cand_regs" 1 (default): each candidate's thresholds are sorted in registers (at most 64
 *               thresholds, ranges below 2^24); 0: by insertion in shared memory (same tables);
 *   "upload_copy" 1 (default): training images in pinned host memory, and pd_sample's staged
 *               batches, are copied to the device by an SM kernel reading over the host link;
 *               0: by the copy engine (pageable memory always is). */
int pd_ctx_set_tuning(pd_ctx *ctx, const char *name, int64_t value);
/* The launch shape chosen by pd_autotune. */
typedef struct {
  int32_t chunk, hist_spi, fuse_max, cand_order, persist;
  double ms_start;   /* tree time with the settings the call started from */
  double ms_best;    /* tree time with the chosen settings */
  int32_t trials;    /* settings timed (0 when the cache had the key) */
  int32_t from_cache;
} pd_tuning;
/* Autotuner of the launch-shape knobs above (no counterpart in the reference,
 * whose tunables are compile-time constants, cl_tree_trainer_impl.hpp:47-68):
 * coordinate descent over chunk {4096..32768}, persist, hist_spi {4, 8},
 * fuse_max {1024..8192} and cand_order, each setting timed as the best of two
 * trees of end_depth levels with `params` on the uploaded training set (at
 * most max_trials settings; 0 = no limit), every tree checked equal to the
 * first.  The winner is applied to the context and, with cache_path, appended
 * to that text file under a key of (GPU, SM count, configuration, F, T,
 * training-set size class, depth, min samples per leaf); a later call with the
 * same key applies the cached setting without timing. */
int pd_autotune(pd_ctx *ctx, const pd_train_params *params, uint32_t end_depth, uint32_t max_trials,
                const char *cache_path, pd_tuning *out);
/* Synchronises the context's stream. */
int pd_ctx_sync(pd_ctx *ctx);
/* The CUDA stream (cudaStream_t) the context launches on. */
void *pd_ctx_stream(pd_ctx *ctx);
/* Bytes copied host->device and device->host by this context since creation. */
int pd_ctx_transfer_bytes(pd_ctx *ctx, uint64_t *h2d, uint64_t *d2h);

/* TrainingSet upload (replaces the per-image streaming of
 * cl_tree_trainer_impl_traverse_ts.hpp:127-358): the whole set is kept in HBM. */
int pd_dataset_upload(pd_ctx *ctx, const pd_dataset_desc *ds);
int pd_dataset_info(pd_ctx *ctx, uint64_t *n_samples, uint32_t *n_images);
/* Wall times of the last pd_dataset_upload: the host pass over the samples
 * (checks, positions, classes), then the copies, kernels and synchronisation. */
typedef struct {
  double ms_samples;
  double ms_device;
  double ms_total;
} pd_upload_stats;
int pd_dataset_upload_stats(pd_ctx *ctx, pd_upload_stats *out);

/* Training: CLTreeTrainer::train (cl_tree_trainer_impl.hpp:203-255).
 * Levels start_depth..end_depth-1 are split (start_depth must be 1, as in the
 * reference).  The tree SoA arrays (2^end_depth - 1 nodes; features/thresholds
 * of FeatType) are read and written in place, as the reference mutates Tree&.
 * root_prior (nClasses floats) becomes the root posterior. */
int pd_train_tree(pd_ctx *ctx, const pd_train_params *params, uint32_t tree_id,
                  uint32_t start_depth, uint32_t end_depth, const float *root_prior,
                  int32_t *left_child, void *features, void *thresholds, float *posteriors);
int pd_train_get_stats(pd_ctx *ctx, pd_train_stats *out);
/* Node of every sample after the last pd_train_tree call (n_samples int32). */
int pd_train_sample_nodes(pd_ctx *ctx, int32_t *out);

/* Stage entry points of one depth, for drop-in use and parity testing. ---- */
/* Candidate table (kernels/hist_update.cl:62-114,127-184): features
 * [n_nodes][F][D] and thresholds [n_nodes][F][T], FeatType. */
int pd_candidates(pd_ctx *ctx, const pd_train_params *params, uint32_t tree_id,
                  const int32_t *nodes, uint32_t n_nodes, void *features_out, void *thresholds_out);
/* Class histograms hist[n][l][t][f] = #samples of node nodes[n] with label l
 * whose response to candidate f is <= threshold t (kernels/hist_update.cl:36-187
 * + cl_tree_trainer_impl_traverse_ts.hpp:462-704).  sample_node holds the
 * current node of every uploaded sample. */
int pd_hist(pd_ctx *ctx, const pd_train_params *params, uint32_t tree_id,
            const int32_t *sample_node, const int32_t *nodes, uint32_t n_nodes, uint32_t *hist_out);
/* Best split of each node from its histogram and class totals
 * (kernels/learn_best_feature.cl:22-111 + learn_best_featthr.hpp:101-112).
 * Ties go to the lowest t*F+f; out_t/out_f are -1 for an empty node. */
int pd_split(pd_ctx *ctx, const pd_train_params *params, const uint32_t *hist,
             const uint32_t *class_tot, uint32_t n_nodes, int32_t *out_t, int32_t *out_f,
             double *out_gain);
/* pd_split for callers that cannot allocate device memory.  It has no
 * counterpart in the reference.  A host that only hands out memory from its own
 * pre-allocated pool, or a runtime whose allocator must not be bypassed, cannot
 * let a library call cudaMalloc; this entry point takes DEVICE pointers for its
 * inputs (hist_device: [n_nodes][K][T][F] cumulative counts as pd_split takes
 * them, class_tot_device: [n_nodes][K]) and outputs (out_t/out_f int32,
 * out_gain double, n_nodes each), needs no context, and keeps every
 * intermediate result in one fixed 32 MiB device array inside the library
 * (held by every GPU that loads it until the process exits).  Limits: the
 * working set must fit the array (PD_ERR_UNSUPPORTED otherwise: about
 * n_nodes*T*F*4 bytes plus 8 MiB of log2 table), and every node must hold
 * fewer than 2^20 samples.  The first call on a device sets the array up and
 * synchronises `stream`: make it before any stream capture; cudaDeviceReset on
 * that device afterwards is not supported.  Calls share the array, so calls
 * that overlap on the GPU race; serialise them.  Each call synchronises
 * `stream` (a cudaStream_t, NULL for the default stream) before returning. */
int pd_split_noalloc(const pd_train_params *params, uint32_t n_classes, const uint32_t *hist_device,
                     const uint32_t *class_tot_device, uint32_t n_nodes, int32_t *out_t_device,
                     int32_t *out_f_device, double *out_gain_device, void *stream);
/* Exact per-integer log2 table used by the split: out[n] = log2(n), out[0]=0. */
int pd_log2_table(pd_ctx *ctx, uint32_t n, double *out);

/* Candidate-sharded training ---------------------------------------------------
 * Several ranks (one GPU each) train one tree together: rank r evaluates the
 * candidates [f_begin, f_end) of every node (candidate f of a node is drawn
 * from its own MD5 seed (tree, node, f), hist_update.cl:62-65,127-130, so no
 * rank needs another's candidates), and after the split of each frontier slice
 * `exchange` is called with this rank's best split of every node of the slice:
 * gain_key[i] (an int64 whose order is the order of the exact gains; INT64_MIN
 * when the rank has none), cand_index[i] = t * F + f (-1: none) and
 * left_counts[i * n_classes ...] (its left class counts).  It must return 0 and
 * leave in cand_index / left_counts the global winner of every node: the
 * largest key, ties to the lowest index (the single-GPU rule; for example an
 * all-reduce MAX of the keys, MIN of the indices holding the maximum, and a sum
 * of the owner's counts).  Every rank then applies the same splits and
 * reassignment, so all ranks end with the same tree -- the unsharded one.  The
 * exchange replaces the host argmax of learn_best_featthr.hpp:101-112 across
 * GPUs.  Slices are cut for all params->n_features candidates, the same on
 * every rank. */
typedef int (*pd_exchange_fn)(void *user, uint32_t n_nodes, uint32_t n_classes, int64_t *gain_key,
                              int64_t *cand_index, uint32_t *left_counts);
int pd_train_tree_sharded(pd_ctx *ctx, const pd_train_params *params, uint32_t f_begin, uint32_t f_end,
                          pd_exchange_fn exchange, void *user, uint32_t tree_id, uint32_t start_depth,
                          uint32_t end_depth, const float *root_prior, int32_t *left_child, void *features,
                          void *thresholds, float *posteriors);

/* Learned candidate proposals ------------------------------------------------
 * No counterpart in the reference, which draws every candidate uniformly
 * (kernels/hist_update.cl:62-184).  The plain trainer emits one record per
 * node it splits; a proposal network (a BF16 MLP: the node's depth, log-count
 * and class frequencies in, three hidden layers of 256 with GELU, a
 * 16-component Gaussian mixture over the normalised feature values and
 * threshold out) is fitted to them on the GPU; a tree trained with it draws
 * the first n_proposed of each node's n_features candidates (and each one's
 * thresholds) from the mixture and the rest uniformly as the reference does.
 * Every candidate is still scored by the exact histogram and split kernels. */
typedef struct pd_record {
  uint32_t depth;      /* level of the node (root = 1) */
  uint32_t count;      /* samples at the node */
  uint32_t node;       /* heap index */
  uint32_t tree;
  double gain;         /* exact gain of the winning split */
  int32_t feat[PD_MAX_FEAT_DIM];  /* the winner's feature values */
  int32_t thr;         /* the winner's threshold */
  uint32_t class_count[PD_MAX_CLASSES];
} pd_record;

/* Records of the last pd_train_tree / pd_train_tree_proposed call of a context
 * whose tuning "records" is 1: one per split node, in training order.  Writes
 * min(cap, available) records to out (may be NULL to query) and the number
 * available to *n. */
int pd_train_records(pd_ctx *ctx, pd_record *out, uint64_t cap, uint64_t *n);

typedef struct pd_proposer pd_proposer;
/* A proposal network for the context's configuration (classes, FeatDim) and the
 * value ranges of `bounds` (feature and threshold bounds), with parameters
 * initialised from `seed`.  It runs on the context's GPU and stream. */
int pd_proposer_create(pd_ctx *ctx, const pd_train_params *bounds, uint64_t seed, pd_proposer **out);
int pd_proposer_destroy(pd_proposer *p);
/* dims = {input width, hidden width, hidden layers, output width, mixture
 * components, drawn dimensions}; *n_params = length of the parameter vector. */
int pd_proposer_dims(pd_proposer *p, uint32_t dims[6], uint64_t *n_params);
/* The FP32 parameter vector (W1 [H][IN], b1, W2 [H][H], b2, W3 [H][H], b3,
 * Wo [OUT][H], bo); setting it resets the optimiser state. */
int pd_proposer_get_params(pd_proposer *p, float *out);
int pd_proposer_set_params(pd_proposer *p, const float *in);
/* Network outputs of n input rows (host buffers: x [n][IN], out [n][OUT]). */
int pd_proposer_forward(pd_proposer *p, const float *x, uint32_t n, float *out);
/* Weighted mean mixture negative log-likelihood of targets y [n][DY] (w [n] or
 * NULL for equal weights) and its gradient with respect to the parameter
 * vector (grad: n_params floats); the parameters do not change. */
int pd_proposer_loss_grad(pd_proposer *p, const float *x, const float *y, const float *w, uint32_t n, float *loss,
                          float *grad);
/* Fits the network to n records with Adam (steps steps of `batch` records drawn
 * with replacement, learning rate lr); loss (steps floats, may be NULL) gets
 * the batch loss of every step, *ms (may be NULL) the GPU time of the fit. */
int pd_proposer_fit(pd_proposer *p, const pd_record *records, uint64_t n, uint32_t steps, uint32_t batch, float lr,
                    float *loss, float *ms);
/* pd_train_tree with learned proposals: candidates f < n_proposed of every node
 * are drawn from the network's mixture for that node, f >= n_proposed are the
 * reference's uniform MD5 candidates (params->n_features in total). */
int pd_train_tree_proposed(pd_ctx *ctx, pd_proposer *p, const pd_train_params *params, uint32_t n_proposed,
                           uint32_t tree_id, uint32_t start_depth, uint32_t end_depth, const float *root_prior,
                           int32_t *left_child, void *features, void *thresholds, float *posteriors);

/* Classifier (cl_classifier_impl.hpp) ---------------------------------------- */
int pd_forest_clear(pd_ctx *ctx);
/* CLClassifier::operator<< (cl_classifier_impl.hpp:146-195). */
int pd_forest_add_tree(pd_ctx *ctx, uint32_t depth, const int32_t *left_child,
                       const void *features, const void *thresholds, const float *posteriors);
int pd_forest_size(pd_ctx *ctx, uint32_t *n_trees);
/* CLClassifier::predict(image, posterior, mask) (cl_classifier_impl.hpp:356-557):
 * out is planar [nClasses][H][W] floats; mask may be NULL (all pixels);
 * masked-out pixels are 0. */
int pd_predict_posterior(pd_ctx *ctx, const void *image, uint32_t width, uint32_t height,
                         const uint8_t *mask, float *out);
/* CLClassifier::predict(treeID, image, prediction, mask) (:200-341): leaf node
 * id per pixel; masked-out pixels are 0. */
int pd_predict_leaf(pd_ctx *ctx, uint32_t tree, const void *image, uint32_t width,
                    uint32_t height, const uint8_t *mask, int32_t *out);
/* A batch of n images of mixed sizes (host buffers: images[i] of widths[i] x
 * heights[i], optional masks[i] (masks or an entry may be NULL), outs[i] planar
 * [K][H][W] float) in one kernel launch, captured in a CUDA graph and replayed
 * while the sizes, the masks' presence and the forest stay the same.  The
 * reference predicts image by image (cl_classifier_impl.hpp:356-557); the
 * results are those of pd_predict_posterior per image. */
int pd_predict_posterior_batch(pd_ctx *ctx, uint32_t n, const void *const *images, const uint32_t *widths,
                               const uint32_t *heights, const uint8_t *const *masks, float *const *outs);
/* Batched posterior prediction of n same-size images already in device
 * memory: images n*H*W*C, masks n*H*W (or NULL), out n*K*H*W.  Asynchronous on
 * the context's stream (pd_ctx_stream): order the caller's own work on these
 * buffers with pd_ctx_sync or stream events. */
int pd_predict_posterior_device(pd_ctx *ctx, uint32_t n_images, const void *images_device,
                                uint32_t width, uint32_t height, const uint8_t *masks_device,
                                float *out_device);

/* Pixel samplers (ImageSampler, image_sampler.hpp:31-73) ---------------------- */
#define PD_SAMPLER_UNIFORM 1         /* UniformImageSampler (uniform_image_sampler_impl.hpp:34-63) */
#define PD_SAMPLER_CLASS_WEIGHTED 2  /* ClassWeightedImageSampler (classweighted_image_sampler_impl.hpp:25-120) */
/* Largest number of samples per image a sampler may produce (its stride). */
#define PD_SAMPLER_MAX_STRIDE 16384

/* The sampler's constructor arguments and template parameters. */
typedef struct {
  int32_t kind;            /* PD_SAMPLER_* */
  uint32_t n_samples;      /* nSamples */
  uint32_t seed;           /* seed (XORed into the CRC-32 of the image data) */
  uint32_t n_classes;      /* nClasses (class-weighted; labels 1..nClasses) */
  const float *weights;    /* per-class weights, NULL = 1/nClasses each (class-weighted) */
  uint32_t pixel_bytes;    /* sizeof(type) * nChannels of the sampled images */
} pd_sampler;

/* Counters and CUDA-event times of the last pd_sample / pd_sample_device call. */
typedef struct {
  uint64_t images;
  uint64_t data_bytes;       /* image bytes checksummed */
  uint64_t label_bytes;      /* label bytes read */
  uint64_t kernel_launches;
  uint64_t h2d_bytes;
  uint64_t d2h_bytes;
  double ms_scan;            /* checksum + labelled-pixel count kernel */
  double ms_draw;            /* per-image drawing / reservoir kernel */
  double ms_total;           /* wall time of the call */
} pd_sample_stats;

/* Samples per image the output of pd_sample must hold: nSamples for the
 * uniform sampler, the sum of the class buckets ceil(weight_k * nSamples) for
 * the class-weighted one. */
int pd_sampler_stride(const pd_sampler *s, uint32_t *stride);
/* ImageSampler::sample over a batch of host images (mixed sizes): images[i]
 * of widths[i] x heights[i] pixels of s->pixel_bytes bytes, labels[i] one byte
 * per pixel (0 = unlabelled, class k stored as k+1).  The sorted pixel indices
 * of image i go to samples + i*stride, their number to counts[i] (the value
 * sample() returns; 0 for a uniform sampler on an image without labelled
 * pixels, where the reference draws from an empty buffer).  A label above
 * nClasses is an error for the class-weighted sampler (the reference indexes
 * past its buckets). */
int pd_sample(pd_ctx *ctx, const pd_sampler *s, uint32_t n_images, const void *const *images,
              const uint8_t *const *labels, const uint32_t *widths, const uint32_t *heights,
              uint32_t stride, uint32_t *samples, uint32_t *counts);
/* The same over n same-size images already in device memory (images
 * n*W*H*pixel_bytes, labels n*W*H, samples n*stride, counts n; all device
 * pointers, 16-byte aligned, with W*H*pixel_bytes and W*H multiples of 16). */
int pd_sample_device(pd_ctx *ctx, const pd_sampler *s, uint32_t n_images, const void *images_device,
                     const uint8_t *labels_device, uint32_t width, uint32_t height, uint32_t stride,
                     uint32_t *samples_device, uint32_t *counts_device);
int pd_sample_get_stats(pd_ctx *ctx, pd_sample_stats *out);

/* Label images (CVRGBLabelsLoader, cv_image_loader.hpp:37-52) ------------------ */
/* The colour-to-class step of CVRGBLabelsLoader::load (_rgb2label,
 * cv_image_loader_impl.hpp:233-266) for a batch of host label images:
 * images[i] holds widths[i] x heights[i] pixels of `channels` bytes (3: R, G, B;
 * 4: R, G, B, A -- the reference converts OpenCV's BGR(A) to RGB(A) first),
 * map[3k..3k+2] is the colour of class k (k < n_classes <= 255).  out[i] gets,
 * per pixel, 1 + the first class with the pixel's colour, or 0 (unlabelled). */
int pd_rgb_to_labels(pd_ctx *ctx, uint32_t n_images, const uint8_t *const *images, const uint32_t *widths,
                     const uint32_t *heights, uint32_t channels, const uint8_t *map, uint32_t n_classes,
                     uint8_t *const *out);
/* The same over n_pixels pixels already in device memory (16-byte aligned
 * buffers); *ms (may be NULL) gets the kernel's CUDA-event time. */
int pd_rgb_to_labels_device(pd_ctx *ctx, uint64_t n_pixels, const uint8_t *src_device, uint32_t channels,
                            const uint8_t *map, uint32_t n_classes, uint8_t *dst_device, float *ms);

/* The crop of the ROI loaders (CVImageROILoader, CVRGBLabelsROILoader;
 * _extractROI at cv_image_loader_impl.hpp:268-289), on the host: the bounding
 * rectangle of largest area among the 8-connected components of the pixels
 * whose value is > 0 in the image's element type img_type (PD_IMG_*; the
 * reference's mask img > 0: negative values and -0.0f are background), the
 * one-pixel image border counting as zero; ties go to the component met first
 * in raster order.  The reference takes single-channel images; with channels > 1
 * a pixel counts when any of its channels is > 0.  roi = {x, y, width, height}.
 * No such pixel is an error (the reference indexes an empty contour list then). */
int pd_image_roi(const void *image, uint32_t width, uint32_t height, int32_t img_type, uint32_t channels,
                 uint32_t roi[4]);

/* Measurement ------------------------------------------------------------------ */
/* The rate (adds/s) at which GPU `device` retires conflict-free shared-memory
 * atomic adds -- the histogram kernel's one add per evaluation, in its
 * [class][rank][lane] layout -- measured with CUDA events at 2, 4 and 8 CTAs of
 * 256 threads per SM; the best rate and its CTAs per SM are returned.  No
 * counterpart in the reference (it is the ceiling the histogram kernel is
 * reported against). */
int pd_measure_smem_atomics(int device, double *adds_per_s, int32_t *best_ctas_per_sm);

/* Synthetic data (seeded, bit-identical on every host) ------------------------ */
/* Depth maps: background plane U(3000,4000) mm + N(0,5^2) noise, ellipses at
 * U(800,2500) mm.  parts=0: 3 classes (bg, left half, right half of each
 * ellipse); parts=1: 9 classes (bg + 8 angular sectors).  Samples: with
 * replacement, (1000-bg_permille)/1000 among object pixels, the rest among
 * background, sorted.  Buffers: pixels n*W*H uint16, labels n*W*H, samples
 * n*samples_per_image. */
int pd_synth_depth(uint64_t seed, uint32_t first_image, uint32_t n_images, uint32_t width,
                   uint32_t height, uint32_t min_ellipses, uint32_t max_ellipses,
                   uint32_t parts, uint32_t samples_per_image, uint32_t bg_permille,
                   uint16_t *pixels, uint8_t *labels, uint32_t *samples);
/* RGB Voronoi images: 8-20 cells, classes 0..n_classes-1 with a seeded palette,
 * uniform texture noise +-20 per channel; samples uniform over all pixels. */
int pd_synth_rgb(uint64_t seed, uint32_t first_image, uint32_t n_images, uint32_t width,
                 uint32_t height, uint32_t n_classes, uint32_t samples_per_image,
                 uint8_t *pixels, uint8_t *labels, uint32_t *samples);

#ifdef __cplusplus
}
#endif
#endif
