// Internal state of a pd_ctx: the device-resident training set, the training
// scratch buffers and the forest.
#pragma once

#include <vector>

#include "pd_common.cuh"

// Samples per iteration of the histogram kernel the tuning accepts (2, 4 or 8).
inline bool valid_hist_spi(uint32_t spi) { return spi == 2 || spi == 4 || spi == 8; }

namespace pd {
struct RtcPlugin;  // pd_rtc.cu
}

struct pd_ctx {
  pd_config cfg{};
  int device = 0;
  pd::RtcPlugin *rtc = nullptr;  // the compiled user feature plugin (PD_PLUGIN_USER)
  bool tree_feature = false;     // its computeFeature reads the tree: the node map is kept
  cudaStream_t stream = nullptr;
  uint64_t hist_budget = 8ull << 30;
  uint32_t chunk = 16384;  // samples per histogram work item (at most 65535)
  uint32_t hist_spi = 8;  // samples per iteration of the histogram kernel (2, 4 or 8)
  uint32_t fuse_max = 4096;  // nodes with at most this many samples get the fused split
  bool cand_order = true;    // order each node's candidate columns by first-probe offset
  bool cand_regs = true;     // candidate keys sorted in registers (T <= 64), else in shared memory
  bool persist = false;      // one persistent histogram grid per launch, items pulled largest first
  int upload_copy = 1;       // bulk inputs from pinned host memory: 0 copy engine, 1 SM copy kernel
  int n_sms = 0;             // multiprocessors of the context's GPU
  uint64_t sample_group = 512ull << 20;  // bytes of images + labels pd_sample stages per round trip
  bool collect_records = false;          // keep a pd_record per split node (learned proposals)
  std::vector<pd_record> records;        // of the last training call

  // ---- training set in HBM (cl_tree_trainer_impl_init.hpp:99-154 streams it
  // image by image; here it stays resident) ----
  bool have_dataset = false;
  uint32_t n_images = 0;
  uint64_t n_samples = 0;
  pd::DevBuf pixels;    // concatenated images
  uint64_t pixels_bytes = 0;
  pd::DevBuf img_off;   // uint64 byte offsets
  pd::DevBuf img_wh;    // uint32 w | h << 16
  pd::DevBuf s_xy;      // uint32 x | y << 16 per sample
  pd::DevBuf s_img;     // uint32 image per sample
  pd::DevBuf s_label;   // uint8 class (0..K-1) per sample
  std::vector<uint32_t> root_class_tot;  // samples per class (the root's class totals)
  pd_upload_stats upload_stats{};        // of the last pd_dataset_upload
  pd::HostBuf h_stage;           // pinned staging of the per-sample upload arrays
  pd::HostBuf h_items;           // pinned staging of a histogram launch's work list
  pd::DevBuf log2_tab;  // double log2(n), n < log2_len
  pd::DevBuf xlog2_tab; // float c*log2(c), c < min(log2_len, 65536): the fused split's filter
  pd::DevBuf parent;    // [slots] parent term of the exact gain, for the fused split
  pd::DevBuf split_par; // [slots][D + 1] feature values and threshold of each winner
  pd::DevBuf magic_tab; // uint32 RoundDiv multiplier by depth value (65536)
  uint64_t log2_len = 0;

  // ---- training scratch ----
  pd::DevBuf snode;                  // int32 node per sample
  pd::DevBuf act[2], act_slot[2];    // active samples sorted by frontier slot
  pd::DevBuf act_rec[2];             // their SampleRec, in the same order
  pd::DevBuf s_rec;                  // SampleRec of every uploaded sample
  pd::DevBuf flags;                  // uint8 per active sample
  pd::DevBuf scan_blocks;            // uint64 per scan block
  pd::DevBuf slot_adj;               // int64 [4] per slot: adjL, adjR, kL, kR
  pd::DevBuf scatter_err;            // uint32 error counter
  pd::DevBuf cand_feat, cand_thr, cand_perm;
  pd::DevBuf cand_ord;       // [slots][F] original candidate index of each column
  pd::DevBuf hist, g32;
  pd::DevBuf items, zero_slots, hist_queue;
  pd::DevBuf split_out, split_cl, recheck, split_scratch, fused_scratch;
  pd::DevBuf t_lc, t_feat, t_thr, t_post;  // device copy of the tree being trained
  // ---- node map of features that read the tree (tree_feature) ----
  pd::DevBuf nm_map[2];   // int32 node per pixel of every training image, this depth's and the next
  pd::DevBuf nm_off;      // uint64 [n_images + 1] first pixel of each image in the map
  pd::DevBuf nm_label;    // uint8 label of every pixel (nonzero: the map advances there)
  uint64_t nm_pixels = 0;
  int nm_cur = 0;
  int32_t nm_level = 0, nm_nodes = 0;  // the map's level (the depth being trained), the tree's node count
  pd::DevBuf np_map[2], np_desc;  // prediction: the map of the images predicted, their descriptors
  pd_train_stats stats{};

  // ---- forest (CLClassifier) ----
  std::vector<uint32_t> tree_depth;
  std::vector<uint64_t> tree_off;
  std::vector<int32_t> h_lc;
  std::vector<uint8_t> h_feat, h_thr;  // FeatType bytes
  std::vector<float> h_post;
  bool forest_dirty = true;
  pd::DevBuf f_lc, f_feat, f_thr, f_post, f_meta;
  pd::DevBuf f_cand;                   // NodeRec of every forest node (k_forest_nodes)
  uint64_t cand_version = ~0ull;       // forest_version f_cand was built for
  bool forest_fast = false;            // every node takes the plugin's fast path (built-in plugins)
  pd::DevBuf f_fast;                   // its device flag
  pd::DevBuf p_img, p_mask, p_out;     // staging for host-buffer prediction
  uint64_t forest_version = 0;         // bumped when the forest arrays are uploaded again
  // mixed-size prediction batches: buffers, the layout they were built for and
  // the graph of the batch kernel (pd_predict_posterior_batch)
  pd::DevBuf b_img, b_mask, b_out, b_desc;
  std::vector<uint64_t> batch_key;
  cudaGraphExec_t batch_graph = nullptr;

  // ---- pixel samplers (pd_sample*) ----
  pd::DevBuf sm_data, sm_lab;    // staged image data and labels of a host batch
  pd::DevBuf sm_desc;            // SampImage per image, item -> image map, checksums, counts, error
  pd::DevBuf sm_out;             // samples and counts of a host batch
  pd::HostBuf h_sm, h_sm_desc;   // pinned staging of a host batch and of its descriptors
  // pd_sample's two pipeline slots: a group is staged into one while the device
  // works on the other's (pinned data, descriptors, results; device copies; events
  // around the scan, the draws and the results)
  struct SampSlot {
    pd::HostBuf h_data, h_desc, h_out;
    pd::DevBuf d_data, d_desc, d_out;
    cudaEvent_t ev[4] = {};
  } samp[2];
  pd_sample_stats sample_stats{};
  // ---- label images (pd_rgb_to_labels*) ----
  pd::DevBuf lab_tab, lab_src, lab_dst;
  pd::HostBuf h_lab;

  cudaEvent_t ev[8] = {};
  uint64_t bytes_h2d = 0, bytes_d2h = 0, launches = 0;
};

namespace pd {
// Counted copies on the context stream.
inline cudaError_t h2d(pd_ctx *c, void *dst, const void *src, size_t n) {
  c->bytes_h2d += n;
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, c->stream);
}
inline cudaError_t d2h(pd_ctx *c, void *dst, const void *src, size_t n) {
  c->bytes_d2h += n;
  return cudaMemcpyAsync(dst, src, n, cudaMemcpyDeviceToHost, c->stream);
}
}  // namespace pd

namespace pd {
struct PropSrc;
// The proposal network's mixture for n frontier nodes of depth `depth` (class
// totals d_ctot [n][K] on the device), on the context's stream (pd_propose.cu).
int proposer_infer(pd_proposer *p, const uint32_t *d_ctot, uint32_t n, uint32_t depth, uint32_t n_prop, PropSrc *src);
int ensure_log2_table(pd_ctx *ctx, uint64_t n);
// Host -> device copy of bulk inputs on the context's stream (pd_api.cu).
int upload_bytes(pd_ctx *ctx, void *dst, const void *src, size_t n);
int init_tables(pd_ctx *ctx);
// Prepares the uploaded images for the plugin's eval_train (zero depths).
int map_training_pixels(pd_ctx *ctx, uint64_t bytes);
// The SampleRec of every uploaded sample (after map_training_pixels).
int build_sample_records(pd_ctx *ctx, uint64_t n_samples);
}
