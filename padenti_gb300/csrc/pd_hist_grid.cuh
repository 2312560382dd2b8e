// Launch of the histogram kernel over a work list.  The kernel has one
// instantiation per (plugin, padded threshold rows, samples per iteration); each
// plugin's set is compiled in its own translation unit (pd_hist_<plugin>.cu) so
// that the build compiles them in parallel.
#pragma once

#include "pd_ctx.cuh"
#include "pd_train_kernels.cuh"

namespace pd {

struct HistGrid {
  DevSet ds;
  const SampleRec *rec;   // active samples of the work list's ranges
  const WorkItem *items;  // device work list
  uint64_t n_items;
  const void *cand_feat, *cand_thr;
  uint32_t *hist;
  uint32_t F, T, K, TP;   // TP = threshold rows padded to a power of two above T
  size_t smem;            // dynamic shared memory per CTA
  FusedSplit fs;
  cudaEvent_t ev_before;  // recorded just before the first launch (may be null)
  unsigned *queue;        // persistent launch: the work counter (zeroed here), null: one CTA per item
};

template <class P>
int launch_hist_grid(pd_ctx *ctx, const HistGrid &g);
// The run-time compiled histogram kernel of a user feature (pd_rtc.cu).
int launch_hist_grid_rtc(pd_ctx *ctx, const HistGrid &g);

extern template int launch_hist_grid<DepthDiff2>(pd_ctx *, const HistGrid &);
extern template int launch_hist_grid<DepthDiff1>(pd_ctx *, const HistGrid &);
extern template int launch_hist_grid<ChannelDiff>(pd_ctx *, const HistGrid &);

}  // namespace pd
