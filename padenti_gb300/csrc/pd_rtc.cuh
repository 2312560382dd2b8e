// Run-time compiled feature plugins (PD_PLUGIN_USER): the kernels that depend on
// the feature, compiled by NVRTC from the user's computeFeature and the kernel
// headers embedded in the library, loaded as a CUDA library on the context's
// device.  The host paths of the built-in plugin with the same types and
// dimensions (dispatch_config) run unchanged and launch these kernels instead.
#pragma once

#include "pd_ctx.cuh"

namespace pd {

struct RtcKernels {
  cudaKernel_t reassign = nullptr, build_rec = nullptr, cand_order = nullptr;
  cudaKernel_t predict_posterior = nullptr, predict_leaf = nullptr, predict_batch = nullptr;
  cudaKernel_t forest_nodes = nullptr;
  cudaKernel_t node_map_step = nullptr;  // k_node_map_step (features that read the tree)
  int node_rec_bytes = 0;                // sizeof(NodeRec<UserPlugin>) as compiled
};

// The compiled base kernels; PD_ERR_STATE when pd_plugin_compile has not run.
int rtc_kernels(pd_ctx *ctx, const RtcKernels **out);
// k_hist<UserPlugin, TP, SPI>, compiled on first use.
int rtc_hist_kernel(pd_ctx *ctx, uint32_t TP, int SPI, cudaKernel_t *out);
// Dynamic shared memory limit (and carve-out when pct >= 0) of a kernel.
int rtc_set_smem(pd_ctx *ctx, cudaKernel_t k, size_t smem, int carveout_pct = -1);
int rtc_launch(pd_ctx *ctx, cudaKernel_t k, dim3 grid, dim3 block, size_t smem, void **args);
void rtc_release(pd_ctx *ctx);

inline bool is_user_plugin(const pd_ctx *ctx) { return ctx->cfg.plugin == PD_PLUGIN_USER; }

}  // namespace pd
