// Definition of launch_hist_grid<P>; included only by the per-plugin
// translation units that instantiate it.
#pragma once

#include "pd_hist_grid.cuh"
#include "pd_rtc.cuh"

namespace pd {

template <class P, uint32_t TP, int SPI>
static int launch_hist_grid_as(pd_ctx *ctx, const HistGrid &g) {
  using FeatT = typename P::feat_t;
  auto kern = k_hist<P, TP, SPI>;
  PD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem));
  // carve out only the shared memory the resident CTAs need; the rest stays L1
  // for the probe gathers (resident CTAs are register-limited: 3 at 2 samples
  // per iteration, 2 at 4 or 8)
  const int resident = SPI <= 2 ? 3 : 2;
  cudaFuncAttributes fa;
  PD_CUDA(cudaFuncGetAttributes(&fa, kern));
  const size_t per_cta = g.smem + fa.sharedSizeBytes + 1024;  // dynamic + static + reserved
  const int pct = (int)std::min<size_t>(100, (resident * per_cta * 100 + 233471) / 233472);
  PD_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
  if (g.queue) PD_CUDA(cudaMemsetAsync(g.queue, 0, 4, ctx->stream));
  if (g.ev_before) PD_CUDA(cudaEventRecord(g.ev_before, ctx->stream));
  // Without a queue the grid is the work list and the hardware scheduler keeps
  // every SM full; with one, resident CTAs pull the items in list order.
  for (uint64_t b = 0; b < g.n_items; b += 0x7fffffffull) {
    const uint64_t cnt = std::min<uint64_t>(g.n_items - b, 0x7fffffffull);
    const unsigned grid = g.queue ? (unsigned)std::min<uint64_t>(cnt, (uint64_t)ctx->n_sms * resident)
                                  : (unsigned)cnt;
    kern<<<grid, kHistThreads, g.smem, ctx->stream>>>(
        g.ds, g.rec, g.items + b, (uint32_t)cnt, g.queue, static_cast<const FeatT *>(g.cand_feat),
        static_cast<const FeatT *>(g.cand_thr), g.hist, g.F, g.T, g.K, g.fs);
    PD_CUDA(cudaGetLastError());
    ctx->launches++;
    if (g.queue) break;  // a persistent list holds fewer than 2^31 items
  }
  return PD_OK;
}

template <class P, uint32_t TP>
static int launch_hist_grid_tp(pd_ctx *ctx, const HistGrid &g) {
  switch (ctx->hist_spi) {
    case 2: return launch_hist_grid_as<P, TP, 2>(ctx, g);
    case 4: return launch_hist_grid_as<P, TP, 4>(ctx, g);
    case 8: return launch_hist_grid_as<P, TP, 8>(ctx, g);
    default: return set_error(PD_ERR_INVALID, "hist_spi %u", ctx->hist_spi);
  }
}

template <class P>
int launch_hist_grid(pd_ctx *ctx, const HistGrid &g) {
  switch (g.TP) {
    case 2: return launch_hist_grid_tp<P, 2>(ctx, g);
    case 4: return launch_hist_grid_tp<P, 4>(ctx, g);
    case 8: return launch_hist_grid_tp<P, 8>(ctx, g);
    case 16: return launch_hist_grid_tp<P, 16>(ctx, g);
    case 32: return launch_hist_grid_tp<P, 32>(ctx, g);
    case 64: return launch_hist_grid_tp<P, 64>(ctx, g);
    case 128: return launch_hist_grid_tp<P, 128>(ctx, g);
    case 256: return launch_hist_grid_tp<P, 256>(ctx, g);
    case 512: return launch_hist_grid_tp<P, 512>(ctx, g);
    default: return set_error(PD_ERR_UNSUPPORTED, "n_thresholds %u", g.T);
  }
}

}  // namespace pd
