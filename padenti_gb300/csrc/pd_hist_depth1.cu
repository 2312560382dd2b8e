// Histogram kernel instantiations of the DepthDiff1 plugin.
#include "pd_hist_grid_impl.cuh"

namespace pd {
template int launch_hist_grid<DepthDiff1>(pd_ctx *, const HistGrid &);
}  // namespace pd
