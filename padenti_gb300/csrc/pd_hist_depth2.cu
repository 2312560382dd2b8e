// Histogram kernel instantiations of the DepthDiff2 plugin.
#include "pd_hist_grid_impl.cuh"

namespace pd {
template int launch_hist_grid<DepthDiff2>(pd_ctx *, const HistGrid &);
}  // namespace pd
