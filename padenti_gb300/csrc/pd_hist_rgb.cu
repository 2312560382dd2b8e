// Histogram kernel instantiations of the ChannelDiff plugin.
#include "pd_hist_grid_impl.cuh"

namespace pd {
template int launch_hist_grid<ChannelDiff>(pd_ctx *, const HistGrid &);
}  // namespace pd
