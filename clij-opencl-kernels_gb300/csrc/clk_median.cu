// clk_median.cu - tiled median (placeholder).
#include "clk_common.cuh"
namespace clk {
clk_status fast_median(bool, const Image&, const Image&, const MedianNbhd&, cudaStream_t) {
  return CLK_UNSUPPORTED_DTYPE;
}
}  // namespace clk
