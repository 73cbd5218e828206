// clk_sobel.cu - tiled Sobel (placeholder).
#include "clk_common.cuh"
namespace clk {
clk_status fast_sobel(const Image&, const Image&, const Policy&, cudaStream_t) { return CLK_UNSUPPORTED_DTYPE; }
}  // namespace clk
