// clk_morph.cu - tiled binary morphology (placeholder).
#include "clk_common.cuh"
namespace clk {
clk_status fast_morph(bool, bool, int, const Image&, const Image&, const Policy&, cudaStream_t) {
  return CLK_UNSUPPORTED_DTYPE;
}
}  // namespace clk
