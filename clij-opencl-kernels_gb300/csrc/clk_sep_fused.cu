// clk_sep_fused.cu - fused X+Y+Z separable filters (placeholder).
#include "clk_common.cuh"
namespace clk {
clk_status fused_separable(SepOp, const Image&, const Image&, const SepTaps*, const bool*, const Policy&,
                           cudaStream_t) {
  return CLK_UNSUPPORTED_DTYPE;
}
}  // namespace clk
