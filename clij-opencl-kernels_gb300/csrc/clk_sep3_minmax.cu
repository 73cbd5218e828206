// clk_sep3_minmax.cu - instantiations of the register-ring separable kernel
// (clk_sep3.cuh) for minimum/maximum_separable on 16-bit pixels.
#include "clk_sep3.cuh"

namespace clk {
namespace {

template <int OP, int RMAX>
clk_status minmax_by_radius(int R, int cz, const Image& dst, const Image& src, const sep3::P3& p, cudaStream_t st) {
  if constexpr (RMAX >= 1) {
    if (R == RMAX) {
      return src.dt == CLK_U16 ? sep3::by_cz<uint16_t, OP, RMAX, sep3::kMaxCzInt>(cz, dst, src, p, st)
                               : sep3::by_cz<int16_t, OP, RMAX, sep3::kMaxCzInt>(cz, dst, src, p, st);
    }
    return minmax_by_radius<OP, RMAX - 1>(R, cz, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace

clk_status sep3_minmax(bool is_max, int R, const Image& dst, const Image& src, int cz, cudaStream_t st) {
  if (R < 1 || R > sep3::kMaxRInt || cz < 0 || cz > sep3::kMaxCzInt || src.dt != dst.dt ||
      (src.dt != CLK_U16 && src.dt != CLK_I16) || !sep3::layout_ok(dst, src))
    return CLK_UNSUPPORTED_DTYPE;
  sep3::P3 p{};
  return is_max ? minmax_by_radius<sep3::MAX, sep3::kMaxRInt>(R, cz, dst, src, p, st)
                : minmax_by_radius<sep3::MIN, sep3::kMaxRInt>(R, cz, dst, src, p, st);
}

}  // namespace clk
