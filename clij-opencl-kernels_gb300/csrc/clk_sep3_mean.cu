// clk_sep3_mean.cu - instantiations of the register-ring separable kernel
// (clk_sep3.cuh) for mean_separable on 16-bit pixels (exact int32 sums,
// dst-typed results between passes).
#include "clk_sep3.cuh"

namespace clk {
namespace {

template <int RMAX>
clk_status mean_by_radius(int R, int cz, const Image& dst, const Image& src, const sep3::P3& p, cudaStream_t st) {
  if constexpr (RMAX >= 1) {
    if (R == RMAX) {
      return src.dt == CLK_U16 ? sep3::by_cz<uint16_t, sep3::MEAN, RMAX, sep3::kMaxCzInt>(cz, dst, src, p, st)
                               : sep3::by_cz<int16_t, sep3::MEAN, RMAX, sep3::kMaxCzInt>(cz, dst, src, p, st);
    }
    return mean_by_radius<RMAX - 1>(R, cz, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace

clk_status sep3_mean(int R, const Image& dst, const Image& src, int cz, cudaStream_t st) {
  if (R < 1 || R > sep3::kMaxRInt || cz < 0 || cz > sep3::kMaxCzInt || src.dt != dst.dt ||
      (src.dt != CLK_U16 && src.dt != CLK_I16) || !sep3::layout_ok(dst, src))
    return CLK_UNSUPPORTED_DTYPE;
  sep3::P3 p{};
  p.mx = sep2::recip32(2 * R + 1);
  p.mz = sep2::recip32(2 * cz + 1);
  return mean_by_radius<sep3::kMaxRInt>(R, cz, dst, src, p, st);
}

}  // namespace clk
