// clk_sep2_mean.cu - instantiations of the fused separable kernel (clk_sep2_impl.cuh)
// for mean_separable on 8/16-bit pixels.
#include "clk_sep2_impl.cuh"

namespace clk {

clk_status sep2_mean(int R, const Image& dst, const Image& src, int cz, cudaStream_t st) {
  using namespace sep2;
  if (R < 1 || R > kMaxRIntegers || cz < 0 || cz > kMaxCz || src.dt != dst.dt || !layout_ok(dst, src, 2))
    return CLK_UNSUPPORTED_DTYPE;
  Params p{};
  p.cz = cz;
  p.mx = recip32(2 * R + 1);
  p.mz = recip32(2 * cz + 1);
  switch (src.dt) {
    case CLK_U16: return by_radius<uint16_t, uint16_t, MEAN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_I16: return by_radius<int16_t, int16_t, MEAN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_U8: return by_radius<uint8_t, uint8_t, MEAN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_I8: return by_radius<int8_t, int8_t, MEAN, kMaxRIntegers>(R, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
