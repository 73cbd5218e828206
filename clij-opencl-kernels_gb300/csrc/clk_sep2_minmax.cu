// clk_sep2_minmax.cu - instantiations of the fused separable kernel (clk_sep2_impl.cuh)
// for minimum/maximum_separable on 8/16-bit pixels (16-bit SIMD lanes) and
// float pixels (the reference's comparison order).
#include "clk_sep2_impl.cuh"

namespace clk {

clk_status sep2_minmax(bool is_max, int R, const Image& dst, const Image& src, int cz, cudaStream_t st) {
  using namespace sep2;
  if (R < 1 || R > kMaxRIntegers || cz < 0 || cz > kMaxCz || src.dt != dst.dt || !layout_ok(dst, src, 2))
    return CLK_UNSUPPORTED_DTYPE;
  Params p{};
  p.cz = cz;
  switch (src.dt) {
    case CLK_U16:
      return is_max ? by_radius<uint16_t, uint16_t, MAX, kMaxRIntegers>(R, dst, src, p, st)
                    : by_radius<uint16_t, uint16_t, MIN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_I16:
      return is_max ? by_radius<int16_t, int16_t, MAX, kMaxRIntegers>(R, dst, src, p, st)
                    : by_radius<int16_t, int16_t, MIN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_U8:
      return is_max ? by_radius<uint8_t, uint8_t, MAX, kMaxRIntegers>(R, dst, src, p, st)
                    : by_radius<uint8_t, uint8_t, MIN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_I8:
      return is_max ? by_radius<int8_t, int8_t, MAX, kMaxRIntegers>(R, dst, src, p, st)
                    : by_radius<int8_t, int8_t, MIN, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_F32:  // the reference's comparison order
      return is_max ? by_radius<float, float, MAXF, kMaxRIntegers>(R, dst, src, p, st)
                    : by_radius<float, float, MINF, kMaxRIntegers>(R, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
