// clk_sep2_gauss.cu - instantiations of the fused separable kernel (clk_sep2_impl.cuh)
// for gaussian_blur_separable to float.
#include "clk_sep2_impl.cuh"

namespace clk {

clk_status sep2_gauss(int R, const Image& dst, const Image& src, const float* wx, const float* wy, const float* wz,
                      int cz, cudaStream_t st) {
  using namespace sep2;
  if (R < 1 || R > kMaxRGauss || cz < 0 || cz > kMaxCz || dst.dt != CLK_F32 || !layout_ok(dst, src, 2))
    return CLK_UNSUPPORTED_DTYPE;
  Params p{};
  p.cz = cz;
  for (int k = 0; k <= R; ++k) p.wx[k] = wx[k], p.wy[k] = wy[k];
  for (int k = 0; k <= cz; ++k) p.wz[k] = wz[k];
  switch (src.dt) {
    case CLK_U16: return by_radius<uint16_t, float, GAUSS, kMaxRGauss>(R, dst, src, p, st);
    case CLK_I16: return by_radius<int16_t, float, GAUSS, kMaxRGauss>(R, dst, src, p, st);
    case CLK_U8: return by_radius<uint8_t, float, GAUSS, kMaxRGauss>(R, dst, src, p, st);
    case CLK_I8: return by_radius<int8_t, float, GAUSS, kMaxRGauss>(R, dst, src, p, st);
    case CLK_F32: return by_radius<float, float, GAUSS, kMaxRGauss>(R, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
