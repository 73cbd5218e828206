// clk_sep2_gaussx.cu - instantiations of the fused separable kernel
// (clk_sep2_impl.cuh) for gaussian_blur_separable to 8/16-bit pixels in the
// reference's arithmetic (gaussian_blur_separable_3d_x.cl:22-33: taps in
// order, float multiply then add, division by the float sum of the taps;
// every pass converted to the dst type, as three launches with dst-typed
// temporaries would), bit-exact.
#include "clk_sep2_impl.cuh"

namespace clk {

clk_status sep2_gauss_exact(int R, const Image& dst, const Image& src, const float* const h[3], const float hs[3],
                            int cz, bool rte, cudaStream_t st) {
  using namespace sep2;
  if (R < 1 || R > kMaxRIntegers || cz < 0 || cz > kMaxCz || src.dt != dst.dt || !layout_ok(dst, src, 2))
    return CLK_UNSUPPORTED_DTYPE;
  Params p{};
  p.cz = cz;
  for (int v = 0; v <= 2 * R; ++v) p.hx[v] = h[0][v], p.hy[v] = h[1][v];
  for (int v = 0; v <= 2 * cz; ++v) p.hz[v] = h[2][v];
  for (int d = 0; d < 3; ++d) p.hs[d] = hs[d];
  p.rte = rte ? 1 : 0;
  switch (src.dt) {
    case CLK_U16: return by_radius<uint16_t, uint16_t, GAUSSX, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_I16: return by_radius<int16_t, int16_t, GAUSSX, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_U8: return by_radius<uint8_t, uint8_t, GAUSSX, kMaxRIntegers>(R, dst, src, p, st);
    case CLK_I8: return by_radius<int8_t, int8_t, GAUSSX, kMaxRIntegers>(R, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
