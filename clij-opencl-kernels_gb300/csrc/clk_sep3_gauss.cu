// clk_sep3_gauss.cu - instantiations of the register-ring separable kernel
// (clk_sep3.cuh) for the Gaussian from unsigned 16-bit pixels to float.
#include "clk_sep3.cuh"

namespace clk {
namespace {

template <int RMAX>
clk_status gauss_by_radius(int R, int cz, const Image& dst, const Image& src, const sep3::P3& p, cudaStream_t st) {
  if constexpr (RMAX >= 1) {
    if (R == RMAX) return sep3::by_cz<uint16_t, sep3::GAUSS, RMAX, sep3::kMaxCzGauss>(cz, dst, src, p, st);
    return gauss_by_radius<RMAX - 1>(R, cz, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

uint64_t pair(float w) {
  uint32_t u;
  memcpy(&u, &w, 4);
  return (uint64_t)u | ((uint64_t)u << 32);
}

}  // namespace

// wx, wy, wz: folded taps (w[0] the centre, w[k] for +-k), already divided
// by their sums
clk_status sep3_gauss(int R, const Image& dst, const Image& src, const float* wx, const float* wy, const float* wz,
                      int cz, cudaStream_t st) {
  if (R < 1 || R > sep3::kMaxRGauss || cz < 0 || cz > sep3::kMaxCzGauss || src.dt != CLK_U16 ||
      dst.dt != CLK_F32 || !sep3::layout_ok(dst, src))
    return CLK_UNSUPPORTED_DTYPE;
  sep3::P3 p{};
  for (int k = 0; k <= R; ++k) p.wx[k] = pair(wx[k]), p.wy[k] = pair(wy[k]);
  for (int k = 0; k <= cz; ++k) p.wz[k] = pair(wz[k]);
  return gauss_by_radius<sep3::kMaxRGauss>(R, cz, dst, src, p, st);
}

}  // namespace clk
