// clk_sep_fused.cu - fused X -> Y -> Z separable filters: one HBM round trip
// (read src once, write dst once) instead of the reference's three launches
// with two temporaries (gaussian_blur_separable_3d_x.cl, mean_separable_3d_x.cl,
// minimum/maximum_separable_3d_x.cl, one launch per dim).
//
// Layout.  A CTA owns a TX x TY column of outputs and streams along z.  For
// every input plane it stages the (TY+2cy) x (TX+2cx) halo tile in shared
// memory (clamped coordinates = CLK_ADDRESS_CLAMP_TO_EDGE), runs the X pass
// into a row buffer, the Y pass into a ring of the last 2cz+1 planes, and,
// once the ring is full, the Z pass straight to global memory.
//
// Exactness.  Temporaries have the dst pixel type and every pass converts
// to it, so integer outputs equal three launches bit for bit; in "exact"
// mode each pass also sums in the reference's order with separately rounded
// multiply and add.  The "fast" mode (float outputs of gaussian/mean only)
// uses FMA with weights pre-divided by their sum.
#include <algorithm>

#include "clk_common.cuh"
#include "clk_fused_impl.cuh"
#include "clk_sep2.cuh"

namespace clk {

namespace {

using namespace fused;

// CLK_SEP3=0 in the environment keeps the register-ring kernels out (A/B
// timing against the shared-memory-ring kernels); so does CLK_SEP2_TMA=1,
// which asks for the shared-memory-ring kernels' TMA staging
bool sep3_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_SEP3");
    const char* t = getenv("CLK_SEP2_TMA");
    return !(e && e[0] == '0') && !(t && t[0] == '1');
  }();
  return on;
}

template <class S, class D, int OP, bool FAST, int KMAX>
clk_status launch_fused(const Image& dst, const Image& src, const FusedTaps& ft, bool rte, cudaStream_t st) {
  const size_t smem = fused_smem(ft.c[0], ft.c[1], ft.c[2], sizeof(S), sizeof(D));
  auto kern = k_fused_sep<S, D, OP, FAST, KMAX>;
  static size_t configured = 0;  // max dynamic smem already granted to this instantiation
  if (smem > 48 * 1024 && smem > configured) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      return CLK_UNSUPPORTED_DTYPE;  // does not fit: let the caller fall back
    }
    configured = smem;
  }
  const int tiles_x = (dst.w + TX - 1) / TX, tiles_y = (dst.h + TY - 1) / TY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // enough z-chunks that the grid fills the GPU twice over, each chunk long
  // enough that the 2cz halo planes stay a small overhead
  int chunks = 1;
  const int64_t tiles = (int64_t)tiles_x * tiles_y;
  while (tiles * chunks < 4LL * sms && dst.d / (chunks * 2) >= std::max(8, 4 * ft.c[2])) chunks *= 2;
  const int zchunk = (dst.d + chunks - 1) / chunks;
  dim3 grid(tiles_x, tiles_y, (dst.d + zchunk - 1) / zchunk);
  kern<<<grid, NTHREADS, smem, st>>>((const S*)src.ptr, (D*)dst.ptr, dst.w, dst.h, dst.d, zchunk, ft, rte);
  count_launch();
  return check_launch("fused separable");
}

template <class S, class D, int OP, bool FAST>
clk_status launch_bucket(const Image& dst, const Image& src, const FusedTaps& ft, bool rte, cudaStream_t st) {
  const int n = 2 * std::max(ft.c[0], ft.c[1]) + 1;
  if (n <= 12) return launch_fused<S, D, OP, FAST, 12>(dst, src, ft, rte, st);
  if (n <= 24) return launch_fused<S, D, OP, FAST, 24>(dst, src, ft, rte, st);
  return launch_fused<S, D, OP, FAST, 2 * kFusedMaxR + 1>(dst, src, ft, rte, st);
}

template <class S, class D>
clk_status launch_types(SepOp op, bool fast, const Image& dst, const Image& src, const FusedTaps& ft, bool rte,
                        cudaStream_t st) {
  switch (op) {
    case SEP_GAUSS:
      if constexpr (sizeof(D) == 4) {
        if (fast) return launch_bucket<S, D, SEP_GAUSS, true>(dst, src, ft, rte, st);
      }
      return launch_bucket<S, D, SEP_GAUSS, false>(dst, src, ft, rte, st);
    case SEP_MEAN: return launch_bucket<S, D, SEP_MEAN, false>(dst, src, ft, rte, st);
    case SEP_MIN: return launch_bucket<S, D, SEP_MIN, false>(dst, src, ft, rte, st);
    case SEP_MAX: return launch_bucket<S, D, SEP_MAX, false>(dst, src, ft, rte, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace

using namespace fused;

clk_status fused_separable(SepOp op, const Image& dst, const Image& src, const SepTaps taps[3], const bool skip[3],
                           const Policy& p, cudaStream_t st) {
  FusedTaps ft;
  const bool fast = op == SEP_GAUSS && dst.dt == CLK_F32 && !p.exact_order;
  for (int d = 0; d < 3; ++d) {
    const bool sk = skip[d] || (d == 2 && src.ndim == 2);
    const int c = sk ? 0 : taps[d].c;
    if (c < 0 || c > kFusedMaxR) return CLK_UNSUPPORTED_DTYPE;
    ft.c[d] = c;
    if (sk || op != SEP_GAUSS) {
      ft.h[d][0] = 1.0f;  // one tap: a converting copy (copy_3d_x.cl:13-14)
      ft.hsum[d] = 1.0f;
      continue;
    }
    if (fast) {
      double s = 0;
      for (int v = 0; v <= 2 * c; ++v) s += taps[d].h[v];
      for (int v = 0; v <= 2 * c; ++v) ft.h[d][v] = (float)(taps[d].h[v] / s);
      ft.hsum[d] = 1.0f;
    } else {
      for (int v = 0; v <= 2 * c; ++v) ft.h[d][v] = taps[d].h[v];
      ft.hsum[d] = taps[d].hsum;
    }
  }
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  // Isotropic XY radius: the register-window kernels (clk_sep2.cuh).
  if (ft.c[0] == ft.c[1] && ft.c[0] >= 1) {
    const int R = ft.c[0], cz = ft.c[2];
    const bool ints = src.dt == dst.dt && src.dt != CLK_F32;
    clk_status s2 = CLK_UNSUPPORTED_DTYPE;
    if ((op == SEP_MIN || op == SEP_MAX) && (ints || (src.dt == CLK_F32 && dst.dt == CLK_F32))) {
      if (sep3_enabled()) s2 = sep3_minmax(op == SEP_MAX, R, dst, src, cz, st);
      if (s2 == CLK_UNSUPPORTED_DTYPE) s2 = sep2_minmax(op == SEP_MAX, R, dst, src, cz, st);
    } else if (op == SEP_MEAN && ints) {
      if (sep3_enabled()) s2 = sep3_mean(R, dst, src, cz, st);
      if (s2 == CLK_UNSUPPORTED_DTYPE) s2 = sep2_mean(R, dst, src, cz, st);
    } else if (op == SEP_GAUSS && ints) {
      // integer outputs: the reference's order and rounding, pass by pass
      const float* h[3] = {ft.h[0], ft.h[1], ft.h[2]};
      s2 = sep2_gauss_exact(R, dst, src, h, ft.hsum, cz, p.rte, st);
    } else if (fast) {
      // folded taps: w[0] for the centre, w[k] for the pair +-k, all / sum(h)
      float w[3][kFusedMaxR + 1] = {};
      for (int d = 0; d < 3; ++d) {
        const int c = ft.c[d];
        double sum = 0;
        for (int v = 0; v <= 2 * c; ++v) sum += ft.h[d][v];
        for (int k = 0; k <= c; ++k) w[d][k] = (float)(ft.h[d][c + k] / sum);
      }
      if (sep3_enabled()) s2 = sep3_gauss(R, dst, src, w[0], w[1], w[2], cz, st);
      if (s2 == CLK_UNSUPPORTED_DTYPE) s2 = sep2_gauss(R, dst, src, w[0], w[1], w[2], cz, st);
    }
    if (s2 != CLK_UNSUPPORTED_DTYPE) return s2;
  }
  if (prefer_line(op, dst, src, ft.c, p)) return CLK_UNSUPPORTED_DTYPE;  // the caller chains line passes
  if (fused_smem(ft.c[0], ft.c[1], ft.c[2], dtype_size(src.dt), dtype_size(dst.dt)) > 200 * 1024)
    return CLK_UNSUPPORTED_DTYPE;
  const int s = src.dt, d = dst.dt;
  if (s == d) {
    switch (s) {
      case CLK_U8: return launch_types<uint8_t, uint8_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I8: return launch_types<int8_t, int8_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_U16: return launch_types<uint16_t, uint16_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I16: return launch_types<int16_t, int16_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_F32: return launch_types<float, float>(op, fast, dst, src, ft, p.rte, st);
    }
  } else if (d == CLK_F32) {
    switch (s) {
      case CLK_U8: return launch_types<uint8_t, float>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I8: return launch_types<int8_t, float>(op, fast, dst, src, ft, p.rte, st);
      case CLK_U16: return launch_types<uint16_t, float>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I16: return launch_types<int16_t, float>(op, fast, dst, src, ft, p.rte, st);
    }
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
