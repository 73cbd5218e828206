// clk_pointwise.cu - whole-image pointwise and axis-difference kernels:
// copy_{2d,3d} (a
// converting copy, copy_3d_x.cl:7-14) and greater_constant_{2d,3d}
// (greater_constant_3d_x.cl:10-17), for the common case of a full-range
// launch on images of equal extent.  Each thread moves eight pixels per step
// with vector loads and stores (a grid-stride loop over the flat image); the
// values are exactly those of the per-voxel kernels in clk_direct.cu.
#include <algorithm>
#include <type_traits>

#include "clk_common.cuh"
#include "clk_internal.h"

namespace clk {
namespace {

constexpr int kPwBlock = 256;

template <class T> struct alignas(8 * sizeof(T)) Oct {
  T v[8];
};

template <class S> __device__ __forceinline__ float xval(S t) {
  // .x of a read (uint / int / float) converted to float
  if constexpr (std::is_same<S, float>::value) return t;
  else if constexpr (std::is_signed<S>::value) return (float)(int)t;
  else return (float)(unsigned)t;
}

enum PwOp { PW_COPY = 0, PW_GREATER = 1 };

template <class S, class D, int OP>
__global__ void __launch_bounds__(kPwBlock)
    k_pointwise(D* __restrict__ dst, const S* __restrict__ src, int64_t n, float scalar, bool rte) {
  auto f = [&](S t) -> D {
    if constexpr (OP == PW_COPY) return convert_sat<D>(xval(t), rte);
    else return xval(t) > scalar ? (D)1 : (D)0;
  };
  const int64_t nv = n / 8;
  const int64_t stride = (int64_t)gridDim.x * kPwBlock;
  for (int64_t v = blockIdx.x * (int64_t)kPwBlock + threadIdx.x; v < nv; v += stride) {
    const Oct<S> in = reinterpret_cast<const Oct<S>*>(src)[v];
    Oct<D> out;
#pragma unroll
    for (int k = 0; k < 8; ++k) out.v[k] = f(in.v[k]);
    reinterpret_cast<Oct<D>*>(dst)[v] = out;
  }
  for (int64_t i = nv * 8 + blockIdx.x * (int64_t)kPwBlock + threadIdx.x; i < n; i += stride) dst[i] = f(__ldg(src + i));
}

// gradient_{x,y,z}_{2d,3d}_x.cl over whole rows: a thread takes eight
// consecutive outputs of one row; their values B - A come from eight-wide
// loads of the neighbouring rows / planes (y, z) or of the row itself with its
// two clamped end neighbours (x).
template <class S, class D, int AXIS>
__global__ void __launch_bounds__(kPwBlock)
    k_gradient_rows(D* __restrict__ dst, const S* __restrict__ src, int W, int H, int Dz, bool rte) {
  const int nvec = W / 8;
  const int64_t rows = (int64_t)H * Dz, work = rows * nvec;
  const int64_t stride = (int64_t)gridDim.x * kPwBlock;
  for (int64_t t = blockIdx.x * (int64_t)kPwBlock + threadIdx.x; t < work; t += stride) {
    const int64_t row = t / nvec;
    const int xv = (int)(t - row * nvec);
    const int y = (int)(row % H), z = (int)(row / H);
    const int64_t o = row * W + 8 * xv;
    float a[8], b[8];
    if constexpr (AXIS == 0) {
      const Oct<S> c = reinterpret_cast<const Oct<S>*>(src + o)[0];
      const float l = xval(__ldg(src + row * W + max(8 * xv - 1, 0)));
      const float r = xval(__ldg(src + row * W + min(8 * xv + 8, W - 1)));
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        a[k] = k == 0 ? l : xval(c.v[k - 1]);
        b[k] = k == 7 ? r : xval(c.v[k + 1]);
      }
    } else {
      const int64_t step = AXIS == 1 ? (int64_t)W : (int64_t)W * H;
      const int p = AXIS == 1 ? y : z, P = AXIS == 1 ? H : Dz;
      const Oct<S> ca = reinterpret_cast<const Oct<S>*>(src + o - (p > 0 ? step : 0))[0];
      const Oct<S> cb = reinterpret_cast<const Oct<S>*>(src + o + (p < P - 1 ? step : 0))[0];
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = xval(ca.v[k]), b[k] = xval(cb.v[k]);
    }
    Oct<D> out;
#pragma unroll
    for (int k = 0; k < 8; ++k) out.v[k] = convert_sat<D>(__fsub_rn(b[k], a[k]), rte);
    reinterpret_cast<Oct<D>*>(dst + o)[0] = out;
  }
}

}  // namespace

clk_status fast_gradient(int axis, const Image& dst, const Image& src, const Policy& p, cudaStream_t st) {
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d || src.w % 8 != 0) return CLK_UNSUPPORTED_DTYPE;
  if ((uintptr_t)src.ptr % (8 * dtype_size(src.dt)) != 0 || (uintptr_t)dst.ptr % (8 * dtype_size(dst.dt)) != 0)
    return CLK_UNSUPPORTED_DTYPE;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t work = (int64_t)src.h * src.d * (src.w / 8);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + kPwBlock - 1) / kPwBlock,
                                                                         (int64_t)sms * 8));
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    auto* o = (D*)dst.ptr;
    auto* in = (const S*)src.ptr;
    if (axis == 0) k_gradient_rows<S, D, 0><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
    else if (axis == 1) k_gradient_rows<S, D, 1><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
    else k_gradient_rows<S, D, 2><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
  });
  if (!ok) return CLK_UNSUPPORTED_DTYPE;
  count_launch();
  return check_launch("gradient (rows)");
}

clk_status fast_pointwise(bool greater, const Image& dst, const Image& src, float scalar, const Policy& p,
                          cudaStream_t st) {
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  if ((uintptr_t)src.ptr % (8 * dtype_size(src.dt)) != 0 || (uintptr_t)dst.ptr % (8 * dtype_size(dst.dt)) != 0)
    return CLK_UNSUPPORTED_DTYPE;
  const int64_t n = dst.count();
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t want = (n / 8 + kPwBlock - 1) / kPwBlock;
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * 8));
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    if (greater)
      k_pointwise<S, D, PW_GREATER><<<grid, kPwBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, n, scalar, p.rte);
    else
      k_pointwise<S, D, PW_COPY><<<grid, kPwBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, n, scalar, p.rte);
  });
  if (!ok) return CLK_UNSUPPORTED_DTYPE;
  count_launch();
  return check_launch(greater ? "greater_constant (pointwise)" : "copy (pointwise)");
}

}  // namespace clk
