// clk_pointwise.cu - whole-image pointwise kernels: copy_{2d,3d} (a
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

}  // namespace

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
