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

// laplace_diamond_{2d,3d}_x.cl, laplace_box_2d_x.cl and, for signed
// integer pixels, laplace_box_3d_x.cl over whole rows: for integer pixels
// every partial sum of those expressions is an integer far below 2^24, so the
// reference's float / double evaluation equals the int32 sum K*c - sum of the
// neighbours (laplace_box_3d: c - sum of the 26 others, v * -1 being exact
// for signed reads).  A thread takes eight consecutive outputs of one row
// from eight-wide loads of the rows / planes around it and the two clamped
// end neighbours of each.
template <class S> __device__ __forceinline__ void row8(const S* __restrict__ src, int64_t rowoff, int x, int W,
                                                        int (&v)[10]) {
  const Oct<S> c = reinterpret_cast<const Oct<S>*>(src + rowoff + x)[0];
  v[0] = (int)__ldg(src + rowoff + max(x - 1, 0));
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k + 1] = (int)c.v[k];
  v[9] = (int)__ldg(src + rowoff + min(x + 8, W - 1));
}

template <class S, class D, int KIND>
__global__ void __launch_bounds__(kPwBlock)
    k_laplace_rows(D* __restrict__ dst, const S* __restrict__ src, int W, int H, int Dz, bool rte) {
  const int nvec = W / 8;
  const int64_t rows = (int64_t)H * Dz, work = rows * nvec;
  const int64_t stride = (int64_t)gridDim.x * kPwBlock;
  const int64_t plane = (int64_t)W * H;
  for (int64_t t = blockIdx.x * (int64_t)kPwBlock + threadIdx.x; t < work; t += stride) {
    const int64_t row = t / nvec;
    const int x = 8 * (int)(t - row * nvec);
    const int y = (int)(row % H), z = (int)(row / H);
    const int64_t r0 = (int64_t)z * plane + (int64_t)y * W;
    const int64_t up = (int64_t)z * plane + (int64_t)max(y - 1, 0) * W;
    const int64_t dn = (int64_t)z * plane + (int64_t)min(y + 1, H - 1) * W;
    int acc[8];
    int c[10], a[10], b[10];
    row8(src, r0, x, W, c);
    row8(src, up, x, W, a);
    row8(src, dn, x, W, b);
    if constexpr (KIND == ST_LAPLACE_DIAMOND_2D || KIND == ST_LAPLACE_DIAMOND_3D) {
      constexpr int K = KIND == ST_LAPLACE_DIAMOND_2D ? 4 : 6;
#pragma unroll
      for (int k = 0; k < 8; ++k) acc[k] = K * c[k + 1] - c[k] - c[k + 2] - a[k + 1] - b[k + 1];
      if constexpr (KIND == ST_LAPLACE_DIAMOND_3D) {
        const Oct<S> f = reinterpret_cast<const Oct<S>*>(src + (int64_t)max(z - 1, 0) * plane + (int64_t)y * W + x)[0];
        const Oct<S> g = reinterpret_cast<const Oct<S>*>(src + (int64_t)min(z + 1, Dz - 1) * plane + (int64_t)y * W + x)[0];
#pragma unroll
        for (int k = 0; k < 8; ++k) acc[k] -= (int)f.v[k] + (int)g.v[k];
      }
    } else if constexpr (KIND == ST_LAPLACE_BOX_2D) {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        acc[k] = 8 * c[k + 1] - c[k] - c[k + 2] - a[k] - a[k + 1] - a[k + 2] - b[k] - b[k + 1] - b[k + 2];
    } else {  // laplace_box_3d, signed pixels
#pragma unroll
      for (int k = 0; k < 8; ++k)
        acc[k] = 2 * c[k + 1] - c[k] - c[k + 1] - c[k + 2] - a[k] - a[k + 1] - a[k + 2] - b[k] - b[k + 1] - b[k + 2];
#pragma unroll
      for (int dz = -1; dz <= 1; dz += 2) {
        const int zz = min(max(z + dz, 0), Dz - 1);
        int p[10], q[10], u[10];
        row8(src, (int64_t)zz * plane + (int64_t)y * W, x, W, p);
        row8(src, (int64_t)zz * plane + (int64_t)max(y - 1, 0) * W, x, W, q);
        row8(src, (int64_t)zz * plane + (int64_t)min(y + 1, H - 1) * W, x, W, u);
#pragma unroll
        for (int k = 0; k < 8; ++k)
          acc[k] -= p[k] + p[k + 1] + p[k + 2] + q[k] + q[k + 1] + q[k + 2] + u[k] + u[k + 1] + u[k + 2];
      }
    }
    Oct<D> out;
#pragma unroll
    for (int k = 0; k < 8; ++k) out.v[k] = convert_sat<D>((float)acc[k], rte);
    reinterpret_cast<Oct<D>*>(dst + r0 + x)[0] = out;
  }
}

}  // namespace

clk_status fast_laplace(int kind, const Image& dst, const Image& src, const Policy& p, cudaStream_t st) {
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d || src.w % 8 != 0) return CLK_UNSUPPORTED_DTYPE;
  if (src.dt == CLK_F32) return CLK_UNSUPPORTED_DTYPE;  // float pixels: the reference's rounding order
  if (kind == ST_LAPLACE_BOX_3D && (src.dt == CLK_U8 || src.dt == CLK_U16))
    return CLK_UNSUPPORTED_DTYPE;  // unsigned reads wrap: the float sum's order decides
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
    if constexpr (std::is_integral<S>::value) {
      auto* o = (D*)dst.ptr;
      auto* in = (const S*)src.ptr;
      switch (kind) {
        case ST_LAPLACE_DIAMOND_2D:
          k_laplace_rows<S, D, ST_LAPLACE_DIAMOND_2D><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
          break;
        case ST_LAPLACE_DIAMOND_3D:
          k_laplace_rows<S, D, ST_LAPLACE_DIAMOND_3D><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
          break;
        case ST_LAPLACE_BOX_2D:
          k_laplace_rows<S, D, ST_LAPLACE_BOX_2D><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
          break;
        default:
          k_laplace_rows<S, D, ST_LAPLACE_BOX_3D><<<grid, kPwBlock, 0, st>>>(o, in, src.w, src.h, src.d, p.rte);
      }
    }
  });
  if (!ok) return CLK_UNSUPPORTED_DTYPE;
  count_launch();
  return check_launch("laplace (rows)");
}

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
