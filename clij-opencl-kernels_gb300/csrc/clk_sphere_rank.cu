// clk_sphere_rank.cu - fast minimum / maximum / mean over the small spheres
// (minimum_sphere_3d_x.cl, maximum_sphere_3d_x.cl, mean_sphere_3d_x.cl and
// the 2-D / slice-by-slice kernels) for 8/16-bit pixels with src type = dst
// type: radius 1 (the 7- or 5-point cross) and radius 2 (the 33-point sphere,
// 13-point disk).
//
// With equal pixel types every value semantics of the reference kernels
// (float running value, dst-typed CONVERT, dst-typed cast) reduces to the
// exact integer operation, and the mean's float sum of integers is exact
// (|sum| < 2^24), so CONVERT(sum / n) = trunc(sum / n) is computed by the
// exact multiply-high division.  A thread owns two x-outputs (two 16-bit
// lanes, packed min/max) at one row and walks along z; per input plane it
// reduces the in-plane part once (the 3x3 block, the cross arms, the points
// at distance 2) and the z neighbours come from a register ring of planes.
#include "clk_internal.h"
#include "clk_median_impl.cuh"

namespace clk {
namespace srank {
namespace {

using med::BX;
using med::BY;
using med::Px;

enum Op { MIN = 0, MAX = 1, MEAN = 2 };

// per-lane accumulator: packed lanes for min/max, two int32 sums for the mean
template <class T, int OP> struct Acc {
  typedef typename Px<T>::V V;
  V v;
};
template <class T> struct Acc<T, MEAN> {
  int lo, hi;
};

template <class T, int OP> __device__ __forceinline__ Acc<T, OP> from(typename Px<T>::V v) {
  Acc<T, OP> a;
  if constexpr (OP == MEAN) {
    if constexpr (std::is_signed<T>::value) a.lo = (int)(int16_t)(v.v & 0xFFFFu), a.hi = (int)v.v >> 16;
    else a.lo = (int)(v.v & 0xFFFFu), a.hi = (int)(v.v >> 16);
  } else {
    a.v = v;
  }
  return a;
}
template <class T, int OP> __device__ __forceinline__ Acc<T, OP> join(Acc<T, OP> a, Acc<T, OP> b) {
  if constexpr (OP == MEAN) {
    a.lo += b.lo, a.hi += b.hi;
  } else if constexpr (OP == MIN) {
    a.v = med::vmin(a.v, b.v);
  } else {
    a.v = med::vmax(a.v, b.v);
  }
  return a;
}

// exact truncating division of a lane sum by n (m = ceil(2^32 / n))
__device__ __forceinline__ int qdiv(int s, uint32_t m) {
  const uint32_t a = (uint32_t)(s < 0 ? -s : s);
  const int q = (int)__umulhi(a, m);
  return s < 0 ? -q : q;
}

// What one input plane contributes, at this thread's pair (x, x+1), row y.
template <class T, int OP> struct PlaneVals {
  Acc<T, OP> inplane;  // R=1: the in-plane cross (5); R=2: the 3x3 block
  Acc<T, OP> extra;    // R=2: x-2, x+2, y-2, y+2 of the plane
  Acc<T, OP> centre;   // (x, y) of the plane
};

template <class T, int OP, int R, bool ODD>
__device__ __forceinline__ PlaneVals<T, OP> plane_vals(const T* pl, int x, int y, int W, int H) {
  using V = typename Px<T>::V;
  PlaneVals<T, OP> p;
  V a, b, c, fl, fr;
  med::row_cols<T, ODD>(pl + (int64_t)y * W, x, W, a, b, c, &fl, &fr);
  p.centre = from<T, OP>(b);
  const T* rup = pl + (int64_t)clampi(y - 1, H - 1) * W;
  const T* rdn = pl + (int64_t)clampi(y + 1, H - 1) * W;
  if constexpr (R == 1) {
    Acc<T, OP> s = join<T, OP>(join<T, OP>(from<T, OP>(b), from<T, OP>(a)), from<T, OP>(c));
    s = join<T, OP>(s, from<T, OP>(med::load_pair<T, ODD>(rup, x, W)));
    p.inplane = join<T, OP>(s, from<T, OP>(med::load_pair<T, ODD>(rdn, x, W)));
  } else {
    Acc<T, OP> s = join<T, OP>(join<T, OP>(from<T, OP>(a), from<T, OP>(b)), from<T, OP>(c));
    V ua, ub, uc, da, db, dc;
    med::row_cols<T, ODD>(rup, x, W, ua, ub, uc);
    med::row_cols<T, ODD>(rdn, x, W, da, db, dc);
    s = join<T, OP>(s, join<T, OP>(join<T, OP>(from<T, OP>(ua), from<T, OP>(ub)), from<T, OP>(uc)));
    p.inplane = join<T, OP>(s, join<T, OP>(join<T, OP>(from<T, OP>(da), from<T, OP>(db)), from<T, OP>(dc)));
    // x-2 / x+2 of the outputs x, x+1: the far pairs (x-2, x-1) and
    // (x+2, x+3), lane by lane
    Acc<T, OP> e = join<T, OP>(from<T, OP>(fl), from<T, OP>(fr));
    e = join<T, OP>(e, from<T, OP>(med::load_pair<T, ODD>(pl + (int64_t)clampi(y - 2, H - 1) * W, x, W)));
    p.extra = join<T, OP>(e, from<T, OP>(med::load_pair<T, ODD>(pl + (int64_t)clampi(y + 2, H - 1) * W, x, W)));
  }
  return p;
}

// output = the reduction at (x..x+1, y, zo) of the sphere; ZN: with z
// neighbours (3-D spheres), else the plane alone (2-D / slice by slice)
template <class T, int OP, int R, bool ZN, bool ODD>
__global__ void __launch_bounds__(BX * BY) k_sphere_rank(const T* __restrict__ src, T* __restrict__ dst, int W, int H,
                                                         int D, int zchunk, uint32_t recip) {
  const int x = 2 * (blockIdx.x * BX + (int)threadIdx.x % BX);
  const int y = blockIdx.y * BY + (int)threadIdx.x / BX;
  if (x >= W || y >= H) return;
  const int z0 = blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto pl = [&](int z) { return src + (int64_t)clampi(z, D - 1) * plane; };
  auto store = [&](int zo, Acc<T, OP> r) {
    typename Px<T>::V v;
    if constexpr (OP == MEAN) {
      v = Px<T>::template make<int>(qdiv(r.lo, recip), qdiv(r.hi, recip));
    } else {
      v = r.v;
    }
    med::store_pair<T, ODD>(dst + (int64_t)zo * plane + (int64_t)y * W, x, W, v);
  };
  if constexpr (!ZN) {
    for (int zo = z0; zo < z1; ++zo) {
      const PlaneVals<T, OP> p = plane_vals<T, OP, R, ODD>(pl(zo), x, y, W, H);
      store(zo, R == 1 ? p.inplane : join<T, OP>(p.inplane, p.extra));
    }
  } else if constexpr (R == 1) {
    // cross: in-plane cross of zo, centres of zo-1 and zo+1
    Acc<T, OP> cprev = plane_vals<T, OP, R, ODD>(pl(z0 - 1), x, y, W, H).centre;
    PlaneVals<T, OP> cur = plane_vals<T, OP, R, ODD>(pl(z0), x, y, W, H);
    for (int zo = z0; zo < z1; ++zo) {
      const PlaneVals<T, OP> nxt = plane_vals<T, OP, R, ODD>(pl(zo + 1), x, y, W, H);
      store(zo, join<T, OP>(join<T, OP>(cur.inplane, cprev), nxt.centre));
      cprev = cur.centre;
      cur = nxt;
    }
  } else {
    // sphere r=2: blocks of zo-1, zo, zo+1; extras of zo; centres of zo-2, zo+2
    PlaneVals<T, OP> pm2 = plane_vals<T, OP, R, ODD>(pl(z0 - 2), x, y, W, H);
    PlaneVals<T, OP> pm1 = plane_vals<T, OP, R, ODD>(pl(z0 - 1), x, y, W, H);
    PlaneVals<T, OP> p0 = plane_vals<T, OP, R, ODD>(pl(z0), x, y, W, H);
    PlaneVals<T, OP> pp1 = plane_vals<T, OP, R, ODD>(pl(z0 + 1), x, y, W, H);
    for (int zo = z0; zo < z1; ++zo) {
      const PlaneVals<T, OP> pp2 = plane_vals<T, OP, R, ODD>(pl(zo + 2), x, y, W, H);
      Acc<T, OP> r = join<T, OP>(join<T, OP>(pm1.inplane, p0.inplane), pp1.inplane);
      r = join<T, OP>(join<T, OP>(r, p0.extra), join<T, OP>(pm2.centre, pp2.centre));
      store(zo, r);
      pm2 = pm1, pm1 = p0, p0 = pp1, pp1 = pp2;
    }
  }
}

template <class T, int OP, int R, bool ZN>
clk_status launch(const Image& dst, const Image& src, uint32_t recip, cudaStream_t st) {
  const dim3 block(BX * BY);
  const int tx = ((src.w + 1) / 2 + BX - 1) / BX, ty = (src.h + BY - 1) / BY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 8LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
  if (src.w & 1)
    k_sphere_rank<T, OP, R, ZN, true><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d,
                                                              zchunk, recip);
  else
    k_sphere_rank<T, OP, R, ZN, false><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d,
                                                               zchunk, recip);
  count_launch();
  return check_launch("sphere rank (fast)");
}

template <class T, int OP>
clk_status by_shape(int R, bool zn, const Image& dst, const Image& src, uint32_t recip, cudaStream_t st) {
  if (R == 1) return zn ? launch<T, OP, 1, true>(dst, src, recip, st) : launch<T, OP, 1, false>(dst, src, recip, st);
  return zn ? launch<T, OP, 2, true>(dst, src, recip, st) : launch<T, OP, 2, false>(dst, src, recip, st);
}

template <class T>
clk_status by_op(RankOp op, int R, bool zn, const Image& dst, const Image& src, uint32_t recip, cudaStream_t st) {
  switch (op) {
    case RANK_MIN: return by_shape<T, MIN>(R, zn, dst, src, recip, st);
    case RANK_MAX: return by_shape<T, MAX>(R, zn, dst, src, recip, st);
    case RANK_MEAN: return by_shape<T, MEAN>(R, zn, dst, src, recip, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace
}  // namespace srank

clk_status fast_sphere_rank(RankOp op, bool planar, const Image& dst, const Image& src, const MedianNbhd& m,
                            cudaStream_t st) {
  using namespace srank;
  if (src.dt != dst.dt || src.dt == CLK_F32) return CLK_UNSUPPORTED_DTYPE;
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  if ((((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % (2 * dtype_size(src.dt))) != 0) return CLK_UNSUPPORTED_DTYPE;
  const bool zn = src.ndim == 3 && !planar;
  int R = 0;
  if (zn) {
    if (m.ex == 1 && m.ey == 1 && m.ez == 1 && m.n == 7) R = 1;
    else if (m.ex == 2 && m.ey == 2 && m.ez == 2 && m.n == 33) R = 2;
  } else {
    if (m.ex == 1 && m.ey == 1 && m.ez == 0 && m.n == 5) R = 1;
    else if (m.ex == 2 && m.ey == 2 && m.ez == 0 && m.n == 13) R = 2;
  }
  if (!R) return CLK_UNSUPPORTED_DTYPE;
  const uint32_t recip = (uint32_t)((((uint64_t)1 << 32) + (uint64_t)m.n - 1) / (uint64_t)m.n);
  switch (src.dt) {
    case CLK_U16: return by_op<uint16_t>(op, R, zn, dst, src, recip, st);
    case CLK_I16: return by_op<int16_t>(op, R, zn, dst, src, recip, st);
    case CLK_U8: return by_op<uint8_t>(op, R, zn, dst, src, recip, st);
    case CLK_I8: return by_op<int8_t>(op, R, zn, dst, src, recip, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
