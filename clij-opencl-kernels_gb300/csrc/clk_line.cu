// clk_line.cu - one pass of a separable filter along one axis, for radii
// beyond the fused kernels (clk_sep2.cuh: XY radius <= 8 / 12).  The
// whole-filter call (clk_separable) chains one pass per axis with dst-typed
// temporaries -- exactly the three launches of the reference kernels
// (gaussian_blur_separable_3d_x.cl:6-35, mean_separable_3d_x.cl:3-30,
// minimum_separable_3d_x.cl:3-24, maximum_separable_3d_x.cl:3-24).
//
// A CTA owns a tile of 64 lines along the axis x 64 columns across it (two
// columns per thread, the two lanes of every operation), stages the tile and
// its 2R-line halo in shared memory (float pixels by cp.async, all of a
// thread's copies in flight at once), and each thread computes 8 consecutive
// outputs with a register window that slides one staged line per tap: every
// tap costs one shared-memory read per 8 outputs, whatever the radius.
//
//   min / max (any pixel type): the reference's loop exactly -- start at the
//     centre, then taps v = -R..R in order with `t < r ? t : r` -- on values
//     widened to int or float; bit-exact, NaN behaviour included.
//   mean (integer pixels): exact int32 sums, exact division (the 32-bit
//     multiply-high equal to trunc(fl(S / N)), |S| < 2^24, N < 256).
//   Gaussian to float: taps pre-divided by their sum, fma.rn.f32x2; within
//     the float tolerance of the FP64 oracle.
#include <cstring>
#include <type_traits>

#include "clk_common.cuh"
#include "clk_internal.h"

namespace clk {
namespace line {
namespace {

constexpr int NT = 256;
// M: outputs per thread along the axis (a template argument: 8, or 16 for
// the Gaussian along long lines); a tile holds 8 M outputs along the axis,
// one group of M per warp
constexpr int TC = 64;   // columns per tile across the axis (32 lane pairs)
constexpr int kMaxR = 127;

struct Params {
  // Gaussian: normalised taps of v = -R..R, each as the f32x2 pair (w, w)
  // that the packed FMA takes straight from the parameter space
  uint64_t w2[2 * kMaxR + 1];
  uint32_t mrecip;         // mean: ceil(2^32 / N)
  int R;
};

template <class S> struct Val { typedef int T; };  // staged value type
template <> struct Val<float> { typedef float T; };

__device__ __forceinline__ uint64_t f2(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 f2_split(uint64_t v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

enum Op { MIN = 0, MAX = 1, MEAN = 2, GAUSS = 3 };

// (a, b) to o[0], o[1] as one store; o aligned to the pair
__device__ __forceinline__ void store_pair(float* o, float a, float b) { *reinterpret_cast<float2*>(o) = make_float2(a, b); }
__device__ __forceinline__ void store_pair(uint16_t* o, uint16_t a, uint16_t b) {
  *reinterpret_cast<uint32_t*>(o) = (uint32_t)a | ((uint32_t)b << 16);
}
__device__ __forceinline__ void store_pair(int16_t* o, int16_t a, int16_t b) {
  *reinterpret_cast<uint32_t*>(o) = (uint32_t)(uint16_t)a | ((uint32_t)(uint16_t)b << 16);
}
__device__ __forceinline__ void store_pair(uint8_t* o, uint8_t a, uint8_t b) {
  *reinterpret_cast<uint16_t*>(o) = (uint16_t)(a | (b << 8));
}
__device__ __forceinline__ void store_pair(int8_t* o, int8_t a, int8_t b) {
  *reinterpret_cast<uint16_t*>(o) = (uint16_t)((uint8_t)a | ((uint8_t)b << 8));
}

// One lane pair of a window / an accumulator.
template <int OP, class T> struct Lane {
  T a, b;
};
template <class T> struct Lane<GAUSS, T> {
  uint64_t v;
};

// AXIS 0: lines along x; the tile's columns are 64 rows (y), lanes = rows
//   r and r + 32.  AXIS 1 / 2: lines along y / z; columns are 64 x
//   positions, lanes = x and x + 1.
template <class S, class D, int OP, int AXIS, int M>
__global__ void __launch_bounds__(NT) k_line(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                            const __grid_constant__ Params p) {
  using T = typename Val<S>::T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  constexpr int TL = 8 * M;
  const int R = p.R;
  const int KP = (2 * R + 1 + M - 1) / M * M;  // taps rounded up to whole chunks
  const int NLS = TL + KP;                     // staged lines
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = warp;  // line group: outputs g*M .. g*M+M-1 of the tile

  // tile coordinates: l0 = first output line, c0 = first column; o = the
  // third coordinate (fixed for the CTA)
  const int L = AXIS == 0 ? W : AXIS == 1 ? H : Dz;
  int l0, c0, o;
  if constexpr (AXIS == 0) {
    l0 = blockIdx.x * TL, c0 = blockIdx.y * TC, o = blockIdx.z;  // c = y, o = z
  } else if constexpr (AXIS == 1) {
    c0 = blockIdx.x * TC, l0 = blockIdx.y * TL, o = blockIdx.z;  // c = x, o = z
  } else {
    c0 = blockIdx.x * TC, l0 = blockIdx.y * TL, o = blockIdx.z;  // c = x, o = y
  }
  const int C = AXIS == 0 ? H : W;  // extent of the column coordinate
  const int64_t plane = (int64_t)W * H;
  // element (line l, column c) of the image (both clamped by the caller)
  auto at = [&](int l, int c) -> int64_t {
    if constexpr (AXIS == 0) return (int64_t)o * plane + (int64_t)c * W + l;
    else if constexpr (AXIS == 1) return (int64_t)o * plane + (int64_t)l * W + c;
    else return (int64_t)l * plane + (int64_t)o * W + c;
  };

  // stage lines l0 - R .. l0 - R + NLS - 1 (clamped) x the tile's columns
  // AXIS 0: columns c and c + 32 (a thread's two rows) interleaved,
  // sm[((c % 32) * NP + l) * 2 + c / 32], so that one 8-byte read fetches
  // both lanes (odd pitch NP: a warp's reads hit distinct banks); AXIS 1/2:
  // sm[l * TC + c] (lane pairs adjacent)
  // Loads are batched U deep so that each thread has U in flight.
  constexpr int U = 8;
  const int NP = NLS | 1;
  if constexpr (std::is_same<S, T>::value) {
    // float pixels are staged as they are: 4-byte cp.async copies, every one
    // of the thread's copies in flight at once and no registers held
    auto cp4 = [](T* d, const S* g) {
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(d)), "l"(g)
                   : "memory");
    };
    if constexpr (AXIS == 0) {
      for (int l = lane; l < NLS; l += 32) {
        const int ll = clampi(l0 - R + l, L - 1);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const int c = warp + 8 * u;
          cp4(sm + ((c & 31) * NP + l) * 2 + (c >> 5), src + at(ll, min(c0 + c, C - 1)));
        }
      }
    } else {
      const int total = NLS * TC;
      for (int i = tid; i < total; i += NT)
        cp4(sm + i, src + at(clampi(l0 - R + (i >> 6), L - 1), min(c0 + (i & 63), C - 1)));
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else if constexpr (AXIS == 0) {
    // warp w stages columns (rows of the image) w + 8u, u = 0..7
    for (int l = lane; l < NLS; l += 32) {
      const int ll = clampi(l0 - R + l, L - 1);
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) v[u] = (T)__ldg(src + at(ll, min(c0 + warp + 8 * u, C - 1)));
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int c = warp + 8 * u;
        sm[((c & 31) * NP + l) * 2 + (c >> 5)] = v[u];
      }
    }
  } else {
    const int total = NLS * TC;  // element i = (line i / 64, column i % 64) = sm[i]
    for (int b0 = 0; b0 < total; b0 += NT * U) {
      T v[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = b0 + u * NT + tid;
        if (i < total) v[u] = (T)__ldg(src + at(clampi(l0 - R + (i >> 6), L - 1), min(c0 + (i & 63), C - 1)));
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = b0 + u * NT + tid;
        if (i < total) sm[i] = v[u];
      }
    }
  }
  __syncthreads();

  // the thread's lane pair of staged line l
  const int ca = AXIS == 0 ? lane : 2 * lane, cb = AXIS == 0 ? lane + 32 : 2 * lane + 1;
  auto get = [&](int l) -> Lane<OP, T> {
    T a, b;
    typedef typename std::conditional<std::is_same<T, float>::value, float2, int2>::type P2;
    if constexpr (AXIS == 0) {  // rows ca, cb = ca + 32, interleaved: one 8-byte read
      const P2 v = *reinterpret_cast<const P2*>(sm + (ca * NP + l) * 2);
      a = v.x, b = v.y;
    } else {  // the adjacent pair as one 8-byte read
      const P2 v = *reinterpret_cast<const P2*>(sm + l * TC + ca);
      a = v.x, b = v.y;
    }
    Lane<OP, T> r;
    if constexpr (OP == GAUSS) r.v = f2((float)a, (float)b);
    else r.a = a, r.b = b;
    return r;
  };

  const int base = g * M;  // staged line of tap k = 0 for output j = 0 is base + j
  // outputs: lines l0 + base + j, columns c0 + ca / c0 + cb
  auto store_out = [&](const D (&ra)[M], const D (&rb)[M]) {
    if constexpr (AXIS == 0) {
      // the lanes are rows: transpose through shared memory so that the
      // stores run along x
      D* so = reinterpret_cast<D*>(smem_raw);
      constexpr int OP_ = TL + 1;  // odd pitch
      __syncthreads();             // everyone is done with the staged tile
#pragma unroll
      for (int j = 0; j < M; ++j) so[ca * OP_ + base + j] = ra[j], so[cb * OP_ + base + j] = rb[j];
      __syncthreads();
      for (int c = warp; c < TC; c += NT / 32) {
        if (c0 + c >= C) break;
#pragma unroll
        for (int h = 0; h < TL / 32; ++h) {
          const int l = lane + 32 * h;
          if (l0 + l < L) dst[at(l0 + l, c0 + c)] = so[c * OP_ + l];
        }
      }
    } else {
      // adjacent pair as one store where the rows keep pairs aligned
      const bool pair = (W & 1) == 0 && c0 + cb < C && ((uintptr_t)dst & (2 * sizeof(D) - 1)) == 0;
#pragma unroll
      for (int j = 0; j < M; ++j) {
        const int l = l0 + base + j;
        if (l >= L) break;
        D* o = dst + at(l, c0 + ca);
        if (pair) {
          store_pair(o, ra[j], rb[j]);
        } else {
          if (c0 + ca < C) o[0] = ra[j];
          if (c0 + cb < C) o[1] = rb[j];
        }
      }
    }
  };
  if constexpr (OP == MIN || OP == MAX) {
    if (2 * R >= M) {
      // van Herk / Gil-Werman over the window lines base .. base+2R+M-1:
      // out[j] = first(suffix of lines j..M-1, prefix of lines M..j+2R),
      // with first(a, b) = the earlier operand unless the later one is
      // strictly smaller (MIN) / larger (MAX) or the earlier one is NaN --
      // an associative "leftmost extreme, NaN never chosen".  The
      // reference's loop (res = centre, then res = x < res ? x : res over
      // the taps) returns the leftmost extreme of (centre, taps), or NaN
      // when the centre is NaN: first(centre, out[j]) unless the centre is
      // NaN.  2R + 2M - 2 operations for M outputs instead of (2R+1) M.
      auto first = [](T a, T b) -> T {
        if constexpr (std::is_same<T, float>::value) {
          const bool take = (OP == MIN ? b < a : a < b) || a != a;
          return take ? b : a;
        } else {
          return OP == MIN ? (b < a ? b : a) : (a < b ? b : a);
        }
      };
      // Float pixels: fminf / fmaxf (one instruction, NaN never chosen) give
      // first()'s value wherever that value is not a zero: equal nonzero
      // floats are the same bits, and a zero can be the extreme only when the
      // result is one.  So outputs whose centre is NaN take the centre and
      // zero results (the sign of a zero depends on which one comes first)
      // rerun the reference's loop over their window.
      auto firstl = [&](const Lane<OP, T>& a, const Lane<OP, T>& b) {
        Lane<OP, T> r;
        if constexpr (std::is_same<T, float>::value) {
          r.a = OP == MIN ? fminf(a.a, b.a) : fmaxf(a.a, b.a);
          r.b = OP == MIN ? fminf(a.b, b.b) : fmaxf(a.b, b.b);
        } else {
          r.a = first(a.a, b.a), r.b = first(a.b, b.b);
        }
        return r;
      };
      auto exact = [&](int t, int ln) -> T {  // the reference's loop for output t, lane ln
        const Lane<OP, T> c = get(base + t + R);
        T r = ln ? c.b : c.a;
        for (int k = 0; k <= 2 * R; ++k) {
          const Lane<OP, T> v = get(base + t + k);
          const T x = ln ? v.b : v.a;
          r = (OP == MIN ? x < r : r < x) ? x : r;
        }
        return r;
      };
      (void)exact;
      Lane<OP, T> suf[M];
      suf[M - 1] = get(base + M - 1);
#pragma unroll
      for (int j = M - 2; j >= 0; --j) suf[j] = firstl(get(base + j), suf[j + 1]);
      Lane<OP, T> pre = get(base + M);
      for (int k = M + 1; k < 2 * R; ++k) pre = firstl(pre, get(base + k));
      D ra[M], rb[M];
#pragma unroll
      for (int t = 0; t < M; ++t) {
        const int k = 2 * R + t;
        if (k > M) pre = firstl(pre, get(base + k));
        Lane<OP, T> o = firstl(suf[t], pre);
        if constexpr (std::is_same<T, float>::value) {  // a NaN centre is the result; zeros exactly
          const Lane<OP, T> c = get(base + t + R);
          if (c.a != c.a) o.a = c.a;
          else if (o.a == 0.f) o.a = exact(t, 0);
          if (c.b != c.b) o.b = c.b;
          else if (o.b == 0.f) o.b = exact(t, 1);
        }
        ra[t] = (D)o.a, rb[t] = (D)o.b;
      }
      store_out(ra, rb);
      return;
    }
  }
  Lane<OP, T> acc[M], win[M];
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if constexpr (OP == MIN || OP == MAX) acc[j] = get(base + j + R);  // the centre
    else if constexpr (OP == MEAN) acc[j].a = acc[j].b = 0;
    else acc[j].v = 0ull;
    win[j] = get(base + j);
  }
  // a group whose outputs all lie beyond the line (the last tile of a line
  // that is not a whole number of tiles) skips the taps
  const int kend = l0 + base < L ? KP : 0;
  for (int kk = 0; kk < kend; kk += M) {
#pragma unroll
    for (int t = 0; t < M; ++t) {
      const int k = kk + t;
      if (k <= 2 * R) {
        uint64_t wk = 0;
        if constexpr (OP == GAUSS) wk = p.w2[k];
#pragma unroll
        for (int j = 0; j < M; ++j) {
          const Lane<OP, T>& v = win[(j + t) % M];
          if constexpr (OP == MIN) {
            acc[j].a = v.a < acc[j].a ? v.a : acc[j].a;
            acc[j].b = v.b < acc[j].b ? v.b : acc[j].b;
          } else if constexpr (OP == MAX) {
            acc[j].a = acc[j].a < v.a ? v.a : acc[j].a;
            acc[j].b = acc[j].b < v.b ? v.b : acc[j].b;
          } else if constexpr (OP == MEAN) {
            acc[j].a += v.a;
            acc[j].b += v.b;
          } else {
            acc[j].v = f2_fma(wk, v.v, acc[j].v);
          }
        }
      }
      win[t] = get(base + k + M);  // line base+k leaves the window, base+k+M enters
    }
  }

  // outputs: lines l0 + base + j, columns c0 + ca / c0 + cb
  D ra[M], rb[M];
#pragma unroll
  for (int j = 0; j < M; ++j) {
    if constexpr (OP == GAUSS) {
      const float2 f = f2_split(acc[j].v);
      ra[j] = (D)f.x, rb[j] = (D)f.y;
    } else if constexpr (OP == MEAN) {
      auto q = [&](int s) -> int {
        const uint32_t a = (uint32_t)(s < 0 ? -s : s);
        const int v = p.mrecip ? (int)__umulhi(a, p.mrecip) : (int)a;
        return s < 0 ? -v : v;
      };
      ra[j] = (D)q(acc[j].a), rb[j] = (D)q(acc[j].b);
    } else {
      ra[j] = (D)acc[j].a, rb[j] = (D)acc[j].b;
    }
  }
  store_out(ra, rb);
}

template <class S, class D, int OP, int M>
clk_status launch(const Image& dst, const Image& src, int axis, const Params& p, cudaStream_t st) {
  constexpr int TL = 8 * M;
  const int KP = (2 * p.R + 1 + M - 1) / M * M, NLS = TL + KP;
  const size_t smem = axis == 0 ? (size_t)TC * (NLS | 1) * 4 : (size_t)NLS * TC * 4;
  const int W = src.w, H = src.h, Dz = src.d;
  dim3 grid;
  if (axis == 0) grid = dim3((W + TL - 1) / TL, (H + TC - 1) / TC, Dz);
  else if (axis == 1) grid = dim3((W + TC - 1) / TC, (H + TL - 1) / TL, Dz);
  else grid = dim3((W + TC - 1) / TC, (Dz + TL - 1) / TL, H);
  if (grid.y > 65535 || grid.z > 65535) return CLK_UNSUPPORTED_DTYPE;
  auto go = [&](auto kern) -> clk_status {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      return CLK_UNSUPPORTED_DTYPE;
    }
    kern<<<grid, NT, smem, st>>>((const S*)src.ptr, (D*)dst.ptr, W, H, Dz, p);
    count_launch();
    return check_launch("separable (line pass)");
  };
  if (axis == 0) return go(k_line<S, D, OP, 0, M>);
  if (axis == 1) return go(k_line<S, D, OP, 1, M>);
  return go(k_line<S, D, OP, 2, M>);
}
// The Gaussian along lines of at least 256 voxels takes 16 outputs per
// thread (half the window reads and tap loads per FMA, half the halo per
// tile); other operations, and short lines, take 8
template <class S, class D, int OP>
clk_status launch(const Image& dst, const Image& src, int axis, const Params& p, cudaStream_t st) {
  if constexpr (OP == GAUSS) {
    const int L = axis == 0 ? src.w : axis == 1 ? src.h : src.d;
    if (L >= 256) return launch<S, D, OP, 16>(dst, src, axis, p, st);
  }
  return launch<S, D, OP, 8>(dst, src, axis, p, st);
}

template <int OP> clk_status by_type(const Image& dst, const Image& src, int axis, const Params& p, cudaStream_t st) {
  if constexpr (OP == GAUSS) {
    switch (src.dt) {
      case CLK_U8: return launch<uint8_t, float, OP>(dst, src, axis, p, st);
      case CLK_I8: return launch<int8_t, float, OP>(dst, src, axis, p, st);
      case CLK_U16: return launch<uint16_t, float, OP>(dst, src, axis, p, st);
      case CLK_I16: return launch<int16_t, float, OP>(dst, src, axis, p, st);
      case CLK_F32: return launch<float, float, OP>(dst, src, axis, p, st);
    }
  } else {
    switch (src.dt) {
      case CLK_U8: return launch<uint8_t, uint8_t, OP>(dst, src, axis, p, st);
      case CLK_I8: return launch<int8_t, int8_t, OP>(dst, src, axis, p, st);
      case CLK_U16: return launch<uint16_t, uint16_t, OP>(dst, src, axis, p, st);
      case CLK_I16: return launch<int16_t, int16_t, OP>(dst, src, axis, p, st);
      case CLK_F32:
        if constexpr (OP != MEAN) return launch<float, float, OP>(dst, src, axis, p, st);
        break;
    }
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace
}  // namespace line

bool line_eligible(SepOp op, const Image& dst, const Image& src, const Policy& pol) {
  if (op == SEP_GAUSS) return dst.dt == CLK_F32 && !pol.exact_order;
  if (src.dt != dst.dt) return false;
  if (op == SEP_MEAN) return src.dt != CLK_F32;  // float means keep the reference's summation order
  return true;
}

clk_status line_pass(SepOp op, const Image& dst, const Image& src, int axis, const SepTaps& taps, const Policy& pol,
                     cudaStream_t st) {
  using namespace line;
  if (!line_eligible(op, dst, src, pol) || taps.c < 1 || taps.c > kMaxR) return CLK_UNSUPPORTED_DTYPE;
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  static thread_local Params p;
  p.R = taps.c;
  p.mrecip = 0;
  if (op == SEP_GAUSS) {
    double s = 0;
    for (int v = 0; v <= 2 * taps.c; ++v) s += taps.h[v];
    for (int v = 0; v <= 2 * taps.c; ++v) {
      const float w = (float)(taps.h[v] / s);
      uint32_t u;
      memcpy(&u, &w, 4);
      p.w2[v] = (uint64_t)u | ((uint64_t)u << 32);
    }
  } else if (op == SEP_MEAN) {
    const uint64_t n = 2 * (uint64_t)taps.c + 1;
    p.mrecip = (uint32_t)((((uint64_t)1 << 32) + n - 1) / n);
  }
  switch (op) {
    case SEP_MIN: return by_type<MIN>(dst, src, axis, p, st);
    case SEP_MAX: return by_type<MAX>(dst, src, axis, p, st);
    case SEP_MEAN: return by_type<MEAN>(dst, src, axis, p, st);
    case SEP_GAUSS: return by_type<GAUSS>(dst, src, axis, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
