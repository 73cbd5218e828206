// clk_common.cuh - shared device helpers of the neighbourhood-filter
// kernels: pixel-type traits, the preamble semantics (clamp-to-edge reads,
// saturating convert) and the internal launch descriptors.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "clk_internal.h"

namespace clk {

// Value type of a read's .x (read_imageui / read_imagei / read_imagef,
// README.md:103-116): uint for uchar/ushort, int for char/short, float.
template <class T> struct ReadT;
template <> struct ReadT<uint8_t> { typedef uint32_t type; };
template <> struct ReadT<uint16_t> { typedef uint32_t type; };
template <> struct ReadT<int8_t> { typedef int32_t type; };
template <> struct ReadT<int16_t> { typedef int32_t type; };
template <> struct ReadT<float> { typedef float type; };

template <class T> struct Lim;
template <> struct Lim<uint8_t> { static constexpr float lo = 0.f, hi = 255.f; };
template <> struct Lim<int8_t> { static constexpr float lo = -128.f, hi = 127.f; };
template <> struct Lim<uint16_t> { static constexpr float lo = 0.f, hi = 65535.f; };
template <> struct Lim<int16_t> { static constexpr float lo = -32768.f, hi = 32767.f; };

// CONVERT_dst_PIXEL_TYPE: clij_convert_<T>_sat.  Saturate to the type's
// range; float -> integer truncates toward zero (rte: half to even); NaN -> 0.
template <class D> __device__ __forceinline__ D convert_sat(float v, bool rte) {
  if constexpr (sizeof(D) == 4) {
    return v;
  } else {
    if (v != v) return (D)0;
    if (v <= Lim<D>::lo) return (D)Lim<D>::lo;
    if (v >= Lim<D>::hi) return (D)Lim<D>::hi;
    return (D)(rte ? __float2int_rn(v) : __float2int_rz(v));
  }
}

__device__ __forceinline__ int clampi(int v, int hi) { return min(max(v, 0), hi); }

template <class T> __device__ __forceinline__ float ldf(const T* p, int64_t i) { return (float)__ldg(p + i); }

struct Dims3 {
  int w, h, d;
};

__device__ __forceinline__ int64_t at(const Dims3& s, int x, int y, int z) {
  return (int64_t)x + (int64_t)s.w * ((int64_t)y + (int64_t)s.h * z);
}
__device__ __forceinline__ int64_t atc(const Dims3& s, int x, int y, int z) {
  return at(s, clampi(x, s.w - 1), clampi(y, s.h - 1), clampi(z, s.d - 1));
}

// Calls f(S{}, D{}) for the runtime pixel-type pair; returns false for an
// unknown code.
template <class F> inline bool dispatch_types(int sdt, int ddt, F&& f) {
  auto d = [&](auto s) -> bool {
    switch (ddt) {
      case CLK_U8: f(s, uint8_t{}); return true;
      case CLK_I8: f(s, int8_t{}); return true;
      case CLK_U16: f(s, uint16_t{}); return true;
      case CLK_I16: f(s, int16_t{}); return true;
      case CLK_F32: f(s, float{}); return true;
    }
    return false;
  };
  switch (sdt) {
    case CLK_U8: return d(uint8_t{});
    case CLK_I8: return d(int8_t{});
    case CLK_U16: return d(uint16_t{});
    case CLK_I16: return d(int16_t{});
    case CLK_F32: return d(float{});
  }
  return false;
}

template <class F> inline bool dispatch_type(int dt, F&& f) {
  switch (dt) {
    case CLK_U8: f(uint8_t{}); return true;
    case CLK_I8: f(int8_t{}); return true;
    case CLK_U16: f(uint16_t{}); return true;
    case CLK_I16: f(int16_t{}); return true;
    case CLK_F32: f(float{}); return true;
  }
  return false;
}

inline unsigned grid_1d(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

}  // namespace clk
