// clk_sep2.cuh - fast fused X -> Y -> Z separable filters with a
// compile-time XY radius R (cx = cy = R) and a runtime Z radius.
//
// A CTA owns a 64 x 32 column of outputs and streams along z.  Per input
// plane:
//   stage   the clamped (32+2R) x (64+2R) halo tile into shared memory (the
//           next plane's tile is fetched into registers while this one is
//           filtered);
//   X pass  a thread filters two rows x 8 outputs; the two rows are the two
//           lanes of every packed operation, so each tap is one instruction
//           for two outputs and the window slides along x in registers;
//   Y pass  a thread filters a column pair x 4 outputs, lanes = (x, x+1);
//   Z pass  the Y results enter a ring of the last 2cz+1 planes (shared
//           memory); the same thread reduces its cells along z and writes
//           two outputs with one store.
// Lane types: min/max on 8/16-bit pixels use min/max.{u,s}16x2, the mean
// sums int32 lanes and divides exactly (a 64-bit reciprocal multiply that
// equals truncating fl(S/N) for |S| < 2^24, N < 256), the Gaussian uses
// fma.rn.f32x2 with weights pre-divided by their sum, folded symmetrically.
// Integer temporaries keep the dst pixel type between passes, so integer
// results equal three launches of the reference kernels bit for bit.
#pragma once
#include "clk_common.cuh"

namespace clk {
namespace sep2 {

constexpr int TX = 64, TY = 32, NT = 256;
constexpr int SEGX = 8;     // X-pass outputs per thread along x
constexpr int SEGY = 4;     // Y-pass outputs per thread along y
constexpr int kMaxCz = 31;  // Z radius limit (ring in shared memory)

struct Params {
  float wx[16];        // Gaussian: folded, normalised taps of X (w[0] centre, w[k] for +-k)
  float wy[16];        //           ... of Y
  float wz[kMaxCz + 1];  //         ... of Z
  uint32_t mx, mz;     // mean: reciprocal multipliers (recip32) for N = 2R+1 and 2cz+1
  int cz;
};

// ---------------------------------------------------------------- lanes
__device__ __forceinline__ uint32_t u16x2_min(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t u16x2_max(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t s16x2_min(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("min.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint32_t s16x2_max(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("max.s16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}
__device__ __forceinline__ uint64_t f2_pack(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(uint64_t v) {
  float2 r;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
  return r;
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ uint64_t f2_bcast(float w) { return f2_pack(w, w); }

// Exact truncating division of an integer sum by N: m = ceil(2^32 / N) for
// N >= 2 (m = 0 for N = 1).  For |s| < 2^24 and N < 256,
// floor(|s| * m / 2^32) = floor(|s| / N): the error |s|(m - 2^32/N)/2^32 <
// 2^-8 stays below the 1/N gap to the next quotient.  That quotient also
// equals trunc(fl(s / N)) in float: s/N = q + r/N lies at least 1/N below
// q + 1, more than half a float ulp at that magnitude (q < 2^24 / N).
template <bool SIGNED> __device__ __forceinline__ int div_exact(int s, uint32_t m) {
  if constexpr (SIGNED) {
    const uint32_t a = (uint32_t)(s < 0 ? -s : s);
    const int q = m ? (int)__umulhi(a, m) : (int)a;
    return s < 0 ? -q : q;
  } else {
    return m ? (int)__umulhi((uint32_t)s, m) : s;
  }
}
inline uint32_t recip32(int n) { return n <= 1 ? 0u : (uint32_t)((((uint64_t)1 << 32) + (uint64_t)n - 1) / (uint64_t)n); }

template <class T> struct Is16;  // 16-bit lane traits of 8/16-bit pixels
template <> struct Is16<uint16_t> { static constexpr bool sgn = false; };
template <> struct Is16<int16_t> { static constexpr bool sgn = true; };
template <> struct Is16<uint8_t> { static constexpr bool sgn = false; };
template <> struct Is16<int8_t> { static constexpr bool sgn = true; };

template <class T> __device__ __forceinline__ uint32_t lane16(T v) {
  return Is16<T>::sgn ? (uint32_t)(uint16_t)(int16_t)v : (uint32_t)(uint16_t)v;
}
template <class T> __device__ __forceinline__ T from_lane16(uint32_t l) { return (T)(int16_t)(uint16_t)l; }

}  // namespace sep2

clk_status sep2_minmax(bool is_max, int R, const Image& dst, const Image& src, int cz, cudaStream_t st);
clk_status sep2_mean(int R, const Image& dst, const Image& src, int cz, cudaStream_t st);
clk_status sep2_gauss(int R, const Image& dst, const Image& src, const float* wx, const float* wy, const float* wz,
                      int cz, cudaStream_t st);

}  // namespace clk
