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
//           memory, private to the thread); the same thread reduces its
//           cells along z and writes two outputs with one store.
// Operations: min/max on 8/16-bit pixels use min/max.{u,s}16x2 with the van
// Herk split; float min/max follow the reference's comparison order (the
// van Herk split with its leftmost-extreme tie rule, the centre first); the
// mean sums int32 lanes and divides exactly (a 32-bit reciprocal multiply
// that equals truncating fl(S/N) for |S| < 2^24, N < 256); the Gaussian to
// float uses fma.rn.f32x2 with weights pre-divided by their sum, folded
// symmetrically; the Gaussian to 8/16-bit pixels keeps the reference's
// arithmetic (taps in order, separately rounded products and sums, IEEE
// division).  Integer temporaries keep the dst pixel type between passes,
// so integer results equal three launches of the reference kernels bit for
// bit.
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
  // Gaussian to integer pixels (exact order): the reference's taps h[v],
  // v = -c..c, of each pass and their float sums
  float hx[17], hy[17], hz[2 * kMaxCz + 1];
  float hs[3];
  int rte;
  // TMA staging: polls of the wait for each staged tile before the CTA
  // gives the tile up (tma::kWaitLimit unless CLK_TMA_WAIT_POLLS is set)
  uint32_t tma_polls;
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

// The two 16-bit lanes of w (signed or not) as an f32x2 pair, exactly: the
// float 2^23 + v (+ 2^15 for signed lanes) built by a byte permute, minus
// the same constant.
template <bool SGN> __device__ __forceinline__ uint64_t f2_of_lanes(uint32_t w) {
  constexpr uint32_t K = 0x4B000000u;
  uint32_t a = __byte_perm(w, K, 0x7410), b = __byte_perm(w, K, 0x7432);
  if constexpr (SGN) a ^= 0x8000u, b ^= 0x8000u;
  constexpr float off = 8388608.0f + (SGN ? 32768.0f : 0.0f);
  return f2_add(f2_pack(__uint_as_float(a), __uint_as_float(b)), f2_bcast(-off));
}

// One exact-order Gaussian output pair: sum of h[v] * win[v], v = 0..N-1, in
// that order with separately rounded products and sums (the reference's
// loop), divided by hsum (IEEE), converted to D; returned as 16-bit lanes.
// Scalar __fmul_rn / __fadd_rn per lane: a packed mul.rn.f32x2 followed by
// add.rn.f32x2 gave results that differed from them in the last bit now and
// then (measured: about 1 in 3000 outputs one unit off after conversion).
template <class D, int N> __device__ __forceinline__ uint32_t gauss_exact_pair(const uint64_t* win, const float* h,
                                                                              float hsum, bool rte) {
  float2 f = f2_unpack(win[0]);
  f.x = __fmul_rn(h[0], f.x), f.y = __fmul_rn(h[0], f.y);
#pragma unroll
  for (int v = 1; v < N; ++v) {
    const float2 x = f2_unpack(win[v]);
    f.x = __fadd_rn(f.x, __fmul_rn(h[v], x.x));
    f.y = __fadd_rn(f.y, __fmul_rn(h[v], x.y));
  }
  const D a = convert_sat<D>(__fdiv_rn(f.x, hsum), rte), b = convert_sat<D>(__fdiv_rn(f.y, hsum), rte);
  return lane16(a) | (lane16(b) << 16);
}

}  // namespace sep2

clk_status sep2_minmax(bool is_max, int R, const Image& dst, const Image& src, int cz, cudaStream_t st);
clk_status sep2_mean(int R, const Image& dst, const Image& src, int cz, cudaStream_t st);
clk_status sep2_gauss(int R, const Image& dst, const Image& src, const float* wx, const float* wy, const float* wz,
                      int cz, cudaStream_t st);
// Gaussian with integer temporaries and outputs, bit-exact: h[d] are the
// 2c+1 taps of pass d (v = -c..c), hs[d] their float sums
clk_status sep2_gauss_exact(int R, const Image& dst, const Image& src, const float* const h[3], const float hs[3],
                            int cz, bool rte, cudaStream_t st);

// The register-ring kernels of clk_sep3.cuh (16-bit pixels, x extent a
// multiple of 8, small Z radius); CLK_UNSUPPORTED_DTYPE where they do not
// apply, and the caller takes the kernels above.
clk_status sep3_minmax(bool is_max, int R, const Image& dst, const Image& src, int cz, cudaStream_t st);
clk_status sep3_mean(int R, const Image& dst, const Image& src, int cz, cudaStream_t st);
clk_status sep3_gauss(int R, const Image& dst, const Image& src, const float* wx, const float* wy, const float* wz,
                      int cz, cudaStream_t st);

}  // namespace clk
