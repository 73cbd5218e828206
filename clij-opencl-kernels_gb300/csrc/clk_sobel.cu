// clk_sobel.cu - fast sobel_3d (sobel_3d_x.cl:3-57) to float.
//
// The kernel's 3x3x4 window (dz = -1..+2, the k<=3 loop reading the flat
// arrays one row on, the last tap pinned to 0) decomposes per input plane
// into row sums sx = v(x-1) + 2v(x) + v(x+1) and differences
// dx = v(x-1) - v(x+1):
//   A = dx(y-1) + 2dx(y) + dx(y+1)   B = sx(y-1) - sx(y+1)
//   C = sx(y-1) + 2sx(y) + sx(y+1)   q = 2v(x-1,y+1) + v(x,y+1)
//   Ex = 2dx(y-1) + dx(y) - v(x,y+1) Ey = q - sx(y)   Ez = 2sx(y-1) + sx(y) + q
// and then along z
//   Sx = A(z-1) + 2A(z) + A(z+1) + Ex(z+2)
//   Sy = B(z-1) + 2B(z) + B(z+1) + Ey(z+2)
//   Sz = C(z-1) - C(z+1) + Ez(z+2),
// exact integer sums for integer pixels.  For unsigned pixels the kernel
// multiplies int coefficients by uint reads (C: the product is uint), so
// each negative-coefficient tap with a nonzero pixel contributes 2^32 more:
// sum_c = S_c + K_c * 2^32 with K_c the count of such taps (12, 12, 9 when no
// pixel of the window is 0; counted exactly otherwise).  The float result
// sqrt(sx^2 + sy^2 + sz^2) is within 1e-5 of the FP64 evaluation; integer
// outputs use the generic kernel, which sums in the reference's order.
//
// A thread owns 2 x 2 outputs (x, x+1; y, y+1) and walks along z, keeping
// A, B, C of the last three planes in registers (the z loop is unrolled by
// three so the ring never moves) and the next plane's pixels in flight.
// Rows are read as aligned pixel pairs.  Sums convert to float exactly
// without the I2F unit; the square root is the hardware approximation
// (relative error far below the 1e-5 bound).  Unsigned 16-bit images whose
// rows are whole vectors run the same sums on packed float pairs
// (k_sobel3d_x2), bit-identical to the integer kernel.
#include <cstdlib>
#include <type_traits>

#include "clk_common.cuh"
#include "clk_internal.h"

namespace clk {

namespace {

constexpr int SBX = 32, SBY = 8;  // threads: 64 columns x 16 rows per block

template <class S> struct Num { typedef int type; };
template <> struct Num<float> { typedef float type; };

// v(x-1), v(x), v(x+1), v(x+2) of one row, clamped at the row ends
template <class S>
__device__ __forceinline__ void load4(const S* row, int x, int W, typename Num<S>::type (&v)[4]) {
  using N = typename Num<S>::type;
  v[0] = (N)__ldg(row + (x > 0 ? x - 1 : 0));
  v[1] = (N)__ldg(row + x);
  v[2] = (N)__ldg(row + min(x + 1, W - 1));
  v[3] = (N)__ldg(row + min(x + 2, W - 1));
}

// Exact counts K of the negative-coefficient taps with a nonzero pixel
// (unsigned reads), for a window that contains a zero pixel.
template <class S>
__device__ __noinline__ float3 wrap_counts(const S* __restrict__ src, int W, int H, int D, int gx, int gy, int z) {
  const Dims3 dm{W, H, D};
  auto nz = [&](int ddx, int ddy, int ddz) -> float {
    return __ldg(src + atc(dm, gx + ddx, gy + ddy, z + ddz)) != 0 ? 1.f : 0.f;
  };
  float kx = 0.f, ky = 0.f, kz = 0.f;
  for (int dz = -1; dz <= 1; ++dz)
    for (int d = -1; d <= 1; ++d) {
      kx += nz(1, d, dz);  // gx: dx = +1 taps
      ky += nz(d, 1, dz);  // gy: dy = +1 taps
    }
  for (int ddx = -1; ddx <= 1; ++ddx)
    for (int ddy = -1; ddy <= 1; ++ddy) kz += nz(ddx, ddy, 1);  // gz: dz = +1 taps
  kx += nz(0, 1, 2) + nz(1, -1, 2) + nz(1, 0, 2);   // negative taps of the dz = +2 plane
  ky += nz(-1, 0, 2) + nz(0, 0, 2) + nz(1, 0, 2);
  return make_float3(kx, ky, kz);
}

// Two consecutive pixels (x, x+1), x even, as one aligned load.
template <class S> struct Pair;
template <> struct Pair<uint16_t> {
  typedef uint32_t V;
  static __device__ __forceinline__ int lo(V v) { return (int)(v & 0xFFFFu); }
  static __device__ __forceinline__ int hi(V v) { return (int)(v >> 16); }
};
template <> struct Pair<int16_t> {
  typedef uint32_t V;
  static __device__ __forceinline__ int lo(V v) { return (int)(int16_t)(v & 0xFFFFu); }
  static __device__ __forceinline__ int hi(V v) { return (int)v >> 16; }
};
template <> struct Pair<uint8_t> {
  typedef uint16_t V;
  static __device__ __forceinline__ int lo(V v) { return (int)(v & 0xFFu); }
  static __device__ __forceinline__ int hi(V v) { return (int)(v >> 8); }
};
template <> struct Pair<int8_t> {
  typedef uint16_t V;
  static __device__ __forceinline__ int lo(V v) { return (int)(int8_t)(v & 0xFFu); }
  static __device__ __forceinline__ int hi(V v) { return (int)(int8_t)(v >> 8); }
};
template <> struct Pair<float> {
  typedef float2 V;
  static __device__ __forceinline__ float lo(V v) { return v.x; }
  static __device__ __forceinline__ float hi(V v) { return v.y; }
};

// int -> float without the I2F unit, exact for |v| < 2^22 (every sum here:
// at most 47 * 65535 in magnitude)
__device__ __forceinline__ float exact_float(int v) { return __int_as_float(0x4B400000 + v) - 12582912.0f; }
__device__ __forceinline__ float exact_float(float v) { return v; }

__device__ __forceinline__ float sqrt_approx(float v) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

template <class S, bool WRAP>
__global__ void __launch_bounds__(SBX * SBY, 2) k_sobel3d_fast(const S* __restrict__ src, float* __restrict__ dst,
                                                               int W, int H, int D, int zchunk) {
  using N = typename Num<S>::type;
  using PV = typename Pair<S>::V;
  const int x = 2 * (blockIdx.x * SBX + threadIdx.x);
  const int y = 2 * (blockIdx.y * SBY + threadIdx.y);
  if (x >= W || y >= H) return;
  const int z0 = blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  const bool hasl = x > 0, hasr = x + 2 < W;
  int roff[4];  // rows y-1 .. y+2, clamped
#pragma unroll
  for (int r = 0; r < 4; ++r) roff[r] = clampi(y - 1 + r, H - 1) * W + x;

  // raw pairs (x-2, x-1), (x, x+1), (x+2, x+3) of the four rows of one plane
  PV raw[4][3];
  auto load = [&](int p) {
    const S* sp = src + (int64_t)clampi(p, D - 1) * plane;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const PV* row = reinterpret_cast<const PV*>(sp + roff[r]);
      raw[r][1] = __ldg(row);
      raw[r][0] = hasl ? __ldg(row - 1) : raw[r][1];
      raw[r][2] = hasr ? __ldg(row + 1) : raw[r][1];
    }
  };

  // per output (ox, oy): A, B, C of the three planes before the newest
  N A[3][2][2], B[3][2][2], C[3][2][2];
  N ex[2][2], ey[2][2], ez[2][2];
  uint32_t zflags = 0;  // bit i: a zero pixel among this thread's loads of plane p-i

  // partial sums of the plane held in raw, into ring slot s; E terms too
  auto terms = [&](N (&a)[2][2], N (&b)[2][2], N (&c)[2][2]) {
    N v[4][4];  // rows y-1 .. y+2, columns x-1 .. x+2 (clamped)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      v[r][0] = hasl ? Pair<S>::hi(raw[r][0]) : Pair<S>::lo(raw[r][1]);
      v[r][1] = Pair<S>::lo(raw[r][1]);
      v[r][2] = Pair<S>::hi(raw[r][1]);
      v[r][3] = hasr ? Pair<S>::lo(raw[r][2]) : Pair<S>::hi(raw[r][1]);
    }
    if constexpr (WRAP) {
      N m = v[0][0];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) m = min(m, v[r][c]);
      zflags = (zflags << 1) | (m == 0 ? 1u : 0u);
    }
    N sx[4][2], dx[4][2];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int o = 0; o < 2; ++o) {
        sx[r][o] = v[r][o] + 2 * v[r][o + 1] + v[r][o + 2];
        dx[r][o] = v[r][o] - v[r][o + 2];
      }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int rm = oy, rc = oy + 1, rp = oy + 2;
        a[oy][ox] = dx[rm][ox] + 2 * dx[rc][ox] + dx[rp][ox];
        b[oy][ox] = sx[rm][ox] - sx[rp][ox];
        c[oy][ox] = sx[rm][ox] + 2 * sx[rc][ox] + sx[rp][ox];
        const N q = 2 * v[rp][ox] + v[rp][ox + 1];
        ex[oy][ox] = 2 * dx[rm][ox] + dx[rc][ox] - v[rp][ox + 1];
        ey[oy][ox] = q - sx[rc][ox];
        ez[oy][ox] = 2 * sx[rm][ox] + sx[rc][ox] + q;
      }
  };

  // output plane zo from ring slots (i0, i1, i2) = planes (zo-1, zo, zo+1)
  // and the newest plane zo+2, whose A/B/C then replace slot i0
  auto step = [&](int zo, auto i0c, auto i1c, auto i2c) {
    constexpr int i0 = decltype(i0c)::value, i1 = decltype(i1c)::value, i2 = decltype(i2c)::value;
    N a[2][2], b[2][2], c[2][2];
    terms(a, b, c);
    if (zo + 1 < z1) load(zo + 3);  // the next step's plane, in flight during this one
    float res[2][2];
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const N sxv = A[i0][oy][ox] + 2 * A[i1][oy][ox] + A[i2][oy][ox] + ex[oy][ox];
        const N syv = B[i0][oy][ox] + 2 * B[i1][oy][ox] + B[i2][oy][ox] + ey[oy][ox];
        const N szv = C[i0][oy][ox] - C[i2][oy][ox] + ez[oy][ox];
        float fx = exact_float(sxv), fy = exact_float(syv), fz = exact_float(szv);
        if constexpr (WRAP) {
          float kx = 12.f, ky = 12.f, kz = 9.f;
          if (zflags & 0xFu) {  // a zero pixel in planes zo-1 .. zo+2: count exactly
            const float3 k = wrap_counts<S>(src, W, H, D, x + ox, y + oy, zo);
            kx = k.x, ky = k.y, kz = k.z;
          }
          fx = fmaf(kx, 4294967296.0f, fx);
          fy = fmaf(ky, 4294967296.0f, fy);
          fz = fmaf(kz, 4294967296.0f, fz);
        }
        res[oy][ox] = sqrt_approx(fmaf(fx, fx, fmaf(fy, fy, fz * fz)));
      }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      if (y + oy < H)
        *reinterpret_cast<float2*>(dst + (int64_t)zo * plane + (int64_t)(y + oy) * W + x) =
            make_float2(res[oy][0], res[oy][1]);
    }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) A[i0][oy][ox] = a[oy][ox], B[i0][oy][ox] = b[oy][ox], C[i0][oy][ox] = c[oy][ox];
  };

  load(z0 - 1);
  terms(A[0], B[0], C[0]);
  load(z0);
  terms(A[1], B[1], C[1]);
  load(z0 + 1);
  terms(A[2], B[2], C[2]);
  load(z0 + 2);
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  for (int zo = z0; zo < z1; zo += 3) {  // unrolled by the ring length: slots rotate at compile time
    step(zo, I0{}, I1{}, I2{});
    if (zo + 1 < z1) step(zo + 1, I1{}, I2{}, I0{});
    if (zo + 2 < z1) step(zo + 2, I2{}, I0{}, I1{});
  }
}

// The same computation with each input plane staged once in shared memory:
// a CTA owns 64 x 16 outputs and streams along z; plane p+1 is fetched into
// registers with 16-byte vector loads (vectors wholly outside a row take the
// clamped edge pixel) while plane p is used, and two plane buffers need one
// barrier per plane.  Requires rows of a whole number of vectors.
constexpr int TSX = 64, TSY = 16;  // outputs per CTA; 32 x 8 threads of 2 x 2

template <class S> __device__ __forceinline__ uint4 splat16(S v) {
  uint32_t w;
  if constexpr (sizeof(S) == 4) w = __float_as_uint(v);
  else if constexpr (sizeof(S) == 2) w = (uint32_t)(uint16_t)v * 0x10001u;
  else w = (uint32_t)(uint8_t)v * 0x01010101u;
  return make_uint4(w, w, w, w);
}

template <class S, bool WRAP>
__global__ void __launch_bounds__(256, WRAP ? 2 : 3) k_sobel3d_tile(const S* __restrict__ src, float* __restrict__ dst, int W,
                                                         int H, int D, int zchunk) {
  using N = typename Num<S>::type;
  using PV = typename Pair<S>::V;
  constexpr int VE = 16 / (int)sizeof(S);  // pixels per vector
  constexpr int RA = VE;                   // staged columns x0 - RA .. x0 + 64 + RA - 1
  constexpr int RW = TSX + 2 * RA, RH = TSY + 3;  // rows y0 - 1 .. y0 + 17
  constexpr int SR = RW / VE, NSLOT = RH * SR, PERV = (NSLOT + 255) / 256;
  __shared__ __align__(16) S tile[2][RH * RW];
  const int tid = threadIdx.x, px = tid & 31, py = tid >> 5;
  const int x0 = blockIdx.x * TSX, y0 = blockIdx.y * TSY;
  const int x = x0 + 2 * px, y = y0 + 2 * py;
  const bool act = x < W && y < H;
  const int z0 = blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;

  uint4 pre[PERV];
  auto fetch = [&](int p) {
    const S* sp = src + (int64_t)clampi(p, D - 1) * plane;
#pragma unroll
    for (int k = 0; k < PERV; ++k) {
      const int sl = tid + k * 256;
      if (sl < NSLOT) {
        const int r = sl / SR, v = sl - r * SR;
        const S* rowp = sp + (int64_t)clampi(y0 - 1 + r, H - 1) * W;
        const int gx = x0 - RA + v * VE;
        pre[k] = (gx >= 0 && gx < W) ? __ldg(reinterpret_cast<const uint4*>(rowp + gx))
                                     : splat16<S>(__ldg(rowp + (gx < 0 ? 0 : W - 1)));
      }
    }
  };
  int pn = z0 - 1;  // the next plane to stage (its pixels are in pre)
  PV raw[4][3];
  // stage plane pn, start fetching pn + 1, and read this thread's pairs
  auto next_plane = [&]() {
    S* t = tile[(pn - z0 + 1) & 1];
#pragma unroll
    for (int k = 0; k < PERV; ++k) {
      const int sl = tid + k * 256;
      if (sl < NSLOT) reinterpret_cast<uint4*>(t)[sl] = pre[k];
    }
    if (pn + 1 <= z1 + 1) fetch(pn + 1);
    ++pn;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const PV* row = reinterpret_cast<const PV*>(t + (2 * py + r) * RW + RA + 2 * px - 2);
      raw[r][0] = row[0], raw[r][1] = row[1], raw[r][2] = row[2];
    }
  };

  N A[3][2][2], B[3][2][2], C[3][2][2];
  N ex[2][2], ey[2][2], ez[2][2];
  // unsigned pixels: zero pixels among the negative-coefficient taps, per
  // plane, in the same ring as A, B, C.  Zr: 4-bit counts ZX (column x+1
  // over 3 rows), ZY (row y+1 over 3 columns), ZZ (the 3x3 block) of the
  // ring planes; Ec: EX, EY of the newest plane (its taps at dz = +2); one
  // 16-bit lane per output column ox, one word per output row oy.
  uint32_t Zr[3][2] = {}, Ec[2] = {};
  auto terms = [&](N (&a)[2][2], N (&b)[2][2], N (&c)[2][2], uint32_t (&zq)[2]) {
    N v[4][4];  // rows y-1 .. y+2, columns x-1 .. x+2 (clamped by the staging)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      v[r][0] = Pair<S>::hi(raw[r][0]);
      v[r][1] = Pair<S>::lo(raw[r][1]);
      v[r][2] = Pair<S>::hi(raw[r][1]);
      v[r][3] = Pair<S>::lo(raw[r][2]);
    }
    if constexpr (WRAP) {
      N m = v[0][0];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) m = min(m, v[r][c]);
      zq[0] = zq[1] = Ec[0] = Ec[1] = 0;
      if (m == 0) {  // a zero pixel in this thread's 4 x 4 rows of the plane
        uint32_t zr[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) zr[r][c] = v[r][c] == 0 ? 1u : 0u;
#pragma unroll
        for (int oy = 0; oy < 2; ++oy)
#pragma unroll
          for (int ox = 0; ox < 2; ++ox) {
            const int rm = oy, rc = oy + 1, rp = oy + 2, sh = 16 * ox;
            const uint32_t zx = zr[rm][ox + 2] + zr[rc][ox + 2] + zr[rp][ox + 2];
            const uint32_t zy = zr[rp][ox] + zr[rp][ox + 1] + zr[rp][ox + 2];
            const uint32_t zz = zr[rm][ox] + zr[rm][ox + 1] + zr[rm][ox + 2] + zr[rc][ox] + zr[rc][ox + 1] +
                                zr[rc][ox + 2] + zy;
            const uint32_t e_x = zr[rp][ox + 1] + zr[rm][ox + 2] + zr[rc][ox + 2];
            const uint32_t e_y = zr[rc][ox] + zr[rc][ox + 1] + zr[rc][ox + 2];
            zq[oy] |= (zx | (zy << 4) | (zz << 8)) << sh;
            Ec[oy] |= (e_x | (e_y << 4)) << sh;
          }
      }
    }
    N sx[4][2], dx[4][2];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int o = 0; o < 2; ++o) {
        sx[r][o] = v[r][o] + 2 * v[r][o + 1] + v[r][o + 2];
        dx[r][o] = v[r][o] - v[r][o + 2];
      }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const int rm = oy, rc = oy + 1, rp = oy + 2;
        a[oy][ox] = dx[rm][ox] + 2 * dx[rc][ox] + dx[rp][ox];
        b[oy][ox] = sx[rm][ox] - sx[rp][ox];
        c[oy][ox] = sx[rm][ox] + 2 * sx[rc][ox] + sx[rp][ox];
        const N q = 2 * v[rp][ox] + v[rp][ox + 1];
        ex[oy][ox] = 2 * dx[rm][ox] + dx[rc][ox] - v[rp][ox + 1];
        ey[oy][ox] = q - sx[rc][ox];
        ez[oy][ox] = 2 * sx[rm][ox] + sx[rc][ox] + q;
      }
  };
  auto step = [&](int zo, auto i0c, auto i1c, auto i2c) {
    constexpr int i0 = decltype(i0c)::value, i1 = decltype(i1c)::value, i2 = decltype(i2c)::value;
    N a[2][2], b[2][2], c[2][2];
    uint32_t zq[2];
    next_plane();  // plane zo + 2
    terms(a, b, c, zq);
    float res[2][2];
#pragma unroll
    for (int oy = 0; oy < 2; ++oy)
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) {
        const N sxv = A[i0][oy][ox] + 2 * A[i1][oy][ox] + A[i2][oy][ox] + ex[oy][ox];
        const N syv = B[i0][oy][ox] + 2 * B[i1][oy][ox] + B[i2][oy][ox] + ey[oy][ox];
        const N szv = C[i0][oy][ox] - C[i2][oy][ox] + ez[oy][ox];
        float fx = exact_float(sxv), fy = exact_float(syv), fz = exact_float(szv);
        if constexpr (WRAP) {
          // K = 12, 12, 9 taps minus the zero pixels among them (planes
          // zo-1 .. zo+1 from the ring, the dz = +2 taps from Ec)
          float kx = 12.f, ky = 12.f, kz = 9.f;
          if (Zr[i0][oy] | Zr[i1][oy] | Zr[i2][oy] | Ec[oy]) {
            const int sh = 16 * ox;
            const uint32_t sum = Zr[i0][oy] + Zr[i1][oy] + Zr[i2][oy];  // fields <= 9: no carry between them
            kx = exact_float(12 - (int)(((sum >> sh) & 0xFu) + ((Ec[oy] >> sh) & 0xFu)));
            ky = exact_float(12 - (int)(((sum >> (sh + 4)) & 0xFu) + ((Ec[oy] >> (sh + 4)) & 0xFu)));
            kz = exact_float(9 - (int)((Zr[i2][oy] >> (sh + 8)) & 0xFu));
          }
          fx = fmaf(kx, 4294967296.0f, fx);
          fy = fmaf(ky, 4294967296.0f, fy);
          fz = fmaf(kz, 4294967296.0f, fz);
        }
        res[oy][ox] = sqrt_approx(fmaf(fx, fx, fmaf(fy, fy, fz * fz)));
      }
    if (act) {
#pragma unroll
      for (int oy = 0; oy < 2; ++oy) {
        if (y + oy < H)
          *reinterpret_cast<float2*>(dst + (int64_t)zo * plane + (int64_t)(y + oy) * W + x) =
              make_float2(res[oy][0], res[oy][1]);
      }
    }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      Zr[i0][oy] = zq[oy];
#pragma unroll
      for (int ox = 0; ox < 2; ++ox) A[i0][oy][ox] = a[oy][ox], B[i0][oy][ox] = b[oy][ox], C[i0][oy][ox] = c[oy][ox];
    }
  };

  fetch(z0 - 1);
  next_plane();
  terms(A[0], B[0], C[0], Zr[0]);
  next_plane();
  terms(A[1], B[1], C[1], Zr[1]);
  next_plane();
  terms(A[2], B[2], C[2], Zr[2]);
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  for (int zo = z0; zo < z1; zo += 3) {
    step(zo, I0{}, I1{}, I2{});
    if (zo + 1 < z1) step(zo + 1, I1{}, I2{}, I0{});
    if (zo + 2 < z1) step(zo + 2, I2{}, I0{}, I1{});
  }
}

// ---- 16-bit unsigned pixels on packed float pairs.  A pixel value v as a
// 32-bit word is the float v * 2^-149 (a subnormal), and every partial sum of
// this kernel is an integer of magnitude below 2^22 times 2^-149, which a
// float holds exactly; so the sums run as add / fma .rn.f32x2 on the two
// output columns (x, x+1) of a thread at once, with no conversion from int,
// and give the integer kernel's sums bit for bit.  The three component sums
// are then scaled by 2^100 (exact), the 2^32 wrap terms added as K * 2^-17,
// squared and summed in the integer kernel's order, so every rounding is
// the same at a scale of 2^-49; the root is scaled back by 2^49.  (Subnormal
// operands need the non-flushing forms: no .ftz.)
__device__ __forceinline__ uint64_t u2(uint32_t lo, uint32_t hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(lo), "r"(hi));
  return r;
}
__device__ __forceinline__ uint64_t f2c(float a) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(a));
  return r;
}
__device__ __forceinline__ uint64_t x2add(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t x2sub(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t x2mul(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t x2fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}

template <bool WRAP>
__global__ void __launch_bounds__(256, 3) k_sobel3d_x2(const uint16_t* __restrict__ src, float* __restrict__ dst,
                                                        int W, int H, int D, int zchunk) {
  using S = uint16_t;
  constexpr int VE = 8, RA = VE;
  constexpr int RW = TSX + 2 * RA, RH = TSY + 3;
  constexpr int SR = RW / VE, NSLOT = RH * SR;
  static_assert(NSLOT <= 256, "one staging vector per thread");
  __shared__ __align__(16) S tile[2][RH * RW];
  const int tid = threadIdx.x, px = tid & 31, py = tid >> 5;
  const int x0 = blockIdx.x * TSX, y0 = blockIdx.y * TSY;
  const int x = x0 + 2 * px, y = y0 + 2 * py;
  const bool act = x < W && y < H;
  const int z0 = blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;

  uint4 pre = make_uint4(0, 0, 0, 0);
  auto fetch = [&](int p) {
    const S* sp = src + (int64_t)clampi(p, D - 1) * plane;
    if (tid < NSLOT) {
      const int r = tid / SR, v = tid - r * SR;
      const S* rowp = sp + (int64_t)clampi(y0 - 1 + r, H - 1) * W;
      const int gx = x0 - RA + v * VE;
      pre = (gx >= 0 && gx < W) ? __ldg(reinterpret_cast<const uint4*>(rowp + gx))
                                : splat16<S>(__ldg(rowp + (gx < 0 ? 0 : W - 1)));
    }
  };
  int pn = z0 - 1;  // the next plane to stage (its pixels are in pre)
  uint32_t raw[4][3];
  auto next_plane = [&]() {
    S* t = tile[(pn - z0 + 1) & 1];
    if (tid < NSLOT) reinterpret_cast<uint4*>(t)[tid] = pre;
    if (pn + 1 <= z1 + 1) fetch(pn + 1);
    ++pn;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint32_t* row = reinterpret_cast<const uint32_t*>(t + (2 * py + r) * RW + RA + 2 * px - 2);
      raw[r][0] = row[0], raw[r][1] = row[1], raw[r][2] = row[2];
    }
  };

  const uint64_t two = f2c(2.0f);
  // per output row oy: A, B, C of the ring planes and the newest plane's E
  // terms, as (x, x+1) pairs
  uint64_t A[3][2], B[3][2], C[3][2], ex[2], ey[2], ez[2];
  uint32_t Zr[3][2] = {}, Ec[2] = {};  // zero-pixel counts, as in k_sobel3d_tile
  auto terms = [&](uint64_t (&a)[2], uint64_t (&b)[2], uint64_t (&c)[2], uint32_t (&zq)[2]) {
    uint32_t v[4][4];  // rows y-1 .. y+2, columns x-1 .. x+2
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      v[r][0] = raw[r][0] >> 16;
      v[r][1] = raw[r][1] & 0xFFFFu;
      v[r][2] = raw[r][1] >> 16;
      v[r][3] = raw[r][2] & 0xFFFFu;
    }
    if constexpr (WRAP) {
      // a zero among the 4 x 4 pixels: min over the packed middle words and
      // the outer columns' pairs (x-1, x+2)
      uint32_t m = __byte_perm(raw[0][0], raw[0][2], 0x5432);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        m = __vminu2(m, raw[r][1]);
        if (r) m = __vminu2(m, __byte_perm(raw[r][0], raw[r][2], 0x5432));
      }
      zq[0] = zq[1] = Ec[0] = Ec[1] = 0;
      if ((m & 0xFFFFu) == 0 || (m >> 16) == 0) {
        uint32_t zr[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int c = 0; c < 4; ++c) zr[r][c] = v[r][c] == 0 ? 1u : 0u;
#pragma unroll
        for (int oy = 0; oy < 2; ++oy)
#pragma unroll
          for (int ox = 0; ox < 2; ++ox) {
            const int rm = oy, rc = oy + 1, rp = oy + 2, sh = 16 * ox;
            const uint32_t zx = zr[rm][ox + 2] + zr[rc][ox + 2] + zr[rp][ox + 2];
            const uint32_t zy = zr[rp][ox] + zr[rp][ox + 1] + zr[rp][ox + 2];
            const uint32_t zz = zr[rm][ox] + zr[rm][ox + 1] + zr[rm][ox + 2] + zr[rc][ox] + zr[rc][ox + 1] +
                                zr[rc][ox + 2] + zy;
            const uint32_t e_x = zr[rp][ox + 1] + zr[rm][ox + 2] + zr[rc][ox + 2];
            const uint32_t e_y = zr[rc][ox] + zr[rc][ox + 1] + zr[rc][ox + 2];
            zq[oy] |= (zx | (zy << 4) | (zz << 8)) << sh;
            Ec[oy] |= (e_x | (e_y << 4)) << sh;
          }
      }
    }
    uint64_t p12[4], sx[4], dx[4], p01r[2];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint64_t p01 = u2(v[r][0], v[r][1]), p23 = u2(v[r][2], v[r][3]);
      p12[r] = u2(v[r][1], v[r][2]);
      sx[r] = x2add(x2fma(p12[r], two, p01), p23);
      dx[r] = x2sub(p01, p23);
      if (r >= 2) p01r[r - 2] = p01;
    }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      const int rm = oy, rc = oy + 1, rp = oy + 2;
      a[oy] = x2add(x2fma(dx[rc], two, dx[rm]), dx[rp]);
      b[oy] = x2sub(sx[rm], sx[rp]);
      c[oy] = x2add(x2fma(sx[rc], two, sx[rm]), sx[rp]);
      const uint64_t q = x2fma(p01r[oy], two, p12[rp]);
      ex[oy] = x2sub(x2fma(dx[rm], two, dx[rc]), p12[rp]);
      ey[oy] = x2sub(q, sx[rc]);
      ez[oy] = x2add(x2fma(sx[rm], two, sx[rc]), q);
    }
  };
  auto step = [&](int zo, auto i0c, auto i1c, auto i2c) {
    constexpr int i0 = decltype(i0c)::value, i1 = decltype(i1c)::value, i2 = decltype(i2c)::value;
    uint64_t a[2], b[2], c[2];
    uint32_t zq[2];
    next_plane();  // plane zo + 2
    terms(a, b, c, zq);
    const uint64_t up = f2c(0x1p100f);
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      const uint64_t sxv = x2add(x2add(x2fma(A[i1][oy], two, A[i0][oy]), A[i2][oy]), ex[oy]);
      const uint64_t syv = x2add(x2add(x2fma(B[i1][oy], two, B[i0][oy]), B[i2][oy]), ey[oy]);
      const uint64_t szv = x2add(x2sub(C[i0][oy], C[i2][oy]), ez[oy]);
      uint64_t fx = x2mul(sxv, up), fy = x2mul(syv, up), fz = x2mul(szv, up);
      if constexpr (WRAP) {
        // + K * 2^32 at the scale 2^-49: K = 12, 12, 9 taps minus the zero
        // pixels among them
        uint64_t kx = f2c(12.0f * 0x1p-17f), ky = kx, kz = f2c(9.0f * 0x1p-17f);
        if (Zr[i0][oy] | Zr[i1][oy] | Zr[i2][oy] | Ec[oy]) {
          const uint32_t sum = Zr[i0][oy] + Zr[i1][oy] + Zr[i2][oy];  // fields <= 9: no carry between them
          float k[3][2];
#pragma unroll
          for (int ox = 0; ox < 2; ++ox) {
            const int sh = 16 * ox;
            k[0][ox] = (float)(12 - (int)(((sum >> sh) & 0xFu) + ((Ec[oy] >> sh) & 0xFu))) * 0x1p-17f;
            k[1][ox] = (float)(12 - (int)(((sum >> (sh + 4)) & 0xFu) + ((Ec[oy] >> (sh + 4)) & 0xFu))) * 0x1p-17f;
            k[2][ox] = (float)(9 - (int)((Zr[i2][oy] >> (sh + 8)) & 0xFu)) * 0x1p-17f;
          }
          kx = u2(__float_as_uint(k[0][0]), __float_as_uint(k[0][1]));
          ky = u2(__float_as_uint(k[1][0]), __float_as_uint(k[1][1]));
          kz = u2(__float_as_uint(k[2][0]), __float_as_uint(k[2][1]));
        }
        fx = x2add(fx, kx);
        fy = x2add(fy, ky);
        fz = x2add(fz, kz);
      }
      const uint64_t s = x2fma(fx, fx, x2fma(fy, fy, x2mul(fz, fz)));
      uint32_t s0, s1;
      asm("mov.b64 {%0, %1}, %2;" : "=r"(s0), "=r"(s1) : "l"(s));
      const uint64_t res = x2mul(u2(__float_as_uint(sqrt_approx(__uint_as_float(s0))),
                                    __float_as_uint(sqrt_approx(__uint_as_float(s1)))),
                                 f2c(0x1p49f));
      if (act && y + oy < H)
        *reinterpret_cast<uint64_t*>(dst + (int64_t)zo * plane + (int64_t)(y + oy) * W + x) = res;
    }
#pragma unroll
    for (int oy = 0; oy < 2; ++oy) {
      Zr[i0][oy] = zq[oy];
      A[i0][oy] = a[oy], B[i0][oy] = b[oy], C[i0][oy] = c[oy];
    }
  };

  fetch(z0 - 1);
  next_plane();
  terms(A[0], B[0], C[0], Zr[0]);
  next_plane();
  terms(A[1], B[1], C[1], Zr[1]);
  next_plane();
  terms(A[2], B[2], C[2], Zr[2]);
  using I0 = std::integral_constant<int, 0>;
  using I1 = std::integral_constant<int, 1>;
  using I2 = std::integral_constant<int, 2>;
  for (int zo = z0; zo < z1; zo += 3) {
    step(zo, I0{}, I1{}, I2{});
    if (zo + 1 < z1) step(zo + 1, I1{}, I2{}, I0{});
    if (zo + 2 < z1) step(zo + 2, I2{}, I0{}, I1{});
  }
}

// CLK_SOBEL_X2=0 in the environment keeps 16-bit pixels on the integer
// kernel (A/B timing)
bool x2_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_SOBEL_X2");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <bool WRAP> clk_status launch_sobel_x2(const Image& dst, const Image& src, cudaStream_t st) {
  const int tx = (src.w + TSX - 1) / TSX, ty = (src.h + TSY - 1) / TSY;
  int dev = 0, sms = 152, per_sm = 2;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sobel3d_x2<WRAP>, 256, 0);
  // whole waves of resident CTAs; each chunk re-reads 3 halo planes
  int chunks = wave_chunks((int64_t)tx * ty, src.d, 3, (int64_t)sms * (per_sm > 0 ? per_sm : 1), 1,
                           src.d / 16 > 1 ? src.d / 16 : 1);
  static const int forced = [] {  // CLK_SOBEL_CHUNKS=n fixes the z-chunks per tile (A/B timing)
    const char* e = getenv("CLK_SOBEL_CHUNKS");
    return e ? atoi(e) : 0;
  }();
  if (forced > 0) chunks = forced < src.d ? forced : src.d;
  const int zchunk = (src.d + chunks - 1) / chunks;
  k_sobel3d_x2<WRAP><<<dim3(tx, ty, (src.d + zchunk - 1) / zchunk), 256, 0, st>>>(
      (const uint16_t*)src.ptr, (float*)dst.ptr, src.w, src.h, src.d, zchunk);
  count_launch();
  return check_launch("sobel_3d (float pairs)");
}

template <class S, bool WRAP> clk_status launch_sobel_tile(const Image& dst, const Image& src, cudaStream_t st) {
  const int tx = (src.w + TSX - 1) / TSX, ty = (src.h + TSY - 1) / TSY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 6LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  k_sobel3d_tile<S, WRAP><<<dim3(tx, ty, (src.d + zchunk - 1) / zchunk), 256, 0, st>>>(
      (const S*)src.ptr, (float*)dst.ptr, src.w, src.h, src.d, zchunk);
  count_launch();
  return check_launch("sobel_3d (staged)");
}

template <class S, bool WRAP> clk_status launch_sobel(const Image& dst, const Image& src, cudaStream_t st) {
  const dim3 block(SBX, SBY);
  const int tx = (src.w / 2 + SBX - 1) / SBX, ty = ((src.h + 1) / 2 + SBY - 1) / SBY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 8LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  k_sobel3d_fast<S, WRAP><<<dim3(tx, ty, (src.d + zchunk - 1) / zchunk), block, 0, st>>>(
      (const S*)src.ptr, (float*)dst.ptr, src.w, src.h, src.d, zchunk);
  count_launch();
  return check_launch("sobel_3d (fast)");
}

}  // namespace

clk_status fast_sobel(const Image& dst, const Image& src, const Policy& p, cudaStream_t st) {
  if (src.ndim != 3 || dst.dt != CLK_F32 || src.w % 2 != 0 || src.w != dst.w || src.h != dst.h || src.d != dst.d)
    return CLK_UNSUPPORTED_DTYPE;
  if ((uintptr_t)dst.ptr % 8 != 0 || (uintptr_t)src.ptr % (2 * dtype_size(src.dt)) != 0) return CLK_UNSUPPORTED_DTYPE;
  const bool wrap = !p.sobel_narrow;
  // staged tiles when rows are whole 16-byte vectors
  const int ve = 16 / dtype_size(src.dt);
  if ((uintptr_t)src.ptr % 16 == 0 && src.w % ve == 0) {
    switch (src.dt) {
      case CLK_U16:
        if (x2_enabled()) return wrap ? launch_sobel_x2<true>(dst, src, st) : launch_sobel_x2<false>(dst, src, st);
        return wrap ? launch_sobel_tile<uint16_t, true>(dst, src, st) : launch_sobel_tile<uint16_t, false>(dst, src, st);
      case CLK_U8:
        return wrap ? launch_sobel_tile<uint8_t, true>(dst, src, st) : launch_sobel_tile<uint8_t, false>(dst, src, st);
      case CLK_I16: return launch_sobel_tile<int16_t, false>(dst, src, st);
      case CLK_I8: return launch_sobel_tile<int8_t, false>(dst, src, st);
      case CLK_F32: return launch_sobel_tile<float, false>(dst, src, st);
    }
  }
  switch (src.dt) {
    case CLK_U16: return wrap ? launch_sobel<uint16_t, true>(dst, src, st) : launch_sobel<uint16_t, false>(dst, src, st);
    case CLK_U8: return wrap ? launch_sobel<uint8_t, true>(dst, src, st) : launch_sobel<uint8_t, false>(dst, src, st);
    case CLK_I16: return launch_sobel<int16_t, false>(dst, src, st);
    case CLK_I8: return launch_sobel<int8_t, false>(dst, src, st);
    case CLK_F32: return launch_sobel<float, false>(dst, src, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
