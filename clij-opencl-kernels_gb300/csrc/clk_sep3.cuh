// clk_sep3.cuh - fused X -> Y -> Z separable filters on 16-bit pixels with a
// compile-time XY radius R (cx = cy = R) and Z radius CZ: minimum / maximum
// and mean to the same pixel type, Gaussian to float.
//
// A CTA (256 threads) owns a 64 x 32 column of outputs and streams along z,
// one barrier per plane.  In the phase of plane i it
//   X pass  plane i: a thread filters MX outputs of a ROW PAIR -- rows 2p
//           and 2p+1 packed into the two lanes of each word by one byte
//           permute per column (u16 lanes for min/max; an f32x2 pair for
//           the Gaussian, converted once per staged pixel) -- so that every
//           operation serves two rows; the window slides in registers (van
//           Herk / Gil-Werman split for min/max: 2R + 2M - 2 packed
//           operations for M outputs of both rows; running int32 sums for
//           the mean, one row per task; 8 accumulators for the Gaussian);
//           results go back to plain rows, even and odd rows in two regions
//           so that a warp's 16-byte stores hit distinct banks;
//   Y pass  plane i-1: a thread filters a column pair (x, x+1) x 4 rows;
//   Z pass  the Y results enter a ring of the last 2CZ+1 planes held in the
//           thread's REGISTERS (one copy of the ring step per slot, chosen
//           by the slot counter, so that every slot is a fixed register);
//           the thread reduces its ring and writes two pixels per store.
// Staging: cp.async copies of the raw halo tile (no registers, no
// instructions beyond one per 16-byte vector), rows clamped at the source;
// min / max / mean copy two planes ahead into three buffers and the tiles
// at the x border fill their outside vectors in shared memory; the Gaussian
// converts each landed tile to f32x2 row pairs one phase ahead.
//
// Arithmetic (the same as the generic fused kernels, so the results are too):
// min/max exact; the mean sums exactly in int32 and divides by a 32-bit
// reciprocal multiply equal to truncating fl(S/N) (sep2::div_exact), with
// dst-typed (16-bit) results between passes as the reference's three
// launches have; the Gaussian to float accumulates fma.rn.f32x2 products of
// taps pre-divided by their sum (within the float tolerance of the FP64
// oracle, not in the reference's order).
#pragma once
#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <utility>

#include "clk_sep2.cuh"

namespace clk {
namespace sep3 {
namespace {

using sep2::div_exact;
using sep2::f2_add;
using sep2::f2_fma;
using sep2::f2_pack;
using sep2::f2_unpack;

enum Op { MIN = 0, MAX = 1, MEAN = 2, GAUSS = 3 };
constexpr int TX = 64;  // output columns per tile (32 column pairs: one warp)

// Launch shape: NT threads; the Y/Z pass gives a thread a column pair x
// SEGY rows (threads beyond 32 x TY/SEGY sit out the Y/Z pass); an X task is
// MX outputs of a row pair (the Gaussian: 8); MINB CTAs per SM for the
// register budget.
template <int NT_, int SEGY_, int MX_, int MINB_, int TY_ = 32> struct Cfg {
  static constexpr int NT = NT_, SEGY = SEGY_, MX = MX_, MINB = MINB_, TY = TY_;  // TY: output rows per tile
};
// instantiated radii: XY radius 1..kMaxRInt (min / max / mean) or
// 1..kMaxRGauss, Z radius 0..kMaxCz*; other radii take the generic fused
// kernels
constexpr int kMaxRInt = 8, kMaxCzInt = 3;
constexpr int kMaxRGauss = 12, kMaxCzGauss = 6;

struct P3 {
  // Gaussian: taps w[k] for offsets +-k, pre-divided by their sum, each as
  // an f32x2 pair (w, w)
  uint64_t wx[13], wy[13], wz[8];
  uint32_t mx, mz;  // mean: recip32(2R+1), recip32(2CZ+1)
};

__host__ __device__ constexpr int rup(int v, int m) { return (v + m - 1) / m * m; }

// f(integral_constant<int, s>) for a runtime s in [LO, HI), by binary search:
// ceil(log2(HI - LO)) compares instead of one per value
template <int LO, int HI, class F> __device__ __forceinline__ void dispatch(int s, F&& f) {
  if constexpr (HI - LO == 1) {
    f(std::integral_constant<int, LO>{});
  } else {
    constexpr int MID = (LO + HI) / 2;
    if (s < MID) dispatch<LO, MID>(s, f);
    else dispatch<MID, HI>(s, f);
  }
}

template <int OP, int R, int CZ, class C> struct Geo {
  static constexpr int NT = C::NT, TY = C::TY;
  static constexpr int MX = OP == GAUSS ? 8 : C::MX;  // outputs of an X task
  static constexpr int RA = rup(R, 8);         // staged margin left and right (whole vectors)
  static constexpr int SW = TX + 2 * RA;       // staged columns
  static constexpr int NV = SW / 8;            // 16-byte vectors per staged row
  static constexpr int NR = TY + 2 * R;        // staged rows (even)
  static constexpr int NP = NR / 2;            // row pairs
  static constexpr int XOFF = RA - R;          // first staged column of the X windows
  static constexpr int NZ = 2 * CZ + 1;
  static constexpr bool PAIRS = OP != MEAN;    // X pass on row pairs
  // staging: raw tiles (cp.async destinations), NRAW buffers of NR rows x SW
  // pixels, pitch RWP.  Tasks: the Gaussian (vector, row pair), two copies
  // each; the others (vector, row), one copy each.
  static constexpr int NRAW = OP == GAUSS ? 2 : 3;
  static constexpr int RWP = OP == GAUSS ? SW + 8 : SW;
  static constexpr int RAW_BYTES = rup(NR * RWP * 2, 128);
  static constexpr int NST = OP == GAUSS ? NP * NV : NR * NV;
  static constexpr int PST = (NST + NT - 1) / NT;
  // the Gaussian's converted tile: f32x2 row pairs, pitch CW entries (an odd
  // number of 16-byte units: a warp's X reads, one row pair per thread, fall
  // in distinct banks)
  static constexpr int CW = SW + 2;
  static constexpr int CV_BYTES = OP == GAUSS ? rup(NP * CW * 8, 128) : 0;
  // X results: NR rows x TX of u16 (f32 for GAUSS), pitch XP; the row-pair
  // layouts store even rows and odd rows in two regions (XHALF apart)
  static constexpr int XEL = OP == GAUSS ? 4 : 2;
  static constexpr int XP = OP == GAUSS ? TX + 4 : TX + 8;  // 272 / 144 bytes: an odd number of 16-byte units
  static constexpr int XHALF = NP * XP;
  static constexpr int XS_BYTES = rup(NR * XP * XEL, 128);
  static constexpr int XTASKS = (PAIRS ? NP : NR) * (TX / MX);
  static constexpr int SMEM = NRAW * RAW_BYTES + 2 * CV_BYTES + 2 * XS_BYTES;
  // pixels (Gaussian: f32x2 entries) an X task reads from the start of its segment
  static constexpr int NWX = rup(XOFF + MX + 2 * R, OP == GAUSS ? 2 : 8);
};

template <bool SG, int OP> __device__ __forceinline__ uint32_t mm(uint32_t a, uint32_t b) {
  if constexpr (OP == MIN) return SG ? sep2::s16x2_min(a, b) : sep2::u16x2_min(a, b);
  else return SG ? sep2::s16x2_max(a, b) : sep2::u16x2_max(a, b);
}

// out[j] = op(win[j .. j+2R]) for j < M: the van Herk / Gil-Werman split
// (2R + 2M - 2 operations) when every window contains column M; longer runs
// in pieces of 2R outputs; direct for a single output
template <bool SG, int OP, int M, int R, int O = 0>
__device__ __forceinline__ void slide_minmax(const uint32_t (&win)[M + 2 * R], uint32_t (&out)[M]) {
  constexpr int B = (2 * R < M - O) ? 2 * R : M - O;  // outputs O .. O+B-1 in this piece
  if constexpr (B > 1) {
    uint32_t suf[B];
    suf[B - 1] = win[O + B - 1];
#pragma unroll
    for (int j = B - 2; j >= 0; --j) suf[j] = mm<SG, OP>(win[O + j], suf[j + 1]);
    uint32_t pre = win[O + B];
#pragma unroll
    for (int k = B + 1; k <= 2 * R; ++k) pre = mm<SG, OP>(pre, win[O + k]);
    out[O] = mm<SG, OP>(suf[0], pre);
#pragma unroll
    for (int j = 1; j < B; ++j) {
      pre = mm<SG, OP>(pre, win[O + j + 2 * R]);
      out[O + j] = mm<SG, OP>(suf[j], pre);
    }
  } else {
    uint32_t a = win[O];
#pragma unroll
    for (int k = 1; k <= 2 * R; ++k) a = mm<SG, OP>(a, win[O + k]);
    out[O] = a;
  }
  if constexpr (O + B < M) slide_minmax<SG, OP, M, R, O + B>(win, out);
}

template <bool SG> __device__ __forceinline__ int lane_lo(uint32_t w) {
  return SG ? (int)(w << 16) >> 16 : (int)(w & 0xFFFFu);
}
template <bool SG> __device__ __forceinline__ int lane_hi(uint32_t w) { return SG ? (int)w >> 16 : (int)(w >> 16); }

__device__ __forceinline__ uint32_t splat16(uint16_t v) { return (uint32_t)v * 0x10001u; }

__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// (row a, row b) of element e of two 8-pixel u16 vectors as an exact f32x2:
// the float 2^23 + v built by a byte permute, minus 2^23 (unsigned pixels)
__device__ __forceinline__ uint64_t f2_of_u16(uint32_t wa, uint32_t wb, int lane) {
  constexpr uint32_t K = 0x4B000000u;
  const uint32_t sel = lane ? 0x7432u : 0x7410u;
  const float a = __uint_as_float(__byte_perm(wa, K, sel)), b = __uint_as_float(__byte_perm(wb, K, sel));
  return f2_add(f2_pack(a, b), f2_pack(-8388608.0f, -8388608.0f));
}

template <class S, int OP, int R, int CZ, class C>
__global__ void __launch_bounds__(C::NT, C::MINB)
    k_sep3(const S* __restrict__ src, void* __restrict__ dstv, int W, int H, int Dz, int zchunk,
           const __grid_constant__ P3 p) {
  using G = Geo<OP, R, CZ, C>;
  constexpr int NT = C::NT, SEGY = C::SEGY, MX = G::MX, TY = C::TY;
  constexpr bool SG = std::is_signed<S>::value;
  constexpr int NZ = G::NZ;
  static_assert(G::XTASKS <= NT, "one X task per thread");
  static_assert(NT / 32 * SEGY >= TY, "the Y tasks cover the tile");
  extern __shared__ __align__(128) unsigned char smem[];
  // byte offsets of the buffers in shared memory
  constexpr uint32_t RAW0 = 0, CV0 = G::NRAW * G::RAW_BYTES, XS0 = CV0 + 2 * G::CV_BYTES;

  const int tid = threadIdx.x;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int z0 = blockIdx.z * zchunk, z1 = min(Dz, z0 + zchunk);
  const size_t plane = (size_t)W * H;
  // a tile whose staged columns reach past the image: its outside vectors
  // are filled in shared memory (rows are clamped at the source)
  const bool xborder = x0 - G::RA < 0 || x0 + TX + G::RA > W;

  // ---- staging tasks of this thread (the same for every plane): the
  // in-plane offset of each copied 16-byte vector (rows clamped) and its
  // place in the raw tile; vectors outside their row are not copied (bit k
  // of outside) but repeat the row's edge pixel.  Rows and the staged
  // origin are vector-aligned (W % 8 == 0): a vector is wholly inside or
  // outside.
  uint32_t goff[G::PST], soff[G::PST], eoff[G::PST];
  uint32_t valid = 0, outside = 0;
#pragma unroll
  for (int k = 0; k < G::PST; ++k) {
    const int q = tid + k * NT;
    goff[k] = soff[k] = eoff[k] = 0;
    if (q < G::NST) {
      valid |= 1u << k;
      const int v = q % G::NV, r = q / G::NV;
      const int gx = x0 - G::RA + 8 * v;
      const int ra = OP == GAUSS ? 2 * r : r;  // first staged row of the task
      if (gx < 0 || gx >= W) {
        outside |= 1u << k;
        eoff[k] = (uint32_t)(ra * G::RWP + (gx < 0 ? 0 : W - 1) - (x0 - G::RA)) * 2;  // the row's edge pixel
      }
      goff[k] = (uint32_t)clampi(y0 - R + ra, H - 1) * (uint32_t)W + (uint32_t)min(max(gx, 0), W - 8);
      soff[k] = (uint32_t)(ra * G::RWP + 8 * v) * 2;
    }
  }
  uint32_t goff2[OP == GAUSS ? G::PST : 1];  // the Gaussian's second row
#pragma unroll
  for (int k = 0; k < (OP == GAUSS ? G::PST : 1); ++k) {
    goff2[k] = 0;
    const int q = tid + k * NT;
    if (OP == GAUSS && q < G::NST) {
      const int v = q % G::NV, r = q / G::NV;
      const int gx = x0 - G::RA + 8 * v;
      goff2[k] = (uint32_t)clampi(y0 - R + 2 * r + 1, H - 1) * (uint32_t)W + (uint32_t)min(max(gx, 0), W - 8);
    }
  }
  auto issue_raw = [&](int zv, uint32_t rwo) {
    const S* sp = src + (size_t)clampi(zv, Dz - 1) * plane;
#pragma unroll
    for (int k = 0; k < G::PST; ++k) {
      if ((valid & ~outside) >> k & 1) {
        cp_async16(smem + rwo + soff[k], sp + goff[k]);
        if constexpr (OP == GAUSS) cp_async16(smem + rwo + soff[k] + G::RWP * 2, sp + goff2[k]);
      }
    }
    cp_async_commit();
  };
  // min / max / mean: the outside vectors of a landed raw tile repeat their
  // row's edge pixel (x-border tiles only)
  auto fixup = [&](uint32_t rwo) {
#pragma unroll
    for (int k = 0; k < G::PST; ++k) {
      if (outside >> k & 1) {
        const uint32_t e = splat16(*reinterpret_cast<const uint16_t*>(smem + rwo + eoff[k]));
        *reinterpret_cast<uint4*>(smem + rwo + soff[k]) = make_uint4(e, e, e, e);
      }
    }
  };
  // Gaussian: raw -> f32x2 row pairs, tasks (row pair yp, vector v), yp
  // fastest; a vector outside its row repeats the edge pixel
  uint32_t crd[OP == GAUSS ? G::PST : 1], cwr[OP == GAUSS ? G::PST : 1];
  uint32_t cedge = 0;
#pragma unroll
  for (int k = 0; k < (OP == GAUSS ? G::PST : 1); ++k) {
    const int q = tid + k * NT;
    crd[k] = cwr[k] = 0;
    if (OP == GAUSS && q < G::NST) {
      const int yp = q % G::NP, v = q / G::NP;
      const int gx = x0 - G::RA + 8 * v;
      int col = 8 * v;
      if (gx < 0 || gx >= W) {
        cedge |= 1u << k;
        col = (gx < 0 ? 0 : W - 1) - (x0 - G::RA);  // staged column of the edge pixel
      }
      crd[k] = (uint32_t)((2 * yp) * G::RWP + col) * 2;
      cwr[k] = (uint32_t)(yp * G::CW + 8 * v) * 8;
    }
  }
  auto convert = [&](uint32_t rwo, uint32_t cvo) {
#pragma unroll
    for (int k = 0; k < (OP == GAUSS ? G::PST : 1); ++k) {
      if (valid >> k & 1) {
        const unsigned char* s = smem + rwo + crd[k];
        uint4 a, b;
        if (cedge >> k & 1) {
          const uint32_t ea = splat16(*reinterpret_cast<const uint16_t*>(s));
          const uint32_t eb = splat16(*reinterpret_cast<const uint16_t*>(s + G::RWP * 2));
          a = make_uint4(ea, ea, ea, ea), b = make_uint4(eb, eb, eb, eb);
        } else {
          a = *reinterpret_cast<const uint4*>(s);
          b = *reinterpret_cast<const uint4*>(s + G::RWP * 2);
        }
        const uint32_t wa[4] = {a.x, a.y, a.z, a.w}, wb[4] = {b.x, b.y, b.z, b.w};
        unsigned char* o = smem + cvo + cwr[k];
#pragma unroll
        for (int m = 0; m < 4; ++m)
          reinterpret_cast<ulonglong2*>(o)[m] = make_ulonglong2(f2_of_u16(wa[m], wb[m], 0), f2_of_u16(wa[m], wb[m], 1));
      }
    }
  };

  // ---- X task of this thread (at most one).  Min / max / mean: segment xsg
  // of MX outputs fastest, then the row pair (row for the mean), so a warp's
  // 16-byte reads and writes are contiguous; the Gaussian: row pair fastest
  // (the converted tile's pitch spreads those over the banks).
  const bool xvalid = tid < G::XTASKS;
  uint32_t xrd = 0, xwr = 0;
  {
    const int q = xvalid ? tid : 0;
    if constexpr (OP == GAUSS) {
      const int xr = q % G::NP, xsg = q / G::NP;
      xrd = (uint32_t)(xr * G::CW + 8 * xsg + (G::XOFF & ~1)) * 8;
      xwr = (uint32_t)(xr * G::XP + 8 * xsg) * 4;
    } else {
      constexpr int NSG = TX / MX;
      const int xsg = q % NSG, xr = q / NSG;
      xrd = (uint32_t)((G::PAIRS ? 2 * xr : xr) * G::RWP + MX * xsg) * 2;
      xwr = (uint32_t)(xr * G::XP + MX * xsg) * 2;  // row-pair layouts: even region row xr = tile row 2xr
    }
  }
  auto xpass = [&](uint32_t rwo, uint32_t cvo, uint32_t xso) {
    if (!xvalid) return;
    unsigned char* xe = smem + xso + xwr;
    if constexpr (OP == MIN || OP == MAX) {
      const unsigned char* ra = smem + rwo + xrd;
      const unsigned char* rb = ra + G::RWP * 2;
      uint32_t wa[G::NWX / 2], wb[G::NWX / 2];
#pragma unroll
      for (int m = 0; m < G::NWX / 8; ++m) {
        const uint4 t = reinterpret_cast<const uint4*>(ra)[m], u = reinterpret_cast<const uint4*>(rb)[m];
        wa[4 * m] = t.x, wa[4 * m + 1] = t.y, wa[4 * m + 2] = t.z, wa[4 * m + 3] = t.w;
        wb[4 * m] = u.x, wb[4 * m + 1] = u.y, wb[4 * m + 2] = u.z, wb[4 * m + 3] = u.w;
      }
      // row pairs (row 2yp low lane, row 2yp+1 high lane) of the window
      uint32_t win[MX + 2 * R], o[MX];
#pragma unroll
      for (int j = 0; j < MX + 2 * R; ++j) {
        const int e = G::XOFF + j;
        win[j] = __byte_perm(wa[e >> 1], wb[e >> 1], (e & 1) ? 0x7632 : 0x5410);
      }
      slide_minmax<SG, OP, MX, R>(win, o);
      unsigned char* xo = xe + G::XHALF * 2;  // odd rows
#pragma unroll
      for (int h = 0; h < MX / 8; ++h) {
        const uint32_t* t = o + 8 * h;
        reinterpret_cast<uint4*>(xe)[h] = make_uint4(__byte_perm(t[0], t[1], 0x5410), __byte_perm(t[2], t[3], 0x5410),
                                                     __byte_perm(t[4], t[5], 0x5410), __byte_perm(t[6], t[7], 0x5410));
        reinterpret_cast<uint4*>(xo)[h] = make_uint4(__byte_perm(t[0], t[1], 0x7632), __byte_perm(t[2], t[3], 0x7632),
                                                     __byte_perm(t[4], t[5], 0x7632), __byte_perm(t[6], t[7], 0x7632));
      }
    } else if constexpr (OP == MEAN) {
      const unsigned char* rowp = smem + rwo + xrd;
      uint32_t w[G::NWX / 2];
#pragma unroll
      for (int m = 0; m < G::NWX / 8; ++m) {
        const uint4 t = reinterpret_cast<const uint4*>(rowp)[m];
        w[4 * m] = t.x, w[4 * m + 1] = t.y, w[4 * m + 2] = t.z, w[4 * m + 3] = t.w;
      }
      auto val = [&](int e) { return (e & 1) ? lane_hi<SG>(w[e >> 1]) : lane_lo<SG>(w[e >> 1]); };
      int sum = 0;
#pragma unroll
      for (int j = 0; j <= 2 * R; ++j) sum += val(G::XOFF + j);
      int qv[MX];
      qv[0] = div_exact<SG>(sum, p.mx);
#pragma unroll
      for (int i = 1; i < MX; ++i) {
        sum += val(G::XOFF + i + 2 * R) - val(G::XOFF + i - 1);
        qv[i] = div_exact<SG>(sum, p.mx);
      }
#pragma unroll
      for (int h = 0; h < MX / 8; ++h) {
        const int* t = qv + 8 * h;
        reinterpret_cast<uint4*>(xe)[h] = make_uint4(__byte_perm(t[0], t[1], 0x5410), __byte_perm(t[2], t[3], 0x5410),
                                                     __byte_perm(t[4], t[5], 0x5410), __byte_perm(t[6], t[7], 0x5410));
      }
    } else {  // GAUSS: 8 accumulators, each entry added to every output it reaches
      const unsigned char* rowp = smem + cvo + xrd;
      constexpr int E0 = G::XOFF & ~1;  // first entry read (16-byte aligned)
      uint64_t acc[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) acc[i] = 0;
#pragma unroll
      for (int m = 0; m < (G::NWX - E0) / 2; ++m) {
        const ulonglong2 t = reinterpret_cast<const ulonglong2*>(rowp)[m];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int j = E0 + 2 * m + h - G::XOFF;  // window index of this entry
          const uint64_t e = h ? t.y : t.x;
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const int k = j - i - R;  // tap offset
            if (j >= 0 && j < 8 + 2 * R && k >= -R && k <= R) acc[i] = f2_fma(p.wx[k < 0 ? -k : k], e, acc[i]);
          }
        }
      }
      unsigned char* xo = xe + G::XHALF * 4;
      float2 f[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) f[i] = f2_unpack(acc[i]);
      reinterpret_cast<float4*>(xe)[0] = make_float4(f[0].x, f[1].x, f[2].x, f[3].x);
      reinterpret_cast<float4*>(xe)[1] = make_float4(f[4].x, f[5].x, f[6].x, f[7].x);
      reinterpret_cast<float4*>(xo)[0] = make_float4(f[0].y, f[1].y, f[2].y, f[3].y);
      reinterpret_cast<float4*>(xo)[1] = make_float4(f[4].y, f[5].y, f[6].y, f[7].y);
    }
  };

  // ---- Y task (column pair c, rows SEGY*g ..) + Z ring (registers) + store
  const int c = tid & 31, g = tid >> 5;
  const bool yvalid = SEGY * g < TY;
  typedef typename std::conditional<OP == GAUSS, uint64_t, uint32_t>::type RT;
  RT ring[NZ][SEGY];
  int zsa[OP == MEAN ? SEGY : 1], zsb[OP == MEAN ? SEGY : 1];
#pragma unroll
  for (int j = 0; j < (OP == MEAN ? SEGY : 1); ++j) zsa[j] = zsb[j] = 0;
  const int gx = x0 + 2 * c;
  // X rows this thread reads: rb + k, rb = SEGY*g even; byte offset of row
  // rb's word c (row-pair layouts: even / odd regions)
  const uint32_t yrd = G::PAIRS ? (uint32_t)((SEGY * g / 2) * G::XP + 2 * c) * G::XEL
                                : (uint32_t)((SEGY * g) * G::XP + 2 * c) * G::XEL;
  auto xrow = [&](int k) -> uint32_t {  // byte offset of row rb + k relative to row rb (compile-time)
    if constexpr (G::PAIRS) return ((k & 1) * G::XHALF + (k >> 1) * G::XP) * G::XEL;
    else return k * G::XP * G::XEL;
  };
  // rows of this thread's outputs inside the image: bit j
  uint32_t rowok = 0;
#pragma unroll
  for (int j = 0; j < SEGY; ++j)
    if (gx < W && y0 + SEGY * g + j < H) rowok |= 1u << j;
  typedef typename std::conditional<OP == GAUSS, float, uint16_t>::type DT;
  DT* outp = reinterpret_cast<DT*>(dstv) + (size_t)z0 * plane + (size_t)(y0 + SEGY * g) * W + gx;

  RT y[SEGY];  // Y results of the current plane
  auto ypass = [&](uint32_t xso) {
    const unsigned char* b = smem + xso + yrd;
    if constexpr (OP == MIN || OP == MAX) {
      uint32_t win[SEGY + 2 * R];
#pragma unroll
      for (int k = 0; k < SEGY + 2 * R; ++k) win[k] = *reinterpret_cast<const uint32_t*>(b + xrow(k));
      slide_minmax<SG, OP, SEGY, R>(win, y);
    } else if constexpr (OP == MEAN) {
      int a[SEGY + 2 * R], bb[SEGY + 2 * R];
#pragma unroll
      for (int k = 0; k < SEGY + 2 * R; ++k) {
        const uint32_t w = *reinterpret_cast<const uint32_t*>(b + xrow(k));
        a[k] = lane_lo<SG>(w), bb[k] = lane_hi<SG>(w);
      }
      int sa = 0, sb = 0;
#pragma unroll
      for (int k = 0; k <= 2 * R; ++k) sa += a[k], sb += bb[k];
#pragma unroll
      for (int j = 0; j < SEGY; ++j) {
        if (j > 0) sa += a[j + 2 * R] - a[j - 1], sb += bb[j + 2 * R] - bb[j - 1];
        const int qa = div_exact<SG>(sa, p.mx), qb = div_exact<SG>(sb, p.mx);
        y[j] = __byte_perm((uint32_t)qa, (uint32_t)qb, 0x5410);
        zsa[j] += qa, zsb[j] += qb;
      }
    } else {
      uint64_t acc[SEGY];
#pragma unroll
      for (int j = 0; j < SEGY; ++j) acc[j] = 0;
#pragma unroll
      for (int k = 0; k < SEGY + 2 * R; ++k) {
        const uint64_t e = *reinterpret_cast<const uint64_t*>(b + xrow(k));
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const int t = k - j - R;
          if (t >= -R && t <= R) acc[j] = f2_fma(p.wy[t < 0 ? -t : t], e, acc[j]);
        }
      }
#pragma unroll
      for (int j = 0; j < SEGY; ++j) y[j] = acc[j];
    }
  };
  // the Y results of plane q enter ring slot SL; once the ring holds a
  // whole window, reduce it and store the plane CZ behind
  auto zstep = [&](int q, auto slot_c) {
    constexpr int SL = decltype(slot_c)::value;
#pragma unroll
    for (int j = 0; j < SEGY; ++j) ring[SL][j] = y[j];
    if (q < 2 * CZ) return;  // the ring does not hold a whole window yet
    if constexpr (OP == MIN || OP == MAX) {
#pragma unroll
      for (int j = 0; j < SEGY; ++j) {
        uint32_t m = ring[0][j];
#pragma unroll
        for (int s = 1; s < NZ; ++s) m = mm<SG, OP>(m, ring[s][j]);
        if (rowok >> j & 1) *reinterpret_cast<uint32_t*>(outp + (size_t)j * W) = m;
      }
    } else if constexpr (OP == MEAN) {
      constexpr int OLD = (SL + 1) % NZ;  // plane q - 2CZ
#pragma unroll
      for (int j = 0; j < SEGY; ++j) {
        const int qa = div_exact<SG>(zsa[j], p.mz), qb = div_exact<SG>(zsb[j], p.mz);
        if (rowok >> j & 1)
          *reinterpret_cast<uint32_t*>(outp + (size_t)j * W) = __byte_perm((uint32_t)qa, (uint32_t)qb, 0x5410);
        zsa[j] -= lane_lo<SG>(ring[OLD][j]), zsb[j] -= lane_hi<SG>(ring[OLD][j]);
      }
    } else {
      constexpr int CEN = (SL + NZ - CZ) % NZ;  // plane q - CZ
#pragma unroll
      for (int j = 0; j < SEGY; ++j) {
        uint64_t acc = f2_fma(p.wz[0], ring[CEN][j], 0ull);
#pragma unroll
        for (int k = 1; k <= CZ; ++k)
          acc = f2_fma(p.wz[k], f2_add(ring[(CEN + NZ - k) % NZ][j], ring[(CEN + k) % NZ][j]), acc);
        if (rowok >> j & 1) *reinterpret_cast<uint64_t*>(outp + (size_t)j * W) = acc;
      }
    }
    outp += plane;
  };

  // ---- the plane loop: phase it X-filters plane it and Y/Z-filters plane
  // it-1 while the copy of a later plane is in flight; one barrier per phase
  // (x-border tiles: two, the second after filling the outside vectors).
  // Min / max / mean: three raw buffers, plane it+2 copied during phase it.
  // Gaussian: two raw buffers, plane it+1 converted during phase it.
  const int NPL = (z1 - z0) + 2 * CZ;  // planes z0-CZ .. z1+CZ-1
  if constexpr (OP == GAUSS) {
    issue_raw(z0 - CZ, RAW0);
    if (NPL > 1) issue_raw(z0 - CZ + 1, RAW0 + G::RAW_BYTES);
    cp_async_wait_all();
    __syncthreads();
    convert(RAW0, CV0);
    __syncthreads();
  } else {
    issue_raw(z0 - CZ, RAW0);
    issue_raw(z0 - CZ + 1, RAW0 + G::RAW_BYTES);
    cp_async_wait_1();
    __syncthreads();
    if (xborder) {
      fixup(RAW0);
      __syncthreads();
    }
  }
  int slot = 0;  // ring slot of the next Y plane
  int rcur = 0;  // raw buffer of plane it (min / max / mean: it % 3)
  for (int it = 0; it <= NPL; ++it) {
    const uint32_t cur = it & 1, nxt = cur ^ 1;
    if constexpr (OP == GAUSS) {
      if (it + 1 < NPL) {
        // raw(it), in buffer cur, was converted in phase it-1
        if (it + 2 < NPL) issue_raw(z0 - CZ + it + 2, RAW0 + cur * G::RAW_BYTES);
        convert(RAW0 + nxt * G::RAW_BYTES, CV0 + nxt * G::CV_BYTES);
      }
      if (it < NPL) xpass(0, CV0 + cur * G::CV_BYTES, XS0 + cur * G::XS_BYTES);
    } else {
      // buffer (it+2) % 3 held plane it-1, whose X pass ended in phase it-1
      const int r2 = rcur == 0 ? 2 : rcur - 1;
      if (it + 2 < NPL) issue_raw(z0 - CZ + it + 2, RAW0 + r2 * G::RAW_BYTES);
      else cp_async_commit();  // an empty group keeps the group count per phase at one
      if (it < NPL) xpass(RAW0 + rcur * G::RAW_BYTES, 0, XS0 + cur * G::XS_BYTES);
    }
    if (it >= 1) {
      if (yvalid) {
        ypass(XS0 + nxt * G::XS_BYTES);
        // one copy of the ring step per slot, so that every slot is a fixed register
        dispatch<0, NZ>(slot, [&](auto kc) { zstep(it - 1, kc); });
      }
      slot = slot + 1 == NZ ? 0 : slot + 1;
    }
    if constexpr (OP == GAUSS) {
      cp_async_wait_all();
      __syncthreads();
    } else {
      cp_async_wait_1();  // plane it+1 has landed (plane it+2 may still be in flight)
      __syncthreads();
      const int r1 = rcur == 2 ? 0 : rcur + 1;
      if (xborder && it + 1 < NPL) {
        fixup(RAW0 + r1 * G::RAW_BYTES);
        __syncthreads();
      }
      rcur = r1;
    }
  }
}

template <class K> bool smem_ok(K kern, size_t smem) {
  if (smem > 220 * 1024) return false;
  if (smem <= 48 * 1024) return true;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

// z-chunks: CLK_SEP3_CHUNKS in the environment fixes the count (tuning).
// Otherwise about seven waves of CTAs (ctas_per_sm resident per SM), each
// chunk long enough that its 2CZ halo planes stay a small overhead: at least
// max(16, 24 CZ) planes while the tiles alone fill the SMs (measured on 1024
// x 1024 x 256: minimum r5 0.47 ms with one chunk per tile, 0.29 with four
// to eight; the Gaussian cz = 5 best with two chunks, 1.12 ms against 1.17
// with three).  Small images take the count whose CTAs fill the resident
// slots in whole waves (wave_chunks; 256x256x64 Gaussian s(2,2,1): eight
// chunks, 0.027 ms against 0.035 with five).
inline int chunk_count(int tiles, int depth, int cz, int ctas_per_sm) {
  static const int forced = [] {
    const char* e = getenv("CLK_SEP3_CHUNKS");
    return e && *e ? atoi(e) : 0;
  }();
  if (forced > 0) return std::min(forced, std::max(1, depth));
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (tiles < sms)  // small images: the count that fills the resident slots in whole waves
    return wave_chunks(tiles, depth, 2 * cz, (int64_t)sms * ctas_per_sm, 1, std::max(1, depth / 4));
  const int64_t want = (int64_t)7 * sms * ctas_per_sm;
  int chunks = (int)std::max<int64_t>(1, (want + tiles / 2) / std::max(1, tiles));
  const int minlen = std::max(16, 24 * cz);
  chunks = std::min(chunks, std::max(1, depth / minlen));
  return chunks;
}

// the launch shape of each operation
template <int OP, int CZ> struct DefaultCfg {
  // measured on 1024 x 1024 x 256 u16 (r5, cz 2): min / max 0.290 ms with
  // 8 outputs per X task (van Herk pieces of 8), 0.318 with 16; the mean
  // needs 16 (one X task per thread)
  typedef Cfg<256, 4, OP == MEAN ? 16 : 8, OP == GAUSS ? 2 : CZ >= 3 ? 3 : 4> type;
};

template <class S, int OP, int R, int CZ, class C = typename DefaultCfg<OP, CZ>::type>
clk_status launch(const Image& dst, const Image& src, const P3& p, cudaStream_t st, int chunks = 0) {
  using G = Geo<OP, R, CZ, C>;
  auto kern = k_sep3<S, OP, R, CZ, C>;
  if (!smem_ok(kern, G::SMEM)) return CLK_UNSUPPORTED_DTYPE;
  const int tx = (dst.w + TX - 1) / TX, ty = (dst.h + C::TY - 1) / C::TY;
  if (chunks <= 0) chunks = chunk_count(tx * ty, dst.d, CZ, C::MINB);
  const int zchunk = (dst.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (dst.d + zchunk - 1) / zchunk);
  kern<<<grid, C::NT, G::SMEM, st>>>((const S*)src.ptr, dst.ptr, dst.w, dst.h, dst.d, zchunk, p);
  count_launch();
  return check_launch("separable (fused, sep3)");
}

template <class S, int OP, int R, int CZMAX>
clk_status by_cz(int cz, const Image& dst, const Image& src, const P3& p, cudaStream_t st) {
  if constexpr (CZMAX >= 0) {
    if (cz == CZMAX) return launch<S, OP, R, CZMAX>(dst, src, p, st);
    return by_cz<S, OP, R, CZMAX - 1>(cz, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

// The layouts these kernels assume: 16-bit pixels, x extents a multiple of 8
// (every staged vector wholly inside or outside its row), 16-byte aligned
// bases, equal extents, a plane of fewer than 2^32 pixels.
inline bool layout_ok(const Image& dst, const Image& src) {
  return src.w == dst.w && src.h == dst.h && src.d == dst.d && src.w % 8 == 0 &&
         (uintptr_t)src.ptr % 16 == 0 && (uintptr_t)dst.ptr % 16 == 0 && (int64_t)src.w * src.h < (1LL << 32);
}

}  // namespace
}  // namespace sep3
}  // namespace clk
