// clk_sep2_impl.cuh - the kernel template behind clk_sep2.cuh (see there for
// the layout); included by the three .cu files that instantiate it per
// operation so that they compile in parallel.
#pragma once
#include <algorithm>
#include <cstdlib>
#include <type_traits>

#include "clk_sep2.cuh"
#include "clk_tma.cuh"

namespace clk {
namespace sep2 {
namespace {

// GAUSSX: the Gaussian to 8/16-bit pixels in the reference's arithmetic
// (taps in order, separately rounded, IEEE division, dst-typed temporaries)
// MINF / MAXF: minimum / maximum of float pixels in the reference's order
// (start at the centre, then res = min(res, x) for v = -c..c with OpenCL's
// min: x < res ? x : res), so NaNs and signed zeros come out as they do there
enum Op { MIN = 0, MAX = 1, MEAN = 2, GAUSS = 3, GAUSSX = 4, MINF = 5, MAXF = 6 };

// temporaries: 16-bit lanes for integer pixels, float for the Gaussian
template <class S, int OP> struct Temp;
template <class S> struct Temp<S, MIN> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, MAX> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, MEAN> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, GAUSS> { typedef float T; };
template <class S> struct Temp<S, GAUSSX> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, MINF> { typedef float T; };
template <class S> struct Temp<S, MAXF> { typedef float T; };

// one step of the reference's float min / max loop
template <int OP> __device__ __forceinline__ float seq_step(float res, float x) {
  if constexpr (OP == MINF) return x < res ? x : res;
  else return res < x ? x : res;
}
// the reference's loop over a window w[0..2R] (centre w[R]) for one output
template <int OP, int R> __device__ __forceinline__ float seq_window(const float* w) {
  float res = w[R];
#pragma unroll
  for (int v = 0; v <= 2 * R; ++v) res = seq_step<OP>(res, w[v]);
  return res;
}
// "the earlier operand unless the later one is strictly more extreme or the
// earlier one is NaN": associative (the leftmost extreme, NaN never chosen)
template <int OP> __device__ __forceinline__ float first_op(float a, float b) {
  const bool take = (OP == MINF ? b < a : a < b) || a != a;
  return take ? b : a;
}
// The reference's loop for M consecutive outputs over w[0 .. M+2R-1]: the
// leftmost extreme of each window by the van Herk / Gil-Werman split
// (2R + 2M - 2 operations), then the centre first unless it is NaN -- equal
// to seq_window bit for bit (NaNs and signed zeros included).
template <int OP, int M, int R> __device__ __forceinline__ void window_first(const float* w, float (&out)[M]) {
  if constexpr (2 * R >= M && M > 1) {
    float suf[M];
    suf[M - 1] = w[M - 1];
#pragma unroll
    for (int j = M - 2; j >= 0; --j) suf[j] = first_op<OP>(w[j], suf[j + 1]);
    float pre = w[M];
#pragma unroll
    for (int k = M + 1; k <= 2 * R; ++k) pre = first_op<OP>(pre, w[k]);
    out[0] = first_op<OP>(suf[0], pre);
#pragma unroll
    for (int j = 1; j < M; ++j) {
      pre = first_op<OP>(pre, w[j + 2 * R]);
      out[j] = first_op<OP>(suf[j], pre);
    }
#pragma unroll
    for (int j = 0; j < M; ++j) {
      const float c = w[j + R];
      out[j] = c != c ? c : first_op<OP>(c, out[j]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < M; ++j) out[j] = seq_window<OP, R>(w + j);
  }
}

template <class S, int OP> __device__ __forceinline__ uint32_t mm(uint32_t a, uint32_t b) {
  if constexpr (Is16<S>::sgn) return OP == MIN ? s16x2_min(a, b) : s16x2_max(a, b);
  else return OP == MIN ? u16x2_min(a, b) : u16x2_max(a, b);
}

// pixel -> float without the I2F unit: 2^23 + v as float bits, minus 2^23
template <class S> __device__ __forceinline__ float tofloat(S v) {
  if constexpr (sizeof(S) == 4) {
    return v;
  } else {
    constexpr int bias = Is16<S>::sgn ? 32768 : 0;
    return __int_as_float(0x4B000000 | (uint32_t)((int)v + bias)) - (8388608.0f + (float)bias);
  }
}

// How the halo tile reaches shared memory.
enum Stage {
  STAGE_SCALAR = 0,  // one clamped pixel load per element (any layout)
  STAGE_VEC = 1,     // 8/16-byte vector loads (rows and image base aligned)
  STAGE_TMA = 2      // cp.async.bulk.tensor boxes, double-buffered
};

// Geometry of one tile.  The vector and TMA stagings start the staged row
// RA >= R elements left of the tile, RA rounded up so that every staged
// vector (TMA: the box origin) is aligned; the X pass then reads from column
// RA - R.
template <class S, int OP, int R, int MODE = STAGE_SCALAR, bool PIPE = false> struct Geo {
  typedef typename Temp<S, OP>::T T;
  static constexpr int ES = (int)sizeof(S);
  static constexpr int rnd(int v, int m) { return (v + m - 1) / m * m; }
  // staging vector bytes: 16 unless 8-byte vectors need a narrower margin
  static constexpr int SV = MODE == STAGE_TMA ? 16
                            : MODE == STAGE_VEC ? (rnd(R, 16 / ES) == rnd(R, 8 / ES) ? 16 : 8)
                                                : ES;
  static constexpr int RA = MODE == STAGE_SCALAR ? R : rnd(R, SV / ES);
  static constexpr int RW = TX + 2 * RA, RH = TY + 2 * R;
  static constexpr int NEL = RW * RH;
  static constexpr int PER = (NEL + NT - 1) / NT;
  static constexpr int VE = SV / ES;          // pixels per staging vector
  static constexpr int SR = RW / VE;          // staging vectors per row
  static constexpr int NSLOT = RH * SR;
  static constexpr int PERV = (NSLOT + NT - 1) / NT;
  static constexpr int NBUF = (MODE == STAGE_TMA || PIPE) ? 2 : 1;  // staged tiles
  static constexpr int NXS = PIPE ? 2 : 1;                            // X-pass result buffers
  static constexpr int WIN_X = SEGX + 2 * R;
  static constexpr int WIN_Y = SEGY + 2 * R;
  static constexpr int XOFF = RA - R;         // first staged column the X pass reads
  // X pass of the aligned stagings: 16- (8-bit pixels: 8-) byte smem reads
  // of the words covering columns [XOFF, XOFF + WIN_X) of a segment
  static constexpr int XV = (SEGX * ES) % 16 == 0 ? 16 : 8;
  static constexpr int NWD = rnd((XOFF + WIN_X) * ES, XV) / 4;
  static constexpr size_t buf_bytes() { return ((size_t)NEL * sizeof(S) + 127) & ~size_t(127); }
  static constexpr size_t tin_bytes() { return NBUF * buf_bytes(); }
  // X-pass results, row pitch XP: padded so that the X pass's stores (a warp
  // = 4 row pairs x 8 segments) spread over the banks
  static constexpr int XP = TX + (sizeof(T) == 2 ? 2 : 4);
  static constexpr size_t xs_bytes() { return ((size_t)RH * XP * sizeof(T) + 15) & ~size_t(15); }
  static __host__ __device__ size_t ring_bytes(int cz) { return (size_t)(2 * cz + 1) * TY * TX * sizeof(T); }
  static size_t smem(int cz) { return tin_bytes() + NXS * xs_bytes() + ring_bytes(cz); }
};

// ---------------------------------------------------------------- words
// Element e of a staged row held in 32-bit words w (x fastest), for the
// aligned stagings.  e is a compile-time constant after unrolling, so each
// is a byte permute or a shift pair (plus an AND / XOR / float add).
template <class S, int N> __device__ __forceinline__ uint32_t lanes16_of(const uint32_t (&w0)[N],
                                                                       const uint32_t (&w1)[N], int e) {
  // 16-bit lanes (row 0 low, row 1 high), as lane16 would widen them
  if constexpr (sizeof(S) == 2) {
    return __byte_perm(w0[e >> 1], w1[e >> 1], (e & 1) ? 0x7632 : 0x5410);
  } else {
    const uint32_t b = e & 3;
    if constexpr (Is16<S>::sgn) {  // sign-extended bytes (shifts: __byte_perm has no sign mode)
      const uint32_t lo = (uint32_t)((int)(w0[e >> 2] << (24 - 8 * b)) >> 24) & 0xFFFFu;
      const uint32_t hi = (uint32_t)((int)(w1[e >> 2] << (24 - 8 * b)) >> 24) << 16;
      return lo | hi;
    } else {
      return __byte_perm(w0[e >> 2], w1[e >> 2], b | ((4 + b) << 8)) & 0x00FF00FFu;
    }
  }
}
template <class S, int N> __device__ __forceinline__ int int_of(const uint32_t (&w)[N], int e) {
  if constexpr (sizeof(S) == 2) {
    if constexpr (Is16<S>::sgn) return (e & 1) ? (int)w[e >> 1] >> 16 : (int)(w[e >> 1] << 16) >> 16;
    else return (int)((e & 1) ? w[e >> 1] >> 16 : w[e >> 1] & 0xFFFFu);
  } else {
    const uint32_t b = e & 3;
    if constexpr (Is16<S>::sgn) return (int)(w[e >> 2] << (24 - 8 * b)) >> 24;
    else return (int)__byte_perm(w[e >> 2], 0, b | 0x4440u);
  }
}
// (row 0, row 1) values of element e as an f32x2 pair: float pixels as they
// are; 8/16-bit pixels as the float 2^23 + v (+ bias for signed) built by a
// byte permute, minus the same constant (exact)
template <class S, int N> __device__ __forceinline__ uint64_t f2_of(const uint32_t (&w0)[N], const uint32_t (&w1)[N],
                                                                  int e) {
  if constexpr (sizeof(S) == 4) {
    return f2_pack(__uint_as_float(w0[e]), __uint_as_float(w1[e]));
  } else {
    constexpr uint32_t K = 0x4B000000u;  // bytes 4..7 of the permute: 00 00 00 4B
    uint32_t a, b;
    if constexpr (sizeof(S) == 2) {
      const uint32_t h = 2 * (e & 1), sel = h | ((h + 1) << 4) | 0x7400u;
      a = __byte_perm(w0[e >> 1], K, sel);
      b = __byte_perm(w1[e >> 1], K, sel);
    } else {
      const uint32_t sel = (e & 3) | 0x7440u;
      a = __byte_perm(w0[e >> 2], K, sel);
      b = __byte_perm(w1[e >> 2], K, sel);
    }
    constexpr uint32_t flip = Is16<S>::sgn ? (sizeof(S) == 2 ? 0x8000u : 0x80u) : 0u;
    constexpr float off = 8388608.0f + (Is16<S>::sgn ? (sizeof(S) == 2 ? 32768.0f : 128.0f) : 0.0f);
    if constexpr (flip != 0) a ^= flip, b ^= flip;
    return f2_add(f2_pack(__uint_as_float(a), __uint_as_float(b)), f2_bcast(-off));
  }
}

// a 32-bit word of a pixel value repeated (clamp-to-edge fill of a vector)
template <class S> __device__ __forceinline__ uint32_t splat_word(S v) {
  if constexpr (sizeof(S) == 4) return __float_as_uint(v);
  else if constexpr (sizeof(S) == 2) return (uint32_t)(uint16_t)v * 0x10001u;
  else return (uint32_t)(uint8_t)v * 0x01010101u;
}

// Running min/max of M consecutive windows of 2R+1 packed lanes:
// out[j] = op(win[j .. j+2R]).  When every window contains the split point
// M (2R >= M), out[j] = op(suffix of win[j .. M-1], prefix of win[M .. j+2R])
// (the van Herk / Gil-Werman decomposition): 2R + 2M - 2 operations instead
// of 2R * M.  Exact for min/max, so the result is the same either way.
template <class S, int OP, int M, int R>
__device__ __forceinline__ void window_minmax(const uint32_t (&win)[M + 2 * R], uint32_t (&out)[M]) {
  if constexpr (2 * R >= M && M > 1) {
    uint32_t suf[M];
    suf[M - 1] = win[M - 1];
#pragma unroll
    for (int j = M - 2; j >= 0; --j) suf[j] = mm<S, OP>(win[j], suf[j + 1]);
    uint32_t pre = win[M];
#pragma unroll
    for (int k = M + 1; k <= 2 * R; ++k) pre = mm<S, OP>(pre, win[k]);
    out[0] = mm<S, OP>(suf[0], pre);  // window 0 ends at 2R
#pragma unroll
    for (int j = 1; j < M; ++j) {
      pre = mm<S, OP>(pre, win[j + 2 * R]);
      out[j] = mm<S, OP>(suf[j], pre);
    }
  } else {
#pragma unroll
    for (int j = 0; j < M; ++j) {
      uint32_t a = win[j];
#pragma unroll
      for (int k = 1; k <= 2 * R; ++k) a = mm<S, OP>(a, win[j + k]);
      out[j] = a;
    }
  }
}

// The z ring is private to each thread: for the mean and the Gaussians its
// SEGY (= 4) row results of a plane are contiguous, so a plane's cells move
// as one 16-byte access (two for float, in two halves of the ring plane so
// that a warp's accesses stay contiguous).  4 x 32-bit words of 16-bit
// lanes, or 4 x f32x2.
static_assert(SEGY == 4, "the ring cell layout holds four rows");
template <class T> __device__ __forceinline__ void ring_put(T* slot, int tid, const uint32_t (&w)[4]) {
  reinterpret_cast<uint4*>(slot)[tid] = make_uint4(w[0], w[1], w[2], w[3]);
}
template <class T> __device__ __forceinline__ void ring_get(const T* slot, int tid, uint32_t (&w)[4]) {
  const uint4 v = reinterpret_cast<const uint4*>(slot)[tid];
  w[0] = v.x, w[1] = v.y, w[2] = v.z, w[3] = v.w;
}
__device__ __forceinline__ void ring_put2(float* slot, int tid, const uint64_t (&w)[4]) {
  reinterpret_cast<ulonglong2*>(slot)[tid] = make_ulonglong2(w[0], w[1]);
  reinterpret_cast<ulonglong2*>(slot)[NT + tid] = make_ulonglong2(w[2], w[3]);
}
__device__ __forceinline__ void ring_get2(const float* slot, int tid, uint64_t (&w)[4]) {
  const ulonglong2 a = reinterpret_cast<const ulonglong2*>(slot)[tid];
  const ulonglong2 b = reinterpret_cast<const ulonglong2*>(slot)[NT + tid];
  w[0] = a.x, w[1] = a.y, w[2] = b.x, w[3] = b.y;
}

// One tile (bx, by) x z-chunk bz of one image; the whole CTA takes part.
// smem: dynamic shared memory of at least Geo::smem(p.cz) bytes (128-byte
// aligned).  TMA: map is a 3-D tensor map of src with a (RW, RH, 1) box;
// err receives 1 if a bounded wait for a tile ran out (the tile is then
// abandoned).
template <class S, class D, int OP, int R, int MODE = STAGE_SCALAR, bool PIPE = false>
__device__ __forceinline__ void sep2_tile(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                          int zchunk, const Params& p, int bx, int by, int bz,
                                          unsigned char* smem, const CUtensorMap* map = nullptr,
                                          int* err = nullptr) {
  using G = Geo<S, OP, R, MODE, PIPE>;
  using T = typename G::T;
  constexpr bool TMA = MODE == STAGE_TMA;
  static_assert(!(TMA && PIPE), "the pipelined loop stages from registers");
  S* tin = reinterpret_cast<S*>(smem);
  T* xs = reinterpret_cast<T*>(smem + G::tin_bytes());
  T* ring = reinterpret_cast<T*>(smem + G::tin_bytes() + G::NXS * G::xs_bytes());
  auto tinb = [&](int b) { return reinterpret_cast<S*>(smem + b * G::buf_bytes()); };
  auto xsb = [&](int b) { return reinterpret_cast<T*>(smem + G::tin_bytes() + b * G::xs_bytes()); };
  const int cz = p.cz, NZ = 2 * cz + 1;
  const int tid = threadIdx.x;
  const int x0 = bx * TX, y0 = by * TY;
  const int z0 = bz * zchunk, z1 = min(Dz, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  constexpr int XOFF = G::XOFF;

  // register prefetch of the next plane's halo tile (scalar / vector staging)
  typedef typename std::conditional<G::SV == 16, uint4, uint2>::type VT;
  S pre[MODE == STAGE_SCALAR ? G::PER : 1];
  VT prev[MODE == STAGE_VEC ? G::PERV : 1];
  // vector staging: the in-plane offset of each of this thread's staged
  // vectors -- or, for a vector wholly outside the row, of the row's edge
  // pixel (bit k of vsplat) -- is the same for every plane: computed once
  // (the host keeps W * H below 2^32 for this path)
  uint32_t voff[MODE == STAGE_VEC ? G::PERV : 1];
  uint32_t vsplat = 0;
  if constexpr (MODE == STAGE_VEC) {
#pragma unroll
    for (int k = 0; k < G::PERV; ++k) {
      const int sl = tid + k * NT;
      voff[k] = 0;
      if (k < G::PERV - 1 || sl < G::NSLOT) {
        const int r = sl / G::SR, v = sl - r * G::SR;
        const uint32_t row = (uint32_t)clampi(y0 - R + r, H - 1) * (uint32_t)W;
        const int gx = x0 - G::RA + v * G::VE;
        if (gx >= 0 && gx < W) {
          voff[k] = row + (uint32_t)gx;
        } else {
          voff[k] = row + (uint32_t)(gx < 0 ? 0 : W - 1);
          vsplat |= 1u << k;
        }
      }
    }
  }
  auto fetch = [&](int zv) {
    const S* sp = src + (int64_t)clampi(zv, Dz - 1) * plane;
    if constexpr (MODE == STAGE_SCALAR) {
#pragma unroll
      for (int k = 0; k < G::PER; ++k) {
        const int i = tid + k * NT;
        if (i < G::NEL) {
          const int r = i / G::RW, q = i - r * G::RW;
          pre[k] = __ldg(sp + (int64_t)clampi(y0 - R + r, H - 1) * W + clampi(x0 - R + q, W - 1));
        }
      }
    } else if constexpr (MODE == STAGE_VEC) {
      // a vector lies wholly inside the row or wholly outside it (rows and
      // the staged origin are vector-aligned): load it, or fill it with the
      // clamped edge pixel
#pragma unroll
      for (int k = 0; k < G::PERV; ++k) {
        const int sl = tid + k * NT;
        if (k < G::PERV - 1 || sl < G::NSLOT) {
          if (!(vsplat & (1u << k))) {
            prev[k] = __ldg(reinterpret_cast<const VT*>(sp + voff[k]));
          } else {
            const uint32_t w = splat_word<S>(__ldg(sp + voff[k]));
            if constexpr (G::SV == 16) prev[k] = make_uint4(w, w, w, w);
            else prev[k] = make_uint2(w, w);
          }
        }
      }
    }
  };
  auto commit = [&](S* to) {
    if constexpr (MODE == STAGE_SCALAR) {
#pragma unroll
      for (int k = 0; k < G::PER; ++k) {
        const int i = tid + k * NT;
        if (i < G::NEL) to[i] = pre[k];
      }
    } else if constexpr (MODE == STAGE_VEC) {
#pragma unroll
      for (int k = 0; k < G::PERV; ++k) {
        const int sl = tid + k * NT;
        if (k < G::PERV - 1 || sl < G::NSLOT) reinterpret_cast<VT*>(to)[sl] = prev[k];
      }
    }
  };

  // TMA: two staging buffers, one mbarrier each; thread 0 issues the loads.
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int stalled;
  constexpr uint32_t kBoxBytes = (uint32_t)(G::NEL * sizeof(S));
  auto issue = [&](int zv, int buf) {
    tma::mbar_expect_tx(&bars[buf], kBoxBytes);
    tma::load_3d(reinterpret_cast<unsigned char*>(tin) + buf * G::buf_bytes(), map, &bars[buf], x0 - G::RA,
                 y0 - R, clampi(zv, Dz - 1));
  };
  // clamp-to-edge for a staged tile that reaches past the image: TMA filled
  // those cells with 0; copy the border column / row into them
  const bool border = x0 - G::RA < 0 || x0 + TX + G::RA > W || y0 - R < 0 || y0 + TY + R > H;
  auto fix_border = [&](S* t) {
    const int qlo = max(0, G::RA - x0), qhi = min(G::RW - 1, W - 1 - (x0 - G::RA));
    for (int i = tid; i < G::NEL; i += NT) {
      const int r = i / G::RW, q = i - r * G::RW;
      if (q < qlo) t[i] = t[r * G::RW + qlo];
      else if (q > qhi) t[i] = t[r * G::RW + qhi];
    }
    __syncthreads();
    const int rlo = max(0, R - y0), rhi = min(G::RH - 1, H - 1 - (y0 - R));
    for (int i = tid; i < G::NEL; i += NT) {
      const int r = i / G::RW, q = i - r * G::RW;
      if (r < rlo) t[i] = t[rlo * G::RW + q];
      else if (r > rhi) t[i] = t[rhi * G::RW + q];
    }
  };
  if constexpr (TMA) {
    if (tid == 0) {
      tma::mbar_init(&bars[0], 1);
      tma::mbar_init(&bars[1], 1);
      tma::fence_barrier_init();
      issue(z0 - cz, 0);
      if (z0 - cz + 1 < z1 + cz) issue(z0 - cz + 1, 1);
    }
  } else {
    fetch(z0 - cz);
  }

  // Y/Z ownership: column pair cp, rows sy*SEGY .. +SEGY-1
  const int cp = tid % (TX / 2), sy = tid / (TX / 2);
  int wslot = 0;
  int zs0[SEGY], zs1[SEGY];  // mean: running sums along z of this thread's cells
#pragma unroll
  for (int j = 0; j < SEGY; ++j) zs0[j] = zs1[j] = 0;
  // X pass of the staged tile tcur into the X-result buffer xs
  auto xpass = [&](const S* tcur, T* xs) {
    // ---------------- X pass: rows (rp, rp + RH/2) x outputs sg*SEGX ..
    {
      const int rp = tid / (TX / SEGX), sg = tid % (TX / SEGX);
      constexpr int HALF = G::RH / 2;
      if (rp < HALF) {
        const S* r0 = tcur + rp * G::RW + sg * SEGX + XOFF;
        const S* r1 = r0 + HALF * G::RW;
        T* o0 = xs + rp * G::XP + sg * SEGX;
        T* o1 = o0 + HALF * G::XP;
        // aligned stagings: the segment's words of both rows, read as vectors
        uint32_t w0[MODE == STAGE_SCALAR ? 1 : G::NWD], w1[MODE == STAGE_SCALAR ? 1 : G::NWD];
        if constexpr (MODE != STAGE_SCALAR) {
          const S* a0 = tcur + rp * G::RW + sg * SEGX;
          if constexpr (G::XV == 16) {
#pragma unroll
            for (int v = 0; v < G::NWD / 4; ++v) {
              const uint4 x = reinterpret_cast<const uint4*>(a0)[v];
              const uint4 y = reinterpret_cast<const uint4*>(a0 + HALF * G::RW)[v];
              w0[4 * v] = x.x, w0[4 * v + 1] = x.y, w0[4 * v + 2] = x.z, w0[4 * v + 3] = x.w;
              w1[4 * v] = y.x, w1[4 * v + 1] = y.y, w1[4 * v + 2] = y.z, w1[4 * v + 3] = y.w;
            }
          } else {
#pragma unroll
            for (int v = 0; v < G::NWD / 2; ++v) {
              const uint2 x = reinterpret_cast<const uint2*>(a0)[v];
              const uint2 y = reinterpret_cast<const uint2*>(a0 + HALF * G::RW)[v];
              w0[2 * v] = x.x, w0[2 * v + 1] = x.y;
              w1[2 * v] = y.x, w1[2 * v + 1] = y.y;
            }
          }
        }
        if constexpr (OP == MIN || OP == MAX) {
          uint32_t win[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) {
            if constexpr (MODE == STAGE_SCALAR) win[k] = lane16(r0[k]) | (lane16(r1[k]) << 16);
            else win[k] = lanes16_of<S>(w0, w1, XOFF + k);
          }
          uint32_t out[SEGX];
          window_minmax<S, OP, SEGX, R>(win, out);
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            *reinterpret_cast<uint32_t*>(o0 + j) = __byte_perm(out[j], out[j + 1], 0x5410);
            *reinterpret_cast<uint32_t*>(o1 + j) = __byte_perm(out[j], out[j + 1], 0x7632);
          }
        } else if constexpr (OP == MINF || OP == MAXF) {
          float v0[G::WIN_X], v1[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) {
            if constexpr (MODE == STAGE_SCALAR) v0[k] = r0[k], v1[k] = r1[k];
            else v0[k] = __uint_as_float(w0[XOFF + k]), v1[k] = __uint_as_float(w1[XOFF + k]);
          }
          float q0[SEGX], q1[SEGX];
          window_first<OP, SEGX, R>(v0, q0);
          window_first<OP, SEGX, R>(v1, q1);
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            *reinterpret_cast<float2*>(o0 + j) = make_float2(q0[j], q0[j + 1]);
            *reinterpret_cast<float2*>(o1 + j) = make_float2(q1[j], q1[j + 1]);
          }
        } else if constexpr (OP == MEAN) {
          int v0[G::WIN_X], v1[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) {
            if constexpr (MODE == STAGE_SCALAR) v0[k] = (int)r0[k], v1[k] = (int)r1[k];
            else v0[k] = int_of<S>(w0, XOFF + k), v1[k] = int_of<S>(w1, XOFF + k);
          }
          int s0 = 0, s1 = 0;
#pragma unroll
          for (int k = 0; k <= 2 * R; ++k) s0 += v0[k], s1 += v1[k];
          int q0[SEGX], q1[SEGX];
#pragma unroll
          for (int j = 0; j < SEGX; ++j) {
            if (j > 0) {
              s0 += v0[j + 2 * R] - v0[j - 1];
              s1 += v1[j + 2 * R] - v1[j - 1];
            }
            q0[j] = div_exact<Is16<S>::sgn>(s0, p.mx);
            q1[j] = div_exact<Is16<S>::sgn>(s1, p.mx);
          }
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            *reinterpret_cast<uint32_t*>(o0 + j) = __byte_perm((uint32_t)q0[j], (uint32_t)q0[j + 1], 0x5410);
            *reinterpret_cast<uint32_t*>(o1 + j) = __byte_perm((uint32_t)q1[j], (uint32_t)q1[j + 1], 0x5410);
          }
        } else if constexpr (OP == GAUSSX) {
          uint64_t win[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) {
            if constexpr (MODE == STAGE_SCALAR) win[k] = f2_pack(tofloat(r0[k]), tofloat(r1[k]));
            else win[k] = f2_of<S>(w0, w1, XOFF + k);
          }
          uint32_t q[SEGX];  // lane 0: row 0, lane 1: row 1
#pragma unroll
          for (int j = 0; j < SEGX; ++j) q[j] = gauss_exact_pair<D, 2 * R + 1>(win + j, p.hx, p.hs[0], p.rte);
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            *reinterpret_cast<uint32_t*>(o0 + j) = __byte_perm(q[j], q[j + 1], 0x5410);
            *reinterpret_cast<uint32_t*>(o1 + j) = __byte_perm(q[j], q[j + 1], 0x7632);
          }
        } else {
          uint64_t win[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) {
            if constexpr (MODE == STAGE_SCALAR) win[k] = f2_pack(tofloat(r0[k]), tofloat(r1[k]));
            else win[k] = f2_of<S>(w0, w1, XOFF + k);
          }
          uint64_t out[SEGX];
#pragma unroll
          for (int j = 0; j < SEGX; ++j) {
            uint64_t acc = f2_fma(f2_bcast(p.wx[0]), win[j + R], 0ull);
#pragma unroll
            for (int k = 1; k <= R; ++k) acc = f2_fma(f2_bcast(p.wx[k]), f2_add(win[j + R - k], win[j + R + k]), acc);
            out[j] = acc;
          }
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            const float2 a = f2_unpack(out[j]), b = f2_unpack(out[j + 1]);
            *reinterpret_cast<float2*>(o0 + j) = make_float2(a.x, b.x);
            *reinterpret_cast<float2*>(o1 + j) = make_float2(a.y, b.y);
          }
        }
      }
    }
  };
  // Y pass of the X results xs of plane zi into the ring, then the Z pass
  // of the output plane zi - cz
  auto yzpass = [&](const T* xs, int zi) {
    // ---------------- Y pass: column pair cp x rows sy*SEGY .. -> ring slot
    T* rs = ring + (size_t)wslot * TY * TX;
    {
      const T* col = xs + (sy * SEGY) * G::XP + 2 * cp;
      if constexpr (OP == MIN || OP == MAX) {
        uint32_t win[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) win[k] = *reinterpret_cast<const uint32_t*>(col + k * G::XP);
        uint32_t out[SEGY];
        window_minmax<S, OP, SEGY, R>(win, out);
        // min / max keep the row-major ring (measured faster for them than
        // the per-thread 16-byte cells: 0.589 against 0.622 ms at r = 5)
        T* o = rs + (sy * SEGY) * TX + 2 * cp;
#pragma unroll
        for (int j = 0; j < SEGY; ++j) *reinterpret_cast<uint32_t*>(o + j * TX) = out[j];
      } else if constexpr (OP == MINF || OP == MAXF) {
        float a[G::WIN_Y], b[G::WIN_Y];  // columns x, x+1
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) {
          const float2 v = *reinterpret_cast<const float2*>(col + k * G::XP);
          a[k] = v.x, b[k] = v.y;
        }
        float qa[SEGY], qb[SEGY];
        window_first<OP, SEGY, R>(a, qa);
        window_first<OP, SEGY, R>(b, qb);
        uint64_t out[SEGY];
#pragma unroll
        for (int j = 0; j < SEGY; ++j) out[j] = f2_pack(qa[j], qb[j]);
        ring_put2(rs, tid, out);
      } else if constexpr (OP == MEAN) {
        int w0[G::WIN_Y], w1[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) {  // one word: columns x (low lane), x+1 (high lane)
          const uint32_t w = *reinterpret_cast<const uint32_t*>(col + k * G::XP);
          if constexpr (Is16<S>::sgn) w0[k] = (int)(w << 16) >> 16, w1[k] = (int)w >> 16;
          else w0[k] = (int)(w & 0xFFFFu), w1[k] = (int)(w >> 16);
        }
        uint32_t out[SEGY];
        int s0 = 0, s1 = 0;
#pragma unroll
        for (int k = 0; k <= 2 * R; ++k) s0 += w0[k], s1 += w1[k];
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          if (j > 0) {
            s0 += w0[j + 2 * R] - w0[j - 1];
            s1 += w1[j + 2 * R] - w1[j - 1];
          }
          const int q0 = div_exact<Is16<S>::sgn>(s0, p.mx), q1 = div_exact<Is16<S>::sgn>(s1, p.mx);
          out[j] = __byte_perm((uint32_t)q0, (uint32_t)q1, 0x5410);
          zs0[j] += q0;  // the new plane enters the running z sums
          zs1[j] += q1;
        }
        ring_put(rs, tid, out);
      } else if constexpr (OP == GAUSSX) {
        uint64_t win[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k)
          win[k] = f2_of_lanes<Is16<S>::sgn>(*reinterpret_cast<const uint32_t*>(col + k * G::XP));
        uint32_t out[SEGY];
#pragma unroll
        for (int j = 0; j < SEGY; ++j) out[j] = gauss_exact_pair<D, 2 * R + 1>(win + j, p.hy, p.hs[1], p.rte);
        ring_put(rs, tid, out);
      } else {
        uint64_t win[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) win[k] = *reinterpret_cast<const uint64_t*>(col + k * G::XP);
        uint64_t out[SEGY];
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          uint64_t acc = f2_fma(f2_bcast(p.wy[0]), win[j + R], 0ull);
#pragma unroll
          for (int k = 1; k <= R; ++k) acc = f2_fma(f2_bcast(p.wy[k]), f2_add(win[j + R - k], win[j + R + k]), acc);
          out[j] = acc;
        }
        ring_put2(rs, tid, out);
      }
    }

    // ---------------- Z pass over this thread's own ring cells
    // (ring slots in the outer loop, the thread's SEGY rows in the inner one)
    const int zo = zi - cz;
    const int oldest = wslot + 1 == NZ ? 0 : wslot + 1;
    wslot = oldest;
    if (zo >= z0) {
      constexpr int PL = TY * TX;  // one ring plane, in T elements
      const int gx = x0 + 2 * cp;
      // even widths keep every row pair-aligned: one store for both lanes;
      // odd widths store the lanes separately (the second may lie past W)
      const bool pair = (W & 1) == 0;
      if constexpr (OP == MINF || OP == MAXF) {
        // the centre plane first, then planes zo-cz .. zo+cz in order
        const int centre = oldest + cz >= NZ ? oldest + cz - NZ : oldest + cz;
        uint64_t c[SEGY];
        ring_get2(ring + (size_t)centre * PL, tid, c);
        float ra[SEGY], rb[SEGY];
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const float2 f = f2_unpack(c[j]);
          ra[j] = f.x, rb[j] = f.y;
        }
        int idx = oldest;
        for (int v = 0; v < NZ; ++v) {
          uint64_t w[SEGY];
          ring_get2(ring + (size_t)idx * PL, tid, w);
#pragma unroll
          for (int j = 0; j < SEGY; ++j) {
            const float2 f = f2_unpack(w[j]);
            ra[j] = seq_step<OP>(ra[j], f.x), rb[j] = seq_step<OP>(rb[j], f.y);
          }
          idx = idx + 1 == NZ ? 0 : idx + 1;
        }
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const int gy = y0 + sy * SEGY + j;
          D* out = dst + (int64_t)zo * plane + (int64_t)gy * W + gx;
          if (gy < H && gx < W) {
            if (pair) {
              *reinterpret_cast<float2*>(out) = make_float2(ra[j], rb[j]);
            } else {
              out[0] = ra[j];
              if (gx + 1 < W) out[1] = rb[j];
            }
          }
        }
      } else if constexpr (OP == GAUSSX) {
        // planes zo-cz .. zo+cz in order, from the oldest ring slot on
        float2 acc[SEGY];
        int idx = oldest;
        for (int v = 0; v < NZ; ++v) {
          uint32_t cw[SEGY];
          ring_get(ring + (size_t)idx * PL, tid, cw);
          const float hv = p.hz[v];
#pragma unroll
          for (int j = 0; j < SEGY; ++j) {
            const float2 x = f2_unpack(f2_of_lanes<Is16<S>::sgn>(cw[j]));
            const float mx = __fmul_rn(hv, x.x), my = __fmul_rn(hv, x.y);
            acc[j] = v == 0 ? make_float2(mx, my) : make_float2(__fadd_rn(acc[j].x, mx), __fadd_rn(acc[j].y, my));
          }
          idx = idx + 1 == NZ ? 0 : idx + 1;
        }
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const float2 f = acc[j];
          const D a = convert_sat<D>(__fdiv_rn(f.x, p.hs[2]), p.rte), b = convert_sat<D>(__fdiv_rn(f.y, p.hs[2]), p.rte);
          const int gy = y0 + sy * SEGY + j;
          D* out = dst + (int64_t)zo * plane + (int64_t)gy * W + gx;
          if (gy < H && gx < W) {
            if (pair) {
              if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = lane16(a) | (lane16(b) << 16);
              else *reinterpret_cast<uint16_t*>(out) = (uint16_t)((uint8_t)a | ((uint32_t)(uint8_t)b << 8));
            } else {
              out[0] = a;
              if (gx + 1 < W) out[1] = b;
            }
          }
        }
      } else if constexpr (OP == MIN || OP == MAX) {
        const T* cells = ring + (sy * SEGY) * TX + 2 * cp;
        uint32_t a[SEGY];
        const T* c = cells + (size_t)oldest * PL;
#pragma unroll
        for (int j = 0; j < SEGY; ++j) a[j] = *reinterpret_cast<const uint32_t*>(c + j * TX);
        int idx = oldest;
        for (int v = 1; v < NZ; ++v) {
          idx = idx + 1 == NZ ? 0 : idx + 1;
          c = cells + (size_t)idx * PL;
#pragma unroll
          for (int j = 0; j < SEGY; ++j) a[j] = mm<S, OP>(a[j], *reinterpret_cast<const uint32_t*>(c + j * TX));
        }
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const int gy = y0 + sy * SEGY + j;
          D* out = dst + (int64_t)zo * plane + (int64_t)gy * W + gx;
          if (gy < H && gx < W) {
            if (pair) {
              if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = a[j];
              else *reinterpret_cast<uint16_t*>(out) = (uint16_t)__byte_perm(a[j], 0, 0x0020);
            } else {
              out[0] = from_lane16<D>(a[j] & 0xFFFFu);
              if (gx + 1 < W) out[1] = from_lane16<D>(a[j] >> 16);
            }
          }
        }
      } else if constexpr (OP == MEAN) {
        // zs holds the NZ planes zo-cz .. zo+cz; the oldest (zo-cz) leaves
        uint32_t cw[SEGY];
        ring_get(ring + (size_t)oldest * PL, tid, cw);
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const int q0 = div_exact<Is16<S>::sgn>(zs0[j], p.mz), q1 = div_exact<Is16<S>::sgn>(zs1[j], p.mz);
          if constexpr (Is16<S>::sgn) zs0[j] -= (int)(cw[j] << 16) >> 16, zs1[j] -= (int)cw[j] >> 16;
          else zs0[j] -= (int)(cw[j] & 0xFFFFu), zs1[j] -= (int)(cw[j] >> 16);
          const int gy = y0 + sy * SEGY + j;
          D* out = dst + (int64_t)zo * plane + (int64_t)gy * W + gx;
          if (gy < H && gx < W) {
            if (pair) {
              if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = __byte_perm(q0, q1, 0x5410);
              else *reinterpret_cast<uint16_t*>(out) = (uint16_t)__byte_perm(q0, q1, 0x0040);
            } else {
              out[0] = (D)q0;
              if (gx + 1 < W) out[1] = (D)q1;
            }
          }
        }
      } else {
        const int centre = oldest + cz >= NZ ? oldest + cz - NZ : oldest + cz;
        uint64_t acc[SEGY];
        {
          uint64_t c[SEGY];
          ring_get2(ring + (size_t)centre * PL, tid, c);
#pragma unroll
          for (int j = 0; j < SEGY; ++j) acc[j] = f2_fma(f2_bcast(p.wz[0]), c[j], 0ull);
        }
        int lo = centre, hi = centre;
        for (int k = 1; k <= cz; ++k) {
          lo = lo == 0 ? NZ - 1 : lo - 1;
          hi = hi + 1 == NZ ? 0 : hi + 1;
          uint64_t bl[SEGY], bh[SEGY];
          ring_get2(ring + (size_t)lo * PL, tid, bl);
          ring_get2(ring + (size_t)hi * PL, tid, bh);
          const uint64_t wk = f2_bcast(p.wz[k]);
#pragma unroll
          for (int j = 0; j < SEGY; ++j) acc[j] = f2_fma(wk, f2_add(bl[j], bh[j]), acc[j]);
        }
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          const int gy = y0 + sy * SEGY + j;
          D* out = dst + (int64_t)zo * plane + (int64_t)gy * W + gx;
          if (gy < H && gx < W) {
            if (pair) {
              *reinterpret_cast<uint64_t*>(out) = acc[j];
            } else {
              const float2 f = f2_unpack(acc[j]);
              out[0] = f.x;
              if (gx + 1 < W) out[1] = f.y;
            }
          }
        }
      }
    }
  };

  if constexpr (PIPE) {
    // One barrier per plane: the staged tile and the X results are double
    // buffered, so the X pass of plane i runs in the same phase as the Y/Z
    // passes of plane i-1 (threads idle in the X pass go on to Y/Z).
    const int NPL = z1 + 2 * cz - z0;  // planes z0-cz .. z1+cz-1
    commit(tinb(0));
    if (NPL > 1) fetch(z0 - cz + 1);
    __syncthreads();
    for (int it = 0; it <= NPL; ++it) {
      const int zi = z0 - cz + it;
      if (it < NPL) {
        if (it + 1 < NPL) {
          commit(tinb((it + 1) & 1));
          if (it + 2 < NPL) fetch(zi + 2);
        }
        xpass(tinb(it & 1), xsb(it & 1));
      }
      if (it >= 1) yzpass(xsb((it - 1) & 1), zi - 1);
      __syncthreads();
    }
  } else {
    for (int zi = z0 - cz, it = 0; zi < z1 + cz; ++zi, ++it) {
      S* tcur = tin;
      if constexpr (TMA) {
        const int buf = it & 1;
        tcur = reinterpret_cast<S*>(reinterpret_cast<unsigned char*>(tin) + buf * G::buf_bytes());
        if (tid == 0) stalled = tma::mbar_wait(&bars[buf], (it >> 1) & 1, p.tma_polls) ? 0 : 1;
        __syncthreads();  // tile landed; previous Y pass done with xs
        if (stalled) {    // the copy did not arrive in time: report and give up on this tile
          if (tid == 0) {
            if (err) atomicExch(err, 1);
            // every copy issued into this CTA's shared memory lands before
            // the CTA exits: the abandoned one and the next plane's, each
            // waited for with the full bound (a copy still missing after
            // that is lost to the hardware; the flag already reports the
            // launch as failed)
            tma::mbar_wait(&bars[buf], (it >> 1) & 1);
            if (zi + 1 < z1 + cz) tma::mbar_wait(&bars[buf ^ 1], ((it + 1) >> 1) & 1);
          }
          return;
        }
        if (border) {
          fix_border(tcur);
          __syncthreads();
        }
      } else {  // scalar / vector staging from the register prefetch
        __syncthreads();  // previous X pass done with tin, previous Y pass with xs
        commit(tin);
        if (zi + 1 < z1 + cz) fetch(zi + 1);
        __syncthreads();
      }
      xpass(tcur, xs);
      if constexpr (TMA) {
        if (border) tma::fence_proxy_async();  // this thread's fix-up writes of tcur before the refill
      }
      __syncthreads();
      if constexpr (TMA) {
        if (tid == 0 && zi + 2 < z1 + cz) issue(zi + 2, it & 1);
      }
      yzpass(xs, zi);
    }
  }
}

// CTAs per SM the register budget is sized for (64 / 80 / 128 registers;
// the vector staging holds fewer prefetch registers than the scalar one)
template <int OP, int MODE> constexpr int min_ctas() {
  return (OP == GAUSS || OP == MINF || OP == MAXF) ? 2 : OP == GAUSSX ? (MODE == STAGE_VEC ? 3 : 2)
                                                     : MODE == STAGE_VEC ? 4 : 3;
}

template <class S, class D, int OP, int R, int MODE, bool PIPE = false>
__global__ void __launch_bounds__(NT, min_ctas<OP, MODE>()) k_sep2(const S* __restrict__ src, D* __restrict__ dst, int W,
                                                             int H, int Dz, int zchunk,
                                                             const __grid_constant__ Params p) {
  extern __shared__ __align__(128) unsigned char smem[];
  sep2_tile<S, D, OP, R, MODE, PIPE>(src, dst, W, H, Dz, zchunk, p, blockIdx.x, blockIdx.y, blockIdx.z, smem);
}

// Same tile body with the halo tile staged by TMA, double-buffered: the copy
// of plane z+1 overlaps the X/Y/Z passes of plane z.
template <class S, class D, int OP, int R>
__global__ void __launch_bounds__(NT) k_sep2_tma(const __grid_constant__ CUtensorMap map, D* __restrict__ dst,
                                                 int W, int H, int Dz, int zchunk, const __grid_constant__ Params p,
                                                 int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  sep2_tile<S, D, OP, R, STAGE_TMA>(nullptr, dst, W, H, Dz, zchunk, p, blockIdx.x, blockIdx.y, blockIdx.z, smem,
                                    &map, err);
}

template <class K>
bool smem_ok(K kern, size_t smem) {
  if (smem > 220 * 1024) return false;
  if (smem <= 48 * 1024) return true;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

// CLK_SEP2_TMA=1 in the environment stages with TMA instead of the
// register prefetch
inline bool tma_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_SEP2_TMA");
    return e && e[0] == '1';
  }();
  return on;
}

// CLK_TMA_WAIT_POLLS in the environment (read at every TMA launch): the
// poll limit of the first wait for each staged tile; a test sets it to 0 to
// make those waits run out.  Default tma::kWaitLimit.
inline uint32_t tma_wait_polls() {
  const char* e = getenv("CLK_TMA_WAIT_POLLS");
  if (!e || !*e) return tma::kWaitLimit;
  char* end = nullptr;
  const unsigned long v = strtoul(e, &end, 10);
  return (*end || v > tma::kWaitLimit) ? tma::kWaitLimit : (uint32_t)v;
}

template <class S, class D, int OP, int R>
clk_status launch(const Image& dst, const Image& src, const Params& p_in, cudaStream_t st) {
  Params p = p_in;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tx = (dst.w + TX - 1) / TX, ty = (dst.h + TY - 1) / TY;
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 3LL * sms && dst.d / (chunks * 2) >= std::max(8, 4 * p.cz)) chunks *= 2;
  const int zchunk = (dst.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (dst.d + zchunk - 1) / zchunk);

  using GT = Geo<S, OP, R, STAGE_TMA>;
  CUtensorMap map;
  int* err = wait_flag_device();
  if (tma_enabled() && err && smem_ok(k_sep2_tma<S, D, OP, R>, GT::smem(p.cz)) &&
      tma::make_map_3d(&map, src.ptr, sizeof(S), src.w, src.h, src.d, GT::RW, GT::RH)) {
    p.tma_polls = tma_wait_polls();
    k_sep2_tma<S, D, OP, R><<<grid, NT, GT::smem(p.cz), st>>>(map, (D*)dst.ptr, dst.w, dst.h, dst.d, zchunk, p, err);
    count_launch();
    return check_launch("separable (fused, sep2, tma)");
  }
  // vector staging when the image base and rows are aligned to its vectors;
  // the pipelined loop (double-buffered tiles, one barrier per plane) where
  // its shared memory leaves several CTAs per SM: min / max / mean
  constexpr bool PIPE = OP != GAUSS && OP != MINF && OP != MAXF;  // float tiles: one buffer each
  using GV = Geo<S, OP, R, STAGE_VEC, PIPE>;
  if ((uintptr_t)src.ptr % GV::SV == 0 && ((int64_t)src.w * (int64_t)sizeof(S)) % GV::SV == 0 &&
      (int64_t)src.w * src.h < (1LL << 32) && smem_ok(k_sep2<S, D, OP, R, STAGE_VEC, PIPE>, GV::smem(p.cz))) {
    k_sep2<S, D, OP, R, STAGE_VEC, PIPE><<<grid, NT, GV::smem(p.cz), st>>>((const S*)src.ptr, (D*)dst.ptr, dst.w,
                                                                           dst.h, dst.d, zchunk, p);
    count_launch();
    return check_launch("separable (fused, sep2, vector staging)");
  }
  using G = Geo<S, OP, R, STAGE_SCALAR>;
  if (!smem_ok(k_sep2<S, D, OP, R, STAGE_SCALAR>, G::smem(p.cz))) return CLK_UNSUPPORTED_DTYPE;
  k_sep2<S, D, OP, R, STAGE_SCALAR><<<grid, NT, G::smem(p.cz), st>>>((const S*)src.ptr, (D*)dst.ptr, dst.w, dst.h,
                                                                     dst.d, zchunk, p);
  count_launch();
  return check_launch("separable (fused, sep2)");
}

template <class S, class D, int OP, int RMAX>
clk_status by_radius(int R, const Image& dst, const Image& src, const Params& p, cudaStream_t st) {
  if constexpr (RMAX >= 1) {
    if (R == RMAX) return launch<S, D, OP, RMAX>(dst, src, p, st);
    return by_radius<S, D, OP, RMAX - 1>(R, dst, src, p, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

constexpr int kMaxRIntegers = 8;
constexpr int kMaxRGauss = 12;


bool layout_ok(const Image& dst, const Image& src, int align_elems) {
  return src.w == dst.w && src.h == dst.h && src.d == dst.d &&
         ((uintptr_t)dst.ptr % (align_elems * dtype_size(dst.dt))) == 0 &&
         ((uintptr_t)src.ptr % dtype_size(src.dt)) == 0;
}

}  // namespace
}  // namespace sep2
}  // namespace clk
