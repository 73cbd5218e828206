// clk_sep2_impl.cuh - the kernel template behind clk_sep2.cuh (see there for
// the layout); included by the three .cu files that instantiate it per
// operation so that they compile in parallel.
#pragma once
#include <algorithm>
#include <type_traits>

#include "clk_sep2.cuh"

namespace clk {
namespace sep2 {
namespace {

enum Op { MIN = 0, MAX = 1, MEAN = 2, GAUSS = 3 };

// temporaries: 16-bit lanes for integer pixels, float for the Gaussian
template <class S, int OP> struct Temp;
template <class S> struct Temp<S, MIN> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, MAX> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, MEAN> { typedef typename std::conditional<Is16<S>::sgn, int16_t, uint16_t>::type T; };
template <class S> struct Temp<S, GAUSS> { typedef float T; };

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

template <class S, int OP, int R> struct Geo {
  typedef typename Temp<S, OP>::T T;
  static constexpr int RW = TX + 2 * R, RH = TY + 2 * R;
  static constexpr int NEL = RW * RH;
  static constexpr int PER = (NEL + NT - 1) / NT;
  static constexpr int WIN_X = SEGX + 2 * R;
  static constexpr int WIN_Y = SEGY + 2 * R;
  static constexpr size_t tin_bytes() { return ((size_t)NEL * sizeof(S) + 15) & ~size_t(15); }
  static constexpr size_t xs_bytes() { return ((size_t)RH * TX * sizeof(T) + 15) & ~size_t(15); }
  static __host__ __device__ size_t ring_bytes(int cz) { return (size_t)(2 * cz + 1) * TY * TX * sizeof(T); }
  static size_t smem(int cz) { return tin_bytes() + xs_bytes() + ring_bytes(cz); }
};

// One tile (bx, by) x z-chunk bz of one image; the whole CTA takes part.
// smem: dynamic shared memory of at least Geo::smem(p.cz) bytes.
template <class S, class D, int OP, int R>
__device__ __forceinline__ void sep2_tile(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                          int zchunk, const Params& p, int bx, int by, int bz,
                                          unsigned char* smem) {
  using G = Geo<S, OP, R>;
  using T = typename G::T;
  S* tin = reinterpret_cast<S*>(smem);
  T* xs = reinterpret_cast<T*>(smem + G::tin_bytes());
  T* ring = reinterpret_cast<T*>(smem + G::tin_bytes() + G::xs_bytes());
  const int cz = p.cz, NZ = 2 * cz + 1;
  const int tid = threadIdx.x;
  const int x0 = bx * TX, y0 = by * TY;
  const int z0 = bz * zchunk, z1 = min(Dz, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;

  S pre[G::PER];
  auto fetch = [&](int zv) {
    const S* sp = src + (int64_t)clampi(zv, Dz - 1) * plane;
#pragma unroll
    for (int k = 0; k < G::PER; ++k) {
      const int i = tid + k * NT;
      if (i < G::NEL) {
        const int r = i / G::RW, q = i - r * G::RW;
        pre[k] = __ldg(sp + (int64_t)clampi(y0 - R + r, H - 1) * W + clampi(x0 - R + q, W - 1));
      }
    }
  };
  auto commit = [&]() {
#pragma unroll
    for (int k = 0; k < G::PER; ++k) {
      const int i = tid + k * NT;
      if (i < G::NEL) tin[i] = pre[k];
    }
  };

  // Y/Z ownership: column pair cp, rows sy*SEGY .. +SEGY-1
  const int cp = tid % (TX / 2), sy = tid / (TX / 2);
  int wslot = 0;
  fetch(z0 - cz);
  for (int zi = z0 - cz; zi < z1 + cz; ++zi) {
    __syncthreads();  // previous X pass done with tin, previous Y pass with xs
    commit();
    if (zi + 1 < z1 + cz) fetch(zi + 1);
    __syncthreads();

    // ---------------- X pass: rows (2rp, 2rp+1) x outputs sg*SEGX ..
    {
      const int rp = tid / (TX / SEGX), sg = tid % (TX / SEGX);
      if (rp < G::RH / 2) {
        const S* r0 = tin + (2 * rp) * G::RW + sg * SEGX;
        const S* r1 = r0 + G::RW;
        T* o0 = xs + (2 * rp) * TX + sg * SEGX;
        T* o1 = o0 + TX;
        if constexpr (OP == MIN || OP == MAX) {
          uint32_t win[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) win[k] = lane16(r0[k]) | (lane16(r1[k]) << 16);
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            uint32_t a = win[j], b = win[j + 1];
#pragma unroll
            for (int k = 1; k <= 2 * R; ++k) {
              a = mm<S, OP>(a, win[j + k]);
              b = mm<S, OP>(b, win[j + 1 + k]);
            }
            *reinterpret_cast<uint32_t*>(o0 + j) = __byte_perm(a, b, 0x5410);
            *reinterpret_cast<uint32_t*>(o1 + j) = __byte_perm(a, b, 0x7632);
          }
        } else if constexpr (OP == MEAN) {
          int w0[G::WIN_X], w1[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) w0[k] = (int)r0[k], w1[k] = (int)r1[k];
          int s0 = 0, s1 = 0;
#pragma unroll
          for (int k = 0; k <= 2 * R; ++k) s0 += w0[k], s1 += w1[k];
          int q0[SEGX], q1[SEGX];
#pragma unroll
          for (int j = 0; j < SEGX; ++j) {
            if (j > 0) {
              s0 += w0[j + 2 * R] - w0[j - 1];
              s1 += w1[j + 2 * R] - w1[j - 1];
            }
            q0[j] = div_exact(s0, p.mx);
            q1[j] = div_exact(s1, p.mx);
          }
#pragma unroll
          for (int j = 0; j < SEGX; j += 2) {
            *reinterpret_cast<uint32_t*>(o0 + j) = __byte_perm((uint32_t)q0[j], (uint32_t)q0[j + 1], 0x5410);
            *reinterpret_cast<uint32_t*>(o1 + j) = __byte_perm((uint32_t)q1[j], (uint32_t)q1[j + 1], 0x5410);
          }
        } else {
          uint64_t win[G::WIN_X];
#pragma unroll
          for (int k = 0; k < G::WIN_X; ++k) win[k] = f2_pack(tofloat(r0[k]), tofloat(r1[k]));
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
    __syncthreads();

    // ---------------- Y pass: column pair cp x rows sy*SEGY .. -> ring slot
    T* rs = ring + (size_t)wslot * TY * TX;
    {
      const T* col = xs + (sy * SEGY) * TX + 2 * cp;
      T* o = rs + (sy * SEGY) * TX + 2 * cp;
      if constexpr (OP == MIN || OP == MAX) {
        uint32_t win[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) win[k] = *reinterpret_cast<const uint32_t*>(col + k * TX);
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          uint32_t a = win[j];
#pragma unroll
          for (int k = 1; k <= 2 * R; ++k) a = mm<S, OP>(a, win[j + k]);
          *reinterpret_cast<uint32_t*>(o + j * TX) = a;
        }
      } else if constexpr (OP == MEAN) {
        int w0[G::WIN_Y], w1[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) w0[k] = (int)col[k * TX], w1[k] = (int)col[k * TX + 1];
        int s0 = 0, s1 = 0;
#pragma unroll
        for (int k = 0; k <= 2 * R; ++k) s0 += w0[k], s1 += w1[k];
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          if (j > 0) {
            s0 += w0[j + 2 * R] - w0[j - 1];
            s1 += w1[j + 2 * R] - w1[j - 1];
          }
          *reinterpret_cast<uint32_t*>(o + j * TX) =
              __byte_perm((uint32_t)div_exact(s0, p.mx), (uint32_t)div_exact(s1, p.mx), 0x5410);
        }
      } else {
        uint64_t win[G::WIN_Y];
#pragma unroll
        for (int k = 0; k < G::WIN_Y; ++k) win[k] = *reinterpret_cast<const uint64_t*>(col + k * TX);
#pragma unroll
        for (int j = 0; j < SEGY; ++j) {
          uint64_t acc = f2_fma(f2_bcast(p.wy[0]), win[j + R], 0ull);
#pragma unroll
          for (int k = 1; k <= R; ++k) acc = f2_fma(f2_bcast(p.wy[k]), f2_add(win[j + R - k], win[j + R + k]), acc);
          *reinterpret_cast<uint64_t*>(o + j * TX) = acc;
        }
      }
    }

    // ---------------- Z pass over this thread's own ring cells
    const int zo = zi - cz;
    const int oldest = wslot + 1 == NZ ? 0 : wslot + 1;
    wslot = oldest;
    if (zo >= z0) {
      const int gx = x0 + 2 * cp;
#pragma unroll
      for (int j = 0; j < SEGY; ++j) {
        const int gy = y0 + sy * SEGY + j;
        const size_t cell = (size_t)(sy * SEGY + j) * TX + 2 * cp;
        D* out = dst + (int64_t)zo * plane + (int64_t)gy * W + gx;
        const bool ok = gy < H && gx < W;
        if constexpr (OP == MIN || OP == MAX) {
          uint32_t a = *reinterpret_cast<const uint32_t*>(ring + (size_t)oldest * TY * TX + cell);
          int idx = oldest;
          for (int v = 1; v < NZ; ++v) {
            idx = idx + 1 == NZ ? 0 : idx + 1;
            a = mm<S, OP>(a, *reinterpret_cast<const uint32_t*>(ring + (size_t)idx * TY * TX + cell));
          }
          if (ok) {
            if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = a;
            else *reinterpret_cast<uint16_t*>(out) = (uint16_t)__byte_perm(a, 0, 0x0020);
          }
        } else if constexpr (OP == MEAN) {
          int s0 = 0, s1 = 0, idx = oldest;
          for (int v = 0; v < NZ; ++v) {
            const T* c = ring + (size_t)idx * TY * TX + cell;
            s0 += (int)c[0];
            s1 += (int)c[1];
            idx = idx + 1 == NZ ? 0 : idx + 1;
          }
          const int q0 = div_exact(s0, p.mz), q1 = div_exact(s1, p.mz);
          if (ok) {
            if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = __byte_perm(q0, q1, 0x5410);
            else *reinterpret_cast<uint16_t*>(out) = (uint16_t)__byte_perm(q0, q1, 0x0040);
          }
        } else {
          const int centre = oldest + cz >= NZ ? oldest + cz - NZ : oldest + cz;
          const uint64_t* base = reinterpret_cast<const uint64_t*>(ring + cell);
          const size_t stride = (size_t)TY * TX / 2;  // ring plane in uint64 units
          uint64_t acc = f2_fma(f2_bcast(p.wz[0]), base[centre * stride], 0ull);
          int lo = centre, hi = centre;
          for (int k = 1; k <= cz; ++k) {
            lo = lo == 0 ? NZ - 1 : lo - 1;
            hi = hi + 1 == NZ ? 0 : hi + 1;
            acc = f2_fma(f2_bcast(p.wz[k]), f2_add(base[lo * stride], base[hi * stride]), acc);
          }
          if (ok) *reinterpret_cast<uint64_t*>(out) = acc;
        }
      }
    }
  }
}

template <class S, class D, int OP, int R>
__global__ void __launch_bounds__(NT) k_sep2(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                             int zchunk, const __grid_constant__ Params p) {
  extern __shared__ __align__(16) unsigned char smem[];
  sep2_tile<S, D, OP, R>(src, dst, W, H, Dz, zchunk, p, blockIdx.x, blockIdx.y, blockIdx.z, smem);
}

template <class S, class D, int OP, int R>
clk_status launch(const Image& dst, const Image& src, const Params& p, cudaStream_t st) {
  using G = Geo<S, OP, R>;
  const size_t smem = G::smem(p.cz);
  if (smem > 220 * 1024) return CLK_UNSUPPORTED_DTYPE;
  auto kern = k_sep2<S, D, OP, R>;
  static size_t configured = 48 * 1024;
  if (smem > configured) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      return CLK_UNSUPPORTED_DTYPE;
    }
    configured = smem;
  }
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tx = (dst.w + TX - 1) / TX, ty = (dst.h + TY - 1) / TY;
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 3LL * sms && dst.d / (chunks * 2) >= std::max(8, 4 * p.cz)) chunks *= 2;
  const int zchunk = (dst.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (dst.d + zchunk - 1) / zchunk);
  kern<<<grid, NT, smem, st>>>((const S*)src.ptr, (D*)dst.ptr, dst.w, dst.h, dst.d, zchunk, p);
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

uint64_t recip40(int n) { return (((uint64_t)1 << 40) + (uint64_t)n - 1) / (uint64_t)n; }

bool layout_ok(const Image& dst, const Image& src, int align_elems) {
  return src.w == dst.w && src.h == dst.h && src.d == dst.d && src.w % 2 == 0 &&
         ((uintptr_t)dst.ptr % (align_elems * dtype_size(dst.dt))) == 0 &&
         ((uintptr_t)src.ptr % dtype_size(src.dt)) == 0;
}

}  // namespace
}  // namespace sep2
}  // namespace clk
