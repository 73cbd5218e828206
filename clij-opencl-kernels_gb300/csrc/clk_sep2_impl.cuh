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

// Geometry of one tile.  With TMA the staged row starts RA >= R elements left
// of the tile (RA rounds R up so that the box's x coordinate is 16-byte
// aligned) and the halo tile is double-buffered.
template <class S, int OP, int R, bool TMA = false> struct Geo {
  typedef typename Temp<S, OP>::T T;
  static constexpr int RA = TMA ? (R + (16 / (int)sizeof(S)) - 1) / (16 / (int)sizeof(S)) * (16 / (int)sizeof(S)) : R;
  static constexpr int RW = TX + 2 * RA, RH = TY + 2 * R;
  static constexpr int NEL = RW * RH;
  static constexpr int PER = (NEL + NT - 1) / NT;
  static constexpr int NBUF = TMA ? 2 : 1;
  static constexpr int WIN_X = SEGX + 2 * R;
  static constexpr int WIN_Y = SEGY + 2 * R;
  static constexpr size_t buf_bytes() { return ((size_t)NEL * sizeof(S) + 127) & ~size_t(127); }
  static constexpr size_t tin_bytes() { return NBUF * buf_bytes(); }
  static constexpr size_t xs_bytes() { return ((size_t)RH * TX * sizeof(T) + 15) & ~size_t(15); }
  static __host__ __device__ size_t ring_bytes(int cz) { return (size_t)(2 * cz + 1) * TY * TX * sizeof(T); }
  static size_t smem(int cz) { return tin_bytes() + xs_bytes() + ring_bytes(cz); }
};

// One tile (bx, by) x z-chunk bz of one image; the whole CTA takes part.
// smem: dynamic shared memory of at least Geo::smem(p.cz) bytes (128-byte
// aligned).  TMA: map is a 3-D tensor map of src with a (RW, RH, 1) box;
// err receives 1 if a bounded wait for a tile ran out (the tile is then
// abandoned).
template <class S, class D, int OP, int R, bool TMA = false>
__device__ __forceinline__ void sep2_tile(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                          int zchunk, const Params& p, int bx, int by, int bz,
                                          unsigned char* smem, const CUtensorMap* map = nullptr,
                                          int* err = nullptr) {
  using G = Geo<S, OP, R, TMA>;
  using T = typename G::T;
  S* tin = reinterpret_cast<S*>(smem);
  T* xs = reinterpret_cast<T*>(smem + G::tin_bytes());
  T* ring = reinterpret_cast<T*>(smem + G::tin_bytes() + G::xs_bytes());
  const int cz = p.cz, NZ = 2 * cz + 1;
  const int tid = threadIdx.x;
  const int x0 = bx * TX, y0 = by * TY;
  const int z0 = bz * zchunk, z1 = min(Dz, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  constexpr int XOFF = G::RA - R;  // first staged column the X pass reads

  S pre[G::PER];  // unused (and removed) when TMA stages the tile
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
  for (int zi = z0 - cz, it = 0; zi < z1 + cz; ++zi, ++it) {
    S* tcur = tin;
    if constexpr (TMA) {
      const int buf = it & 1;
      tcur = reinterpret_cast<S*>(reinterpret_cast<unsigned char*>(tin) + buf * G::buf_bytes());
      if (tid == 0) stalled = tma::mbar_wait(&bars[buf], (it >> 1) & 1) ? 0 : 1;
      __syncthreads();  // tile landed; previous Y pass done with xs
      if (stalled) {    // the copy never arrived: report, drain the other buffer, give up on this tile
        if (tid == 0) {
          if (err) atomicExch(err, 1);
          if (zi + 1 < z1 + cz) tma::mbar_wait(&bars[buf ^ 1], ((it + 1) >> 1) & 1);
        }
        return;
      }
      if (border) {
        fix_border(tcur);
        __syncthreads();
      }
    } else {
      __syncthreads();  // previous X pass done with tin, previous Y pass with xs
      commit();
      if (zi + 1 < z1 + cz) fetch(zi + 1);
      __syncthreads();
    }

    // ---------------- X pass: rows (2rp, 2rp+1) x outputs sg*SEGX ..
    {
      const int rp = tid / (TX / SEGX), sg = tid % (TX / SEGX);
      if (rp < G::RH / 2) {
        const S* r0 = tcur + (2 * rp) * G::RW + sg * SEGX + XOFF;
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
    if constexpr (TMA) tma::fence_proxy_async();  // this thread's reads/writes of tcur before the refill
    __syncthreads();
    if constexpr (TMA) {
      if (tid == 0 && zi + 2 < z1 + cz) issue(zi + 2, it & 1);
    }

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
        // even widths keep every row pair-aligned: one store for both lanes;
        // odd widths store the lanes separately (the second may lie past W)
        const bool pair = (W & 1) == 0;
        if constexpr (OP == MIN || OP == MAX) {
          uint32_t a = *reinterpret_cast<const uint32_t*>(ring + (size_t)oldest * TY * TX + cell);
          int idx = oldest;
          for (int v = 1; v < NZ; ++v) {
            idx = idx + 1 == NZ ? 0 : idx + 1;
            a = mm<S, OP>(a, *reinterpret_cast<const uint32_t*>(ring + (size_t)idx * TY * TX + cell));
          }
          if (ok && pair) {
            if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = a;
            else *reinterpret_cast<uint16_t*>(out) = (uint16_t)__byte_perm(a, 0, 0x0020);
          } else if (ok) {
            out[0] = from_lane16<D>(a & 0xFFFFu);
            if (gx + 1 < W) out[1] = from_lane16<D>(a >> 16);
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
          if (ok && pair) {
            if constexpr (sizeof(D) == 2) *reinterpret_cast<uint32_t*>(out) = __byte_perm(q0, q1, 0x5410);
            else *reinterpret_cast<uint16_t*>(out) = (uint16_t)__byte_perm(q0, q1, 0x0040);
          } else if (ok) {
            out[0] = (D)q0;
            if (gx + 1 < W) out[1] = (D)q1;
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
          if (ok && pair) {
            *reinterpret_cast<uint64_t*>(out) = acc;
          } else if (ok) {
            const float2 f = f2_unpack(acc);
            out[0] = f.x;
            if (gx + 1 < W) out[1] = f.y;
          }
        }
      }
    }
  }
}

template <class S, class D, int OP, int R>
__global__ void __launch_bounds__(NT) k_sep2(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                             int zchunk, const __grid_constant__ Params p) {
  extern __shared__ __align__(128) unsigned char smem[];
  sep2_tile<S, D, OP, R>(src, dst, W, H, Dz, zchunk, p, blockIdx.x, blockIdx.y, blockIdx.z, smem);
}

// Same tile body with the halo tile staged by TMA, double-buffered: the copy
// of plane z+1 overlaps the X/Y/Z passes of plane z.
template <class S, class D, int OP, int R>
__global__ void __launch_bounds__(NT) k_sep2_tma(const __grid_constant__ CUtensorMap map, D* __restrict__ dst,
                                                 int W, int H, int Dz, int zchunk, const __grid_constant__ Params p,
                                                 int* err) {
  extern __shared__ __align__(128) unsigned char smem[];
  sep2_tile<S, D, OP, R, true>(nullptr, dst, W, H, Dz, zchunk, p, blockIdx.x, blockIdx.y, blockIdx.z, smem, &map,
                               err);
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

// CLK_SEP2_TMA=0 in the environment keeps the register-prefetch staging
inline bool tma_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_SEP2_TMA");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <class S, class D, int OP, int R>
clk_status launch(const Image& dst, const Image& src, const Params& p, cudaStream_t st) {
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tx = (dst.w + TX - 1) / TX, ty = (dst.h + TY - 1) / TY;
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 3LL * sms && dst.d / (chunks * 2) >= std::max(8, 4 * p.cz)) chunks *= 2;
  const int zchunk = (dst.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (dst.d + zchunk - 1) / zchunk);

  using GT = Geo<S, OP, R, true>;
  CUtensorMap map;
  int* err = wait_flag_device();
  if (tma_enabled() && err && smem_ok(k_sep2_tma<S, D, OP, R>, GT::smem(p.cz)) &&
      tma::make_map_3d(&map, src.ptr, sizeof(S), src.w, src.h, src.d, GT::RW, GT::RH)) {
    k_sep2_tma<S, D, OP, R><<<grid, NT, GT::smem(p.cz), st>>>(map, (D*)dst.ptr, dst.w, dst.h, dst.d, zchunk, p, err);
    count_launch();
    return check_launch("separable (fused, sep2, tma)");
  }
  using G = Geo<S, OP, R>;
  if (!smem_ok(k_sep2<S, D, OP, R>, G::smem(p.cz))) return CLK_UNSUPPORTED_DTYPE;
  k_sep2<S, D, OP, R><<<grid, NT, G::smem(p.cz), st>>>((const S*)src.ptr, (D*)dst.ptr, dst.w, dst.h, dst.d, zchunk,
                                                       p);
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
  return src.w == dst.w && src.h == dst.h && src.d == dst.d &&
         ((uintptr_t)dst.ptr % (align_elems * dtype_size(dst.dt))) == 0 &&
         ((uintptr_t)src.ptr % dtype_size(src.dt)) == 0;
}

}  // namespace
}  // namespace sep2
}  // namespace clk
