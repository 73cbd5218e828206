// clk_morph.cu - binary erode/dilate (box 3x3x3 and the 7-point "sphere"
// cross, erode_box_3d_x.cl:14-37, erode_sphere_3d_x.cl:14-37,
// dilate_box_3d_x.cl:14-37, dilate_sphere_3d_x.cl:14-38) on byte images.
//
// Every kernel writes 1 where its condition holds (erode: all neighbours
// nonzero; dilate: any neighbour nonzero) and 0 elsewhere, which is exactly
// what the early-exit loops produce for integer pixels.  Here a thread owns a
// 16-byte chunk of a row (16 voxels): pixels become byte masks (0xFF where
// nonzero), x-neighbours come from funnel shifts across the chunk, y- and
// z-neighbours from neighbouring chunks staged in shared memory.  The CTA
// streams along z through a ring of three planes.
//
// ITER = 2 fuses two launches of the r=1 kernel (the radius-2 request) in one
// pass.  The intermediate image of the two-launch sequence is read with
// clamp-to-edge, so its value at a virtual position outside the image is
// the value at the clamped position -- not the operator re-evaluated on
// clamped inputs.  The fused kernel therefore copies border rows and planes
// of the intermediate instead of computing them.
#include <cstdlib>

#include "clk_common.cuh"

namespace clk {

namespace {

constexpr int MX = 8;    // chunks (16 voxels) per tile row
constexpr int MY = 32;   // rows per tile
constexpr int MT = 256;  // threads

__device__ __forceinline__ uint4 nzmask(uint4 v) {
  return make_uint4(__vcmpne4(v.x, 0u), __vcmpne4(v.y, 0u), __vcmpne4(v.z, 0u), __vcmpne4(v.w, 0u));
}
// byte i of the result = byte i-1 of c; byte 0 = lb (0 or 0xFF)
__device__ __forceinline__ uint4 shl1(uint4 c, uint32_t lb) {
  return make_uint4((c.x << 8) | lb, __funnelshift_l(c.x, c.y, 8), __funnelshift_l(c.y, c.z, 8),
                    __funnelshift_l(c.z, c.w, 8));
}
// byte i of the result = byte i+1 of c; byte 15 = rb (0 or 0xFF)
__device__ __forceinline__ uint4 shr1(uint4 c, uint32_t rb) {
  return make_uint4(__funnelshift_r(c.x, c.y, 8), __funnelshift_r(c.y, c.z, 8), __funnelshift_r(c.z, c.w, 8),
                    (c.w >> 8) | (rb << 24));
}
template <bool ERODE> __device__ __forceinline__ uint4 comb(uint4 a, uint4 b) {
  return ERODE ? make_uint4(a.x & b.x, a.y & b.y, a.z & b.z, a.w & b.w)
               : make_uint4(a.x | b.x, a.y | b.y, a.z | b.z, a.w | b.w);
}

// x-neighbour combination of chunk c with the left/right neighbour chunks
// (their boundary bytes: the last word of the left chunk, the first of the
// right one); at the image's first/last chunk the clamped neighbour is the
// chunk's own boundary byte.
template <bool ERODE>
__device__ __forceinline__ uint4 xcomb(uint4 c, uint32_t lw, uint32_t rx, bool first, bool last) {
  const uint32_t lb = first ? (c.x & 0xFFu) : (lw >> 24);
  const uint32_t rb = last ? (c.w >> 24) : (rx & 0xFFu);
  return comb<ERODE>(comb<ERODE>(c, shl1(c, lb)), shr1(c, rb));
}
// the boundary words of the chunks left / right of chunk i (4-byte reads)
__device__ __forceinline__ uint32_t lword(const uint4* P, int i) { return reinterpret_cast<const uint32_t*>(P + i - 1)[3]; }
__device__ __forceinline__ uint32_t rword(const uint4* P, int i) { return reinterpret_cast<const uint32_t*>(P + i + 1)[0]; }

// One r=1 step at tile chunk (r, q) of a region whose planes A (z-1), B (z),
// C (z+1) are stored with row pitch `pitch` and one halo chunk/row around.
template <bool ERODE, bool SPHERE>
__device__ __forceinline__ uint4 step(const uint4* A, const uint4* B, const uint4* C, int pitch, int r, int q,
                                      bool first, bool last) {
  const int i = (r + 1) * pitch + (q + 1);
  if constexpr (SPHERE) {
    const uint4 c = B[i];
    uint4 o = xcomb<ERODE>(c, lword(B, i), rword(B, i), first, last);
    o = comb<ERODE>(o, B[i - pitch]);
    o = comb<ERODE>(o, B[i + pitch]);
    o = comb<ERODE>(o, A[i]);
    return comb<ERODE>(o, C[i]);
  } else {
    uint4 o = xcomb<ERODE>(B[i], lword(B, i), rword(B, i), first, last);
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const uint4* pl[3] = {A, B, C};
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        if (p == 1 && dy == 0) continue;
        const int j = i + dy * pitch;
        o = comb<ERODE>(o, xcomb<ERODE>(pl[p][j], lword(pl[p], j), rword(pl[p], j), first, last));
      }
    }
    return o;
  }
}

template <int ITER> struct Geo {
  static constexpr int R1X = ITER == 2 ? MX + 2 : MX;  // region of the first step
  static constexpr int R1Y = ITER == 2 ? MY + 2 : MY;
  static constexpr int IX = R1X + 2, IY = R1Y + 2;    // staged input planes
  static constexpr int SX = MX + 2, SY = MY + 2;      // staged intermediate planes
};

// ITER = 0: one step of the 2-D kernel on every plane of a 3-D image (the
// slice-by-slice kernels, erode_sphere_slice_by_slice_3d_x.cl:14-26 ...).
template <class S, class D, bool ERODE, bool SPHERE, int ITER>
__global__ void __launch_bounds__(MT)
    k_morph_bytes(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz, int zchunk) {
  using G = Geo<ITER>;
  constexpr bool PLANAR = ITER == 0;
  // ITER 0: two input planes; ITER 1: a ring of four; ITER 2: rings of four
  // input and four intermediate planes in dynamic shared memory (49 KiB)
  __shared__ uint4 in[ITER == 2 ? 1 : 4][ITER == 2 ? 1 : G::IY * G::IX];
  extern __shared__ uint4 dsm[];
  const int nxc = W / 16;
  const int xc0 = blockIdx.x * MX, y0 = blockIdx.y * MY;
  const int z0 = blockIdx.z * zchunk, z1 = min(Dz, z0 + zchunk);
  const int tid = threadIdx.x;
  const int64_t plane = (int64_t)W * H;
  const uint4* src4 = reinterpret_cast<const uint4*>(src);
  uint4* dst4 = reinterpret_cast<uint4*>(dst);
  const int hx = PLANAR ? 1 : ITER, hy = hx;  // halo of the staged input around the output tile

  // Input planes are staged strictly in z order.  The next one is always in
  // flight in registers (pf) while the current planes are processed;
  // load_plane(zv, slot) stores plane zv (the prefetched one) as masks and
  // starts fetching zv + 1 if it will be needed.
  constexpr int NS = G::IY * G::IX, PERM = (NS + MT - 1) / MT;
  const int last_in = PLANAR ? z1 - 1 : z1 - 1 + ITER;
  uint4 pf[PERM];
  auto fetch = [&](int zv) {
    const int zc = clampi(zv, Dz - 1);
#pragma unroll
    for (int k = 0; k < PERM; ++k) {
      const int i = tid + k * MT;
      if (i < NS) {
        const int r = i / G::IX, q = i - r * G::IX;
        const int gy = clampi(y0 - hy + r, H - 1), gq = clampi(xc0 - hx + q, nxc - 1);
        pf[k] = __ldg(src4 + ((int64_t)zc * plane + (int64_t)gy * W) / 16 + gq);
      }
    }
  };
  auto stage = [&](int zv, uint4* to) {
#pragma unroll
    for (int k = 0; k < PERM; ++k) {
      const int i = tid + k * MT;
      if (i < NS) to[i] = nzmask(pf[k]);
    }
    if (zv + 1 <= last_in) fetch(zv + 1);
  };
  auto load_plane = [&](int zv, int slot) { stage(zv, in[slot]); };
  fetch(PLANAR ? z0 : z0 - ITER);
  auto store = [&](int zo, int r, int q, uint4 m) {
    const int gy = y0 + r, gq = xc0 + q;
    if (gy < H && gq < nxc) {
      const uint32_t one = 0x01010101u;
      dst4[((int64_t)zo * plane + (int64_t)gy * W) / 16 + gq] = make_uint4(m.x & one, m.y & one, m.z & one, m.w & one);
    }
  };

  if constexpr (PLANAR) {
    // each plane alone, two buffers: one barrier per plane
    for (int zo = z0; zo < z1; ++zo) {
      const int b = (zo - z0) & 1;
      load_plane(zo, b);
      __syncthreads();
      const int r = tid / MX, q = tid % MX;
      const int gq = xc0 + q;
      store(zo, r, q, step<ERODE, SPHERE>(in[b], in[b], in[b], G::IX, r, q, gq == 0, gq == nxc - 1));
    }
  } else if constexpr (ITER == 1) {
    // Phase j stages input j+2 and filters output plane j from inputs
    // j-1 .. j+1 (staged in earlier phases): a ring of four input planes
    // (plane p in slot p & 3) and one barrier per plane.
    for (int j = z0 - 3; j < z1; ++j) {
      if (j + 2 <= last_in) stage(j + 2, in[(j + 2) & 3]);
      if (j >= z0) {
        const int r = tid / MX, q = tid % MX;
        const int gq = xc0 + q;
        store(j, r, q, step<ERODE, SPHERE>(in[(j - 1) & 3], in[j & 3], in[(j + 1) & 3], G::IX, r, q, gq == 0,
                                           gq == nxc - 1));
      }
      __syncthreads();
    }
  } else {
    // Phase j stages input j+4, computes the intermediate (first step) at
    // plane j+2 from inputs j+1 .. j+3, and filters output plane j from the
    // intermediates j-1 .. j+1: rings of four input and four intermediate
    // planes (plane p in slot p & 3), one barrier per plane.
    //
    // The intermediate at a virtual position is the one at the clamped
    // position: rows above / below the image evaluate the first step at the
    // clamped row; plane -1 (Dz) is a copy of plane 0 (Dz - 1), made in the
    // phase after that plane is computed.  Intermediate region rows
    // r = 0..R1Y-1 <-> global rows y0-1+r, chunks q <-> xc0-1+q.
    constexpr int MS = G::SY * G::SX;
    auto ip = [&](int p) { return dsm + (p & 3) * NS; };
    auto mp = [&](int p) { return dsm + 4 * NS + (p & 3) * MS; };
    for (int j = z0 - 6; j < z1; ++j) {
      if (j + 4 <= last_in) stage(j + 4, ip(j + 4));
      const int pm = j + 2;
      if (pm >= z0 - 1 && pm <= z1) {
        if (pm >= 0 && pm < Dz) {
          uint4* M = mp(pm);
          for (int i = tid; i < G::R1Y * G::R1X; i += MT) {
            const int r = i / G::R1X, q = i - r * G::R1X;
            const int gy = y0 - 1 + r;
            const int rr = r + (clampi(gy, H - 1) - gy);
            const int gq = clampi(xc0 - 1 + q, nxc - 1);
            M[r * G::SX + q] = step<ERODE, SPHERE>(ip(pm - 1), ip(pm), ip(pm + 1), G::IX, rr, q, gq == 0,
                                                   gq == nxc - 1);
          }
        } else if (pm >= Dz) {  // plane Dz: copy of Dz - 1 (computed in the previous phase)
          const uint4* Mf = mp(Dz - 1);
          uint4* Mt = mp(pm);
          for (int i = tid; i < MS; i += MT) Mt[i] = Mf[i];
        }
      }
      if (j == -1 && z0 == 0) {  // plane -1: copy of plane 0 (computed in the previous phase)
        const uint4* Mf = mp(0);
        uint4* Mt = mp(-1);
        for (int i = tid; i < MS; i += MT) Mt[i] = Mf[i];
      }
      if (j >= z0) {
        const int r = tid / MX, q = tid % MX;
        const int gq = xc0 + q;
        // output tile (r, q) sits at (r+1, q+1) of the intermediate region
        store(j, r, q, step<ERODE, SPHERE>(mp(j - 1), mp(j), mp(j + 1), G::SX, r, q, gq == 0, gq == nxc - 1));
      }
      __syncthreads();
    }
  }
}

template <class S, class D, bool ERODE, bool SPHERE, int ITER>
clk_status launch_morph(const Image& dst, const Image& src, cudaStream_t st) {
  const int nxc = src.w / 16;
  const int tx = (nxc + MX - 1) / MX, ty = (src.h + MY - 1) / MY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int chunks = 1;
  // z-chunks: enough CTAs for 16 per SM (r=1: 0.115 ms on 1024x1024x256
  // against 0.117 with 8 and 0.135 with 4); the fused radius 2, whose
  // chunks re-stage two more input planes each, is faster with 4 (0.234
  // against 0.240 ms with 8)
  const int64_t want = (ITER == 2 ? 4LL : 16LL) * sms;
  while ((int64_t)tx * ty * chunks < want && src.d / (chunks * 2) >= 8) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
  using G = Geo<ITER>;
  const size_t smem = ITER == 2 ? 4 * sizeof(uint4) * (G::IY * G::IX + G::SY * G::SX) : 0;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_morph_bytes<S, D, ERODE, SPHERE, ITER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return CLK_UNSUPPORTED_DTYPE;
  }
  k_morph_bytes<S, D, ERODE, SPHERE, ITER><<<grid, MT, smem, st>>>((const S*)src.ptr, (D*)dst.ptr, src.w, src.h,
                                                                     src.d, zchunk);
  count_launch();
  return check_launch("morphology (byte tiles)");
}

template <bool ERODE, bool SPHERE, int ITER>
clk_status launch_sel(const Image& dst, const Image& src, cudaStream_t st) {
  const bool su = src.dt == CLK_U8, du = dst.dt == CLK_U8;
  if (su && du) return launch_morph<uint8_t, uint8_t, ERODE, SPHERE, ITER>(dst, src, st);
  if (su) return launch_morph<uint8_t, int8_t, ERODE, SPHERE, ITER>(dst, src, st);
  if (du) return launch_morph<int8_t, uint8_t, ERODE, SPHERE, ITER>(dst, src, st);
  return launch_morph<int8_t, int8_t, ERODE, SPHERE, ITER>(dst, src, st);
}

// CLK_MORPH_BITS=0 in the environment keeps the byte-mask kernels (A/B timing)
bool morph_bits_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_MORPH_BITS");
    return !(e && e[0] == '0');
  }();
  return on;
}

}  // namespace

bool fast_morph_fusable(const Image& dst, const Image& src) {
  const bool bytes = (src.dt == CLK_U8 || src.dt == CLK_I8) && (dst.dt == CLK_U8 || dst.dt == CLK_I8);
  return bytes && src.ndim == 3 && src.w % 16 == 0 && ((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % 16 == 0 &&
         src.w == dst.w && src.h == dst.h && src.d == dst.d;
}

clk_status fast_morph(bool erode, bool sphere, int iterations, const Image& dst, const Image& src, const Policy&,
                      cudaStream_t st, bool planar) {
  if (!fast_morph_fusable(dst, src) || iterations < 1 || iterations > 2) return CLK_UNSUPPORTED_DTYPE;
  if (!planar && morph_bits_enabled()) {
    const clk_status b = morph_bits(erode, sphere, iterations, dst, src, st);
    if (b != CLK_UNSUPPORTED_DTYPE) return b;
  }
  if (planar) {
    if (iterations != 1) return CLK_UNSUPPORTED_DTYPE;
    if (erode) return sphere ? launch_sel<true, true, 0>(dst, src, st) : launch_sel<true, false, 0>(dst, src, st);
    return sphere ? launch_sel<false, true, 0>(dst, src, st) : launch_sel<false, false, 0>(dst, src, st);
  }
  const int sel = (erode ? 4 : 0) | (sphere ? 2 : 0) | (iterations == 2 ? 1 : 0);
  switch (sel) {
    case 0: return launch_sel<false, false, 1>(dst, src, st);
    case 1: return launch_sel<false, false, 2>(dst, src, st);
    case 2: return launch_sel<false, true, 1>(dst, src, st);
    case 3: return launch_sel<false, true, 2>(dst, src, st);
    case 4: return launch_sel<true, false, 1>(dst, src, st);
    case 5: return launch_sel<true, false, 2>(dst, src, st);
    case 6: return launch_sel<true, true, 1>(dst, src, st);
    case 7: return launch_sel<true, true, 2>(dst, src, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
