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
// (their boundary bytes); at the image's first/last chunk the clamped
// neighbour is the chunk's own boundary byte.
template <bool ERODE>
__device__ __forceinline__ uint4 xcomb(uint4 c, uint4 l, uint4 r, bool first, bool last) {
  const uint32_t lb = first ? (c.x & 0xFFu) : (l.w >> 24);
  const uint32_t rb = last ? (c.w >> 24) : (r.x & 0xFFu);
  return comb<ERODE>(comb<ERODE>(c, shl1(c, lb)), shr1(c, rb));
}

// One r=1 step at tile chunk (r, q) of a region whose planes A (z-1), B (z),
// C (z+1) are stored with row pitch `pitch` and one halo chunk/row around.
template <bool ERODE, bool SPHERE>
__device__ __forceinline__ uint4 step(const uint4* A, const uint4* B, const uint4* C, int pitch, int r, int q,
                                      bool first, bool last) {
  const int i = (r + 1) * pitch + (q + 1);
  if constexpr (SPHERE) {
    const uint4 c = B[i];
    uint4 o = xcomb<ERODE>(c, B[i - 1], B[i + 1], first, last);
    o = comb<ERODE>(o, B[i - pitch]);
    o = comb<ERODE>(o, B[i + pitch]);
    o = comb<ERODE>(o, A[i]);
    return comb<ERODE>(o, C[i]);
  } else {
    uint4 o = xcomb<ERODE>(B[i], B[i - 1], B[i + 1], first, last);
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const uint4* pl[3] = {A, B, C};
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        if (p == 1 && dy == 0) continue;
        const int j = i + dy * pitch;
        o = comb<ERODE>(o, xcomb<ERODE>(pl[p][j], pl[p][j - 1], pl[p][j + 1], first, last));
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
  __shared__ uint4 in[3][G::IY * G::IX];
  __shared__ uint4 mid[ITER == 2 ? 3 : 1][ITER == 2 ? G::SY * G::SX : 1];
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
  auto load_plane = [&](int zv, int slot) {
#pragma unroll
    for (int k = 0; k < PERM; ++k) {
      const int i = tid + k * MT;
      if (i < NS) in[slot][i] = nzmask(pf[k]);
    }
    if (zv + 1 <= last_in) fetch(zv + 1);
  };
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
    load_plane(z0 - 1, 0);
    load_plane(z0, 1);
    for (int zo = z0; zo < z1; ++zo) {
      load_plane(zo + 1, (zo + 2 - z0) % 3);
      __syncthreads();
      const uint4* A = in[(zo - z0) % 3];
      const uint4* B = in[(zo + 1 - z0) % 3];
      const uint4* C = in[(zo + 2 - z0) % 3];
      const int r = tid / MX, q = tid % MX;
      const int gq = xc0 + q;
      store(zo, r, q, step<ERODE, SPHERE>(A, B, C, G::IX, r, q, gq == 0, gq == nxc - 1));
      __syncthreads();
    }
  } else {
    // Intermediate plane p (virtual index) is the first step evaluated at
    // clamp(p): rows/planes outside the image are copies of the border
    // row/plane.  Region rows r = 0..R1Y-1 <-> global rows y0-1+r, chunks
    // q <-> xc0-1+q; stored densely with pitch SX (= R1X).
    auto compute_mid = [&](int p, int sa, int sb, int sc) {
      uint4* M = mid[(p - (z0 - 1)) % 3];
      for (int i = tid; i < G::R1Y * G::R1X; i += MT) {
        const int r = i / G::R1X, q = i - r * G::R1X;
        const int gq = clampi(xc0 - 1 + q, nxc - 1);
        M[r * G::SX + q] = step<ERODE, SPHERE>(in[sa], in[sb], in[sc], G::IX, r, q, gq == 0, gq == nxc - 1);
      }
      __syncthreads();
      // rows of the region above / below the image repeat the border row
      for (int i = tid; i < G::R1Y * G::R1X; i += MT) {
        const int r = i / G::R1X, q = i - r * G::R1X;
        const int gy = y0 - 1 + r;
        if (gy < 0 || gy >= H) {
          const int rc = clampi(gy, H - 1) - (y0 - 1);
          M[r * G::SX + q] = M[rc * G::SX + q];
        }
      }
    };
    // input plane zv lives in in[(zv - (z0 - 2)) % 3]
    auto islot = [&](int zv) { return ((zv - (z0 - 2)) % 3 + 3) % 3; };
    auto mslot = [&](int p) { return ((p - (z0 - 1)) % 3 + 3) % 3; };
    // the intermediate at virtual plane p is the one at clamp(p): compute
    // real planes from their own (clamped) inputs, copy for virtual ones
    auto mid_for = [&](int p) {
      const int pc = clampi(p, Dz - 1);
      if (pc != p) return;  // filled by copy below
      compute_mid(p, islot(p - 1), islot(p), islot(p + 1));
    };
    auto copy_mid = [&](int to, int from) {
      uint4* Mt = mid[mslot(to)];
      const uint4* Mf = mid[mslot(from)];
      for (int i = tid; i < G::SY * G::SX; i += MT) Mt[i] = Mf[i];
    };
    // prologue: inputs z0-2 .. z0+1, intermediates z0-1 .. z0
    load_plane(z0 - 2, islot(z0 - 2));
    load_plane(z0 - 1, islot(z0 - 1));
    load_plane(z0, islot(z0));
    for (int zo = z0; zo < z1; ++zo) {
      if (zo == z0) {
        // intermediate z0-1 needs inputs z0-2..z0; intermediate z0 needs z0+1
        __syncthreads();
        if (z0 - 1 >= 0) mid_for(z0 - 1);
        __syncthreads();
        load_plane(z0 + 1, islot(z0 + 1));
        __syncthreads();
        mid_for(z0);
        __syncthreads();
        if (z0 - 1 < 0) copy_mid(z0 - 1, 0);
      }
      // intermediate zo+1 needs input zo+2 (overwrites input zo-1's slot)
      __syncthreads();
      load_plane(zo + 2, islot(zo + 2));
      __syncthreads();
      if (zo + 1 <= Dz - 1) mid_for(zo + 1);
      else copy_mid(zo + 1, Dz - 1);
      __syncthreads();
      const int r = tid / MX, q = tid % MX;
      const int gq = xc0 + q;
      // output tile (r, q) sits at (r+1, q+1) of the intermediate region
      const uint4* A = mid[mslot(zo - 1)];
      const uint4* B = mid[mslot(zo)];
      const uint4* C = mid[mslot(zo + 1)];
      store(zo, r, q, step<ERODE, SPHERE>(A, B, C, G::SX, r, q, gq == 0, gq == nxc - 1));
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
  while ((int64_t)tx * ty * chunks < 8LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
  k_morph_bytes<S, D, ERODE, SPHERE, ITER><<<grid, MT, 0, st>>>((const S*)src.ptr, (D*)dst.ptr, src.w, src.h,
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

}  // namespace

bool fast_morph_fusable(const Image& dst, const Image& src) {
  const bool bytes = (src.dt == CLK_U8 || src.dt == CLK_I8) && (dst.dt == CLK_U8 || dst.dt == CLK_I8);
  return bytes && src.ndim == 3 && src.w % 16 == 0 && ((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % 16 == 0 &&
         src.w == dst.w && src.h == dst.h && src.d == dst.d;
}

clk_status fast_morph(bool erode, bool sphere, int iterations, const Image& dst, const Image& src, const Policy&,
                      cudaStream_t st, bool planar) {
  if (!fast_morph_fusable(dst, src) || iterations < 1 || iterations > 2) return CLK_UNSUPPORTED_DTYPE;
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
