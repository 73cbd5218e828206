// clk_morph_bits.cu - binary erode/dilate (box 3x3x3 and the 7-point
// "sphere" cross, erode_box_3d_x.cl:14-37, erode_sphere_3d_x.cl:14-37,
// dilate_box_3d_x.cl:14-37, dilate_sphere_3d_x.cl:14-38) on byte images
// whose rows are whole 32-voxel words, one or two iterations per pass.
//
// The same results as the byte-mask kernels of clk_morph.cu (1 where the
// condition holds, 0 elsewhere; two iterations with the two-launch clamp
// semantics), with the masks packed 32 voxels to a word: bit k of word w
// of a row is voxel 32w + k nonzero.  A thread converts 32 input bytes to a
// word (the high bit of each byte set where it is nonzero, gathered by one
// multiply per four voxels), the stencil is word-wide AND / OR with the x
// neighbours shifted in from the adjacent words (at the image's first and
// last voxel the clamped neighbour is the voxel itself), and each output
// word expands back to 32 bytes of 0/1 by one multiply per four voxels.
// Shared memory then moves 4 bytes per 32 voxels and step instead of 16
// bytes per 16, so the fused radius 2 costs about what radius 1 does.
//
// Layout: a CTA owns NW words (8: 256 voxels) x TY rows (32) and streams
// along z; the staged input planes carry one halo word left and right and
// ITER halo rows above and below; phase j stages input plane j + 2*ITER
// (prefetched into registers one phase earlier) and filters; one barrier
// per phase.
#include "clk_common.cuh"

namespace clk {

namespace {

constexpr int NW = 8;    // words (32 voxels) per tile row
constexpr int TY = 32;   // rows per tile
constexpr int NT = 256;  // threads

// bit k = byte k of the 4-byte word v nonzero, k = 0..3
__device__ __forceinline__ uint32_t nz4(uint32_t v) {
  const uint32_t t = (((v & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | v) & 0x80808080u;  // bit 7 of each byte: nonzero
  return (t * 0x00204081u) >> 28;                                          // bits 7, 15, 23, 31 -> 28..31
}
// 32 bytes (two 16-byte vectors, x fastest) -> one mask word
__device__ __forceinline__ uint32_t pack32(uint4 a, uint4 b) {
  const uint32_t w[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) m |= nz4(w[k]) << (4 * k);
  return m;
}
// bits 4k .. 4k+3 of m -> four bytes of 0 / 1
__device__ __forceinline__ uint32_t unpack4(uint32_t m, int k) { return ((m >> (4 * k)) & 15u) * 0x00204081u & 0x01010101u; }

template <bool ERODE> __device__ __forceinline__ uint32_t comb(uint32_t a, uint32_t b) { return ERODE ? a & b : a | b; }

// x-neighbour combination of word j of a staged row P (with its left and
// right words); first / last: the word is the image row's first / last
template <bool ERODE>
__device__ __forceinline__ uint32_t xcomb(const uint32_t* P, int j, bool first, bool last) {
  const uint32_t c = P[j];
  const uint32_t lb = first ? (c & 1u) : (P[j - 1] >> 31);
  const uint32_t rb = last ? (c >> 31) : (P[j + 1] & 1u);
  return comb<ERODE>(comb<ERODE>(c, (c << 1) | lb), (c >> 1) | (rb << 31));
}

// One r=1 step at word i of planes A (z-1), B (z), C (z+1), row pitch `pitch`
template <bool ERODE, bool SPHERE>
__device__ __forceinline__ uint32_t step(const uint32_t* A, const uint32_t* B, const uint32_t* C, int pitch, int i,
                                         bool first, bool last) {
  if constexpr (SPHERE) {
    uint32_t o = xcomb<ERODE>(B, i, first, last);
    o = comb<ERODE>(o, B[i - pitch]);
    o = comb<ERODE>(o, B[i + pitch]);
    o = comb<ERODE>(o, A[i]);
    return comb<ERODE>(o, C[i]);
  } else {
    uint32_t o = xcomb<ERODE>(B, i, first, last);
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const uint32_t* pl[3] = {A, B, C};
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        if (p == 1 && dy == 0) continue;
        o = comb<ERODE>(o, xcomb<ERODE>(pl[p], i + dy * pitch, first, last));
      }
    }
    return o;
  }
}

template <int ITER> struct Geo {
  static constexpr int R1X = ITER == 2 ? NW + 2 : NW;  // region of the first step (words)
  static constexpr int R1Y = ITER == 2 ? TY + 2 : TY;
  static constexpr int IX = R1X + 2, IY = R1Y + 2;    // staged input planes
  static constexpr int SX = NW + 2, SY = TY + 2;      // intermediate planes
  static constexpr int NS = IX * IY, PER = (NS + NT - 1) / NT;
  static constexpr int MS = SX * SY;
};

template <class D, bool ERODE, bool SPHERE, int ITER>
__global__ void __launch_bounds__(NT)
    k_morph_bits(const uint8_t* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz, int zchunk) {
  using G = Geo<ITER>;
  __shared__ uint32_t in[4][G::NS];
  __shared__ uint32_t mid[ITER == 2 ? 4 : 1][ITER == 2 ? G::MS : 1];
  const int nxw = W / 32;
  const int w0 = blockIdx.x * NW, y0 = blockIdx.y * TY;
  const int z0 = blockIdx.z * zchunk, z1 = min(Dz, z0 + zchunk);
  const int tid = threadIdx.x;
  const size_t plane = (size_t)W * H;
  const int hy = ITER;  // halo rows of the staged input above / below the tile (one halo word left / right per step)

  // staging tasks (the same for every plane): byte offset of each staged
  // word's 32 bytes inside a plane (rows and words clamped)
  uint32_t goff[G::PER];
#pragma unroll
  for (int k = 0; k < G::PER; ++k) {
    const int i = tid + k * NT;
    goff[k] = 0;
    if (i < G::NS) {
      const int r = i / G::IX, q = i - r * G::IX;
      const int gy = clampi(y0 - hy + r, H - 1), gw = clampi(w0 - (G::IX - NW) / 2 + q, nxw - 1);
      goff[k] = (uint32_t)gy * (uint32_t)W + (uint32_t)gw * 32u;
    }
  }
  const int last_in = z1 - 1 + ITER;
  uint4 pa[G::PER], pb[G::PER];
  auto fetch = [&](int zv) {
    const uint8_t* sp = src + (size_t)clampi(zv, Dz - 1) * plane;
#pragma unroll
    for (int k = 0; k < G::PER; ++k) {
      if (tid + k * NT < G::NS) {
        const uint4* v = reinterpret_cast<const uint4*>(sp + goff[k]);
        pa[k] = __ldg(v);
        pb[k] = __ldg(v + 1);
      }
    }
  };
  auto stage = [&](int zv, uint32_t* to) {
#pragma unroll
    for (int k = 0; k < G::PER; ++k) {
      const int i = tid + k * NT;
      if (i < G::NS) to[i] = pack32(pa[k], pb[k]);
    }
    if (zv + 1 <= last_in) fetch(zv + 1);
  };
  fetch(z0 - ITER);

  // output word (r, q) of the tile; a warp owns rows 4w .. 4w+3 of it
  const int orow = tid / NW, oq = tid % NW;
  const int ogw = w0 + oq;
  const bool ofirst = ogw == 0, olast = ogw == nxw - 1;
  // Each store instruction of a warp writes two whole 256-byte row segments
  // of the warp's four output rows: lane l writes 16-byte chunk l % 16 of
  // row 2k + l / 16 and takes the mask word holding it from the lane that
  // computed it (one shuffle per instruction).  A thread writing its own 32
  // bytes would cover half of each 128-byte line per instruction, which
  // halves the rate of stores into host-mapped memory (measured: 80 against
  // 190 GB/s over the host link).
  const int lane = tid & 31, warp = tid >> 5;
  auto store = [&](int zo, uint32_t m) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int rw = 2 * k + lane / 16, c = lane % 16;  // row of the warp's four, chunk of that row
      const uint32_t v = __shfl_sync(0xFFFFFFFFu, m, 8 * rw + c / 2) >> (16 * (c & 1));
      const int gy = y0 + 4 * warp + rw, gw = w0 + c / 2;
      if (gy < H && gw < nxw)
        *reinterpret_cast<uint4*>(dst + (size_t)zo * plane + (size_t)gy * W + (size_t)w0 * 32 + c * 16) =
            make_uint4(unpack4(v, 0), unpack4(v, 1), unpack4(v, 2), unpack4(v, 3));
    }
  };

  if constexpr (ITER == 1) {
    // phase j stages input j+2 and filters output plane j from inputs
    // j-1 .. j+1: a ring of four input planes (plane p in slot p & 3)
    const int i = (orow + 1) * G::IX + (oq + 1);
    for (int j = z0 - 3; j < z1; ++j) {
      if (j + 2 <= last_in) stage(j + 2, in[(j + 2) & 3]);
      if (j >= z0) store(j, step<ERODE, SPHERE>(in[(j - 1) & 3], in[j & 3], in[(j + 1) & 3], G::IX, i, ofirst, olast));
      __syncthreads();
    }
  } else {
    // phase j stages input j+4, computes the intermediate (first step) at
    // plane j+2 from inputs j+1 .. j+3 and filters output plane j from the
    // intermediates j-1 .. j+1: rings of four input and four intermediate
    // planes.  The intermediate at a virtual position is the one at the
    // clamped position: rows outside the image evaluate the first step at
    // the clamped row; plane -1 (Dz) is a copy of plane 0 (Dz - 1), made in
    // the phase after that plane is computed.  Intermediate region rows
    // r = 0..R1Y-1 <-> rows y0-1+r, words q <-> w0-1+q.
    for (int j = z0 - 6; j < z1; ++j) {
      if (j + 4 <= last_in) stage(j + 4, in[(j + 4) & 3]);
      const int pm = j + 2;
      if (pm >= z0 - 1 && pm <= z1) {
        uint32_t* M = mid[pm & 3];
        if (pm >= 0 && pm < Dz) {
          for (int t = tid; t < G::R1Y * G::R1X; t += NT) {
            const int r = t / G::R1X, q = t - r * G::R1X;
            const int gy = y0 - 1 + r;
            const int rr = r + (clampi(gy, H - 1) - gy);
            const int gw = w0 - 1 + q;
            M[r * G::SX + q] = step<ERODE, SPHERE>(in[(pm - 1) & 3], in[pm & 3], in[(pm + 1) & 3], G::IX,
                                                   (rr + 1) * G::IX + (q + 1), gw <= 0, gw >= nxw - 1);
          }
        } else if (pm >= Dz) {  // plane Dz: copy of Dz - 1 (computed in the previous phase)
          const uint32_t* Mf = mid[(Dz - 1) & 3];
          for (int t = tid; t < G::MS; t += NT) M[t] = Mf[t];
        }
      }
      if (j == -1 && z0 == 0) {  // plane -1: copy of plane 0 (computed in the previous phase)
        const uint32_t* Mf = mid[0];
        uint32_t* Mt = mid[3];
        for (int t = tid; t < G::MS; t += NT) Mt[t] = Mf[t];
      }
      if (j >= z0)
        store(j, step<ERODE, SPHERE>(mid[(j - 1) & 3], mid[j & 3], mid[(j + 1) & 3], G::SX,
                                     (orow + 1) * G::SX + (oq + 1), ofirst, olast));
      __syncthreads();
    }
  }
}

template <class D, bool ERODE, bool SPHERE, int ITER>
clk_status launch_bits(const Image& dst, const Image& src, cudaStream_t st) {
  const int nxw = src.w / 32;
  const int tx = (nxw + NW - 1) / NW, ty = (src.h + TY - 1) / TY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // z-chunks: about eight CTAs per SM in flight, chunks of at least 16 planes
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 8LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
  k_morph_bits<D, ERODE, SPHERE, ITER><<<grid, NT, 0, st>>>((const uint8_t*)src.ptr, (D*)dst.ptr, src.w, src.h,
                                                             src.d, zchunk);
  count_launch();
  return check_launch("morphology (bit words)");
}

template <bool ERODE, bool SPHERE, int ITER>
clk_status sel_dst(const Image& dst, const Image& src, cudaStream_t st) {
  return dst.dt == CLK_U8 ? launch_bits<uint8_t, ERODE, SPHERE, ITER>(dst, src, st)
                          : launch_bits<int8_t, ERODE, SPHERE, ITER>(dst, src, st);
}

}  // namespace

// 8-bit 3-D images whose rows are whole words (W % 32 == 0), 16-byte
// aligned, one or two iterations; CLK_UNSUPPORTED_DTYPE otherwise (the byte
// kernels take those).  The nonzero test reads bytes, so signed and
// unsigned pixels are the same here.
clk_status morph_bits(bool erode, bool sphere, int iterations, const Image& dst, const Image& src, cudaStream_t st) {
  const bool bytes = (src.dt == CLK_U8 || src.dt == CLK_I8) && (dst.dt == CLK_U8 || dst.dt == CLK_I8);
  if (!bytes || src.ndim != 3 || src.w % 32 != 0 || ((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % 16 != 0 ||
      src.w != dst.w || src.h != dst.h || src.d != dst.d || iterations < 1 || iterations > 2 ||
      (int64_t)src.w * src.h >= (1LL << 32))
    return CLK_UNSUPPORTED_DTYPE;
  const int sel = (erode ? 4 : 0) | (sphere ? 2 : 0) | (iterations == 2 ? 1 : 0);
  switch (sel) {
    case 0: return sel_dst<false, false, 1>(dst, src, st);
    case 1: return sel_dst<false, false, 2>(dst, src, st);
    case 2: return sel_dst<false, true, 1>(dst, src, st);
    case 3: return sel_dst<false, true, 2>(dst, src, st);
    case 4: return sel_dst<true, false, 1>(dst, src, st);
    case 5: return sel_dst<true, false, 2>(dst, src, st);
    case 6: return sel_dst<true, true, 1>(dst, src, st);
    case 7: return sel_dst<true, true, 2>(dst, src, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
