// clk_fused_impl.cuh - the generic fused X -> Y -> Z separable kernel (runtime
// radii up to 31, reference-order arithmetic for integer outputs); see
// clk_sep_fused.cu for the layout.  Shared by the plain launcher and the
// batch engine.
#pragma once
#include "clk_common.cuh"

namespace clk {
namespace fused {

constexpr int TX = 64, TY = 16, NTHREADS = 256, P = 4;
constexpr int kFusedMaxR = 31;  // per-axis radius limit of the fused path

struct FusedTaps {
  float h[3][2 * kFusedMaxR + 1];  // per-axis taps (exact: h; fast: h / hsum)
  float hsum[3];                    // exact mode: divisor of each pass
  int c[3];                         // radius per axis
};

template <class D> struct TempT { typedef D type; };

template <int OP> __device__ __forceinline__ float op_init(float center) {
  return (OP == SEP_MIN || OP == SEP_MAX) ? center : 0.f;
}

// One pass over a register window buf[j + v], v = 0..2c, for P outputs.
// ctr[j] is the window's centre (min/max start from it, as the kernels do);
// it is passed separately because c is a runtime value and indexing buf with
// it would move the window out of registers.
template <int OP, bool FAST, int KMAX>
__device__ __forceinline__ void pass_window(const float (&buf)[KMAX + P - 1], const float (&ctr)[P], int c,
                                            const float* __restrict__ h, float hsum, float (&out)[P]) {
  const int n = 2 * c + 1;
#pragma unroll
  for (int j = 0; j < P; ++j) out[j] = op_init<OP>(ctr[j]);
#pragma unroll
  for (int v = 0; v < KMAX; ++v) {
    if (v < n) {
#pragma unroll
      for (int j = 0; j < P; ++j) {
        const float x = buf[j + v];
        if constexpr (OP == SEP_GAUSS) {
          out[j] = FAST ? fmaf(h[v], x, out[j]) : __fadd_rn(out[j], __fmul_rn(h[v], x));
        } else if constexpr (OP == SEP_MEAN) {
          out[j] = __fadd_rn(out[j], x);
        } else if constexpr (OP == SEP_MIN) {
          out[j] = x < out[j] ? x : out[j];
        } else {
          out[j] = out[j] < x ? x : out[j];
        }
      }
    }
  }
  if constexpr (OP == SEP_GAUSS) {
    if (!FAST) {
#pragma unroll
      for (int j = 0; j < P; ++j) out[j] = __fdiv_rn(out[j], hsum);
    }
  } else if constexpr (OP == SEP_MEAN) {
#pragma unroll
    for (int j = 0; j < P; ++j) out[j] = __fdiv_rn(out[j], (float)n);
  }
}

template <class T> __device__ __forceinline__ T to_temp(float v, bool rte) { return convert_sat<T>(v, rte); }

// One tile (bx, by) x z-chunk bz of one image; the whole CTA takes part.
template <class S, class D, int OP, bool FAST, int KMAX>
__device__ __forceinline__ void fused_tile(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz,
                                           int zchunk, const FusedTaps& taps, bool rte, int bx, int by, int bz,
                                           unsigned char* smem_raw) {
  using T = D;  // temporaries carry the dst pixel type (float for float)
  const int cx = taps.c[0], cy = taps.c[1], cz = taps.c[2];
  const int RW = TX + 2 * cx;  // staged row width
  const int RH = TY + 2 * cy;  // staged rows
  const int NZ = 2 * cz + 1;
  S* tin = reinterpret_cast<S*>(smem_raw);
  size_t off = ((size_t)RH * RW * sizeof(S) + 15) & ~size_t(15);
  T* xs = reinterpret_cast<T*>(smem_raw + off);
  off += ((size_t)RH * TX * sizeof(T) + 15) & ~size_t(15);
  T* zr = reinterpret_cast<T*>(smem_raw + off);

  const int x0 = bx * TX, y0 = by * TY;
  const int z0 = bz * zchunk, z1 = min(Dz, z0 + zchunk);
  const int tid = threadIdx.x;
  // Y / Z pass ownership: column x = tid % TX, rows yq .. yq+P-1
  const int ox = tid % TX, oy = (tid / TX) * P;
  const int64_t plane = (int64_t)W * H;
  const int warp = tid / 32, lane = tid % 32;
  int wslot = 0;  // ring slot of the plane staged in this iteration

  for (int zi = z0 - cz; zi < z1 + cz; ++zi) {
    const int zc = clampi(zi, Dz - 1);
    // ---- stage the clamped halo tile of plane zc (a warp per row)
    const S* sp = src + (int64_t)zc * plane;
    for (int r = warp; r < RH; r += NTHREADS / 32) {
      const S* srow = sp + (int64_t)clampi(y0 - cy + r, H - 1) * W;
      for (int q = lane; q < RW; q += 32) tin[r * RW + q] = __ldg(srow + clampi(x0 - cx + q, W - 1));
    }
    __syncthreads();
    // ---- X pass: RH rows x TX outputs, strips of P along x
    for (int s = tid; s < RH * (TX / P); s += NTHREADS) {
      const int r = s / (TX / P), xq = (s % (TX / P)) * P;
      float buf[KMAX + P - 1];
      const S* row = tin + r * RW + xq;
#pragma unroll
      for (int k = 0; k < KMAX + P - 1; ++k)
        if (k < 2 * cx + P) buf[k] = (float)row[k];
      float ctr[P], out[P];
#pragma unroll
      for (int j = 0; j < P; ++j) ctr[j] = (float)row[cx + j];
      pass_window<OP, FAST, KMAX>(buf, ctr, cx, taps.h[0], taps.hsum[0], out);
#pragma unroll
      for (int j = 0; j < P; ++j) xs[r * TX + xq + j] = to_temp<T>(out[j], rte);
    }
    __syncthreads();
    // ---- Y pass: TY x TX outputs, strips of P along y -> ring slot
    {
      float buf[KMAX + P - 1];
#pragma unroll
      for (int k = 0; k < KMAX + P - 1; ++k)
        if (k < 2 * cy + P) buf[k] = (float)xs[(oy + k) * TX + ox];
      float ctr[P], out[P];
#pragma unroll
      for (int j = 0; j < P; ++j) ctr[j] = (float)xs[(oy + j + cy) * TX + ox];
      pass_window<OP, FAST, KMAX>(buf, ctr, cy, taps.h[1], taps.hsum[1], out);
#pragma unroll
      for (int j = 0; j < P; ++j) zr[((size_t)wslot * TY + oy + j) * TX + ox] = to_temp<T>(out[j], rte);
    }
    __syncthreads();
    // ---- Z pass for output plane zo once the ring holds zo-cz .. zo+cz;
    // the oldest of them (zo - cz) sits in the slot after the newest
    const int zo = zi - cz;
    const int oldest = wslot + 1 == NZ ? 0 : wslot + 1;
    wslot = oldest;
    if (zo >= z0) {
      const int gx = x0 + ox;
      const int centre = oldest + cz >= NZ ? oldest + cz - NZ : oldest + cz;
#pragma unroll
      for (int j = 0; j < P; ++j) {
        const int gy = y0 + oy + j;
        const int cell = (oy + j) * TX + ox;
        float acc = op_init<OP>((float)zr[(size_t)centre * TY * TX + cell]);
        int idx = oldest;
        for (int v = 0; v < NZ; ++v) {
          const float x = (float)zr[(size_t)idx * TY * TX + cell];
          idx = idx + 1 == NZ ? 0 : idx + 1;
          if constexpr (OP == SEP_GAUSS) {
            acc = FAST ? fmaf(taps.h[2][v], x, acc) : __fadd_rn(acc, __fmul_rn(taps.h[2][v], x));
          } else if constexpr (OP == SEP_MEAN) {
            acc = __fadd_rn(acc, x);
          } else if constexpr (OP == SEP_MIN) {
            acc = x < acc ? x : acc;
          } else {
            acc = acc < x ? x : acc;
          }
        }
        if constexpr (OP == SEP_GAUSS) {
          if (!FAST) acc = __fdiv_rn(acc, taps.hsum[2]);
        } else if constexpr (OP == SEP_MEAN) {
          acc = __fdiv_rn(acc, (float)NZ);
        }
        if (gx < W && gy < H) dst[(int64_t)zo * plane + (int64_t)gy * W + gx] = convert_sat<D>(acc, rte);
      }
    }
  }
}

template <class S, class D, int OP, bool FAST, int KMAX>
__global__ void __launch_bounds__(NTHREADS, KMAX > 24 ? 1 : 2)
    k_fused_sep(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz, int zchunk,
                const __grid_constant__ FusedTaps taps, bool rte) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  fused_tile<S, D, OP, FAST, KMAX>(src, dst, W, H, Dz, zchunk, taps, rte, blockIdx.x, blockIdx.y, blockIdx.z,
                                   smem_raw);
}

inline size_t fused_smem(int cx, int cy, int cz, int ssz, int tsz) {
  const int RW = TX + 2 * cx, RH = TY + 2 * cy;
  size_t b = ((size_t)RH * RW * ssz + 15) & ~size_t(15);
  b += ((size_t)RH * TX * tsz + 15) & ~size_t(15);
  b += (size_t)(2 * cz + 1) * TY * TX * tsz;
  return b;
}

}  // namespace fused
}  // namespace clk
