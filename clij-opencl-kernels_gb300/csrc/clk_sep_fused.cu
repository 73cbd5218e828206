// clk_sep_fused.cu - fused X -> Y -> Z separable filters: one HBM round trip
// (read src once, write dst once) instead of the reference's three launches
// with two temporaries (gaussian_blur_separable_3d_x.cl, mean_separable_3d_x.cl,
// minimum/maximum_separable_3d_x.cl, one launch per dim).
//
// Layout.  A CTA owns a TX x TY column of outputs and streams along z.  For
// every input plane it stages the (TY+2cy) x (TX+2cx) halo tile in shared
// memory (clamped coordinates = CLK_ADDRESS_CLAMP_TO_EDGE), runs the X pass
// into a row buffer, the Y pass into a ring of the last 2cz+1 planes, and,
// once the ring is full, the Z pass straight to global memory.
//
// Exactness.  Temporaries have the dst pixel type and every pass converts
// to it, so integer outputs equal three launches bit for bit; in "exact"
// mode each pass also sums in the reference's order with separately rounded
// multiply and add.  The "fast" mode (float outputs of gaussian/mean only)
// uses FMA with weights pre-divided by their sum.
#include <algorithm>

#include "clk_common.cuh"
#include "clk_sep2.cuh"

namespace clk {

namespace {

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

template <class S, class D, int OP, bool FAST, int KMAX>
__global__ void __launch_bounds__(NTHREADS, KMAX > 24 ? 1 : 2)
    k_fused_sep(const S* __restrict__ src, D* __restrict__ dst, int W, int H, int Dz, int zchunk,
                const __grid_constant__ FusedTaps taps, bool rte) {
  using T = D;  // temporaries carry the dst pixel type (float for float)
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int cx = taps.c[0], cy = taps.c[1], cz = taps.c[2];
  const int RW = TX + 2 * cx;  // staged row width
  const int RH = TY + 2 * cy;  // staged rows
  const int NZ = 2 * cz + 1;
  S* tin = reinterpret_cast<S*>(smem_raw);
  size_t off = ((size_t)RH * RW * sizeof(S) + 15) & ~size_t(15);
  T* xs = reinterpret_cast<T*>(smem_raw + off);
  off += ((size_t)RH * TX * sizeof(T) + 15) & ~size_t(15);
  T* zr = reinterpret_cast<T*>(smem_raw + off);

  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int z0 = blockIdx.z * zchunk, z1 = min(Dz, z0 + zchunk);
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

size_t fused_smem(int cx, int cy, int cz, int ssz, int tsz) {
  const int RW = TX + 2 * cx, RH = TY + 2 * cy;
  size_t b = ((size_t)RH * RW * ssz + 15) & ~size_t(15);
  b += ((size_t)RH * TX * tsz + 15) & ~size_t(15);
  b += (size_t)(2 * cz + 1) * TY * TX * tsz;
  return b;
}

template <class S, class D, int OP, bool FAST, int KMAX>
clk_status launch_fused(const Image& dst, const Image& src, const FusedTaps& ft, bool rte, cudaStream_t st) {
  const size_t smem = fused_smem(ft.c[0], ft.c[1], ft.c[2], sizeof(S), sizeof(D));
  auto kern = k_fused_sep<S, D, OP, FAST, KMAX>;
  static size_t configured = 0;  // max dynamic smem already granted to this instantiation
  if (smem > 48 * 1024 && smem > configured) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
      cudaGetLastError();
      return CLK_UNSUPPORTED_DTYPE;  // does not fit: let the caller fall back
    }
    configured = smem;
  }
  const int tiles_x = (dst.w + TX - 1) / TX, tiles_y = (dst.h + TY - 1) / TY;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // enough z-chunks that the grid fills the GPU twice over, each chunk long
  // enough that the 2cz halo planes stay a small overhead
  int chunks = 1;
  const int64_t tiles = (int64_t)tiles_x * tiles_y;
  while (tiles * chunks < 4LL * sms && dst.d / (chunks * 2) >= std::max(8, 4 * ft.c[2])) chunks *= 2;
  const int zchunk = (dst.d + chunks - 1) / chunks;
  dim3 grid(tiles_x, tiles_y, (dst.d + zchunk - 1) / zchunk);
  kern<<<grid, NTHREADS, smem, st>>>((const S*)src.ptr, (D*)dst.ptr, dst.w, dst.h, dst.d, zchunk, ft, rte);
  count_launch();
  return check_launch("fused separable");
}

template <class S, class D, int OP, bool FAST>
clk_status launch_bucket(const Image& dst, const Image& src, const FusedTaps& ft, bool rte, cudaStream_t st) {
  const int n = 2 * std::max(ft.c[0], ft.c[1]) + 1;
  if (n <= 12) return launch_fused<S, D, OP, FAST, 12>(dst, src, ft, rte, st);
  if (n <= 24) return launch_fused<S, D, OP, FAST, 24>(dst, src, ft, rte, st);
  return launch_fused<S, D, OP, FAST, 2 * kFusedMaxR + 1>(dst, src, ft, rte, st);
}

template <class S, class D>
clk_status launch_types(SepOp op, bool fast, const Image& dst, const Image& src, const FusedTaps& ft, bool rte,
                        cudaStream_t st) {
  switch (op) {
    case SEP_GAUSS:
      if constexpr (sizeof(D) == 4) {
        if (fast) return launch_bucket<S, D, SEP_GAUSS, true>(dst, src, ft, rte, st);
      }
      return launch_bucket<S, D, SEP_GAUSS, false>(dst, src, ft, rte, st);
    case SEP_MEAN: return launch_bucket<S, D, SEP_MEAN, false>(dst, src, ft, rte, st);
    case SEP_MIN: return launch_bucket<S, D, SEP_MIN, false>(dst, src, ft, rte, st);
    case SEP_MAX: return launch_bucket<S, D, SEP_MAX, false>(dst, src, ft, rte, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace

clk_status fused_separable(SepOp op, const Image& dst, const Image& src, const SepTaps taps[3], const bool skip[3],
                           const Policy& p, cudaStream_t st) {
  FusedTaps ft;
  const bool fast = op == SEP_GAUSS && dst.dt == CLK_F32 && !p.exact_order;
  for (int d = 0; d < 3; ++d) {
    const bool sk = skip[d] || (d == 2 && src.ndim == 2);
    const int c = sk ? 0 : taps[d].c;
    if (c < 0 || c > kFusedMaxR) return CLK_UNSUPPORTED_DTYPE;
    ft.c[d] = c;
    if (sk || op != SEP_GAUSS) {
      ft.h[d][0] = 1.0f;  // one tap: a converting copy (copy_3d_x.cl:13-14)
      ft.hsum[d] = 1.0f;
      continue;
    }
    if (fast) {
      double s = 0;
      for (int v = 0; v <= 2 * c; ++v) s += taps[d].h[v];
      for (int v = 0; v <= 2 * c; ++v) ft.h[d][v] = (float)(taps[d].h[v] / s);
      ft.hsum[d] = 1.0f;
    } else {
      for (int v = 0; v <= 2 * c; ++v) ft.h[d][v] = taps[d].h[v];
      ft.hsum[d] = taps[d].hsum;
    }
  }
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  // Isotropic XY radius: the register-window kernels (clk_sep2.cuh).
  if (ft.c[0] == ft.c[1] && ft.c[0] >= 1) {
    const int R = ft.c[0], cz = ft.c[2];
    const bool ints = src.dt == dst.dt && src.dt != CLK_F32;
    clk_status s2 = CLK_UNSUPPORTED_DTYPE;
    if ((op == SEP_MIN || op == SEP_MAX) && ints) {
      s2 = sep2_minmax(op == SEP_MAX, R, dst, src, cz, st);
    } else if (op == SEP_MEAN && ints) {
      s2 = sep2_mean(R, dst, src, cz, st);
    } else if (fast) {
      // folded taps: w[0] for the centre, w[k] for the pair +-k, all / sum(h)
      float w[3][kFusedMaxR + 1] = {};
      for (int d = 0; d < 3; ++d) {
        const int c = ft.c[d];
        double sum = 0;
        for (int v = 0; v <= 2 * c; ++v) sum += ft.h[d][v];
        for (int k = 0; k <= c; ++k) w[d][k] = (float)(ft.h[d][c + k] / sum);
      }
      s2 = sep2_gauss(R, dst, src, w[0], w[1], w[2], cz, st);
    }
    if (s2 != CLK_UNSUPPORTED_DTYPE) return s2;
  }
  if (fused_smem(ft.c[0], ft.c[1], ft.c[2], dtype_size(src.dt), dtype_size(dst.dt)) > 200 * 1024)
    return CLK_UNSUPPORTED_DTYPE;
  const int s = src.dt, d = dst.dt;
  if (s == d) {
    switch (s) {
      case CLK_U8: return launch_types<uint8_t, uint8_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I8: return launch_types<int8_t, int8_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_U16: return launch_types<uint16_t, uint16_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I16: return launch_types<int16_t, int16_t>(op, fast, dst, src, ft, p.rte, st);
      case CLK_F32: return launch_types<float, float>(op, fast, dst, src, ft, p.rte, st);
    }
  } else if (d == CLK_F32) {
    switch (s) {
      case CLK_U8: return launch_types<uint8_t, float>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I8: return launch_types<int8_t, float>(op, fast, dst, src, ft, p.rte, st);
      case CLK_U16: return launch_types<uint16_t, float>(op, fast, dst, src, ft, p.rte, st);
      case CLK_I16: return launch_types<int16_t, float>(op, fast, dst, src, ft, p.rte, st);
    }
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
