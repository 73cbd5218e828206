// clk_direct.cu - generic kernels: one thread per output voxel, every
// pixel-type pair, float arithmetic in the reference's own order with
// explicitly rounded operations (__fmul_rn / __fadd_rn never contract into
// FMA), so their results are bit-identical to the reference's.  They back
// clk_execute's single-pass drop-in and every case the fused fast paths do
// not cover.
#include <type_traits>

#include "clk_common.cuh"

namespace clk {

namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ void decode(int64_t i, const Range& r, int& x, int& y, int& z) {
  const int64_t xy = (int64_t)r.x * r.y;
  z = (int)(i / xy);
  const int64_t rem = i - (int64_t)z * xy;
  y = (int)(rem / r.x);
  x = (int)(rem - (int64_t)y * r.x);
}

inline unsigned grid_for(int64_t n) {
  const int64_t g = (n + kBlock - 1) / kBlock;
  return (unsigned)(g < 152 * 64 ? (g < 1 ? 1 : g) : 152 * 64);
}

// One separable pass (gaussian_blur_separable_3d_x.cl:14-34,
// mean_separable_3d_x.cl:12-29, minimum/maximum_separable_3d_x.cl:12-23).
template <class S, class D, int OP>
__global__ void __launch_bounds__(kBlock)
    k_sep_pass(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, int dim,
               const __grid_constant__ SepTaps taps, bool rte) {
  const int dx = dim == 0, dy = dim == 1, dz = dim == 2;
  const int c = taps.c;
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    float res;
    if constexpr (OP == SEP_GAUSS) {
      res = 0.f;
      for (int v = -c; v <= c; ++v)
        res = __fadd_rn(res, __fmul_rn(taps.h[v + c], ldf(src, atc(sd, x + v * dx, y + v * dy, z + v * dz))));
      res = __fdiv_rn(res, taps.hsum);
    } else if constexpr (OP == SEP_MEAN) {
      res = 0.f;
      for (int v = -c; v <= c; ++v) res = __fadd_rn(res, ldf(src, atc(sd, x + v * dx, y + v * dy, z + v * dz)));
      res = __fdiv_rn(res, c >= 0 ? (float)(2 * c + 1) : 0.f);
    } else {
      res = ldf(src, atc(sd, x, y, z));
      for (int v = -c; v <= c; ++v) {
        const float t = ldf(src, atc(sd, x + v * dx, y + v * dy, z + v * dz));
        if constexpr (OP == SEP_MIN) res = t < res ? t : res;
        else res = res < t ? t : res;
      }
    }
    dst[at(dd, x, y, z)] = convert_sat<D>(res, rte);
  }
}

// copy_3d_x.cl:13-14: float through, then CONVERT.
template <class S, class D>
__global__ void __launch_bounds__(kBlock)
    k_copy(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool rte) {
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    dst[at(dd, x, y, z)] = convert_sat<D>(ldf(src, atc(sd, x, y, z)), rte);
  }
}

// median_box/sphere (median_box_3d_x.cl:3-20,41-64): gather, stable
// insertion sort, element n/2.
template <class T, int CAP>
__global__ void __launch_bounds__(kBlock)
    k_median(T* __restrict__ dst, const T* __restrict__ src, Dims3 sd, Dims3 dd, Range r,
             const __grid_constant__ MedianNbhd m) {
  T a[CAP];
  const int n = m.n;
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    for (int k = 0; k < n; ++k) {
      const char4 o = m.off[k];
      a[k] = __ldg(src + atc(sd, x + o.x, y + o.y, z + o.z));
    }
    for (int k = 1; k < n; ++k) {
      const T t = a[k];
      int j = k - 1;
      while (j >= 0 && t < a[j]) {
        a[j + 1] = a[j];
        --j;
      }
      a[j + 1] = t;
    }
    dst[at(dd, x, y, z)] = a[n / 2];
  }
}

// READ(..).x * -1 in the read's own type: for the uint reads of unsigned
// pixels the product wraps to 2^32 - v (0 stays 0), as the reference's does
template <class V> __device__ __forceinline__ V times_minus_one(V v) { return v * (V)-1; }

// .x of a read: uint for unsigned pixels, int for signed, float for float
template <class S> __device__ __forceinline__ auto readx(const S* p, int64_t i) {
  const S t = __ldg(p + i);
  if constexpr (std::is_same<S, float>::value) return t;
  else if constexpr (std::is_signed<S>::value) return (int)t;
  else return (unsigned)t;
}

// minimum/maximum/mean over the sphere offsets in loop order (x, y, z):
// minimum/maximum_sphere_3d_x.cl:15-49 (RANK_FLOAT: float running value,
// CONVERT at the end), maximum_sphere_2d_x.cl:16-45 and
// minimum/maximum_slice_by_slice_sphere_3d_x.cl:15-38 (RANK_CONVERT: dst-typed
// value, CONVERT of every read), minimum_sphere_2d_x.cl:16-47 (RANK_CAST: the
// reads C-cast to the dst type), mean_sphere_{2d,3d}_x.cl and
// mean_slice_by_slice_sphere_3d_x.cl (float sum in loop order,
// CONVERT(sum / count)).
template <class S, class D, int OP, int MODE>
__global__ void __launch_bounds__(kBlock)
    k_rank(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r,
           const __grid_constant__ MedianNbhd m, bool rte) {
  const int n = m.n;
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    D res;
    if constexpr (OP == RANK_MEAN) {
      float sum = 0.f;
      for (int k = 0; k < n; ++k) {
        const char4 o = m.off[k];
        sum = __fadd_rn(sum, (float)readx(src, atc(sd, x + o.x, y + o.y, z + o.z)));
      }
      res = convert_sat<D>(__fdiv_rn(sum, (float)n), rte);
    } else if constexpr (MODE == RANK_FLOAT) {
      float v = (float)readx(src, atc(sd, x, y, z));
      for (int k = 0; k < n; ++k) {
        const char4 o = m.off[k];
        const float t = (float)readx(src, atc(sd, x + o.x, y + o.y, z + o.z));
        if (OP == RANK_MIN ? t < v : t > v) v = t;
      }
      res = convert_sat<D>(v, rte);
    } else {
      D v = convert_sat<D>((float)readx(src, atc(sd, x, y, z)), rte);
      for (int k = 0; k < n; ++k) {
        const char4 o = m.off[k];
        const auto rv = readx(src, atc(sd, x + o.x, y + o.y, z + o.z));
        const D t = MODE == RANK_CAST ? (D)rv : convert_sat<D>((float)rv, rte);
        if (OP == RANK_MIN ? t < v : t > v) v = t;
      }
      res = v;
    }
    dst[at(dd, x, y, z)] = res;
  }
}

// gradient_{x,y,z}_{2d,3d}_x.cl: CONVERT(READ(+1).x - READ(-1).x) in float.
template <class S, class D, int AXIS>
__global__ void __launch_bounds__(kBlock)
    k_gradient(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool rte) {
  constexpr int dx = AXIS == 0, dy = AXIS == 1, dz = AXIS == 2;
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    const float a = (float)readx(src, atc(sd, x - dx, y - dy, z - dz));
    const float b = (float)readx(src, atc(sd, x + dx, y + dy, z + dz));
    dst[at(dd, x, y, z)] = convert_sat<D>(__fsub_rn(b, a), rte);
  }
}

// laplace_diamond_{2d,3d}_x.cl, laplace_box_2d_x.cl: centre * K + each
// neighbour * -1.0 in the expression's order, in double (the literals are
// double), stored to float, converted.  KIND: 0 diamond 2-D, 1 diamond 3-D,
// 2 box 2-D.
template <class S, class D, int KIND>
__global__ void __launch_bounds__(kBlock)
    k_laplace_expr(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool rte) {
  constexpr int NB = KIND == 0 ? 4 : KIND == 1 ? 6 : 8;
  constexpr double K = KIND == 0 ? 4.0 : KIND == 1 ? 6.0 : 8.0;
  // right, left, top, bottom, then front, back (3-D) or the corners A..D
  constexpr signed char ox[8] = {1, -1, 0, 0, KIND == 1 ? 0 : -1, KIND == 1 ? 0 : 1, -1, 1};
  constexpr signed char oy[8] = {0, 0, -1, 1, KIND == 1 ? 0 : -1, KIND == 1 ? 0 : -1, 1, 1};
  constexpr signed char oz[8] = {0, 0, 0, 0, KIND == 1 ? 1 : 0, KIND == 1 ? -1 : 0, 0, 0};
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    float res;
    if constexpr (std::is_integral<S>::value) {
      // integer pixels: every partial sum is an integer far below 2^53, so the
      // double evaluation is exact and equals this int32 sum
      int acc = (int)readx(src, atc(sd, x, y, z)) * (int)K;
#pragma unroll
      for (int k = 0; k < NB; ++k) acc -= (int)readx(src, atc(sd, x + ox[k], y + oy[k], z + oz[k]));
      res = (float)acc;
    } else {
      double acc = __dmul_rn((double)(float)readx(src, atc(sd, x, y, z)), K);
#pragma unroll
      for (int k = 0; k < NB; ++k)
        acc = __dadd_rn(acc, __dmul_rn((double)(float)readx(src, atc(sd, x + ox[k], y + oy[k], z + oz[k])), -1.0));
      res = __double2float_rn(acc);
    }
    dst[at(dd, x, y, z)] = convert_sat<D>(res, rte);
  }
}

// laplace_box_3d_x.cl:13-25: float result over ax, ay, az; the centre adds
// READ(..).x, the other taps READ(..).x * -1, which wraps for the uint reads
// of unsigned pixels (2^32 - v).
template <class S, class D>
__global__ void __launch_bounds__(kBlock)
    k_laplace_box3d(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool rte) {
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    float result = 0.f;
    for (int ax = -1; ax <= 1; ++ax)
      for (int ay = -1; ay <= 1; ++ay)
        for (int az = -1; az <= 1; ++az) {
          const auto v = readx(src, atc(sd, x + ax, y + ay, z + az));
          result = __fadd_rn(result, (ax == 0 && ay == 0 && az == 0) ? (float)v : (float)times_minus_one(v));
        }
    dst[at(dd, x, y, z)] = convert_sat<D>(result, rte);
  }
}

// The same sum over whole images, tiled: a CTA owns 128 x 8 outputs of a
// z-chunk; each staged input plane holds t(v) = (float)(v * -1) of every
// pixel of the (8+2) x (128+2) halo region once (the conversion that the
// per-voxel kernel repeats for 26 taps); a thread takes four consecutive
// outputs of a row, keeps the 9 (y, z) rows of its 6 columns in registers
// and adds the 27 taps in the reference's order (ax, ay, az, az fastest),
// the centre as (float)v.  Planes sit in a ring of four slots (plane p in
// slot p & 3) so each plane costs one barrier; the next plane's pixels are
// loaded before the current plane's sums.
constexpr int LBX = 128, LBY = 8, LBP = LBX + 4;  // tile, staged row pitch (floats; 130 used)
template <class S, class D>
__global__ void __launch_bounds__(256)
    k_laplace_box3d_tile(D* __restrict__ dst, const S* __restrict__ src, int W, int H, int Dz, int zchunk, bool rte) {
  __shared__ __align__(16) float ring[4][(LBY + 2) * LBP];
  constexpr int NS = (LBY + 2) * (LBX + 2), PER = (NS + 255) / 256;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  const int x0 = blockIdx.x * LBX, y0 = blockIdx.y * LBY;
  const int z0 = blockIdx.z * zchunk, z1 = min(Dz, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  const int xo = x0 + 4 * tx, yo = y0 + ty;  // this thread's first output
  // staged cell i <-> region row i / (LBX + 2), column i % (LBX + 2); the
  // in-plane offset of its clamped pixel is the same for every plane
  int soff[PER];
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    const int i = tid + k * 256;
    const int r = i / (LBX + 2), c = i - r * (LBX + 2);
    soff[k] = i < NS ? clampi(y0 - 1 + r, H - 1) * W + clampi(x0 - 1 + c, W - 1) : 0;
  }
  decltype(readx(src, 0)) pre[PER];
  auto fetch = [&](int p) {
    const S* sp = src + (int64_t)clampi(p, Dz - 1) * plane;
#pragma unroll
    for (int k = 0; k < PER; ++k)
      if (tid + k * 256 < NS) pre[k] = readx(sp, soff[k]);
  };
  auto commit = [&](int p) {
    float* t = ring[p & 3];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int i = tid + k * 256;
      if (i < NS) {
        const int r = i / (LBX + 2), c = i - r * (LBX + 2);
        t[r * LBP + c] = (float)times_minus_one(pre[k]);
      }
    }
  };
  // planes z0-1 .. z0+1 staged before the first output plane
  for (int p = z0 - 1; p <= z0 + 1; ++p) {
    fetch(p);
    commit(p);
  }
  __syncthreads();
  for (int z = z0; z < z1; ++z) {
    const bool more = z + 1 < z1;
    if (more) fetch(z + 2);
    // centres, as (float)v
    float cen[4];
    const S* cp = src + (int64_t)z * plane + (int64_t)min(yo, H - 1) * W;
#pragma unroll
    for (int k = 0; k < 4; ++k) cen[k] = (float)readx(cp, min(xo + k, W - 1));
    // the 9 (y, z) rows of columns xo-1 .. xo+4 (region columns 4tx .. 4tx+5)
    float v[3][3][6];  // [ay][az][column]
#pragma unroll
    for (int az = 0; az < 3; ++az) {
      const float* t = ring[(z - 1 + az) & 3];
#pragma unroll
      for (int ay = 0; ay < 3; ++ay) {
        const float* row = t + (ty + ay) * LBP + 4 * tx;
        const float4 a = *reinterpret_cast<const float4*>(row);
        const float2 b = *reinterpret_cast<const float2*>(row + 4);
        v[ay][az][0] = a.x, v[ay][az][1] = a.y, v[ay][az][2] = a.z, v[ay][az][3] = a.w;
        v[ay][az][4] = b.x, v[ay][az][5] = b.y;
      }
    }
    if (yo < H) {
      D* o = dst + (int64_t)z * plane + (int64_t)yo * W;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        float result = 0.f;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax)
#pragma unroll
          for (int ay = 0; ay < 3; ++ay)
#pragma unroll
            for (int az = 0; az < 3; ++az)
              result = __fadd_rn(result, (ax == 1 && ay == 1 && az == 1) ? cen[k] : v[ay][az][k + ax]);
        if (xo + k < W) o[xo + k] = convert_sat<D>(result, rte);
      }
    }
    if (more) commit(z + 2);
    __syncthreads();
  }
}

// convolve_{2d,3d}_x.cl:17-31: c = kernel extent / 2; x, y, z over -c..c:
// sum = sum + kernel(c + offset) * src(coord + offset), float multiply then
// float add (no contraction), both reads clamped; CONVERT(sum).
template <class S, class D>
__global__ void __launch_bounds__(kBlock)
    k_convolve(D* __restrict__ dst, const S* __restrict__ src, const float* __restrict__ kern, Dims3 sd, Dims3 kd,
               Dims3 dd, Range r, bool rte) {
  const int cx = kd.w / 2, cy = kd.h / 2, cz = kd.d / 2;
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    float sum = 0.f;
    for (int a = -cx; a <= cx; ++a)
      for (int b = -cy; b <= cy; ++b)
        for (int c = -cz; c <= cz; ++c) {
          const float kv = __ldg(kern + atc(kd, cx + a, cy + b, cz + c));
          sum = __fadd_rn(sum, __fmul_rn(kv, (float)readx(src, atc(sd, x + a, y + b, z + c))));
        }
    dst[at(dd, x, y, z)] = convert_sat<D>(sum, rte);
  }
}

// greater_constant_{2d,3d}_x.cl:10-17
template <class S, class D>
__global__ void __launch_bounds__(kBlock)
    k_greater_constant(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, float scalar) {
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    const float in = (float)readx(src, atc(sd, x, y, z));
    dst[at(dd, x, y, z)] = in > scalar ? (D)1 : (D)0;
  }
}

// erode/dilate box/sphere (erode_box_3d_x.cl:14-37, erode_sphere_3d_x.cl:
// 14-37, dilate_box_3d_x.cl:14-37, dilate_sphere_3d_x.cl:14-38 and the _2d
// files), replaying the early-exit read order so the written value,
// including the sign of a float zero, is the one the kernel writes.
template <class S, class D, bool ERODE, bool SPHERE, bool THREE>
__global__ void __launch_bounds__(kBlock)
    k_morph(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool rte) {
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    float value = ldf(src, atc(sd, x, y, z));
    const bool go = ERODE ? (value != 0.f) : ((THREE && !SPHERE) ? (value < 1.f) : (value == 0.f));
    if (go) {
      if constexpr (SPHERE) {
        const int fx[6] = {1, -1, 0, 0, 0, 0}, fy[6] = {0, 0, 1, -1, 0, 0}, fz[6] = {0, 0, 0, 0, 1, -1};
#pragma unroll
        for (int k = 0; k < (THREE ? 6 : 4); ++k) {
          value = ldf(src, atc(sd, x + fx[k], y + fy[k], z + fz[k]));
          if (ERODE ? (value == 0.f) : (value != 0.f)) break;
        }
      } else {
        constexpr int zr = THREE ? 1 : 0;
        bool stop = false;
        for (int ax = -1; ax <= 1 && !stop; ++ax)
          for (int ay = -1; ay <= 1 && !stop; ++ay)
            for (int az = -zr; az <= zr && !stop; ++az) {
              value = ldf(src, atc(sd, x + ax, y + ay, z + az));
              stop = ERODE ? (value == 0.f) : (value != 0.f);
            }
      }
    }
    if (value != 0.f) value = 1.f;
    dst[at(dd, x, y, z)] = convert_sat<D>(value, rte);
  }
}

// sobel_2d_x.cl:14-41: the weighted sums are double-promoted (double
// literals) and stored to float.
template <class S, class D>
__global__ void __launch_bounds__(kBlock)
    k_sobel2d(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool rte) {
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    auto v = [&](int ddx, int ddy) -> double { return (double)ldf(src, atc(sd, x + ddx, y + ddy, 0)); };
    const double tl = v(-1, -1), tr = v(1, -1), bl = v(-1, 1), br = v(1, 1);
    const double l = v(-1, 0), rr = v(1, 0), t = v(0, -1), b = v(0, 1);
    double ax = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(-tl, l * -2.0), -bl), tr), rr * 2.0), br);
    double ay = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(-tl, t * -2.0), -tr), bl), b * 2.0), br);
    const float rx = __double2float_rn(ax), ry = __double2float_rn(ay);
    const float res = __fsqrt_rn(__fadd_rn(__fmul_rn(rx, rx), __fmul_rn(ry, ry)));
    dst[at(dd, x, y, z)] = convert_sat<D>(res, rte);
  }
}

// Coefficient of tap (m, n, k), k = 0..3, of the 3x3x4 window of
// sobel_3d_x.cl:44-52 for component comp: the arrays of :33-41 read through
// their flat layout, the one element past the array pinned to 0.
__host__ __device__ constexpr int sobel3d_coef(int comp, int m, int n, int k) {
  const int flat = 9 * m + 3 * n + k;
  if (flat >= 27) return 0;
  const int mm = flat / 9, nn = (flat / 3) % 3, kk = flat % 3;
  const int h0 = mm == 1 ? 2 : 1, h1 = nn == 1 ? 2 : 1, h2 = kk == 1 ? 2 : 1;
  const int p0 = 1 - mm, p1 = 1 - nn, p2 = 1 - kk;  // hp = {1, 0, -1}
  return comp == 0 ? p0 * h1 * h2 : (comp == 1 ? h0 * p1 * h2 : h0 * h1 * p2);
}

// sobel_3d_x.cl:43-56, sums in the kernel's order.  A term's type follows C:
// int * uint is uint (negative coefficients wrap), int * int is int,
// int * float is float; each term is added to a float sum.
template <class S, class D>
__global__ void __launch_bounds__(kBlock)
    k_sobel3d(D* __restrict__ dst, const S* __restrict__ src, Dims3 sd, Dims3 dd, Range r, bool narrow, bool rte) {
  for (int64_t i = blockIdx.x * (int64_t)kBlock + threadIdx.x; i < r.count(); i += (int64_t)gridDim.x * kBlock) {
    int x, y, z;
    decode(i, r, x, y, z);
    float sum[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int n = 0; n < 3; ++n)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const S raw = __ldg(src + atc(sd, x + m - 1, y + n - 1, z + k - 1));
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const int co = sobel3d_coef(c, m, n, k);
            float term;
            if constexpr (sizeof(S) == 4) {
              term = __fmul_rn((float)co, raw);
            } else if constexpr (S(-1) > S(0)) {  // unsigned pixel type
              term = narrow ? __int2float_rn(co * (int)raw) : __uint2float_rn((uint32_t)co * (uint32_t)raw);
            } else {
              term = __int2float_rn(co * (int)raw);
            }
            sum[c] = __fadd_rn(sum[c], term);
          }
        }
    const float res = __fsqrt_rn(
        __fadd_rn(__fadd_rn(__fmul_rn(sum[0], sum[0]), __fmul_rn(sum[1], sum[1])), __fmul_rn(sum[2], sum[2])));
    dst[at(dd, x, y, z)] = convert_sat<D>(res, rte);
  }
}

inline Dims3 dims(const Image& im) { return Dims3{im.w, im.h, im.d}; }

}  // namespace

clk_status direct_sep_pass(SepOp op, const Image& dst, const Image& src, int dim, const SepTaps& taps, Range r,
                           const Policy& p, cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    auto* o = (D*)dst.ptr;
    auto* in = (const S*)src.ptr;
    switch (op) {
      case SEP_GAUSS: k_sep_pass<S, D, SEP_GAUSS><<<g, kBlock, 0, st>>>(o, in, dims(src), dims(dst), r, dim, taps, p.rte); break;
      case SEP_MEAN: k_sep_pass<S, D, SEP_MEAN><<<g, kBlock, 0, st>>>(o, in, dims(src), dims(dst), r, dim, taps, p.rte); break;
      case SEP_MIN: k_sep_pass<S, D, SEP_MIN><<<g, kBlock, 0, st>>>(o, in, dims(src), dims(dst), r, dim, taps, p.rte); break;
      case SEP_MAX: k_sep_pass<S, D, SEP_MAX><<<g, kBlock, 0, st>>>(o, in, dims(src), dims(dst), r, dim, taps, p.rte); break;
    }
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "separable pass: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("separable pass");
}

clk_status direct_copy(const Image& dst, const Image& src, Range r, const Policy& p, cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    k_copy<S, D><<<grid_for(r.count()), kBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, dims(src), dims(dst), r,
                                                         p.rte);
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "copy: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("copy");
}

clk_status direct_rank(RankOp op, RankMode mode, const Image& dst, const Image& src, const MedianNbhd& m, Range r,
                       const Policy& p, cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  if (mode == RANK_CAST && src.dt == CLK_F32 && dst.dt != CLK_F32)
    return fail(CLK_UNSUPPORTED_DTYPE, "minimum_sphere_2d: float to integer (the kernel's C cast of an out-of-range "
                                       "float is undefined)");
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    auto* o = (D*)dst.ptr;
    auto* in = (const S*)src.ptr;
    const Dims3 a = dims(src), b = dims(dst);
    if (op == RANK_MEAN) k_rank<S, D, RANK_MEAN, RANK_FLOAT><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
    else if (op == RANK_MIN && mode == RANK_FLOAT) k_rank<S, D, RANK_MIN, RANK_FLOAT><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
    else if (op == RANK_MAX && mode == RANK_FLOAT) k_rank<S, D, RANK_MAX, RANK_FLOAT><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
    else if (op == RANK_MIN && mode == RANK_CONVERT) k_rank<S, D, RANK_MIN, RANK_CONVERT><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
    else if (op == RANK_MAX && mode == RANK_CONVERT) k_rank<S, D, RANK_MAX, RANK_CONVERT><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
    else if (op == RANK_MIN) k_rank<S, D, RANK_MIN, RANK_CAST><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
    else k_rank<S, D, RANK_MAX, RANK_CAST><<<g, kBlock, 0, st>>>(o, in, a, b, r, m, p.rte);
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "rank filter: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("rank filter");
}

clk_status direct_stencil(StencilKind kind, const Image& dst, const Image& src, Range r, const Policy& p,
                          cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    auto* o = (D*)dst.ptr;
    auto* in = (const S*)src.ptr;
    const Dims3 a = dims(src), b = dims(dst);
    switch (kind) {
      case ST_GRADIENT_X: k_gradient<S, D, 0><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case ST_GRADIENT_Y: k_gradient<S, D, 1><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case ST_GRADIENT_Z: k_gradient<S, D, 2><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case ST_LAPLACE_DIAMOND_2D: k_laplace_expr<S, D, 0><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case ST_LAPLACE_DIAMOND_3D: k_laplace_expr<S, D, 1><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case ST_LAPLACE_BOX_2D: k_laplace_expr<S, D, 2><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case ST_LAPLACE_BOX_3D: k_laplace_box3d<S, D><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
    }
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "stencil: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("stencil");
}

clk_status fast_laplace_box3d(const Image& dst, const Image& src, const Policy& p, cudaStream_t st) {
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d || (int64_t)src.w * src.h >= (1LL << 31))
    return CLK_UNSUPPORTED_DTYPE;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int tx = (src.w + LBX - 1) / LBX, ty = (src.h + LBY - 1) / LBY;
  int chunks = 1;
  while ((int64_t)tx * ty * chunks < 4LL * sms && src.d / (chunks * 2) >= 8) chunks *= 2;
  const int zchunk = (src.d + chunks - 1) / chunks;
  const dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    k_laplace_box3d_tile<S, D><<<grid, 256, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, src.w, src.h, src.d, zchunk,
                                                     p.rte);
  });
  if (!ok) return CLK_UNSUPPORTED_DTYPE;
  count_launch();
  return check_launch("laplace_box_3d (tiles)");
}

clk_status direct_convolve(const Image& dst, const Image& src, const Image& kern, Range r, const Policy& p,
                           cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  if (kern.dt != CLK_F32) return fail(CLK_UNSUPPORTED_DTYPE, "convolve: the kernel image must be float");
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    k_convolve<S, D><<<g, kBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, (const float*)kern.ptr, dims(src),
                                           dims(kern), dims(dst), r, p.rte);
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "convolve: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("convolve");
}

clk_status direct_greater_constant(const Image& dst, const Image& src, float scalar, Range r, cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    k_greater_constant<S, D><<<g, kBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, dims(src), dims(dst), r, scalar);
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "greater_constant: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("greater_constant");
}

clk_status direct_median(const Image& dst, const Image& src, const MedianNbhd& m, Range r, cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  if (src.dt != dst.dt)
    return fail(CLK_UNSUPPORTED_DTYPE, "median: src and dst pixel types must match (the kernel's dst-typed array "
                                       "makes other pairs implementation-defined)");
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_type(src.dt, [&](auto t) {
    using T = decltype(t);
    if (m.n <= 32)
      k_median<T, 32><<<g, kBlock, 0, st>>>((T*)dst.ptr, (const T*)src.ptr, dims(src), dims(dst), r, m);
    else if (m.n <= 128)
      k_median<T, 128><<<g, kBlock, 0, st>>>((T*)dst.ptr, (const T*)src.ptr, dims(src), dims(dst), r, m);
    else
      k_median<T, kMaxMedian><<<g, kBlock, 0, st>>>((T*)dst.ptr, (const T*)src.ptr, dims(src), dims(dst), r, m);
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "median: pixel type %d", src.dt);
  count_launch();
  return check_launch("median");
}

clk_status direct_morph(bool erode, bool sphere, const Image& dst, const Image& src, Range r, const Policy& p,
                        cudaStream_t st, bool planar) {
  if (r.count() == 0) return CLK_OK;
  const unsigned g = grid_for(r.count());
  const bool three = src.ndim == 3 && !planar;  // slice-by-slice: the 2-D kernel on every plane
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    auto* o = (D*)dst.ptr;
    auto* in = (const S*)src.ptr;
    const Dims3 a = dims(src), b = dims(dst);
    const int sel = (erode ? 4 : 0) | (sphere ? 2 : 0) | (three ? 1 : 0);
    switch (sel) {
      case 0: k_morph<S, D, false, false, false><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 1: k_morph<S, D, false, false, true><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 2: k_morph<S, D, false, true, false><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 3: k_morph<S, D, false, true, true><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 4: k_morph<S, D, true, false, false><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 5: k_morph<S, D, true, false, true><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 6: k_morph<S, D, true, true, false><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
      case 7: k_morph<S, D, true, true, true><<<g, kBlock, 0, st>>>(o, in, a, b, r, p.rte); break;
    }
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "morphology: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("morphology");
}

clk_status direct_sobel(const Image& dst, const Image& src, Range r, const Policy& p, cudaStream_t st) {
  if (r.count() == 0) return CLK_OK;
  const unsigned g = grid_for(r.count());
  const bool ok = dispatch_types(src.dt, dst.dt, [&](auto s, auto d) {
    using S = decltype(s);
    using D = decltype(d);
    if (src.ndim == 2)
      k_sobel2d<S, D><<<g, kBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, dims(src), dims(dst), r, p.rte);
    else
      k_sobel3d<S, D><<<g, kBlock, 0, st>>>((D*)dst.ptr, (const S*)src.ptr, dims(src), dims(dst), r,
                                            p.sobel_narrow, p.rte);
  });
  if (!ok) return fail(CLK_UNSUPPORTED_DTYPE, "sobel: pixel types %d -> %d", src.dt, dst.dt);
  count_launch();
  return check_launch("sobel");
}

}  // namespace clk
