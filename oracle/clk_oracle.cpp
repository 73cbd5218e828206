// clk_oracle.cpp - TEST INFRASTRUCTURE ONLY.
//
// CPU restatement ("port") of the reference's neighbourhood-filter kernels
// and of the host orchestration around them.  Only tests/, the smoke check
// and bench.py's CPU-baseline leg load it, and only as the checker.  It is
// written from the kernels' semantics, one function per family, each citing
// the .cl lines it restates; oracle/_ref (the .cl text itself compiled on the
// host) pins it.
//
// Shared semantics (the preamble, README.md:25-141, restated):
//  * reads clamp each coordinate to [0, extent-1] (CLK_ADDRESS_CLAMP_TO_EDGE,
//    line 1 of every hot file);
//  * a read's .x is uint for uchar/ushort, int for char/short, float for
//    float (the read_imageui / read_imagei / read_imagef families);
//  * CONVERT_dst_PIXEL_TYPE saturates to the type's range and truncates
//    toward zero (NaN -> 0); flag CLKO_RTE rounds half to even instead;
//  * float arithmetic is evaluated exactly as written: no FMA contraction
//    (compile with -ffp-contract=off), left-to-right, float exp taken as the
//    correctly rounded float of exp.
//
// The FP64 oracle (clko_fp64) evaluates the float-output filters in double
// with double temporaries; tests compare float outputs against it.
#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

namespace {

enum { U8 = 0, I8 = 1, U16 = 2, I16 = 3, F32 = 4 };
enum { CLKO_RTE = 1, CLKO_SOBEL_NARROW = 2 };

struct Vol {
  void* p;
  int dt;
  int w, h, d;
};

static inline int clampi(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }
static inline long vidx(const Vol& v, int x, int y, int z) {
  return (long)clampi(x, v.w - 1) + (long)v.w * ((long)clampi(y, v.h - 1) + (long)v.h * clampi(z, v.d - 1));
}

template <class T> struct Lim;
template <> struct Lim<uint8_t> { static constexpr double lo = 0, hi = 255; };
template <> struct Lim<int8_t> { static constexpr double lo = -128, hi = 127; };
template <> struct Lim<uint16_t> { static constexpr double lo = 0, hi = 65535; };
template <> struct Lim<int16_t> { static constexpr double lo = -32768, hi = 32767; };

// CONVERT_dst_PIXEL_TYPE (clij_convert_<T>_sat, README.md:35-43).
template <class D> static inline D convert_sat(double v, int flags) {
  if constexpr (std::is_same<D, float>::value) {
    return (float)v;
  } else {
    if (v != v) return (D)0;
    if (v <= Lim<D>::lo) return (D)Lim<D>::lo;
    if (v >= Lim<D>::hi) return (D)Lim<D>::hi;
    if (flags & CLKO_RTE) return (D)std::nearbyint(v);  // default FE mode: half to even
    return (D)(long long)v;
  }
}

// Gaussian weight h = exp((v*v)/n), n = -2*s*s, all in float as at
// gaussian_blur_separable_3d_x.cl:24,29; exp correctly rounded to float.
static inline float gauss_weight(int v, float s) {
  const float n = (-2.0f * s) * s;
  const float q = (float)(v * v) / n;
  return (float)std::exp((double)q);
}

template <class S> static inline float readf(const Vol& v, int x, int y, int z) {
  return (float)((const S*)v.p)[vidx(v, x, y, z)];
}

// One separable pass along dim (gaussian_blur_separable_3d_x.cl:14-34,
// mean_separable_3d_x.cl:12-29, minimum_separable_3d_x.cl:12-23,
// maximum_separable_3d_x.cl:12-23; the _2d files are the same with z = 0;
// minimum/maximum_separable_2d_x.cl:20-23 skip v = 0, which re-reads the
// centre they start from, so the result is identical).
enum SepOp { GAUSS, MEAN, MINI, MAXI };

template <class S, class D>
static void sep_pass(SepOp op, const Vol& dst, const Vol& src, int dim, int N, float s, const int g[3], int flags,
                     int nt) {
  const int c = (N - 1) / 2;  // C division, as in the kernel
  const int dx = dim == 0, dy = dim == 1, dz = dim == 2;
  std::vector<float> h;
  if (op == GAUSS)
    for (int v = -c; v <= c; ++v) h.push_back(gauss_weight(v, s));
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      float res = 0.0f;
      if (op == GAUSS) {
        float hsum = 0.0f;
        for (int v = -c; v <= c; ++v) {
          const float hv = h[v + c];
          const float prod = hv * readf<S>(src, x + v * dx, y + v * dy, z + v * dz);
          res = res + prod;
          hsum = hsum + hv;
        }
        res = res / hsum;
      } else if (op == MEAN) {
        float count = 0.0f;
        for (int v = -c; v <= c; ++v) {
          res = res + readf<S>(src, x + v * dx, y + v * dy, z + v * dz);
          count = count + 1.0f;
        }
        res = res / count;
      } else {
        res = readf<S>(src, x, y, z);
        for (int v = -c; v <= c; ++v) {
          const float t = readf<S>(src, x + v * dx, y + v * dy, z + v * dz);
          if (op == MINI) res = t < res ? t : res;
          else res = res < t ? t : res;
        }
      }
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>(res, flags);
    }
  }
}

// copy_3d_x.cl:7-14: float out = READ(src).x; WRITE(dst, CONVERT(out)).
template <class S, class D> static void copy_conv(const Vol& dst, const Vol& src, int flags, int nt) {
  const long n = (long)dst.w * dst.h * dst.d;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long i = 0; i < n; ++i) ((D*)dst.p)[i] = convert_sat<D>((float)((const S*)src.p)[i], flags);
}

// Neighbourhood offsets of median_box/median_sphere in the kernels' loop
// order (x outer, then y, then z; median_sphere_3d_x.cl:55-72), with the
// sphere test evaluated in float exactly as written (:42-61).
// guard = false: median_slice_by_slice_sphere_3d_x.cl:39-45 has no FLT_MIN
// guard, so a zero semi-axis gives 0/0 and an empty neighbourhood.
static std::vector<int> median_offsets(bool sphere, int ndim, int Nx, int Ny, int Nz, bool guard = true) {
  const int ex = (Nx - 1) / 2, ey = (Ny - 1) / 2, ez = ndim == 3 ? (Nz - 1) / 2 : 0;
  float a2 = (float)(ex * ex), b2 = (float)(ey * ey), c2 = (float)(ez * ez);
  if (guard && a2 == 0) a2 = FLT_MIN;
  if (guard && b2 == 0) b2 = FLT_MIN;
  if (guard && c2 == 0) c2 = FLT_MIN;
  std::vector<int> off;
  for (int x = -ex; x <= ex; ++x) {
    const float xs = (float)(x * x);
    for (int y = -ey; y <= ey; ++y) {
      const float ys = (float)(y * y);
      for (int z = -ez; z <= ez; ++z) {
        const float zs = (float)(z * z);
        bool in = true;
        if (sphere) {
          float t = xs / a2 + ys / b2;
          if (ndim == 3) t = t + zs / c2;
          in = t <= 1.0f;
        }
        if (in) {
          off.push_back(x);
          off.push_back(y);
          off.push_back(z);
        }
      }
    }
  }
  return off;
}

// median_box/sphere_{2d,3d}: gather into a dst-typed array, stable insertion
// sort, take element n/2 (median_box_3d_x.cl:3-20, :41-64).
template <class S, class D>
static void median(const Vol& dst, const Vol& src, const std::vector<int>& off, const int g[3], int nt) {
  const int n = (int)off.size() / 3;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    std::vector<D> a(n > 0 ? n : 1);
    for (int x = 0; x < g[0]; ++x) {
      for (int i = 0; i < n; ++i)
        a[i] = (D)((const S*)src.p)[vidx(src, x + off[3 * i], y + off[3 * i + 1], z + off[3 * i + 2])];
      std::stable_sort(a.begin(), a.begin() + n, [](D p, D q) { return p < q; });
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = a[n / 2];
    }
  }
}

// erode/dilate_{box,sphere}_{2d,3d} (erode_box_3d_x.cl:14-37,
// erode_sphere_3d_x.cl:14-37, dilate_box_3d_x.cl:14-37,
// dilate_sphere_3d_x.cl:14-38), replaying the early-exit loops so that the
// zero that is finally written (its sign, for float images) is the same one.
// The slice-by-slice variants (erode_box_slice_by_slice_3d_x.cl:14-31,
// erode_sphere_slice_by_slice_3d_x.cl:14-26, dilate_box_slice_by_slice_3d_x.cl,
// dilate_sphere_slice_by_slice_3d_x.cl) are the 2-D kernels on every plane of a
// 3-D image: ndim = 2 semantics with z unchanged.
template <class S, class D>
static void morph(bool erode, bool sphere, int ndim, const Vol& dst, const Vol& src, const int g[3], int flags,
                  int nt) {
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    const int zr = ndim == 3 ? 1 : 0;
    for (int x = 0; x < g[0]; ++x) {
      float value = readf<S>(src, x, y, z);
      // erode continues while values are nonzero, dilate while they are 0
      // (dilate_box_3d_x.cl:15 tests value < 1, which re-reads the centre in
      // the loop and therefore ends the same way as == 0).
      const bool go = erode ? (value != 0) : (ndim == 3 && !sphere ? (value < 1) : (value == 0));
      if (go) {
        if (sphere) {
          static const int fx[6] = {1, -1, 0, 0, 0, 0}, fy[6] = {0, 0, 1, -1, 0, 0}, fz[6] = {0, 0, 0, 0, 1, -1};
          const int nf = ndim == 3 ? 6 : 4;
          for (int i = 0; i < nf; ++i) {
            value = readf<S>(src, x + fx[i], y + fy[i], z + fz[i]);
            if (erode ? !(value != 0) : (value != 0)) break;
          }
        } else {
          bool stop = false;
          for (int ax = -1; ax <= 1 && !stop; ++ax)
            for (int ay = -1; ay <= 1 && !stop; ++ay)
              for (int az = -zr; az <= zr && !stop; ++az) {
                value = readf<S>(src, x + ax, y + ay, z + az);
                stop = erode ? (value == 0) : (value != 0);
              }
        }
      }
      if (value != 0) value = 1;
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>(value, flags);
    }
  }
}

// sobel_2d_x.cl:14-41: float reads, double-promoted weighted sums stored to
// float, float magnitude.
template <class S, class D>
static void sobel2d(const Vol& dst, const Vol& src, const int g[3], int flags, int nt) {
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long y = 0; y < g[1]; ++y) {
    for (int x = 0; x < g[0]; ++x) {
      const int yy = (int)y;
      const float c_r = readf<S>(src, x + 1, yy, 0), c_l = readf<S>(src, x - 1, yy, 0);
      const float c_b = readf<S>(src, x, yy + 1, 0), c_t = readf<S>(src, x, yy - 1, 0);
      const float tl = readf<S>(src, x - 1, yy - 1, 0), tr = readf<S>(src, x + 1, yy - 1, 0);
      const float bl = readf<S>(src, x - 1, yy + 1, 0), br = readf<S>(src, x + 1, yy + 1, 0);
      const float rx = (float)((double)tl * -1.0 + (double)c_l * -2.0 + (double)bl * -1.0 + (double)tr * 1.0 +
                               (double)c_r * 2.0 + (double)br * 1.0);
      const float ry = (float)((double)tl * -1.0 + (double)c_t * -2.0 + (double)tr * -1.0 + (double)bl * 1.0 +
                               (double)c_b * 2.0 + (double)br * 1.0);
      const float rxx = rx * rx, ryy = ry * ry;
      const float res = std::sqrt(rxx + ryy);
      ((D*)dst.p)[(long)x + (long)dst.w * y] = convert_sat<D>(res, flags);
    }
  }
}

// The 3x3x4 window of sobel_3d_x.cl:44-52: coefficient of tap (m, n, k),
// k = 0..3, for component c (0 = x, 1 = y, 2 = z), from the arrays built at
// :33-41 read through their flat layout (k = 3 reads element 9m+3n+3; the
// one element past the array, m = n = 2, is pinned to 0).
static int sobel3d_coef(int comp, int m, int n, int k) {
  static const int h[3] = {1, 2, 1}, hp[3] = {1, 0, -1};
  int flat = 9 * m + 3 * n + k;
  if (flat >= 27) return 0;
  const int mm = flat / 9, nn = (flat / 3) % 3, kk = flat % 3;
  if (comp == 0) return hp[mm] * h[nn] * h[kk];
  if (comp == 1) return h[mm] * hp[nn] * h[kk];
  return h[mm] * h[nn] * hp[kk];
}

// sobel_3d_x.cl:43-56: sum_c += g_c[m][n][k] * READ(...).x in float.  The
// product's type follows C: int * uint is uint (wraps for negative
// coefficients), int * int is int, int * float is float.
template <class S, class D>
static void sobel3d(const Vol& dst, const Vol& src, const int g[3], int flags, int nt) {
  int cf[3][36];
  for (int c = 0; c < 3; ++c)
    for (int m = 0; m < 3; ++m)
      for (int n = 0; n < 3; ++n)
        for (int k = 0; k < 4; ++k) cf[c][12 * m + 4 * n + k] = sobel3d_coef(c, m, n, k);
  const bool narrow = (flags & CLKO_SOBEL_NARROW) != 0;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      float sum[3] = {0.0f, 0.0f, 0.0f};
      for (int m = 0; m < 3; ++m)
        for (int n = 0; n < 3; ++n)
          for (int k = 0; k < 4; ++k) {
            const S raw = ((const S*)src.p)[vidx(src, x + m - 1, y + n - 1, z + k - 1)];
            for (int c = 0; c < 3; ++c) {
              const int co = cf[c][12 * m + 4 * n + k];
              float term;
              if constexpr (std::is_same<S, float>::value) {
                term = (float)co * raw;
              } else if constexpr (std::is_same<S, uint8_t>::value || std::is_same<S, uint16_t>::value) {
                if (narrow) term = (float)(co * (int)raw);
                else term = (float)((uint32_t)co * (uint32_t)raw);
              } else {
                term = (float)(co * (int)raw);
              }
              sum[c] = sum[c] + term;
            }
          }
      const float res = std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>(res, flags);
    }
  }
}

// minimum/maximum/mean_sphere_{2d,3d} and the slice-by-slice sphere
// variants: a reduction over the ellipsoid (ellipse) offsets in the kernels'
// loop order (x outer, then y, then z).  The variants differ in the type the
// running value lives in:
//   RANK_FLOAT    float, values (float)READ(..).x, result CONVERT(value)
//                 (minimum/maximum_sphere_3d_x.cl:15-49);
//   RANK_CONVERT  dst type, centre and values CONVERT(READ(..).x), result
//                 the value (maximum_sphere_2d_x.cl:16-45,
//                 minimum/maximum_slice_by_slice_sphere_3d_x.cl:15-38);
//   RANK_CAST     dst type, centre CONVERT, values the C cast
//                 (IMAGE_dst_PIXEL_TYPE)READ(..).x (minimum_sphere_2d_x.cl:16-47);
// and the mean sums READ(..).x into a float in loop order and writes
// CONVERT(sum / count) (mean_sphere_3d_x.cl:16-56, mean_sphere_2d_x.cl,
// mean_slice_by_slice_sphere_3d_x.cl:16-41).
enum RankOp { RANK_MIN, RANK_MAX, RANK_MEAN };
enum RankMode { RANK_FLOAT, RANK_CONVERT, RANK_CAST };

template <class S> static inline auto readx(const Vol& v, int x, int y, int z) {
  // .x of a read: uint for unsigned, int for signed, float for float
  const S t = ((const S*)v.p)[vidx(v, x, y, z)];
  if constexpr (std::is_same<S, float>::value) return t;
  else if constexpr (std::is_signed<S>::value) return (int)t;
  else return (unsigned)t;
}

template <class S, class D>
static void rank_filter(RankOp op, RankMode mode, const Vol& dst, const Vol& src, const std::vector<int>& off,
                        const int g[3], int flags, int nt) {
  const int n = (int)off.size() / 3;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      D res;
      if (op == RANK_MEAN) {
        float sum = 0;
        int count = 0;
        for (int i = 0; i < n; ++i) {
          sum = sum + (float)readx<S>(src, x + off[3 * i], y + off[3 * i + 1], z + off[3 * i + 2]);
          count++;
        }
        res = convert_sat<D>((double)(sum / (float)count), flags);
      } else if (mode == RANK_FLOAT) {
        float m = (float)readx<S>(src, x, y, z);
        for (int i = 0; i < n; ++i) {
          const float v = (float)readx<S>(src, x + off[3 * i], y + off[3 * i + 1], z + off[3 * i + 2]);
          if (op == RANK_MIN ? v < m : v > m) m = v;
        }
        res = convert_sat<D>((double)m, flags);
      } else {
        D m = convert_sat<D>((double)readx<S>(src, x, y, z), flags);
        for (int i = 0; i < n; ++i) {
          const auto r = readx<S>(src, x + off[3 * i], y + off[3 * i + 1], z + off[3 * i + 2]);
          const D v = mode == RANK_CAST ? (D)r : convert_sat<D>((double)r, flags);
          if (op == RANK_MIN ? v < m : v > m) m = v;
        }
        res = m;
      }
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = res;
    }
  }
}

// greater_constant_{2d,3d}_x.cl:10-17: (float)READ(src1).x > scalar ? 1 : 0.
template <class S, class D>
static void greater_constant(const Vol& dst, const Vol& src, float scalar, const int g[3], int nt) {
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      const float in = (float)readx<S>(src, x, y, z);
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = in > scalar ? (D)1 : (D)0;
    }
  }
}

// gradient_{x,y,z}_{2d,3d}_x.cl: CONVERT(READ(+1).x - READ(-1).x), float
// values and a float difference, along the kernel's axis.
template <class S, class D>
static void gradient(int axis, const Vol& dst, const Vol& src, const int g[3], int flags, int nt) {
  const int dx = axis == 0, dy = axis == 1, dz = axis == 2;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      const float a = (float)readx<S>(src, x - dx, y - dy, z - dz);
      const float b = (float)readx<S>(src, x + dx, y + dy, z + dz);
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>((double)(b - a), flags);
    }
  }
}

// laplace_diamond_{2d,3d}_x.cl and laplace_box_2d_x.cl: float values, then
// centre * K + each neighbour * -1.0 in the expression's order; the
// literals are double, so the sum is evaluated in double and stored to float.
template <class S, class D>
static void laplace_expr(const std::vector<int>& nb, double k, const Vol& dst, const Vol& src, const int g[3],
                         int flags, int nt) {
  const int n = (int)nb.size() / 3;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      double r = (double)(float)readx<S>(src, x, y, z) * k;
      for (int i = 0; i < n; ++i)
        r = r + (double)(float)readx<S>(src, x + nb[3 * i], y + nb[3 * i + 1], z + nb[3 * i + 2]) * -1.0;
      const float res = (float)r;
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>((double)res, flags);
    }
  }
}

// laplace_box_3d_x.cl:13-25: float result, loop ax, ay, az; the centre adds
// READ(..).x, every other tap READ(..).x * -1 -- an int times the read's .x,
// which for unsigned pixels is a uint product that wraps (2^32 - v).
template <class S, class D>
static void laplace_box3d(const Vol& dst, const Vol& src, const int g[3], int flags, int nt) {
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      float result = 0;
      for (int ax = -1; ax <= 1; ++ax)
        for (int ay = -1; ay <= 1; ++ay)
          for (int az = -1; az <= 1; ++az) {
            const auto v = readx<S>(src, x + ax, y + ay, z + az);
            if (ax == 0 && ay == 0 && az == 0) result = result + v;
            else result = result + v * -1;
          }
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>((double)result, flags);
    }
  }
}

// convolve_{2d,3d}_x.cl:17-31: c = kernel extent / 2 per axis; for x, y, z
// in -c..c: sum = sum + (float)kernel(c + offset) * (float)src(coord + offset),
// both reads clamped; CONVERT(sum).
template <class S, class D>
static void convolve(const Vol& dst, const Vol& src, const float* kern, const int kshape[3], const int g[3],
                     int flags, int nt) {
  const int cx = kshape[0] / 2, cy = kshape[1] / 2, cz = kshape[2] / 2;
  const Vol K{(void*)kern, F32, kshape[0], kshape[1], kshape[2]};
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < (long)g[2] * g[1]; ++zy) {
    const int z = (int)(zy / g[1]), y = (int)(zy % g[1]);
    for (int x = 0; x < g[0]; ++x) {
      float sum = 0;
      for (int a = -cx; a <= cx; ++a)
        for (int b = -cy; b <= cy; ++b)
          for (int c = -cz; c <= cz; ++c) {
            const float kv = kern[vidx(K, cx + a, cy + b, cz + c)];
            sum = sum + kv * (float)readx<S>(src, x + a, y + b, z + c);
          }
      ((D*)dst.p)[(long)x + (long)dst.w * ((long)y + (long)dst.h * z)] = convert_sat<D>((double)sum, flags);
    }
  }
}

// ---------------------------------------------------------------- dispatch
template <class F> static int with_types(int sdt, int ddt, F f) {
  auto d = [&](auto s) -> int {
    switch (ddt) {
      case U8: return f(s, uint8_t{});
      case I8: return f(s, int8_t{});
      case U16: return f(s, uint16_t{});
      case I16: return f(s, int16_t{});
      case F32: return f(s, float{});
    }
    return -1;
  };
  switch (sdt) {
    case U8: return d(uint8_t{});
    case I8: return d(int8_t{});
    case U16: return d(uint16_t{});
    case I16: return d(int16_t{});
    case F32: return d(float{});
  }
  return -1;
}

static bool starts(const std::string& s, const char* p) { return s.rfind(p, 0) == 0; }

static int sep_op(const std::string& k, SepOp* op) {
  if (starts(k, "gaussian_blur_separable_")) *op = GAUSS;
  else if (starts(k, "mean_separable_")) *op = MEAN;
  else if (starts(k, "minimum_separable_")) *op = MINI;
  else if (starts(k, "maximum_separable_")) *op = MAXI;
  else return -1;
  return 0;
}

template <class T> static double fp64_read(const Vol& v, int x, int y, int z) {
  return (double)((const T*)v.p)[vidx(v, x, y, z)];
}

}  // namespace

extern "C" {

// One kernel launch of the named reference kernel over global range g.
// ia/fa: the kernel's int / float parameters in declaration order.
int clko_execute(const char* kernel, int sdt, int ddt, const void* src, const int sshape[3], void* dst,
                 const int dshape[3], const int g[3], const int* ia, const float* fa, int flags, int nthreads) {
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  const std::string k(kernel);
  const int ndim = k.size() > 3 && k.compare(k.size() - 2, 2, "2d") == 0 ? 2 : 3;
  Vol S{(void*)src, sdt, sshape[0], sshape[1], sshape[2]};
  Vol D{dst, ddt, dshape[0], dshape[1], dshape[2]};
  SepOp op;
  if (sep_op(k, &op) == 0) {
    return with_types(sdt, ddt, [&](auto s, auto d) {
      sep_pass<decltype(s), decltype(d)>(op, D, S, ia[0], ia[1], fa[0], g, flags, nt);
      return 0;
    });
  }
  // slice-by-slice kernels: a 2-D neighbourhood on every plane of a 3-D image
  const bool planar = k.find("slice_by_slice") != std::string::npos;
  const int nbdim = planar ? 2 : ndim;
  if (starts(k, "minimum_sphere_") || starts(k, "maximum_sphere_") || starts(k, "mean_sphere_") ||
      starts(k, "minimum_slice_by_slice_sphere") || starts(k, "maximum_slice_by_slice_sphere") ||
      starts(k, "mean_slice_by_slice_sphere")) {
    const RankOp op = starts(k, "minimum") ? RANK_MIN : starts(k, "maximum") ? RANK_MAX : RANK_MEAN;
    const RankMode mode = (ndim == 3 && !planar) ? RANK_FLOAT : (k == "minimum_sphere_2d" ? RANK_CAST : RANK_CONVERT);
    if (mode == RANK_CAST && sdt == F32 && ddt != F32) return -2;  // C cast of an out-of-range float: undefined
    const auto off = median_offsets(true, nbdim, ia[0], ia[1], nbdim == 3 ? ia[2] : 1);
    return with_types(sdt, ddt, [&](auto s, auto d) {
      rank_filter<decltype(s), decltype(d)>(op, mode, D, S, off, g, flags, nt);
      return 0;
    });
  }
  if (starts(k, "gradient_")) {
    const int axis = k[9] - 'x';
    return with_types(sdt, ddt, [&](auto s, auto d) {
      gradient<decltype(s), decltype(d)>(axis, D, S, g, flags, nt);
      return 0;
    });
  }
  if (k == "laplace_box_3d")
    return with_types(sdt, ddt, [&](auto s, auto d) {
      laplace_box3d<decltype(s), decltype(d)>(D, S, g, flags, nt);
      return 0;
    });
  if (starts(k, "laplace_")) {
    // neighbours in the expression's order: right, left, top, bottom(, front, back | A, B, C, D)
    std::vector<int> nb = {1, 0, 0, -1, 0, 0, 0, -1, 0, 0, 1, 0};
    double kc = 4.0;
    if (k == "laplace_diamond_3d") {
      nb.insert(nb.end(), {0, 0, 1, 0, 0, -1});
      kc = 6.0;
    } else if (k == "laplace_box_2d") {
      nb.insert(nb.end(), {-1, -1, 0, 1, -1, 0, -1, 1, 0, 1, 1, 0});
      kc = 8.0;
    }
    return with_types(sdt, ddt, [&](auto s, auto d) {
      laplace_expr<decltype(s), decltype(d)>(nb, kc, D, S, g, flags, nt);
      return 0;
    });
  }
  if (starts(k, "greater_constant_"))
    return with_types(sdt, ddt, [&](auto s, auto d) {
      greater_constant<decltype(s), decltype(d)>(D, S, fa[0], g, nt);
      return 0;
    });
  if (k == "copy_2d" || k == "copy_3d")
    return with_types(sdt, ddt, [&](auto s, auto d) {
      copy_conv<decltype(s), decltype(d)>(D, S, flags, nt);
      return 0;
    });
  if (starts(k, "median_")) {
    if (sdt != ddt) return -2;
    const bool sphere = k.find("sphere") != std::string::npos;
    const auto off = median_offsets(sphere, nbdim, ia[0], ia[1], nbdim == 3 ? ia[2] : 1,
                                    k != "median_slice_by_slice_sphere_3d");
    if (off.empty()) return -3;  // the kernel would read an uninitialised array element
    return with_types(sdt, ddt, [&](auto s, auto d) {
      median<decltype(s), decltype(d)>(D, S, off, g, nt);
      return 0;
    });
  }
  if (starts(k, "erode_") || starts(k, "dilate_")) {
    const bool erode = starts(k, "erode_");
    const bool sphere = k.find("sphere") != std::string::npos;
    return with_types(sdt, ddt, [&](auto s, auto d) {
      morph<decltype(s), decltype(d)>(erode, sphere, nbdim, D, S, g, flags, nt);
      return 0;
    });
  }
  if (k == "sobel_2d")
    return with_types(sdt, ddt, [&](auto s, auto d) {
      sobel2d<decltype(s), decltype(d)>(D, S, g, flags, nt);
      return 0;
    });
  if (k == "sobel_3d")
    return with_types(sdt, ddt, [&](auto s, auto d) {
      sobel3d<decltype(s), decltype(d)>(D, S, g, flags, nt);
      return 0;
    });
  return -1;
}

// convolve_{2d,3d}: src * a float kernel image over global range g.
int clko_convolve(int sdt, int ddt, const void* src, const int sshape[3], const float* kern, const int kshape[3],
                  void* dst, const int dshape[3], const int g[3], int flags, int nthreads) {
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  Vol S{(void*)src, sdt, sshape[0], sshape[1], sshape[2]};
  Vol D{dst, ddt, dshape[0], dshape[1], dshape[2]};
  return with_types(sdt, ddt, [&](auto s, auto d) {
    convolve<decltype(s), decltype(d)>(D, S, kern, kshape, g, flags, nt);
    return 0;
  });
}

// Orchestrated separable filter: passes X, Y(, Z) with dst-typed
// temporaries; an axis with N <= 1 (gaussian: or s <= 0) is a converting
// copy (copy_3d_x.cl:7-14).
int clko_separable(const char* kernel, int sdt, int ddt, const void* src, void* dst, const int shape[3], int ndim,
                   const int N[3], const float s[3], int flags, int nthreads) {
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  SepOp op;
  if (sep_op(kernel, &op) != 0) return -1;
  static const int esz[5] = {1, 1, 2, 2, 4};
  const long n = (long)shape[0] * shape[1] * shape[2];
  std::vector<char> t0(n * esz[ddt]), t1(n * esz[ddt]);
  Vol cur{(void*)src, sdt, shape[0], shape[1], shape[2]};
  char* bufs[2] = {t0.data(), t1.data()};
  const int g[3] = {shape[0], shape[1], shape[2]};
  for (int d = 0; d < ndim; ++d) {
    const bool last = d == ndim - 1;
    Vol out{last ? dst : (void*)bufs[d & 1], ddt, shape[0], shape[1], shape[2]};
    const bool skip = N[d] <= 1 || (op == GAUSS && !(s[d] > 0));
    const int r = with_types(cur.dt, ddt, [&](auto a, auto b) {
      if (skip) copy_conv<decltype(a), decltype(b)>(out, cur, flags, nt);
      else sep_pass<decltype(a), decltype(b)>(op, out, cur, d, N[d], s[d], g, flags, nt);
      return 0;
    });
    if (r) return r;
    cur = out;
  }
  return 0;
}

// FP64 oracle for float outputs.  kernel: gaussian_blur_separable_{2d,3d} /
// mean_separable_{2d,3d} (whole X->Y->Z filter, double temporaries, same
// skip rule as clko_separable), sobel_2d, sobel_3d.  out = value; scale = a
// per-voxel magnitude bound of the terms summed (the same filter applied to
// |src|, for sobel the norm of the per-component sums of |coef * value|),
// the natural error scale of any float evaluation.
int clko_fp64(const char* kernel, int sdt, const void* src, const int shape[3], int ndim, const int N[3],
              const float s[3], int flags, double* out, double* scale, int nthreads) {
  const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
  const std::string k(kernel);
  const long n = (long)shape[0] * shape[1] * shape[2];
  const int W = shape[0], H = shape[1], Dd = shape[2];
  Vol S{(void*)src, sdt, W, H, Dd};
  auto rd = [&](int x, int y, int z) -> double {
    switch (sdt) {
      case U8: return fp64_read<uint8_t>(S, x, y, z);
      case I8: return fp64_read<int8_t>(S, x, y, z);
      case U16: return fp64_read<uint16_t>(S, x, y, z);
      case I16: return fp64_read<int16_t>(S, x, y, z);
      default: return fp64_read<float>(S, x, y, z);
    }
  };
  auto at = [&](int x, int y, int z) { return (long)x + (long)W * ((long)y + (long)H * z); };
  SepOp op;
  if (sep_op(k, &op) == 0) {
    if (op != GAUSS && op != MEAN) return -1;
    std::vector<double> cur(n), cura(n), nxt(n), nxta(n);
#pragma omp parallel for num_threads(nt)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / ((long)W * H));
      cur[i] = rd(x, y, z);
      cura[i] = std::fabs(cur[i]);
    }
    for (int d = 0; d < ndim; ++d) {
      const bool skip = N[d] <= 1 || (op == GAUSS && !(s[d] > 0));
      if (skip) continue;
      const int c = (N[d] - 1) / 2;
      std::vector<double> h;
      for (int v = -c; v <= c; ++v)
        h.push_back(op == GAUSS ? std::exp(-(double)v * v / (2.0 * (double)s[d] * (double)s[d])) : 1.0);
      double hs = 0;
      for (double q : h) hs += q;
      const int ext = d == 0 ? W : (d == 1 ? H : Dd);
#pragma omp parallel for num_threads(nt)
      for (long i = 0; i < n; ++i) {
        const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / ((long)W * H));
        const int p = d == 0 ? x : (d == 1 ? y : z);
        double a = 0, b = 0;
        for (int v = -c; v <= c; ++v) {
          const int q = clampi(p + v, ext - 1);
          const long j = d == 0 ? at(q, y, z) : (d == 1 ? at(x, q, z) : at(x, y, q));
          a += h[v + c] * cur[j];
          b += h[v + c] * cura[j];
        }
        nxt[i] = a / hs;
        nxta[i] = b / hs;
      }
      cur.swap(nxt);
      cura.swap(nxta);
    }
    std::memcpy(out, cur.data(), n * sizeof(double));
    std::memcpy(scale, cura.data(), n * sizeof(double));
    return 0;
  }
  if (k == "sobel_2d") {
#pragma omp parallel for num_threads(nt)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % W), y = (int)((i / W) % H);
      auto v = [&](int dx, int dy) { return (double)(float)rd(x + dx, y + dy, 0); };
      const double gx = -v(-1, -1) - 2 * v(-1, 0) - v(-1, 1) + v(1, -1) + 2 * v(1, 0) + v(1, 1);
      const double gy = -v(-1, -1) - 2 * v(0, -1) - v(1, -1) + v(-1, 1) + 2 * v(0, 1) + v(1, 1);
      const double ax = std::fabs(v(-1, -1)) + 2 * std::fabs(v(-1, 0)) + std::fabs(v(-1, 1)) + std::fabs(v(1, -1)) +
                        2 * std::fabs(v(1, 0)) + std::fabs(v(1, 1));
      const double ay = std::fabs(v(-1, -1)) + 2 * std::fabs(v(0, -1)) + std::fabs(v(1, -1)) + std::fabs(v(-1, 1)) +
                        2 * std::fabs(v(0, 1)) + std::fabs(v(1, 1));
      out[i] = std::sqrt(gx * gx + gy * gy);
      scale[i] = std::sqrt(ax * ax + ay * ay);
    }
    return 0;
  }
  if (k == "sobel_3d") {
    const bool narrow = (flags & CLKO_SOBEL_NARROW) != 0;
    const bool uns = sdt == U8 || sdt == U16;
#pragma omp parallel for num_threads(nt)
    for (long i = 0; i < n; ++i) {
      const int x = (int)(i % W), y = (int)((i / W) % H), z = (int)(i / ((long)W * H));
      double sum[3] = {0, 0, 0}, asum[3] = {0, 0, 0};
      for (int m = 0; m < 3; ++m)
        for (int nn = 0; nn < 3; ++nn)
          for (int kk = 0; kk < 4; ++kk) {
            const double v = rd(x + m - 1, y + nn - 1, z + kk - 1);
            for (int c = 0; c < 3; ++c) {
              const int co = sobel3d_coef(c, m, nn, kk);
              double t = (double)co * v;
              if (uns && !narrow) t = (double)((uint32_t)co * (uint32_t)v);
              sum[c] += t;
              asum[c] += std::fabs(t);
            }
          }
      out[i] = std::sqrt(sum[0] * sum[0] + sum[1] * sum[1] + sum[2] * sum[2]);
      scale[i] = std::sqrt(asum[0] * asum[0] + asum[1] * asum[1] + asum[2] * asum[2]);
    }
    return 0;
  }
  return -1;
}

// Offsets of the median neighbourhood (x, y, z triples in the kernel's loop
// order); returns the count, writes up to cap triples.
int clko_median_offsets(int sphere, int ndim, int Nx, int Ny, int Nz, int* out, int cap) {
  const auto off = median_offsets(sphere != 0, ndim, Nx, Ny, Nz);
  const int n = (int)off.size() / 3;
  for (int i = 0; i < n && i < cap; ++i)
    for (int j = 0; j < 3; ++j) out[3 * i + j] = off[3 * i + j];
  return n;
}

}  // extern "C"
