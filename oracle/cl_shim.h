// cl_shim.h - TEST INFRASTRUCTURE ONLY (oracle).  Lets the reference's
// CLIJ-dialect OpenCL C kernels (kernels/*.cl) compile unchanged as C++ so
// that they can run on the host as the "reference" CPU implementation.
//
// What it supplies, and why each choice:
//  * OpenCL qualifiers (__kernel, __constant, __global) as no-ops, and
//    sampler_t / the CLK_* sampler flags as plain ints: every neighbourhood
//    kernel declares CLK_ADDRESS_CLAMP_TO_EDGE (e.g. sobel_3d_x.cl:1), which
//    the read below always applies.
//  * int2 / int4 aggregates with the + and scalar * the kernels use
//    (coord + v*dir at gaussian_blur_separable_3d_x.cl:30).
//  * get_global_id(d): a thread-local id set by the host loop.
//  * exp / sqrt / min / max with OpenCL's float overloads.  exp(float) is the
//    correctly rounded float of exp (computed through double); the library's
//    host code uses the same rule for Gaussian weights.
//  * The preamble placeholders (README.md:25-141), restated:
//      READ_<img>_IMAGE(img, sampler, pos).x  - buffer read with the
//        coordinate clamped to [0, extent-1] per axis; .x has the type of
//        read_imageui / read_imagei / read_imagef (README.md:103-116):
//        uint for uchar/ushort, int for char/short, float for float.
//      WRITE_<img>_IMAGE(img, pos, v)         - buffer store.
//      CONVERT_<img>_PIXEL_TYPE(x)            - clij_convert_<T>_sat: clamp
//        to the type's range, truncate toward zero, NaN -> 0.
//  The per-image macros refer to the type names SRC_T / DST_T, which the
//  generated translation unit typedefs in one namespace per pixel-type pair.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>

#define __kernel
#define __constant static const
#define __global
#define __private
#define __read_only
#define __write_only

namespace clkcl {

typedef int sampler_t;
enum { CLK_NORMALIZED_COORDS_FALSE = 0, CLK_ADDRESS_CLAMP_TO_EDGE = 0, CLK_FILTER_NEAREST = 0 };
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;

struct int2 { int x, y; };
struct int4 { int x, y, z, w; };
static inline int2 operator+(int2 a, int2 b) { return int2{a.x + b.x, a.y + b.y}; }
static inline int4 operator+(int4 a, int4 b) { return int4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
static inline int2 operator*(int a, int2 b) { return int2{a * b.x, a * b.y}; }
static inline int4 operator*(int a, int4 b) { return int4{a * b.x, a * b.y, a * b.z, a * b.w}; }
static inline int2 operator*(int2 b, int a) { return a * b; }
static inline int4 operator*(int4 b, int a) { return a * b; }

extern thread_local int clk_gid[3];
static inline int get_global_id(int d) { return clk_gid[d]; }

static inline float exp(float x) { return (float)std::exp((double)x); }
static inline double exp(double x) { return std::exp(x); }
static inline float sqrt(float x) { return std::sqrt(x); }
static inline double sqrt(double x) { return std::sqrt(x); }
// OpenCL C min/max: min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x.
template <class T> static inline T min(T x, T y) { return y < x ? y : x; }
template <class T> static inline T max(T x, T y) { return x < y ? y : x; }

template <class T> struct clk_img {
  T* p;
  int w, h, d;
};

template <class T> struct clk_read_type;
template <> struct clk_read_type<uint8_t> { typedef uint type; };
template <> struct clk_read_type<uint16_t> { typedef uint type; };
template <> struct clk_read_type<int8_t> { typedef int type; };
template <> struct clk_read_type<int16_t> { typedef int type; };
template <> struct clk_read_type<float> { typedef float type; };

template <class R> struct clk_texel { R x; };

static inline int clk_clampi(int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); }

template <class T>
static inline clk_texel<typename clk_read_type<T>::type> clk_read(const clk_img<T>& im, int2 p) {
  const long x = clk_clampi(p.x, im.w - 1), y = clk_clampi(p.y, im.h - 1);
  return {(typename clk_read_type<T>::type)im.p[x + (long)im.w * y]};
}
template <class T>
static inline clk_texel<typename clk_read_type<T>::type> clk_read(const clk_img<T>& im, int4 p) {
  const long x = clk_clampi(p.x, im.w - 1), y = clk_clampi(p.y, im.h - 1), z = clk_clampi(p.z, im.d - 1);
  return {(typename clk_read_type<T>::type)im.p[x + (long)im.w * (y + (long)im.h * z)]};
}
template <class T, class V> static inline void clk_write(clk_img<T>& im, int2 p, V v) {
  im.p[p.x + (long)im.w * p.y] = (T)v;
}
template <class T, class V> static inline void clk_write(clk_img<T>& im, int4 p, V v) {
  im.p[p.x + (long)im.w * (p.y + (long)im.h * p.z)] = (T)v;
}

template <class D> struct clk_limits;
template <> struct clk_limits<uint8_t> { static constexpr double lo = 0, hi = 255; };
template <> struct clk_limits<int8_t> { static constexpr double lo = -128, hi = 127; };
template <> struct clk_limits<uint16_t> { static constexpr double lo = 0, hi = 65535; };
template <> struct clk_limits<int16_t> { static constexpr double lo = -32768, hi = 32767; };

template <class D, class X> static inline D clk_convert_sat(X x) {
  const double v = (double)x;
  if (v != v) return (D)0;
  if (v <= clk_limits<D>::lo) return (D)clk_limits<D>::lo;
  if (v >= clk_limits<D>::hi) return (D)clk_limits<D>::hi;
  return (D)(long long)v;  // truncation toward zero
}
template <> inline float clk_convert_sat<float, float>(float x) { return x; }
template <> inline float clk_convert_sat<float, double>(double x) { return (float)x; }
template <> inline float clk_convert_sat<float, int>(int x) { return (float)x; }
template <> inline float clk_convert_sat<float, uint>(uint x) { return (float)x; }

// sobel_3d_x.cl:17-19 declares int g?[3][3][3] and its k<=3 loop (:46) reads
// g?[m][n][3], i.e. flat element 9m+3n+3, which for m=n=2 lies past the
// array.  The oracle backs each array with one zero element after it so that
// this single out-of-range tap reads 0 (the pinned policy); every other k=3
// tap reads the next row exactly as the flat layout implies.
struct clk_sobel_array {
  int a[3][3][3];
  int pad;
};
#define CLK_SOBEL_ARRAY(name)      \
  clk_sobel_array name##_storage{}; \
  int(&name)[3][3][3] = name##_storage.a

}  // namespace clkcl

#define IMAGE_src_TYPE clk_img<SRC_T>
#define IMAGE_dst_TYPE clk_img<DST_T>
#define IMAGE_src_PIXEL_TYPE SRC_T
#define IMAGE_dst_PIXEL_TYPE DST_T
#define READ_src_IMAGE(img, smp, ...) clk_read(img, __VA_ARGS__)
// convolve_{2d,3d}_x.cl: a float kernel image and the untyped accessors
#define IMAGE_kernelImage_TYPE clk_img<float>
#define READ_IMAGE(img, smp, ...) clk_read(img, __VA_ARGS__)
#define WRITE_IMAGE(img, ...) clk_write(img, __VA_ARGS__)
#define GET_IMAGE_WIDTH(img) ((img).w)
#define GET_IMAGE_HEIGHT(img) ((img).h)
#define GET_IMAGE_DEPTH(img) ((img).d)
// greater_constant_{2d,3d}_x.cl name their input src1
#define IMAGE_src1_TYPE clk_img<SRC_T>
#define IMAGE_src1_PIXEL_TYPE SRC_T
#define READ_src1_IMAGE(img, smp, ...) clk_read(img, __VA_ARGS__)
#define WRITE_dst_IMAGE(img, ...) clk_write(img, __VA_ARGS__)
#define CONVERT_dst_PIXEL_TYPE(x) clk_convert_sat<DST_T>(x)
#ifndef MAX_ARRAY_SIZE
#define MAX_ARRAY_SIZE 1024
#endif
