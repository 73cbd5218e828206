// clk_median.cu - fast median_box_3d 3x3x3, median_sphere_3d radius 2
// (33 voxels) and median_box_2d 3x3 for 8/16-bit integer images.
//
// The reference gathers the neighbourhood into an array and insertion-sorts
// it per voxel (median_box_3d_x.cl:3-20, median_sphere_3d_x.cl:3-20); the
// result is the element of rank n/2.  For integer pixels any exact
// selection of that rank gives the same value, so these kernels use pruned
// odd-even merge networks (clk_median_networks.cuh) and share work between
// neighbouring outputs:
//  * a thread computes two adjacent x outputs at once: 16-bit pixels sit in
//    the two halves of a 32-bit word and every min/max is one min.u16x2 /
//    min.s16x2 instruction (8-bit pixels are widened to 16-bit lanes);
//  * it walks along z; for every plane it sorts the 3x3 block around its
//    outputs once (three sorted columns merged into a sorted 9), which the
//    outputs of the planes above and below reuse;
//  * box: the merge of planes z and z+1 (ranks 4..13) serves the outputs at
//    z and z+1; each then needs one rank-9 selection against the third plane.
// Borders clamp exactly as the reference's reads do.
#include "clk_common.cuh"
#include "clk_median_networks.cuh"

namespace clk {

namespace {

// Two 16-bit lanes with unsigned or signed order.
template <bool SIGNED> struct Lanes {
  uint32_t v;
};
template <bool S> __device__ __forceinline__ Lanes<S> vmin(Lanes<S> a, Lanes<S> b) {
  Lanes<S> d;
  if constexpr (S) asm("min.s16x2 %0, %1, %2;" : "=r"(d.v) : "r"(a.v), "r"(b.v));
  else asm("min.u16x2 %0, %1, %2;" : "=r"(d.v) : "r"(a.v), "r"(b.v));
  return d;
}
template <bool S> __device__ __forceinline__ Lanes<S> vmax(Lanes<S> a, Lanes<S> b) {
  Lanes<S> d;
  if constexpr (S) asm("max.s16x2 %0, %1, %2;" : "=r"(d.v) : "r"(a.v), "r"(b.v));
  else asm("max.u16x2 %0, %1, %2;" : "=r"(d.v) : "r"(a.v), "r"(b.v));
  return d;
}

template <class T> struct LaneOf;
template <> struct LaneOf<uint16_t> { static constexpr bool S = false; };
template <> struct LaneOf<int16_t> { static constexpr bool S = true; };
template <> struct LaneOf<uint8_t> { static constexpr bool S = false; };
template <> struct LaneOf<int8_t> { static constexpr bool S = true; };

// Pixels (x, x+1) of a row as two 16-bit lanes; x even, x+1 < W.
template <class T> __device__ __forceinline__ uint32_t load_pair(const T* row, int x) {
  if constexpr (sizeof(T) == 2) {
    return __ldg(reinterpret_cast<const uint32_t*>(row + x));
  } else {
    const uint32_t w = __ldg(reinterpret_cast<const uint16_t*>(row + x));
    return LaneOf<T>::S ? __byte_perm(w, 0, 0x9180) : __byte_perm(w, 0, 0x4140);
  }
}
template <class T> __device__ __forceinline__ void store_pair(T* row, int x, uint32_t v) {
  if constexpr (sizeof(T) == 2) reinterpret_cast<uint32_t*>(row + x)[0] = v;
  else reinterpret_cast<uint16_t*>(row + x)[0] = (uint16_t)__byte_perm(v, 0, 0x0020);
}

// Lanes for the columns x-1, x, x+1 of the pair's outputs in one row:
// a = (x-1, x), b = (x, x+1), c = (x+1, x+2), clamped at the row ends.
template <class T>
__device__ __forceinline__ void row_cols(const T* row, int x, int W, uint32_t& a, uint32_t& b, uint32_t& c,
                                         uint32_t* far_l = nullptr, uint32_t* far_r = nullptr) {
  b = load_pair(row, x);
  const uint32_t l = x >= 2 ? load_pair(row, x - 2) : __byte_perm(b, 0, 0x1010);  // (x-2, x-1) clamped
  const uint32_t r = x + 2 < W ? load_pair(row, x + 2) : __byte_perm(b, 0, 0x3232);  // (x+2, x+3) clamped
  a = __byte_perm(l, b, 0x5432);
  c = __byte_perm(b, r, 0x5432);
  if (far_l) *far_l = l;
  if (far_r) *far_r = r;
}

template <class V, int N, int M> __device__ __forceinline__ void pick(const V (&w)[N], const int (&idx)[M], V (&o)[M]) {
#pragma unroll
  for (int k = 0; k < M; ++k) o[k] = w[idx[k]];
}

// Sorted 9 of the 3x3 block of plane (rows y-1..y+1, columns x-1..x+1) for
// both lanes, plus optionally the extra values the sphere needs.
template <class T, class V>
__device__ __forceinline__ void block9(const T* plane, int x, int y, int W, int H, V (&p)[9]) {
  V w[9];
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) {
    const T* row = plane + (int64_t)clampi(y + dy, H - 1) * W;
    uint32_t a, b, c;
    row_cols(row, x, W, a, b, c);
    w[dy + 1].v = a;
    w[dy + 4].v = b;
    w[dy + 7].v = c;
  }
  {
    V t[3] = {w[0], w[1], w[2]};
    net_sort3_raw(t);
    w[0] = t[net_sort3_out[0]], w[1] = t[net_sort3_out[1]], w[2] = t[net_sort3_out[2]];
  }
  {
    V t[3] = {w[3], w[4], w[5]};
    net_sort3_raw(t);
    w[3] = t[net_sort3_out[0]], w[4] = t[net_sort3_out[1]], w[5] = t[net_sort3_out[2]];
  }
  {
    V t[3] = {w[6], w[7], w[8]};
    net_sort3_raw(t);
    w[6] = t[net_sort3_out[0]], w[7] = t[net_sort3_out[1]], w[8] = t[net_sort3_out[2]];
  }
  net_merge333_raw(w);
  pick(w, net_merge333_out, p);
}

template <class V> __device__ __forceinline__ void merge_mid(const V (&a)[9], const V (&b)[9], V (&m)[10]) {
  V w[18];
#pragma unroll
  for (int k = 0; k < 9; ++k) w[k] = a[k], w[9 + k] = b[k];
  net_merge99_mid_raw(w);
  pick(w, net_merge99_mid_out, m);
}

template <class V> __device__ __forceinline__ V final27(const V (&m)[10], const V (&p)[9]) {
  V w[19];
#pragma unroll
  for (int k = 0; k < 10; ++k) w[k] = m[k];
#pragma unroll
  for (int k = 0; k < 9; ++k) w[10 + k] = p[k];
  net_box27_final_raw(w);
  return w[net_box27_final_out[0]];
}

constexpr int BX = 32;  // threads (= pairs) per row of a tile
constexpr int BY = 8;   // rows per tile

template <class T>
__global__ void __launch_bounds__(BX * BY) k_median_box27(const T* __restrict__ src, T* __restrict__ dst, int W,
                                                          int H, int D, int zchunk) {
  using V = Lanes<LaneOf<T>::S>;
  const int x = 2 * (blockIdx.x * BX + threadIdx.x);
  const int y = blockIdx.y * BY + threadIdx.y;
  if (x >= W || y >= H) return;
  const int z0 = blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  V pm1[9], p0[9];
  block9<T>(src + (int64_t)clampi(z0 - 1, D - 1) * plane, x, y, W, H, pm1);
  block9<T>(src + (int64_t)z0 * plane, x, y, W, H, p0);
  for (int zo = z0; zo < z1; zo += 2) {
    V p1[9], p2[9], m[10];
    block9<T>(src + (int64_t)clampi(zo + 1, D - 1) * plane, x, y, W, H, p1);
    block9<T>(src + (int64_t)clampi(zo + 2, D - 1) * plane, x, y, W, H, p2);
    merge_mid(p0, p1, m);
    store_pair(dst + (int64_t)zo * plane + (int64_t)y * W, x, final27(m, pm1).v);
    if (zo + 1 < z1) store_pair(dst + (int64_t)(zo + 1) * plane + (int64_t)y * W, x, final27(m, p2).v);
#pragma unroll
    for (int k = 0; k < 9; ++k) pm1[k] = p1[k], p0[k] = p2[k];
  }
}

// median_sphere_3d with Nx = Ny = Nz = 5: per output the 3x3 blocks of
// planes z-1, z, z+1, the four voxels at distance 2 in plane z and the two
// at distance 2 along z (33 = 9 + 9 + 9 + 4 + 2).
template <class T>
__global__ void __launch_bounds__(BX * BY) k_median_sphere33(const T* __restrict__ src, T* __restrict__ dst, int W,
                                                             int H, int D, int zchunk) {
  using V = Lanes<LaneOf<T>::S>;
  const int x = 2 * (blockIdx.x * BX + threadIdx.x);
  const int y = blockIdx.y * BY + threadIdx.y;
  if (x >= W || y >= H) return;
  const int z0 = blockIdx.z * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto centre = [&](int z) {
    V c;
    c.v = load_pair(src + (int64_t)clampi(z, D - 1) * plane + (int64_t)y * W, x);
    return c;
  };
  V pm1[9], p0[9];
  block9<T>(src + (int64_t)clampi(z0 - 1, D - 1) * plane, x, y, W, H, pm1);
  block9<T>(src + (int64_t)z0 * plane, x, y, W, H, p0);
  V cm2 = centre(z0 - 2);
  for (int zo = z0; zo < z1; ++zo) {
    V p1[9];
    const T* pz = src + (int64_t)clampi(zo + 1, D - 1) * plane;
    block9<T>(pz, x, y, W, H, p1);
    const T* pc = src + (int64_t)zo * plane;
    V w[33];
#pragma unroll
    for (int k = 0; k < 9; ++k) w[k] = pm1[k], w[9 + k] = p1[k], w[18 + k] = p0[k];
    {
      uint32_t a, b, c, fl, fr;
      row_cols(pc + (int64_t)y * W, x, W, a, b, c, &fl, &fr);
      w[27].v = fl;
      w[28].v = fr;
      w[29].v = load_pair(pc + (int64_t)clampi(y - 2, H - 1) * W, x);
      w[30].v = load_pair(pc + (int64_t)clampi(y + 2, H - 1) * W, x);
    }
    w[31] = cm2;
    w[32] = centre(zo + 2);
    const V cm1 = centre(zo - 1);
    net_sphere33_final_raw(w);
    store_pair(dst + (int64_t)zo * plane + (int64_t)y * W, x, w[net_sphere33_final_out[0]].v);
    cm2 = cm1;
#pragma unroll
    for (int k = 0; k < 9; ++k) pm1[k] = p0[k], p0[k] = p1[k];
  }
}

// median_box_2d 3x3.
template <class T>
__global__ void __launch_bounds__(BX * BY) k_median_box9_2d(const T* __restrict__ src, T* __restrict__ dst, int W,
                                                            int H) {
  using V = Lanes<LaneOf<T>::S>;
  const int x = 2 * (blockIdx.x * BX + threadIdx.x);
  const int y = blockIdx.y * BY + threadIdx.y;
  if (x >= W || y >= H) return;
  V w[9];
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) {
    uint32_t a, b, c;
    row_cols(src + (int64_t)clampi(y + dy, H - 1) * W, x, W, a, b, c);
    w[dy + 1].v = a;
    w[dy + 4].v = b;
    w[dy + 7].v = c;
  }
#pragma unroll
  for (int col = 0; col < 3; ++col) {
    V t[3] = {w[3 * col], w[3 * col + 1], w[3 * col + 2]};
    net_sort3_raw(t);
#pragma unroll
    for (int k = 0; k < 3; ++k) w[3 * col + k] = t[net_sort3_out[k]];
  }
  net_med9_raw(w);
  store_pair(dst + (int64_t)y * W, x, w[net_med9_out[0]].v);
}

enum Shape { BOX27, SPHERE33, BOX9_2D, OTHER };

Shape classify(bool sphere, const MedianNbhd& m, int ndim) {
  if (ndim == 3 && !sphere && m.ex == 1 && m.ey == 1 && m.ez == 1 && m.n == 27) return BOX27;
  if (ndim == 3 && sphere && m.ex == 2 && m.ey == 2 && m.ez == 2 && m.n == 33) return SPHERE33;
  if (ndim == 2 && m.ex == 1 && m.ey == 1 && m.n == 9) return BOX9_2D;  // box, or the 3x3 "sphere" that is a box
  return OTHER;
}

template <class T> clk_status launch(Shape sh, const Image& dst, const Image& src, cudaStream_t st) {
  const dim3 block(BX, BY);
  const int tx = (src.w / 2 + BX - 1) / BX, ty = (src.h + BY - 1) / BY;
  if (sh == BOX9_2D) {
    k_median_box9_2d<T><<<dim3(tx, ty), block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h);
  } else {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int chunks = 1;
    while ((int64_t)tx * ty * chunks < 8LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
    int zchunk = (src.d + chunks - 1) / chunks;
    zchunk += zchunk & 1;  // box: outputs come in z pairs
    const dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
    if (sh == BOX27)
      k_median_box27<T><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d, zchunk);
    else
      k_median_sphere33<T><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d, zchunk);
  }
  count_launch();
  return check_launch("median (networks)");
}

}  // namespace

clk_status fast_median(bool sphere, const Image& dst, const Image& src, const MedianNbhd& m, cudaStream_t st) {
  const Shape sh = classify(sphere, m, src.ndim);
  if (sh == OTHER || src.dt != dst.dt || src.dt == CLK_F32) return CLK_UNSUPPORTED_DTYPE;
  if (src.w % 2 != 0 || src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  const int align = dtype_size(src.dt) * 2;
  if (((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % align != 0) return CLK_UNSUPPORTED_DTYPE;
  switch (src.dt) {
    case CLK_U16: return launch<uint16_t>(sh, dst, src, st);
    case CLK_I16: return launch<int16_t>(sh, dst, src, st);
    case CLK_U8: return launch<uint8_t>(sh, dst, src, st);
    case CLK_I8: return launch<int8_t>(sh, dst, src, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
