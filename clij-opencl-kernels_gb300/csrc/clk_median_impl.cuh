// clk_median_impl.cuh - device code of the network medians (see clk_median.cu):
// lane types, pixel-pair access, the tile bodies and their kernels.  Shared
// by the plain launcher and the batch engine.
#pragma once
#include "clk_common.cuh"
#include "clk_median_networks.cuh"

namespace clk {
namespace med {

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

// Two order-preserving 32-bit keys of float pixels: the bits with the sign
// flipped for non-negative values and all bits flipped for negative ones, so
// unsigned order is float order (with -0 below +0 and NaNs at the ends).
struct Keys {
  uint32_t lo, hi;
};
__device__ __forceinline__ Keys vmin(Keys a, Keys b) { return Keys{min(a.lo, b.lo), min(a.hi, b.hi)}; }
__device__ __forceinline__ Keys vmax(Keys a, Keys b) { return Keys{max(a.lo, b.lo), max(a.hi, b.hi)}; }
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fval(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Pixel pairs (x, x+1) as network values: load/store, and the lane shuffles
// row_cols needs: lolo = (b.lo, b.lo), hihi = (b.hi, b.hi), hilo = (l.hi, b.lo).
template <class T> struct Px;
template <bool SG, int BYTES> struct Px16 {
  typedef Lanes<SG> V;
  static __device__ __forceinline__ V load(const void* row, int x) {
    V v;
    if constexpr (BYTES == 2) {
      v.v = __ldg(reinterpret_cast<const uint32_t*>(row) + x / 2);
    } else {
      const uint32_t w = __ldg(reinterpret_cast<const uint16_t*>(row) + x / 2);
      if constexpr (SG)  // sign-extend each byte to its 16-bit lane
        v.v = ((uint32_t)((int)(w << 24) >> 24) & 0xFFFFu) | ((uint32_t)((int)(w << 16) >> 24) << 16);
      else
        v.v = __byte_perm(w, 0, 0x4140);
    }
    return v;
  }
  static __device__ __forceinline__ void store(void* row, int x, V v) {
    if constexpr (BYTES == 2) reinterpret_cast<uint32_t*>(row)[x / 2] = v.v;
    else reinterpret_cast<uint16_t*>(row)[x / 2] = (uint16_t)__byte_perm(v.v, 0, 0x0020);
  }
  static __device__ __forceinline__ V lolo(V b) { return V{__byte_perm(b.v, 0, 0x1010)}; }
  static __device__ __forceinline__ V hihi(V b) { return V{__byte_perm(b.v, 0, 0x3232)}; }
  static __device__ __forceinline__ V hilo(V l, V b) { return V{__byte_perm(l.v, b.v, 0x5432)}; }
  template <class T> static __device__ __forceinline__ V make(T a, T b) {
    return V{(uint32_t)(uint16_t)(int16_t)a | ((uint32_t)(uint16_t)(int16_t)b << 16)};
  }
  template <class T> static __device__ __forceinline__ T lane(V v, int k) {
    return (T)(int16_t)(uint16_t)(k ? v.v >> 16 : v.v);
  }
};
template <> struct Px<uint16_t> : Px16<false, 2> {};
template <> struct Px<int16_t> : Px16<true, 2> {};
template <> struct Px<uint8_t> : Px16<false, 1> {};
template <> struct Px<int8_t> : Px16<true, 1> {};
template <> struct Px<float> {
  typedef Keys V;
  static __device__ __forceinline__ V load(const void* row, int x) {
    const float2 f = __ldg(reinterpret_cast<const float2*>(row) + x / 2);
    return Keys{fkey(f.x), fkey(f.y)};
  }
  static __device__ __forceinline__ void store(void* row, int x, V v) {
    reinterpret_cast<float2*>(row)[x / 2] = make_float2(fval(v.lo), fval(v.hi));
  }
  static __device__ __forceinline__ V lolo(V b) { return Keys{b.lo, b.lo}; }
  static __device__ __forceinline__ V hihi(V b) { return Keys{b.hi, b.hi}; }
  static __device__ __forceinline__ V hilo(V l, V b) { return Keys{l.hi, b.lo}; }
  template <class T> static __device__ __forceinline__ V make(T a, T b) { return Keys{fkey(a), fkey(b)}; }
  template <class T> static __device__ __forceinline__ T lane(V v, int k) { return fval(k ? v.hi : v.lo); }
};

// Pixels (x, x+1) of a row (x even, x < W).  ODD is the parity of W: rows
// of an even-width image are pair-aligned and load/store as one word; for an
// odd width they take two scalar accesses, x+1 clamped to the row on loads
// and skipped on stores.  (The parity is a template argument so that the
// even-width kernels carry no scalar path and no extra registers.)
template <class T, bool ODD> __device__ __forceinline__ typename Px<T>::V load_pair(const T* row, int x, int W) {
  if constexpr (!ODD) return Px<T>::load(row, x);
  else return Px<T>::template make<T>(__ldg(row + x), __ldg(row + min(x + 1, W - 1)));
}
template <class T, bool ODD>
__device__ __forceinline__ void store_pair(T* row, int x, int W, typename Px<T>::V v) {
  if constexpr (!ODD) {
    Px<T>::store(row, x, v);
  } else {
    row[x] = Px<T>::template lane<T>(v, 0);
    if (x + 1 < W) row[x + 1] = Px<T>::template lane<T>(v, 1);
  }
}

// Values for the columns x-1, x, x+1 of the pair's outputs in one row:
// a = (x-1, x), b = (x, x+1), c = (x+1, x+2), clamped at the row ends; far_l
// = (x-2, x-1) and far_r = (x+2, x+3), also clamped.
template <class T, bool ODD, class V = typename Px<T>::V>
__device__ __forceinline__ void row_cols(const T* row, int x, int W, V& a, V& b, V& c, V* far_l = nullptr,
                                         V* far_r = nullptr) {
  b = load_pair<T, ODD>(row, x, W);
  const V l = x >= 2 ? load_pair<T, ODD>(row, x - 2, W) : Px<T>::lolo(b);
  const V r = x + 2 < W ? load_pair<T, ODD>(row, x + 2, W) : Px<T>::hihi(b);
  a = Px<T>::hilo(l, b);
  c = Px<T>::hilo(b, r);
  if (far_l) *far_l = l;
  if (far_r) *far_r = r;
}

template <class V, int N, int M> __device__ __forceinline__ void pick(const V (&w)[N], const int (&idx)[M], V (&o)[M]) {
#pragma unroll
  for (int k = 0; k < M; ++k) o[k] = w[idx[k]];
}

// The 3x3 block of plane (rows y-1..y+1, columns x-1..x+1) for both lanes,
// unsorted (load9), and sorted (sort9 of those values; block9 = both).
template <class T, bool ODD, class V>
__device__ __forceinline__ void load9(const T* plane, int x, int y, int W, int H, V (&w)[9]) {
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) {
    const T* row = plane + (int64_t)clampi(y + dy, H - 1) * W;
    row_cols<T, ODD>(row, x, W, w[dy + 1], w[dy + 4], w[dy + 7]);
  }
}
template <class V> __device__ __forceinline__ void sort9(V (&w)[9], V (&p)[9]);
template <class T, bool ODD, class V>
__device__ __forceinline__ void block9(const T* plane, int x, int y, int W, int H, V (&p)[9]) {
  V w[9];
  load9<T, ODD>(plane, x, y, W, H, w);
  sort9(w, p);
}
template <class V> __device__ __forceinline__ void sort9(V (&w)[9], V (&p)[9]) {
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

// Tile bodies: tile (bx, by) x z-chunk bz, threads of a 256-thread CTA map to
// BX pairs x BY rows.  ODD must equal W & 1.
template <class T, bool ODD>
__device__ __forceinline__ void box27_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H, int D,
                                           int zchunk, int bx, int by, int bz) {
  using V = typename Px<T>::V;
  const int x = 2 * (bx * BX + (int)threadIdx.x % BX);
  const int y = by * BY + (int)threadIdx.x / BX;
  if (x >= W || y >= H) return;
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  V pm1[9], p0[9], r1[9], r2[9];
  block9<T, ODD>(src + (int64_t)clampi(z0 - 1, D - 1) * plane, x, y, W, H, pm1);
  block9<T, ODD>(src + (int64_t)z0 * plane, x, y, W, H, p0);
  load9<T, ODD>(src + (int64_t)clampi(z0 + 1, D - 1) * plane, x, y, W, H, r1);
  load9<T, ODD>(src + (int64_t)clampi(z0 + 2, D - 1) * plane, x, y, W, H, r2);
  for (int zo = z0; zo < z1; zo += 2) {
    // planes zo+1, zo+2 were loaded one pair ahead; the loads of zo+3,
    // zo+4 go out before this pair's networks
    V p1[9], p2[9], m[10];
    sort9(r1, p1);
    sort9(r2, p2);
    if (zo + 2 < z1) {
      load9<T, ODD>(src + (int64_t)clampi(zo + 3, D - 1) * plane, x, y, W, H, r1);
      load9<T, ODD>(src + (int64_t)clampi(zo + 4, D - 1) * plane, x, y, W, H, r2);
    }
    merge_mid(p0, p1, m);
    store_pair<T, ODD>(dst + (int64_t)zo * plane + (int64_t)y * W, x, W, final27(m, pm1));
    if (zo + 1 < z1) store_pair<T, ODD>(dst + (int64_t)(zo + 1) * plane + (int64_t)y * W, x, W, final27(m, p2));
#pragma unroll
    for (int k = 0; k < 9; ++k) pm1[k] = p1[k], p0[k] = p2[k];
  }
}

// median_box_3d 3x3x3 for 8/16-bit pixels with y pairs: a thread computes
// rows y and y+1 (and, as above, two x lanes and z pairs).  Their blocks
// share rows y and y+1: per plane the four rows y-1 .. y+2 are sorted along
// x once (net_sort3 of the lane words (x-1,x), (x,x+1), (x+1,x+2)), the two
// shared rows merged once (net_merge33) and each block completed with its
// own third row (net_merge63): 84 min/max for two sorted blocks instead of
// 108.
template <class T, bool ODD, class V>
__device__ __forceinline__ void load_rows4(const T* plane, int x, int y, int W, int H, V (&q)[12]) {
#pragma unroll
  for (int r = 0; r < 4; ++r)
    row_cols<T, ODD>(plane + (int64_t)clampi(y - 1 + r, H - 1) * W, x, W, q[3 * r], q[3 * r + 1], q[3 * r + 2]);
}
template <class V> __device__ __forceinline__ void blocks_ypair(V (&q)[12], V (&b0)[9], V (&b1)[9]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {  // each row's x-triple sorted in place
    V t[3] = {q[3 * r], q[3 * r + 1], q[3 * r + 2]};
    net_sort3_raw(t);
#pragma unroll
    for (int k = 0; k < 3; ++k) q[3 * r + k] = t[net_sort3_out[k]];
  }
  V m[6];
  {
    V w[6] = {q[3], q[4], q[5], q[6], q[7], q[8]};  // rows y, y+1
    net_merge33_raw(w);
    pick(w, net_merge33_out, m);
  }
  {
    V w[9] = {m[0], m[1], m[2], m[3], m[4], m[5], q[0], q[1], q[2]};  // + row y-1
    net_merge63_raw(w);
    pick(w, net_merge63_out, b0);
  }
  {
    V w[9] = {m[0], m[1], m[2], m[3], m[4], m[5], q[9], q[10], q[11]};  // + row y+2
    net_merge63_raw(w);
    pick(w, net_merge63_out, b1);
  }
}

constexpr int BYP = 2 * BY;  // rows per tile of the y-pair kernel

template <class T, bool ODD>
__device__ __forceinline__ void box27_ypair_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H, int D,
                                                 int zchunk, int bx, int by, int bz) {
  using V = typename Px<T>::V;
  const int x = 2 * (bx * BX + (int)threadIdx.x % BX);
  const int y = by * BYP + 2 * ((int)threadIdx.x / BX);
  if (x >= W || y >= H) return;
  const bool two = y + 1 < H;
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto pl = [&](int z) { return src + (int64_t)clampi(z, D - 1) * plane; };
  V am1[9], bm1[9], a0[9], b0[9];  // sorted blocks (row y: a, row y+1: b) of planes zo-1, zo
  V q1[12], q2[12];                // unsorted rows of planes zo+1, zo+2 (loaded one pair ahead)
  load_rows4<T, ODD>(pl(z0 - 1), x, y, W, H, q1);
  blocks_ypair(q1, am1, bm1);
  load_rows4<T, ODD>(pl(z0), x, y, W, H, q1);
  blocks_ypair(q1, a0, b0);
  load_rows4<T, ODD>(pl(z0 + 1), x, y, W, H, q1);
  load_rows4<T, ODD>(pl(z0 + 2), x, y, W, H, q2);
  for (int zo = z0; zo < z1; zo += 2) {
    V a1[9], b1[9], a2[9], b2[9];
    blocks_ypair(q1, a1, b1);
    blocks_ypair(q2, a2, b2);
    if (zo + 2 < z1) {
      load_rows4<T, ODD>(pl(zo + 3), x, y, W, H, q1);
      load_rows4<T, ODD>(pl(zo + 4), x, y, W, H, q2);
    }
    T* o0 = dst + (int64_t)zo * plane + (int64_t)y * W;
    {
      V m[10];
      merge_mid(a0, a1, m);
      store_pair<T, ODD>(o0, x, W, final27(m, am1));
      if (zo + 1 < z1) store_pair<T, ODD>(o0 + plane, x, W, final27(m, a2));
    }
    if (two) {
      V m[10];
      merge_mid(b0, b1, m);
      store_pair<T, ODD>(o0 + W, x, W, final27(m, bm1));
      if (zo + 1 < z1) store_pair<T, ODD>(o0 + plane + W, x, W, final27(m, b2));
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) am1[k] = a1[k], bm1[k] = b1[k], a0[k] = a2[k], b0[k] = b2[k];
  }
}

// The y-pair box median with each plane staged in shared memory (16-bit
// pixels, rows of whole 16-byte vectors): a CTA copies the clamped rows
// y0-1 .. y0+BYP of its 64 + 16 columns with cp.async, two planes ahead,
// into a ring of four plane buffers; tiles at the x border fill their
// outside vectors with the row's edge pixel, so a thread reads its words
// (x-2, x-1), (x, x+1), (x+2, x+3) from shared memory without clamping.
// The rows' loads then wait on shared memory instead of L1 / L2.
constexpr int SMR = BYP + 2;                 // staged rows
constexpr int SMW = 2 * BX + 16;             // staged pixels per row (8 each side)
constexpr int SMV = SMW / 8;                 // 16-byte vectors per staged row

__device__ __forceinline__ void med_cp_async16(void* sdst, const void* gsrc) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(sdst)),
               "l"(gsrc)
               : "memory");
}

// rows y0-HY .. y0-HY+NR-1 (clamped) of a plane, one vector per thread
template <int NR, int HY, class T>
__device__ __forceinline__ void stage_plane_async(const T* plane, int x0, int y0, int W, int H, uint16_t* buf) {
  static_assert(NR * SMV <= BX * BY, "one staging vector per thread");
  const int t = threadIdx.x;
  if (t < NR * SMV) {
    const int r = t / SMV, v = t - r * SMV;
    const int gx = x0 - 8 + 8 * v;
    if (gx >= 0 && gx < W)  // vectors outside the row are filled once landed
      med_cp_async16(buf + r * SMW + 8 * v, plane + (int64_t)clampi(y0 - HY + r, H - 1) * W + gx);
  }
}
template <int NR> __device__ __forceinline__ void fill_plane(uint16_t* buf, int x0, int W) {
  const int t = threadIdx.x;
  if (t < NR * SMV) {
    const int r = t / SMV, v = t - r * SMV;
    const int gx = x0 - 8 + 8 * v;
    if (gx < 0 || gx >= W) {
      const uint32_t e = (uint32_t)buf[r * SMW + (gx < 0 ? 0 : W - 1) - (x0 - 8)] * 0x10001u;
      *reinterpret_cast<uint4*>(buf + r * SMW + 8 * v) = make_uint4(e, e, e, e);
    }
  }
}
// rows y-1 .. y+2 of a staged plane as the lane words a, b, c of each row
template <class V> __device__ __forceinline__ void rows4_smem(const uint16_t* buf, int px, int py, V (&q)[12]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t* w = reinterpret_cast<const uint32_t*>(buf + (2 * py + r) * SMW) + px + 3;
    const uint32_t l = w[0], b = w[1], c = w[2];
    q[3 * r] = V{__byte_perm(l, b, 0x5432)};
    q[3 * r + 1] = V{b};
    q[3 * r + 2] = V{__byte_perm(b, c, 0x5432)};
  }
}

template <class T>
__device__ __forceinline__ void box27_staged_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H, int D,
                                                  int zchunk, int bx, int by, int bz) {
  static_assert(sizeof(T) == 2, "16-bit pixels");
  using V = typename Px<T>::V;
  __shared__ __align__(16) uint16_t buf[4][SMR * SMW];
  const int px = (int)threadIdx.x % BX, py = (int)threadIdx.x / BX;
  const int x0 = bx * 2 * BX, y0 = by * BYP;
  const int x = x0 + 2 * px, y = y0 + 2 * py;
  const bool act = x < W && y < H, two = y + 1 < H;
  const bool xb = x0 - 8 < 0 || x0 + SMW - 8 > W;  // outside vectors to fill
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto pl = [&](int z) { return src + (int64_t)clampi(z, D - 1) * plane; };
  V am1[9], bm1[9], a0[9], b0[9];  // sorted blocks (row y: a, row y+1: b) of planes zo-1, zo
  V q1[12], q2[12];
  stage_plane_async<SMR, 1>(pl(z0 - 1), x0, y0, W, H, buf[0]);
  stage_plane_async<SMR, 1>(pl(z0), x0, y0, W, H, buf[1]);
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 0;" ::: "memory");
  __syncthreads();
  if (xb) {
    fill_plane<SMR>(buf[0], x0, W);
    fill_plane<SMR>(buf[1], x0, W);
    __syncthreads();
  }
  rows4_smem(buf[0], px, py, q1);
  blocks_ypair(q1, am1, bm1);
  rows4_smem(buf[1], px, py, q1);
  blocks_ypair(q1, a0, b0);
  stage_plane_async<SMR, 1>(pl(z0 + 1), x0, y0, W, H, buf[2]);
  stage_plane_async<SMR, 1>(pl(z0 + 2), x0, y0, W, H, buf[3]);
  asm volatile("cp.async.commit_group;" ::: "memory");
  int slot = 2;  // buffers of planes zo+1, zo+2
  // one z pair: the blocks of planes zo-1, zo (pm1, p0; row y: a, row y+1:
  // b) are read, those of zo+1, zo+2 written to p1, p2.  Two calls per loop
  // trip with the sets swapped, so the blocks never move between registers.
  typedef V Blk[9];
  auto pair = [&](int zo, const Blk& am1_, const Blk& bm1_, const Blk& a0_, const Blk& b0_, Blk& a1_, Blk& b1_,
                  Blk& a2_, Blk& b2_) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();  // planes zo+1, zo+2 landed; the other pair's last reads are done
    if (xb) {
      fill_plane<SMR>(buf[slot], x0, W);
      fill_plane<SMR>(buf[slot + 1], x0, W);
      __syncthreads();
    }
    const int nslot = slot ^ 2;
    if (zo + 2 < z1) {
      stage_plane_async<SMR, 1>(pl(zo + 3), x0, y0, W, H, buf[nslot]);
      stage_plane_async<SMR, 1>(pl(zo + 4), x0, y0, W, H, buf[nslot + 1]);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    rows4_smem(buf[slot], px, py, q1);
    rows4_smem(buf[slot + 1], px, py, q2);
    blocks_ypair(q1, a1_, b1_);
    blocks_ypair(q2, a2_, b2_);
    T* o0 = dst + (int64_t)zo * plane + (int64_t)y * W;
    if (act) {
      V m[10];
      merge_mid(a0_, a1_, m);
      store_pair<T, false>(o0, x, W, final27(m, am1_));
      if (zo + 1 < z1) store_pair<T, false>(o0 + plane, x, W, final27(m, a2_));
    }
    if (act && two) {
      V m[10];
      merge_mid(b0_, b1_, m);
      store_pair<T, false>(o0 + W, x, W, final27(m, bm1_));
      if (zo + 1 < z1) store_pair<T, false>(o0 + plane + W, x, W, final27(m, b2_));
    }
    slot = nslot;
  };
  V a1[9], b1[9], a2[9], b2[9];
  for (int zo = z0; zo < z1; zo += 4) {
    pair(zo, am1, bm1, a0, b0, a1, b1, a2, b2);
    if (zo + 2 >= z1) break;
    pair(zo + 2, a1, b1, a2, b2, am1, bm1, a0, b0);
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// median_sphere_3d with Nx = Ny = Nz = 5: per output the 3x3 blocks of
// planes z-1, z, z+1, the four voxels at distance 2 in plane z and the two
// at distance 2 along z (33 = 9 + 9 + 9 + 4 + 2).
template <class T, bool ODD>
__device__ __forceinline__ void sphere33_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H, int D,
                                              int zchunk, int bx, int by, int bz) {
  using V = typename Px<T>::V;
  const int x = 2 * (bx * BX + (int)threadIdx.x % BX);
  const int y = by * BY + (int)threadIdx.x / BX;
  if (x >= W || y >= H) return;
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto centre = [&](int z) {
    return load_pair<T, ODD>(src + (int64_t)clampi(z, D - 1) * plane + (int64_t)y * W, x, W);
  };
  V pm1[9], p0[9];
  block9<T, ODD>(src + (int64_t)clampi(z0 - 1, D - 1) * plane, x, y, W, H, pm1);
  block9<T, ODD>(src + (int64_t)z0 * plane, x, y, W, H, p0);
  V cm2 = centre(z0 - 2);
  for (int zo = z0; zo < z1; ++zo) {
    V p1[9];
    const T* pz = src + (int64_t)clampi(zo + 1, D - 1) * plane;
    block9<T, ODD>(pz, x, y, W, H, p1);
    const T* pc = src + (int64_t)zo * plane;
    V w[33];
#pragma unroll
    for (int k = 0; k < 9; ++k) w[k] = pm1[k], w[9 + k] = p1[k], w[18 + k] = p0[k];
    {
      V a, b, c;
      row_cols<T, ODD>(pc + (int64_t)y * W, x, W, a, b, c, &w[27], &w[28]);
      w[29] = load_pair<T, ODD>(pc + (int64_t)clampi(y - 2, H - 1) * W, x, W);
      w[30] = load_pair<T, ODD>(pc + (int64_t)clampi(y + 2, H - 1) * W, x, W);
    }
    w[31] = cm2;
    w[32] = centre(zo + 2);
    const V cm1 = centre(zo - 1);
    net_sphere33_final_raw(w);
    store_pair<T, ODD>(dst + (int64_t)zo * plane + (int64_t)y * W, x, W, w[net_sphere33_final_out[0]]);
    cm2 = cm1;
#pragma unroll
    for (int k = 0; k < 9; ++k) pm1[k] = p0[k], p0[k] = p1[k];
  }
}

// median_sphere_3d r=2 in z pairs: outputs z and z+1 both use the sorted
// blocks of planes z and z+1, so their merge (net_merge99_r1_16) is computed
// once; each output then takes rank 15 of those 16, the sorted block of its
// other plane and its six singles (net_sphere33_pair_final).  187 min/max per
// output instead of 220.
template <class T, bool ODD>
__device__ __forceinline__ void sphere33_pair_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H,
                                                   int D, int zchunk, int bx, int by, int bz) {
  using V = typename Px<T>::V;
  const int x = 2 * (bx * BX + (int)threadIdx.x % BX);
  const int y = by * BY + (int)threadIdx.x / BX;
  if (x >= W || y >= H) return;
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto pl = [&](int z) { return src + (int64_t)clampi(z, D - 1) * plane; };
  auto centre = [&](int z) { return load_pair<T, ODD>(pl(z) + (int64_t)y * W, x, W); };
  // the six singles of output z: x -+ 2 and y -+ 2 in plane z, z -+ 2
  auto singles = [&](int z, V (&s)[6]) {
    const T* pc = pl(z);
    V a, b, c;
    row_cols<T, ODD>(pc + (int64_t)y * W, x, W, a, b, c, &s[0], &s[1]);
    s[2] = load_pair<T, ODD>(pc + (int64_t)clampi(y - 2, H - 1) * W, x, W);
    s[3] = load_pair<T, ODD>(pc + (int64_t)clampi(y + 2, H - 1) * W, x, W);
    s[4] = centre(z - 2);
    s[5] = centre(z + 2);
  };
  auto final = [&](const V (&m)[16], const V (&b)[9], const V (&s)[6]) {
    V w[31];
#pragma unroll
    for (int k = 0; k < 16; ++k) w[k] = m[k];
#pragma unroll
    for (int k = 0; k < 9; ++k) w[16 + k] = b[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[25 + k] = s[k];
    net_sphere33_pair_final_raw(w);
    return w[net_sphere33_pair_final_out[0]];
  };
  V bm1[9], b0[9], b1[9], b2[9];  // sorted blocks of planes zo-1 .. zo+2
  block9<T, ODD>(pl(z0 - 1), x, y, W, H, bm1);
  block9<T, ODD>(pl(z0), x, y, W, H, b0);
  block9<T, ODD>(pl(z0 + 1), x, y, W, H, b1);
  block9<T, ODD>(pl(z0 + 2), x, y, W, H, b2);
  V s0[6];
  singles(z0, s0);
  for (int zo = z0; zo < z1; zo += 2) {
    // the next pair's blocks (planes zo+3, zo+4) are loaded before this
    // pair's networks run and sorted after them: their latency hides
    // behind the merge and the two finals
    const bool more = zo + 2 < z1;
    V r3[9], r4[9];
    if (more) {
      load9<T, ODD>(pl(zo + 3), x, y, W, H, r3);
      load9<T, ODD>(pl(zo + 4), x, y, W, H, r4);
    }
    V m[16];
    {
      V w[18];
#pragma unroll
      for (int k = 0; k < 9; ++k) w[k] = b0[k], w[9 + k] = b1[k];
      net_merge99_r1_16_raw(w);
      pick(w, net_merge99_r1_16_out, m);
    }
    V s1[6];
    if (zo + 1 < z1) singles(zo + 1, s1);
    store_pair<T, ODD>(dst + (int64_t)zo * plane + (int64_t)y * W, x, W, final(m, bm1, s0));
    if (more) singles(zo + 2, s0);
    if (zo + 1 < z1) store_pair<T, ODD>(dst + (int64_t)(zo + 1) * plane + (int64_t)y * W, x, W, final(m, b2, s1));
    if (more) {
#pragma unroll
      for (int k = 0; k < 9; ++k) bm1[k] = b1[k], b0[k] = b2[k];
      sort9(r3, b1);
      sort9(r4, b2);
    }
  }
}

// The z-pair sphere median for 16-bit images whose rows are whole 16-byte
// vectors, its planes staged in shared memory: rows y0-2 .. y0+BY+1 of the
// tile's 64 + 16 columns (outside vectors filled with the row's edge pixel),
// in a ring of eight plane buffers.  The pair (zo, zo+1) reads planes zo-1 ..
// zo+4 while zo+5 and zo+6 land; every read is then a shared-memory word at a
// fixed offset, with no clamping and no row addressing per load.
constexpr int SPR = BY + 4;  // staged rows of a sphere tile
template <class T>
__device__ __forceinline__ void sphere33_staged_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H,
                                                     int D, int zchunk, int bx, int by, int bz) {
  static_assert(sizeof(T) == 2, "16-bit pixels");
  using V = typename Px<T>::V;
  __shared__ __align__(16) uint16_t buf[8][SPR * SMW];
  const int px = (int)threadIdx.x % BX, py = (int)threadIdx.x / BX;
  const int x0 = bx * 2 * BX, y0 = by * BY;
  const int x = x0 + 2 * px, y = y0 + py;
  const bool act = x < W && y < H;
  const bool xb = x0 - 8 < 0 || x0 + SMW - 8 > W;  // outside vectors to fill
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  auto slot = [&](int z) { return buf[(z - z0 + 2) & 7]; };  // planes z0-2 .. z1+4
  auto stage = [&](int z) { stage_plane_async<SPR, 2>(src + (int64_t)clampi(z, D - 1) * plane, x0, y0, W, H, slot(z)); };
  // the words (x-2, x-1), (x, x+1), (x+2, x+3) of row y+dy of plane z
  auto row = [&](int z, int dy) {
    return reinterpret_cast<const uint32_t*>(slot(z) + (py + 2 + dy) * SMW) + px + 3;
  };
  auto blk = [&](int z, V (&p)[9]) {
    V w[9];
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const uint32_t* r = row(z, dy);
      const uint32_t l = r[0], b = r[1], c = r[2];
      w[dy + 1] = V{__byte_perm(l, b, 0x5432)};
      w[dy + 4] = V{b};
      w[dy + 7] = V{__byte_perm(b, c, 0x5432)};
    }
    sort9(w, p);
  };
  auto centre = [&](int z) { return V{row(z, 0)[1]}; };
  auto singles = [&](int z, V (&s)[6]) {  // x -+ 2 and y -+ 2 in plane z, z -+ 2
    const uint32_t* r = row(z, 0);
    s[0] = V{r[0]};
    s[1] = V{r[2]};
    s[2] = V{row(z, -2)[1]};
    s[3] = V{row(z, 2)[1]};
    s[4] = centre(z - 2);
    s[5] = centre(z + 2);
  };
  auto final = [&](const V (&m)[16], const V (&b)[9], const V (&s)[6]) {
    V w[31];
#pragma unroll
    for (int k = 0; k < 16; ++k) w[k] = m[k];
#pragma unroll
    for (int k = 0; k < 9; ++k) w[16 + k] = b[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[25 + k] = s[k];
    net_sphere33_pair_final_raw(w);
    return w[net_sphere33_pair_final_out[0]];
  };
  for (int z = z0 - 2; z <= z0 + 2; ++z) stage(z);
  asm volatile("cp.async.commit_group;" ::: "memory");
  stage(z0 + 3);
  stage(z0 + 4);
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 1;" ::: "memory");
  __syncthreads();
  if (xb) {
    for (int z = z0 - 2; z <= z0 + 2; ++z) fill_plane<SPR>(slot(z), x0, W);
    __syncthreads();
  }
  V bm1[9], b0[9], b1[9], b2[9];  // sorted blocks of planes zo-1 .. zo+2
  blk(z0 - 1, bm1);
  blk(z0, b0);
  blk(z0 + 1, b1);
  blk(z0 + 2, b2);
  V s0[6];
  singles(z0, s0);
  // one z pair from the blocks of planes zo-1 .. zo+2 (pm1, p0, p1, p2); the
  // next pair's zo+3, zo+4 replace pm1, p0.  Two calls per loop trip with
  // the sets swapped, so the blocks never move between registers.
  typedef V Blk[9];
  auto pair = [&](int zo, Blk& pm1, Blk& p0, const Blk& p1, const Blk& p2) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();  // planes zo+3, zo+4 landed; the reads of zo-3, zo-2 are done
    if (xb) {
      fill_plane<SPR>(slot(zo + 3), x0, W);
      fill_plane<SPR>(slot(zo + 4), x0, W);
      __syncthreads();
    }
    const bool more = zo + 2 < z1;
    if (more) {  // the next pair's planes zo+5, zo+6 into the buffers of zo-3, zo-2
      stage(zo + 5);
      stage(zo + 6);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    V m[16];
    {
      V w[18];
#pragma unroll
      for (int k = 0; k < 9; ++k) w[k] = p0[k], w[9 + k] = p1[k];
      net_merge99_r1_16_raw(w);
      pick(w, net_merge99_r1_16_out, m);
    }
    V s1[6];
    if (zo + 1 < z1) singles(zo + 1, s1);
    T* o = dst + (int64_t)zo * plane + (int64_t)y * W;
    if (act) store_pair<T, false>(o, x, W, final(m, pm1, s0));
    if (more) singles(zo + 2, s0);
    if (act && zo + 1 < z1) store_pair<T, false>(o + plane, x, W, final(m, p2, s1));
    if (more) {
      blk(zo + 3, pm1);
      blk(zo + 4, p0);
    }
  };
  for (int zo = z0; zo < z1; zo += 4) {
    pair(zo, bm1, b0, b1, b2);
    if (zo + 2 >= z1) break;
    pair(zo + 2, b1, b2, bm1, b0);
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// The same z-pair sphere median for float images whose rows are whole
// 16-byte vectors: one output column per thread (a 32 x 8 tile), each
// pixel's order-preserving key computed once in shared memory by the thread
// that copied it (cp.async lands the raw floats; the copying thread waits for
// its own group, converts its vector in place, and the barrier publishes the
// keys).  Outside vectors hold the key of the row's edge pixel, read from
// global memory when the plane is issued.  Rows y0-2 .. y0+BY+1, columns
// x0-4 .. x0+35, in the same ring of eight planes.
struct Key1 {
  uint32_t v;
};
__device__ __forceinline__ Key1 vmin(Key1 a, Key1 b) { return Key1{min(a.v, b.v)}; }
__device__ __forceinline__ Key1 vmax(Key1 a, Key1 b) { return Key1{max(a.v, b.v)}; }
constexpr int FSW = BX + 8;    // staged floats per row
constexpr int FSV = FSW / 4;   // 16-byte vectors per row
static_assert(SPR * FSV <= BX * BY, "one staging vector per thread");

__device__ __forceinline__ void sphere33_staged_f32_tile(const float* __restrict__ src, float* __restrict__ dst,
                                                         int W, int H, int D, int zchunk, int bx, int by, int bz) {
  using V = Key1;
  __shared__ __align__(16) uint32_t buf[8][SPR * FSW];
  const int tid = threadIdx.x, px = tid % BX, py = tid / BX;
  const int x0 = bx * BX, y0 = by * BY;
  const int x = x0 + px, y = y0 + py;
  const bool act = x < W && y < H;
  const int z0 = bz * zchunk, z1 = min(D, z0 + zchunk);
  const int64_t plane = (int64_t)W * H;
  // this thread's staging vector: row sr, columns x0-4+4sv .. +3
  const int sr = tid / FSV, sv = tid - sr * FSV, sgx = x0 - 4 + 4 * sv;
  const bool stager = tid < SPR * FSV, inside = sgx >= 0 && sgx < W;
  const int64_t srow = (int64_t)clampi(y0 - 2 + sr, H - 1) * W;
  auto slot = [&](int z) { return buf[(z - z0 + 2) & 7]; };
  auto stage = [&](int z) {
    if (!stager) return;
    const float* p = src + (int64_t)clampi(z, D - 1) * plane + srow;
    uint32_t* b = slot(z) + sr * FSW + 4 * sv;
    if (inside) {
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(b)),
                   "l"(p + sgx)
                   : "memory");
    } else {
      const uint32_t k = fkey(__ldg(p + (sgx < 0 ? 0 : W - 1)));
      *reinterpret_cast<uint4*>(b) = make_uint4(k, k, k, k);
    }
  };
  auto convert = [&](int z) {  // after this thread's copies landed: floats to keys in place
    if (!stager || !inside) return;
    uint4* b = reinterpret_cast<uint4*>(slot(z) + sr * FSW + 4 * sv);
    const uint4 f = *b;
    *b = make_uint4(fkey(__uint_as_float(f.x)), fkey(__uint_as_float(f.y)), fkey(__uint_as_float(f.z)),
                    fkey(__uint_as_float(f.w)));
  };
  auto row = [&](int z, int dy) { return slot(z) + (py + 2 + dy) * FSW + px + 4; };  // key of (x, y+dy)
  auto blk = [&](int z, V (&p)[9]) {
    V w[9];
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
      const uint32_t* r = row(z, dy);
      w[dy + 1] = V{r[-1]};
      w[dy + 4] = V{r[0]};
      w[dy + 7] = V{r[1]};
    }
    sort9(w, p);
  };
  auto centre = [&](int z) { return V{row(z, 0)[0]}; };
  auto singles = [&](int z, V (&s)[6]) {
    const uint32_t* r = row(z, 0);
    s[0] = V{r[-2]};
    s[1] = V{r[2]};
    s[2] = V{row(z, -2)[0]};
    s[3] = V{row(z, 2)[0]};
    s[4] = centre(z - 2);
    s[5] = centre(z + 2);
  };
  auto final = [&](const V (&m)[16], const V (&b)[9], const V (&s)[6]) {
    V w[31];
#pragma unroll
    for (int k = 0; k < 16; ++k) w[k] = m[k];
#pragma unroll
    for (int k = 0; k < 9; ++k) w[16 + k] = b[k];
#pragma unroll
    for (int k = 0; k < 6; ++k) w[25 + k] = s[k];
    net_sphere33_pair_final_raw(w);
    return w[net_sphere33_pair_final_out[0]];
  };
  for (int z = z0 - 2; z <= z0 + 2; ++z) stage(z);
  asm volatile("cp.async.commit_group;" ::: "memory");
  stage(z0 + 3);
  stage(z0 + 4);
  asm volatile("cp.async.commit_group;" ::: "memory");
  asm volatile("cp.async.wait_group 1;" ::: "memory");
  for (int z = z0 - 2; z <= z0 + 2; ++z) convert(z);
  __syncthreads();
  V bm1[9], b0[9], b1[9], b2[9];  // sorted blocks of planes zo-1 .. zo+2
  blk(z0 - 1, bm1);
  blk(z0, b0);
  blk(z0 + 1, b1);
  blk(z0 + 2, b2);
  V s0[6];
  singles(z0, s0);
  typedef V Blk[9];  // z pairs with the block sets swapped, as in the 16-bit kernel
  auto pair = [&](int zo, Blk& pm1, Blk& p0, const Blk& p1, const Blk& p2) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    convert(zo + 3);
    convert(zo + 4);
    __syncthreads();  // planes zo+3, zo+4 hold keys; the reads of zo-3, zo-2 are done
    const bool more = zo + 2 < z1;
    if (more) {  // the next pair's planes zo+5, zo+6 into the buffers of zo-3, zo-2
      stage(zo + 5);
      stage(zo + 6);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
    V m[16];
    {
      V w[18];
#pragma unroll
      for (int k = 0; k < 9; ++k) w[k] = p0[k], w[9 + k] = p1[k];
      net_merge99_r1_16_raw(w);
      pick(w, net_merge99_r1_16_out, m);
    }
    V s1[6];
    if (zo + 1 < z1) singles(zo + 1, s1);
    float* o = dst + (int64_t)zo * plane + (int64_t)y * W + x;
    if (act) *o = fval(final(m, pm1, s0).v);
    if (more) singles(zo + 2, s0);
    if (act && zo + 1 < z1) o[plane] = fval(final(m, p2, s1).v);
    if (more) {
      blk(zo + 3, pm1);
      blk(zo + 4, p0);
    }
  };
  for (int zo = z0; zo < z1; zo += 4) {
    pair(zo, bm1, b0, b1, b2);
    if (zo + 2 >= z1) break;
    pair(zo + 2, b1, b2, bm1, b0);
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// median_box_2d 3x3.
template <class T, bool ODD>
__device__ __forceinline__ void box9_2d_tile(const T* __restrict__ src, T* __restrict__ dst, int W, int H, int bx,
                                             int by) {
  using V = typename Px<T>::V;
  const int x = 2 * (bx * BX + (int)threadIdx.x % BX);
  const int y = by * BY + (int)threadIdx.x / BX;
  if (x >= W || y >= H) return;
  V w[9];
#pragma unroll
  for (int dy = -1; dy <= 1; ++dy) row_cols<T, ODD>(src + (int64_t)clampi(y + dy, H - 1) * W, x, W, w[dy + 1], w[dy + 4], w[dy + 7]);
#pragma unroll
  for (int col = 0; col < 3; ++col) {
    V t[3] = {w[3 * col], w[3 * col + 1], w[3 * col + 2]};
    net_sort3_raw(t);
#pragma unroll
    for (int k = 0; k < 3; ++k) w[3 * col + k] = t[net_sort3_out[k]];
  }
  net_med9_raw(w);
  store_pair<T, ODD>(dst + (int64_t)y * W, x, W, w[net_med9_out[0]]);
}

template <class T, bool ODD>
__global__ void __launch_bounds__(BX * BY) k_median_box27(const T* __restrict__ src, T* __restrict__ dst, int W,
                                                          int H, int D, int zchunk) {
  box27_tile<T, ODD>(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <class T, bool ODD>
__global__ void __launch_bounds__(BX * BY, 2) k_median_box27_yp(const T* __restrict__ src, T* __restrict__ dst,
                                                                 int W, int H, int D, int zchunk) {
  box27_ypair_tile<T, ODD>(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <class T>
__global__ void __launch_bounds__(BX * BY, 2) k_median_box27_st(const T* __restrict__ src, T* __restrict__ dst,
                                                                 int W, int H, int D, int zchunk) {
  box27_staged_tile<T>(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
// 16-bit pixels fit the sphere network in 64 registers without spilling:
// four CTAs per SM instead of three
template <class T> constexpr int sphere_min_ctas() { return sizeof(T) == 2 ? 4 : sizeof(T) == 1 ? 3 : 2; }

// the z-pair kernel holds four sorted blocks and the shared merge
template <class T> constexpr int sphere_pair_min_ctas() { return 2; }

template <class T, bool ODD>
__global__ void __launch_bounds__(BX * BY, sphere_pair_min_ctas<T>()) k_median_sphere33_pair(const T* __restrict__ src,
                                                                                     T* __restrict__ dst, int W,
                                                                                     int H, int D, int zchunk) {
  sphere33_pair_tile<T, ODD>(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <class T>
__global__ void __launch_bounds__(BX * BY, 2) k_median_sphere33_st(const T* __restrict__ src, T* __restrict__ dst,
                                                                    int W, int H, int D, int zchunk) {
  sphere33_staged_tile<T>(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <class T>  // T = float (a template: this header is included by several translation units)
__global__ void __launch_bounds__(BX * BY, 2) k_median_sphere33_stf(const T* __restrict__ src, T* __restrict__ dst,
                                                                     int W, int H, int D, int zchunk) {
  sphere33_staged_f32_tile(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <class T, bool ODD>
__global__ void __launch_bounds__(BX * BY, sphere_min_ctas<T>()) k_median_sphere33(const T* __restrict__ src, T* __restrict__ dst, int W,
                                                             int H, int D, int zchunk) {
  sphere33_tile<T, ODD>(src, dst, W, H, D, zchunk, blockIdx.x, blockIdx.y, blockIdx.z);
}
template <class T, bool ODD>
__global__ void __launch_bounds__(BX * BY) k_median_box9_2d(const T* __restrict__ src, T* __restrict__ dst, int W,
                                                            int H) {
  // one plane per blockIdx.z: a 2-D image, or a 3x3 neighbourhood on every
  // plane of a 3-D image (Nz = 1, slice by slice)
  const int64_t plane = (int64_t)W * H * blockIdx.z;
  box9_2d_tile<T, ODD>(src + plane, dst + plane, W, H, blockIdx.x, blockIdx.y);
}

}  // namespace med
}  // namespace clk
