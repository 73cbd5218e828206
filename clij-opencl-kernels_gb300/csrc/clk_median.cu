// clk_median.cu - fast median_box_3d 3x3x3, median_sphere_3d radius 2
// (33 voxels) and median_box_2d 3x3 (also the 3x3 of every plane of the
// slice-by-slice box) for 8/16-bit integer images and, on 32-bit
// order-preserving keys, float images.
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
//    z and z+1; each then needs one rank-9 selection against the third plane;
//    8/16-bit pixels also pair rows y and y+1, whose blocks share two sorted
//    rows (k_median_box27_yp); 16-bit images whose rows are whole 16-byte
//    vectors stage each plane tile in shared memory with cp.async, two
//    planes ahead, and read the rows from there (k_median_box27_st);
//  * sphere (8/16-bit): likewise the merge of planes z and z+1 (16 ranks)
//    serves z and z+1, each adding its other plane's block and six singles;
//    16-bit rows of whole vectors read staged planes from a ring of eight in
//    shared memory (k_median_sphere33_st); float rows of whole vectors run
//    the same pairs on one column per thread, with the keys computed once in
//    shared memory (k_median_sphere33_stf);
//  * the staged kernels alternate two register sets of sorted blocks from
//    one z pair to the next instead of moving them;
//  * the next z-pair's planes are loaded before the current pair's networks.
// Borders clamp exactly as the reference's reads do.
#include <cstdlib>

#include "clk_median_impl.cuh"

namespace clk {

namespace {

using namespace med;

enum Shape { BOX27, SPHERE33, BOX9_2D, OTHER };

Shape classify(bool sphere, const MedianNbhd& m, int ndim) {
  if (ndim == 3 && !sphere && m.ex == 1 && m.ey == 1 && m.ez == 1 && m.n == 27) return BOX27;
  if (ndim == 3 && sphere && m.ex == 2 && m.ey == 2 && m.ez == 2 && m.n == 33) return SPHERE33;
  // 3x3 in every plane: the 2-D box (or the 3x3 "sphere" that is a box), a
  // 3-D box with Nz = 1, the slice-by-slice box
  if (m.ex == 1 && m.ey == 1 && m.ez == 0 && m.n == 9) return BOX9_2D;
  return OTHER;
}

// CLK_MEDIAN_YPAIR=0 in the environment keeps the box median on the
// one-row kernel (A/B timing)
bool ypair_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_MEDIAN_YPAIR");
    return !(e && e[0] == '0');
  }();
  return on;
}

// CLK_MEDIAN_STAGED=0 in the environment keeps the medians' rows on global
// loads (A/B timing)
bool staged_enabled() {
  static const bool on = [] {
    const char* e = getenv("CLK_MEDIAN_STAGED");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <class T, bool ODD> clk_status launch(Shape sh, const Image& dst, const Image& src, cudaStream_t st) {
  const dim3 block(BX * BY);
  const int tx = ((src.w + 1) / 2 + BX - 1) / BX, ty = (src.h + BY - 1) / BY;
  if (sh == BOX9_2D) {
    k_median_box9_2d<T, ODD><<<dim3(tx, ty, src.d), block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h);
  } else {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int chunks = 1;
    while ((int64_t)tx * ty * chunks < 8LL * sms && src.d / (chunks * 2) >= 16) chunks *= 2;
    int zchunk = (src.d + chunks - 1) / chunks;
    zchunk += zchunk & 1;  // outputs come in z pairs
    const dim3 grid(tx, ty, (src.d + zchunk - 1) / zchunk);
    bool done = false;
    if constexpr (sizeof(T) == 2 && !ODD) {  // planes staged in shared memory: 16-bit rows of whole vectors
      if (sh == BOX27 && ypair_enabled() && staged_enabled() && src.w % 8 == 0 &&
          ((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % 16 == 0) {
        const dim3 gy(tx, (src.h + BYP - 1) / BYP, grid.z);
        k_median_box27_st<T><<<gy, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d, zchunk);
        done = true;
      } else if (sh == SPHERE33 && staged_enabled() && src.w % 8 == 0 &&
                 ((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % 16 == 0) {
        k_median_sphere33_st<T><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d, zchunk);
        done = true;
      }
    }
    if constexpr (sizeof(T) <= 2) {  // y pairs: 8/16-bit lanes (float keys would spill)
      if (!done && sh == BOX27 && ypair_enabled()) {
        const dim3 gy(tx, (src.h + BYP - 1) / BYP, grid.z);
        k_median_box27_yp<T, ODD><<<gy, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d,
                                                        zchunk);
        done = true;
      }
    }
    if constexpr (sizeof(T) == 4) {  // float rows of whole vectors: keys staged in shared memory
      if (sh == SPHERE33 && staged_enabled() && src.w % 4 == 0 &&
          ((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % 16 == 0) {
        const dim3 gf((src.w + BX - 1) / BX, grid.y, grid.z);
        k_median_sphere33_stf<float><<<gf, block, 0, st>>>((const float*)src.ptr, (float*)dst.ptr, src.w, src.h, src.d,
                                                    zchunk);
        done = true;
      }
    }
    if (done) {
    } else if (sh == BOX27)
      k_median_box27<T, ODD><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d, zchunk);
    else if constexpr (sizeof(T) == 4)  // float keys: the pair kernel's registers would leave one CTA per SM
      k_median_sphere33<T, ODD><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d, zchunk);
    else
      k_median_sphere33_pair<T, ODD><<<grid, block, 0, st>>>((const T*)src.ptr, (T*)dst.ptr, src.w, src.h, src.d,
                                                             zchunk);
  }
  count_launch();
  return check_launch("median (networks)");
}

}  // namespace

clk_status fast_median(bool sphere, const Image& dst, const Image& src, const MedianNbhd& m, cudaStream_t st) {
  const Shape sh = classify(sphere, m, src.ndim);
  if (sh == OTHER || src.dt != dst.dt) return CLK_UNSUPPORTED_DTYPE;
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d) return CLK_UNSUPPORTED_DTYPE;
  const int align = dtype_size(src.dt) * 2;
  if (((uintptr_t)src.ptr | (uintptr_t)dst.ptr) % align != 0) return CLK_UNSUPPORTED_DTYPE;
  const bool odd = src.w & 1;
  switch (src.dt) {
    case CLK_U16: return odd ? launch<uint16_t, true>(sh, dst, src, st) : launch<uint16_t, false>(sh, dst, src, st);
    case CLK_I16: return odd ? launch<int16_t, true>(sh, dst, src, st) : launch<int16_t, false>(sh, dst, src, st);
    case CLK_U8: return odd ? launch<uint8_t, true>(sh, dst, src, st) : launch<uint8_t, false>(sh, dst, src, st);
    case CLK_I8: return odd ? launch<int8_t, true>(sh, dst, src, st) : launch<int8_t, false>(sh, dst, src, st);
    case CLK_F32: return odd ? launch<float, true>(sh, dst, src, st) : launch<float, false>(sh, dst, src, st);
  }
  return CLK_UNSUPPORTED_DTYPE;
}

}  // namespace clk
