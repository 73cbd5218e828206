// clk_batch.cuh - the batch engine's device-side descriptors and the
// persistent kernels that walk a tile work list over many images.
#pragma once
#include <type_traits>

#include "clk_fused_impl.cuh"
#include "clk_median_impl.cuh"
#include "clk_sep2_impl.cuh"

namespace clk {
namespace batch {

// Tile bodies a work item can run (chosen per image on the host exactly as
// the plain path chooses them, so batched results equal plain ones).
enum Algo : int {
  A_SEP2 = 1,         // register-window kernel, isotropic XY radius (clk_sep2_impl.cuh)
  A_FUSED_EXACT = 2,  // generic fused kernel, reference order (clk_fused_impl.cuh)
  A_FUSED_FAST = 3,   // generic fused kernel, FMA (float Gaussian)
  A_MED27 = 4,        // median networks (clk_median_impl.cuh)
  A_MED9 = 5,
  A_MED33 = 6,
  // even widths, as the plain launcher chooses them:
  A_MED27Y = 7,   // box median with row pairs (8/16-bit pixels)
  A_MED27S = 8,   // the same with staged plane tiles (16-bit rows of whole vectors, aligned)
  A_MED33P = 9,   // sphere median in z pairs (8/16-bit pixels)
  A_MED33S = 10,  // the same with staged plane tiles (16-bit rows of whole vectors, aligned)
  A_MED33F = 11   // float sphere median, staged keys (rows of whole vectors, aligned)
};
// the median bodies that take their outputs in z pairs (even z-chunks)
constexpr bool med_z_pairs(int algo) { return algo == A_MED27 || algo >= A_MED27Y; }

struct WorkItem {
  int img;
  int bx, by, bz;
};

struct SepDesc {
  const void* src;
  void* dst;
  int W, H, D, zchunk;
  int dt, algo, rte;
  sep2::Params p2;
  fused::FusedTaps ft;
};

struct MedDesc {
  const void* src;
  void* dst;
  int W, H, D, zchunk;
  int dt, algo;
};

// SepOp (clk_internal.h) -> sep2's operation codes
template <int OP> struct S2Op;
template <> struct S2Op<SEP_MIN> { static constexpr int v = sep2::MIN; };
template <> struct S2Op<SEP_MAX> { static constexpr int v = sep2::MAX; };
template <> struct S2Op<SEP_MEAN> { static constexpr int v = sep2::MEAN; };
template <> struct S2Op<SEP_GAUSS> { static constexpr int v = sep2::GAUSS; };
// ... for pixel type T: the Gaussian to 8/16-bit pixels is the exact-order
// one, float min / max the reference-order ones
template <int OP, class T> struct S2OpT {
  static constexpr int v = (OP == SEP_GAUSS && sizeof(T) < 4)  ? (int)sep2::GAUSSX
                           : (OP == SEP_MIN && sizeof(T) == 4) ? (int)sep2::MINF
                           : (OP == SEP_MAX && sizeof(T) == 4) ? (int)sep2::MAXF
                                                               : S2Op<OP>::v;
};

constexpr int kmax_for(int R) { return R == 0 ? 63 : (2 * R + 1 <= 12 ? 12 : 24); }

// One work item of a separable step; the pixel type picks the body.
template <int OP, int R, class T>
__device__ __forceinline__ void sep_item_t(const SepDesc& d, const WorkItem& it, unsigned char* smem) {
  constexpr int KMAX = kmax_for(R);
  const T* s = static_cast<const T*>(d.src);
  T* o = static_cast<T*>(d.dst);
  if constexpr (sizeof(T) == 4 && OP == SEP_GAUSS) {
    if (d.algo == A_FUSED_FAST) {
      fused::fused_tile<T, T, OP, true, KMAX>(s, o, d.W, d.H, d.D, d.zchunk, d.ft, d.rte, it.bx, it.by, it.bz, smem);
      return;
    }
  }
  fused::fused_tile<T, T, OP, false, KMAX>(s, o, d.W, d.H, d.D, d.zchunk, d.ft, d.rte, it.bx, it.by, it.bz, smem);
}

// One persistent kernel per step, pixel type and body: the register-window
// tiles (A_SEP2) and the generic fused tiles run as separate kernels, since
// a kernel's register budget is that of its largest branch.
template <int OP, int R, class T>
__global__ void __launch_bounds__(256, 2) k_batch_sep2(const WorkItem* __restrict__ items, int n,
                                                       const SepDesc* __restrict__ descs) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const WorkItem it = items[i];
    const SepDesc& d = descs[it.img];
    sep2::sep2_tile<T, T, S2OpT<OP, T>::v, R>(static_cast<const T*>(d.src), static_cast<T*>(d.dst), d.W, d.H, d.D,
                                               d.zchunk, d.p2, it.bx, it.by, it.bz, smem);
    __syncthreads();  // the next item reuses shared memory
  }
}
// The generic fused tiles of a step and pixel type.
template <int OP, int R, class T>
__global__ void __launch_bounds__(256) k_batch_sep(const WorkItem* __restrict__ items, int n,
                                                   const SepDesc* __restrict__ descs) {
  extern __shared__ __align__(16) unsigned char smem[];
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const WorkItem it = items[i];
    sep_item_t<OP, R, T>(descs[it.img], it, smem);
    __syncthreads();  // the next item reuses shared memory
  }
}

// One work item of a median step; ALGO picks the body at compile time, so
// that each kernel carries one network (and that network's registers).
template <class T, int ALGO> __device__ __forceinline__ void med_item_t(const MedDesc& d, const WorkItem& it) {
  const T* s = static_cast<const T*>(d.src);
  T* o = static_cast<T*>(d.dst);
  if constexpr (ALGO == A_MED27 || ALGO == A_MED33 || ALGO == A_MED9) {
    if (d.W & 1) {
      if constexpr (ALGO == A_MED27) med::box27_tile<T, true>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
      else if constexpr (ALGO == A_MED33) med::sphere33_tile<T, true>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
      else med::box9_2d_tile<T, true>(s, o, d.W, d.H, it.bx, it.by);
    } else {
      if constexpr (ALGO == A_MED27) med::box27_tile<T, false>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
      else if constexpr (ALGO == A_MED33)
        med::sphere33_tile<T, false>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
      else med::box9_2d_tile<T, false>(s, o, d.W, d.H, it.bx, it.by);
    }
  } else if constexpr (ALGO == A_MED27Y) {
    med::box27_ypair_tile<T, false>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
  } else if constexpr (ALGO == A_MED33P) {
    med::sphere33_pair_tile<T, false>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
  } else if constexpr (ALGO == A_MED27S) {
    med::box27_staged_tile<T>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
  } else if constexpr (ALGO == A_MED33S) {
    med::sphere33_staged_tile<T>(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
  } else {
    med::sphere33_staged_f32_tile(s, o, d.W, d.H, d.D, d.zchunk, it.bx, it.by, it.bz);
  }
}

// the CTAs per SM each body's registers allow (as the plain kernels launch them)
template <int ALGO> constexpr int med_min_ctas() { return ALGO >= A_MED27Y ? 2 : 1; }

template <class T, int ALGO>
__global__ void __launch_bounds__(256, med_min_ctas<ALGO>()) k_batch_median(const WorkItem* __restrict__ items,
                                                                             int n, const MedDesc* __restrict__ descs) {
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const WorkItem it = items[i];
    med_item_t<T, ALGO>(descs[it.img], it);
    if constexpr (ALGO == A_MED27S || ALGO == A_MED33S || ALGO == A_MED33F)
      __syncthreads();  // the staged bodies reuse their shared-memory planes for the next item
  }
}

// host: the kernel for (op, R, pixel type); R = 0 is the generic-radius
// variant.  nullptr if not instantiated.
const void* batch_sep_kernel(int op, int R, int dt);
template <int OP> const void* batch_sep_kernel_op(int R, int dt);  // one file per OP
// the register-window kernel for (op, R >= 1, pixel type); nullptr if none
const void* batch_sep2_kernel(int op, int R, int dt);
template <int OP> const void* batch_sep2_kernel_op(int R, int dt);
const void* batch_median_kernel(int dt, int algo);  // nullptr if not instantiated
constexpr int kBatchRadii[] = {2, 3, 4, 5, 6};  // instantiated XY radii besides 0

}  // namespace batch
}  // namespace clk
