// clk_tma.cuh - Tensor Memory Accelerator staging: host-side tensor maps and
// the device-side mbarrier / cp.async.bulk.tensor primitives.
//
// A tile load copies a box of a 3-D image (x fastest) into shared memory and
// signals an mbarrier with the byte count.  Out-of-range coordinates are
// filled with zeros by the hardware; the kernels that use these loads replace
// those with the clamp-to-edge values themselves.  Waits are bounded: after
// a limit of polls the waiter gives up and reports it, so a lost transfer can
// never hang the device.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

namespace clk {
namespace tma {

constexpr uint32_t kWaitLimit = 1u << 26;  // polls of try_wait (each may suspend briefly)

// ---------------------------------------------------------------- host
// Encode a tiled tensor map over a W x H x D image of 1/2/4-byte pixels with
// a (bx, by, 1) box.  Returns false if the layout is not expressible (row
// pitch not a multiple of 16 bytes, unaligned base, box too large) or the
// driver entry point is unavailable; callers then stage without TMA.
inline bool make_map_3d(CUtensorMap* map, const void* base, int elem_bytes, int W, int H, int D, int bx, int by) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    cudaGetLastError();
  }
  if (!encode) return false;
  if (((uintptr_t)base % 16) != 0 || ((int64_t)W * elem_bytes) % 16 != 0) return false;
  if (bx <= 0 || by <= 0 || bx > 256 || by > 256 || (bx * elem_bytes) % 16 != 0) return false;
  const CUtensorMapDataType t = elem_bytes == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                : elem_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
                                                  : CU_TENSOR_MAP_DATA_TYPE_UINT32;  // bits only
  const cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D};
  const cuuint64_t strides[2] = {(cuuint64_t)W * elem_bytes, (cuuint64_t)W * H * elem_bytes};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return encode(map, t, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// ---------------------------------------------------------------- device
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (TMA) writes to the same memory
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// Poll the barrier's phase `parity` at most `limit` times; true once it
// completed, false if the limit ran out (limit 0: false at once).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// One box of a 3-D tensor map at element coordinates (x, y, z) into smem.
__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

}  // namespace tma
}  // namespace clk
