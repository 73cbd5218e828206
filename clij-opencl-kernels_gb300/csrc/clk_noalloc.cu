// clk_noalloc.cu - clk_separable_noalloc: the whole separable filter for
// callers that must not have the library allocate device memory.
//
// The pass-by-pass form of a separable filter needs two temporaries of the
// dst pixel type (X result, Y result).  clk_separable takes them from the
// stream-ordered allocator; this entry point instead uses one fixed array
// in device memory, declared below at file scope, so a call performs no
// cudaMalloc / cudaFree and no allocating library routine.  Every GPU that
// loads the library holds the array (kNoAllocScratchBytes) until the process
// exits.
//
// The host cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the first call on each device looks the
// address up with cudaGetSymbolAddress while that device is current and
// caches it; make that first call outside any stream capture.
//
// All calls share the array and it keeps the last call's contents.  The
// passes write every voxel of a temporary before any pass reads it, so no
// part of it has to start at zero.  Calls whose work overlaps on the GPU
// (different streams, no ordering between them) race on the array.
#include <mutex>

#include "clk_common.cuh"

namespace clk {

namespace {

// two temporaries of at most half this size each
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_ptr[kMaxDevices] = {};

clk_status scratch_for_current_device(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(CLK_NO_DEVICE, "clk_separable_noalloc: no current CUDA device");
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return fail(CLK_LAUNCH_FAILED, "clk_separable_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                  cudaGetErrorString(e));
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return CLK_OK;
}

}  // namespace

}  // namespace clk

using namespace clk;

extern "C" clk_status clk_separable_noalloc(const char* kernel_name, const clk_image* dst_img,
                                            const clk_image* src_img, const int32_t N[3], const float s[3],
                                            const clk_define* defines, size_t ndefines, void* stream) {
  static thread_local SepPlan plan;  // ~12 KB of taps: kept off the caller's stack
  clk_status st = separable_plan(kernel_name, dst_img, src_img, N, s, defines, ndefines, &plan);
  if (st) return st;
  const size_t bytes = (size_t)plan.dst.count() * dtype_size(plan.dst.dt);
  const size_t half = kNoAllocScratchBytes / 2;
  if (bytes > half)
    return fail(CLK_BAD_ARG,
                "clk_separable_noalloc: a %zu-byte temporary exceeds the fixed scratch limit of %zu bytes per "
                "temporary (dst voxels x dst pixel size); use clk_separable",
                bytes, half);
  void* scratch = nullptr;
  if ((st = scratch_for_current_device(&scratch))) return st;
  cudaStream_t stm = (cudaStream_t)stream;
  void* tmp[2] = {scratch, (unsigned char*)scratch + half};
  const Range r{plan.dst.w, plan.dst.h, plan.dst.d};
  Image cur = plan.src;
  for (int d = 0; d < plan.ndim && st == CLK_OK; ++d) {
    Image out = plan.dst;
    if (d != plan.ndim - 1) out.ptr = tmp[d & 1];
    st = plan.skip[d] ? direct_copy(out, cur, r, plan.pol, stm)
                      : sep_pass(plan.op, out, cur, d, plan.taps[d], r, plan.pol, stm);
    cur = out;
  }
  return st;
}
