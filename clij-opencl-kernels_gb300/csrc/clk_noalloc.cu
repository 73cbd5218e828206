// clk_noalloc.cu - clk_separable_noalloc: the whole separable filter for
// callers that must not have the library allocate memory.
//
// Who needs it: a host application that owns the whole device-memory budget
// and allows no allocation it did not make itself (an imaging system that
// reserves the GPU at start-up), a processing loop that must never stall on
// or fail with an allocation halfway through an acquisition, or a plugin
// whose host hands it only the input and output buffers.
//
// The call first tries the fused kernels, which read src once and write dst
// once and need no temporaries at all.  Where they do not apply (pixel-type
// pairs without a fused kernel, radii above the fused limit) the filter runs
// pass by pass, and the two dst-typed temporaries of that form live in one
// fixed array in device memory declared below at file scope instead of the
// stream-ordered allocator.  So a call performs no cudaMalloc / cudaFree, no
// pinned host allocation and no allocating library routine.  Every GPU that
// loads the library holds the array (kNoAllocScratchBytes) until the process
// exits.
//
// The host cannot use the array's name as a device address (in host code it
// names a host-side stand-in), so the address is looked up with
// cudaGetSymbolAddress while the device is current, on the first call in
// each CUDA context, and cached per context: a new context (after
// cudaDeviceReset, say) gets a fresh lookup.  That first call should come
// before any stream capture.
//
// All calls share the array and it keeps the last call's contents.  The
// passes write every voxel of a temporary before any pass reads it, so no
// part of it has to start at zero.  Calls whose work overlaps on the GPU
// (different streams, no ordering between them) race on the array.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "clk_common.cuh"

namespace clk {

namespace {

// two temporaries of at most half this size each
constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
struct ScratchEntry {
  unsigned long long ctx_id;  // context the address belongs to (0: unknown)
  void* ptr;
};
std::mutex g_scratch_mu;
ScratchEntry g_scratch[kMaxDevices] = {};

// Unique id of the calling thread's current CUDA context, 0 if there is none
// yet or the driver entry points are unavailable.
unsigned long long current_context_id() {
  static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
  static PFN_cuCtxGetId_v12000 get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(fn);
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(fn);
    cudaGetLastError();
  });
  if (!get_current || !get_id) return 0;
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
  return id;
}

clk_status scratch_for_current_device(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return fail(CLK_NO_DEVICE, "clk_separable_noalloc: no current CUDA device");
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  ScratchEntry& e = g_scratch[dev];
  const unsigned long long ctx = current_context_id();
  if (!e.ptr || (ctx && ctx != e.ctx_id)) {
    void* p = nullptr;
    const cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess || !p) {
      cudaGetLastError();
      return fail(CLK_LAUNCH_FAILED, "clk_separable_noalloc: cudaGetSymbolAddress failed on device %d: %s", dev,
                  cudaGetErrorString(err));
    }
    e.ptr = p;
    e.ctx_id = current_context_id();  // the lookup made the context current if it was not yet
  }
  *out = e.ptr;
  return CLK_OK;
}

}  // namespace

}  // namespace clk

using namespace clk;

extern "C" clk_status clk_separable_noalloc(const char* kernel_name, const clk_image* dst_img,
                                            const clk_image* src_img, const int32_t N[3], const float s[3],
                                            const clk_define* defines, size_t ndefines, void* stream) {
  clear_error();
  static thread_local SepPlan plan;  // ~12 KB of taps: kept off the caller's stack
  clk_status st = separable_plan(kernel_name, dst_img, src_img, N, s, defines, ndefines, &plan,
                                 /*may_allocate=*/false);
  if (st) return st;
  cudaStream_t stm = (cudaStream_t)stream;
  // one HBM round trip, no temporaries: the same choice clk_separable makes
  st = fused_separable(plan.op, plan.dst, plan.src, plan.taps, plan.skip, plan.pol, stm);
  if (st != CLK_UNSUPPORTED_DTYPE) return st;
  clear_error();
  const size_t bytes = (size_t)plan.dst.count() * dtype_size(plan.dst.dt);
  const size_t half = kNoAllocScratchBytes / 2;
  if (bytes > half)
    return fail(CLK_BAD_ARG,
                "clk_separable_noalloc: a %zu-byte temporary exceeds the fixed scratch limit of %zu bytes per "
                "temporary (dst voxels x dst pixel size); use clk_separable",
                bytes, half);
  void* scratch = nullptr;
  if ((st = scratch_for_current_device(&scratch))) return st;
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
