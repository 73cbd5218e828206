// clk_api.cpp - the C ABI (include/clk.h): kernel-name registry, binding of
// named arguments, the preamble/host policies, and the separable
// orchestration.  Host code only; kernels live in the .cu files.
#include <cuda_runtime_api.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "clk_internal.h"

namespace clk {

namespace {
thread_local std::string t_error;
std::atomic<uint64_t> g_launches{0};
}  // namespace

clk_status fail(clk_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_error = buf;
  return st;
}

void clear_error() { t_error.clear(); }

bool alloc_failure_injected() {
  const char* e = getenv("CLK_INJECT_ALLOC_FAILURE");
  return e && e[0] == '1' && e[1] == 0;
}

TraceRange::TraceRange(const char* name) { nvtxRangePushA(name ? name : "clk"); }
TraceRange::~TraceRange() { nvtxRangePop(); }

clk_status check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(CLK_LAUNCH_FAILED, "%s: %s", what, cudaGetErrorString(e));
  return CLK_OK;
}

void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }
void uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }

int dtype_size(int dt) {
  switch (dt) {
    case CLK_U8:
    case CLK_I8: return 1;
    case CLK_U16:
    case CLK_I16: return 2;
    case CLK_F32: return 4;
  }
  return 0;
}

// h = exp((v*v)/n), n = -2*s*s, in float exactly as
// gaussian_blur_separable_3d_x.cl:24,29 computes it (exp correctly rounded
// to float), and hsum accumulated in the same v = -c..c order (:31).
bool gauss_taps(int N, float s, SepTaps* t) {
  const int c = (N - 1) / 2;
  if (2 * c + 1 > kMaxTaps) return false;
  t->c = c;
  const float n = (-2.0f * s) * s;
  float hsum = 0.0f;
  for (int v = -c; v <= c; ++v) {
    const float q = (float)(v * v) / n;
    const float h = (float)std::exp((double)q);
    t->h[v + c] = h;
    hsum = hsum + h;
  }
  t->hsum = hsum;
  return true;
}

void box_taps(int N, SepTaps* t) {
  t->c = (N - 1) / 2;
  t->hsum = 0.0f;
}

// The median neighbourhood in the kernels' loop order (x, then y, then z;
// median_sphere_3d_x.cl:55-72); the ellipsoid test in float as written
// (:42-61), with FLT_MIN for a zero semi-axis.
bool median_nbhd(bool sphere, int ndim, int Nx, int Ny, int Nz, MedianNbhd* m, bool guard) {
  const int ex = (Nx - 1) / 2, ey = (Ny - 1) / 2, ez = ndim == 3 ? (Nz - 1) / 2 : 0;
  if (ex > 127 || ey > 127 || ez > 127) return false;
  float a2 = (float)(ex * ex), b2 = (float)(ey * ey), c2 = (float)(ez * ez);
  if (guard && a2 == 0) a2 = 1.17549435e-38f;
  if (guard && b2 == 0) b2 = 1.17549435e-38f;
  if (guard && c2 == 0) c2 = 1.17549435e-38f;
  int n = 0;
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
        if (!in) continue;
        if (n >= kMaxMedian) return false;
        char4 o;
        o.x = (signed char)x;
        o.y = (signed char)y;
        o.z = (signed char)z;
        o.w = 0;
        m->off[n++] = o;
      }
    }
  }
  m->n = n;
  m->ex = ex;
  m->ey = ey;
  m->ez = ez;
  return true;
}

namespace {

enum Family { F_SEP, F_MEDIAN, F_MORPH, F_SOBEL, F_RANK, F_THRESH, F_COPY, F_STENCIL, F_CONV };
// sub bits of the families that take a neighbourhood
// (F_RANK keeps its operation in bits 0-1 and its value mode in bits 2-3)
constexpr int kSphere = 1;      // F_MEDIAN
constexpr int kPlanar = 16;     // F_MEDIAN / F_MORPH / F_RANK: 2-D neighbourhood on each plane of a 3-D image
constexpr int kNoGuard = 32;    // F_MEDIAN: no FLT_MIN guard for a zero semi-axis
constexpr int rank_sub(RankOp op, RankMode mode, bool planar) { return (int)op | ((int)mode << 2) | (planar ? kPlanar : 0); }

struct ParamSpec {
  const char* name;
  int kind;  // clk_arg_kind
};

struct KernelInfo {
  const char* name;
  Family fam;
  int ndim;
  int sub;  // SEP: SepOp; MEDIAN: sphere; MORPH: erode*2 + sphere
  ParamSpec params[5];
  int nparams;
};

constexpr ParamSpec kDst{"dst", CLK_ARG_IMAGE}, kSrc{"src", CLK_ARG_IMAGE};
constexpr ParamSpec kDim{"dim", CLK_ARG_INT}, kN{"N", CLK_ARG_INT}, kS{"s", CLK_ARG_FLOAT};
constexpr ParamSpec kNx{"Nx", CLK_ARG_INT}, kNy{"Ny", CLK_ARG_INT}, kNz{"Nz", CLK_ARG_INT};
constexpr ParamSpec kSrc1{"src1", CLK_ARG_IMAGE}, kScalar{"scalar", CLK_ARG_FLOAT};
constexpr ParamSpec kKernelImage{"kernelImage", CLK_ARG_IMAGE};

// Parameter lists in the .cl declaration order.
const KernelInfo kRegistry[] = {
    {"gaussian_blur_separable_2d", F_SEP, 2, SEP_GAUSS, {kDst, kSrc, kDim, kN, kS}, 5},  // _2d_x.cl:6-13
    {"gaussian_blur_separable_3d", F_SEP, 3, SEP_GAUSS, {kDst, kSrc, kDim, kN, kS}, 5},  // _3d_x.cl:6-12
    {"mean_separable_2d", F_SEP, 2, SEP_MEAN, {kDst, kSrc, kDim, kN, kS}, 5},            // _2d_x.cl:3-10
    {"mean_separable_3d", F_SEP, 3, SEP_MEAN, {kDst, kSrc, kDim, kN, kS}, 5},            // _3d_x.cl:3-10
    {"minimum_separable_2d", F_SEP, 2, SEP_MIN, {kDst, kSrc, kDim, kN, kS}, 5},
    {"minimum_separable_3d", F_SEP, 3, SEP_MIN, {kDst, kSrc, kDim, kN, kS}, 5},
    {"maximum_separable_2d", F_SEP, 2, SEP_MAX, {kDst, kSrc, kDim, kN, kS}, 5},
    {"maximum_separable_3d", F_SEP, 3, SEP_MAX, {kDst, kSrc, kDim, kN, kS}, 5},
    {"median_box_2d", F_MEDIAN, 2, 0, {kDst, kSrc, kNx, kNy}, 4},         // median_box_2d_x.cl:22-28
    {"median_box_3d", F_MEDIAN, 3, 0, {kDst, kSrc, kNx, kNy, kNz}, 5},    // median_box_3d_x.cl:23-30
    {"median_sphere_2d", F_MEDIAN, 2, 1, {kDst, kSrc, kNx, kNy}, 4},      // median_sphere_2d_x.cl:22-28
    {"median_sphere_3d", F_MEDIAN, 3, 1, {kDst, kSrc, kNx, kNy, kNz}, 5}, // median_sphere_3d_x.cl:22-29
    {"erode_box_2d", F_MORPH, 2, 2, {kSrc, kDst}, 2},                     // erode_box_2d_x.cl:3-6
    {"erode_box_3d", F_MORPH, 3, 2, {kSrc, kDst}, 2},
    {"erode_sphere_2d", F_MORPH, 2, 3, {kSrc, kDst}, 2},
    {"erode_sphere_3d", F_MORPH, 3, 3, {kSrc, kDst}, 2},
    {"dilate_box_2d", F_MORPH, 2, 0, {kSrc, kDst}, 2},
    {"dilate_box_3d", F_MORPH, 3, 0, {kSrc, kDst}, 2},
    {"dilate_sphere_2d", F_MORPH, 2, 1, {kSrc, kDst}, 2},
    {"dilate_sphere_3d", F_MORPH, 3, 1, {kSrc, kDst}, 2},
    {"sobel_2d", F_SOBEL, 2, 0, {kDst, kSrc}, 2},  // sobel_2d_x.cl:3-7
    {"sobel_3d", F_SOBEL, 3, 0, {kDst, kSrc}, 2},  // sobel_3d_x.cl:3-7
    // the neighbourhood filters either side of the path
    {"minimum_sphere_2d", F_RANK, 2, rank_sub(RANK_MIN, RANK_CAST, false), {kDst, kSrc, kNx, kNy}, 4},  // :3-9
    {"minimum_sphere_3d", F_RANK, 3, rank_sub(RANK_MIN, RANK_FLOAT, false), {kDst, kSrc, kNx, kNy, kNz}, 5},
    {"maximum_sphere_2d", F_RANK, 2, rank_sub(RANK_MAX, RANK_CONVERT, false), {kDst, kSrc, kNx, kNy}, 4},
    {"maximum_sphere_3d", F_RANK, 3, rank_sub(RANK_MAX, RANK_FLOAT, false), {kDst, kSrc, kNx, kNy, kNz}, 5},
    {"mean_sphere_2d", F_RANK, 2, rank_sub(RANK_MEAN, RANK_FLOAT, false), {kDst, kSrc, kNx, kNy}, 4},
    {"mean_sphere_3d", F_RANK, 3, rank_sub(RANK_MEAN, RANK_FLOAT, false), {kDst, kSrc, kNx, kNy, kNz}, 5},
    {"minimum_slice_by_slice_sphere_3d", F_RANK, 3, rank_sub(RANK_MIN, RANK_CONVERT, true), {kDst, kSrc, kNx, kNy}, 4},
    {"maximum_slice_by_slice_sphere_3d", F_RANK, 3, rank_sub(RANK_MAX, RANK_CONVERT, true), {kDst, kSrc, kNx, kNy}, 4},
    {"mean_slice_by_slice_sphere_3d", F_RANK, 3, rank_sub(RANK_MEAN, RANK_FLOAT, true), {kDst, kSrc, kNx, kNy}, 4},
    {"median_slice_by_slice_box_3d", F_MEDIAN, 3, kPlanar, {kDst, kSrc, kNx, kNy}, 4},
    {"median_slice_by_slice_sphere_3d", F_MEDIAN, 3, kSphere | kPlanar | kNoGuard, {kDst, kSrc, kNx, kNy}, 4},
    {"erode_box_slice_by_slice_3d", F_MORPH, 3, 2 | kPlanar, {kSrc, kDst}, 2},
    {"erode_sphere_slice_by_slice_3d", F_MORPH, 3, 3 | kPlanar, {kSrc, kDst}, 2},
    {"dilate_box_slice_by_slice_3d", F_MORPH, 3, 0 | kPlanar, {kSrc, kDst}, 2},
    {"dilate_sphere_slice_by_slice_3d", F_MORPH, 3, 1 | kPlanar, {kSrc, kDst}, 2},
    {"greater_constant_2d", F_THRESH, 2, 0, {kSrc1, kScalar, kDst}, 3},  // greater_constant_2d_x.cl:3-7
    {"greater_constant_3d", F_THRESH, 3, 0, {kSrc1, kScalar, kDst}, 3},
    {"copy_2d", F_COPY, 2, 0, {kDst, kSrc}, 2},  // copy_2d_x.cl
    {"copy_3d", F_COPY, 3, 0, {kDst, kSrc}, 2},  // copy_3d_x.cl:3-6
    {"gradient_x_2d", F_STENCIL, 2, ST_GRADIENT_X, {kDst, kSrc}, 2},  // gradient_x_2d_x.cl:1-5
    {"gradient_y_2d", F_STENCIL, 2, ST_GRADIENT_Y, {kDst, kSrc}, 2},
    {"gradient_x_3d", F_STENCIL, 3, ST_GRADIENT_X, {kDst, kSrc}, 2},
    {"gradient_y_3d", F_STENCIL, 3, ST_GRADIENT_Y, {kDst, kSrc}, 2},
    {"gradient_z_3d", F_STENCIL, 3, ST_GRADIENT_Z, {kDst, kSrc}, 2},
    {"laplace_box_2d", F_STENCIL, 2, ST_LAPLACE_BOX_2D, {kDst, kSrc}, 2},  // laplace_box_2d_x.cl:3-7
    {"laplace_box_3d", F_STENCIL, 3, ST_LAPLACE_BOX_3D, {kDst, kSrc}, 2},
    {"laplace_diamond_2d", F_STENCIL, 2, ST_LAPLACE_DIAMOND_2D, {kDst, kSrc}, 2},
    {"laplace_diamond_3d", F_STENCIL, 3, ST_LAPLACE_DIAMOND_3D, {kDst, kSrc}, 2},
    {"convolve_2d", F_CONV, 2, 0, {kSrc, kKernelImage, kDst}, 3},  // convolve_2d_x.cl:1-5
    {"convolve_3d", F_CONV, 3, 0, {kSrc, kKernelImage, kDst}, 3},  // convolve_3d_x.cl:1-5
};
constexpr int kRegistrySize = sizeof(kRegistry) / sizeof(kRegistry[0]);

const KernelInfo* find_kernel(const char* name) {
  if (!name) return nullptr;
  for (const auto& k : kRegistry)
    if (std::strcmp(k.name, name) == 0) return &k;
  return nullptr;
}

volatile int* g_wait_flag_host = nullptr;
int* g_wait_flag_dev = nullptr;

std::once_flag g_wait_flag_once;

// CLK_OK if a device exists; reports (and clears) a wait that ran out in an
// earlier launch once the wait flag is mapped.
clk_status device_present() {
  static int count = -1;
  if (count < 0) {
    if (cudaGetDeviceCount(&count) != cudaSuccess) count = 0;
    cudaGetLastError();
  }
  if (count <= 0) return fail(CLK_NO_DEVICE, "no CUDA device available");
  if (g_wait_flag_host && *g_wait_flag_host) {
    *g_wait_flag_host = 0;
    return fail(CLK_TIMEOUT, "a bounded wait for a staged tile ran out in an earlier launch; its output is incomplete");
  }
  return CLK_OK;
}

clk_status device_ready() {
  clk_status st = device_present();
  if (st) return st;
  std::call_once(g_wait_flag_once, [] {
    void* h = nullptr;
    void* d = nullptr;
    if (cudaHostAlloc(&h, sizeof(int), cudaHostAllocMapped | cudaHostAllocPortable) == cudaSuccess &&
        cudaHostGetDevicePointer(&d, h, 0) == cudaSuccess) {
      *(volatile int*)h = 0;
      g_wait_flag_host = (volatile int*)h;
      g_wait_flag_dev = (int*)d;
    }
    cudaGetLastError();
  });
  return CLK_OK;
}

clk_status to_image(const clk_image& a, int ndim, const char* role, Image* out) {
  if (a.dtype < CLK_U8 || a.dtype > CLK_F32) return fail(CLK_UNSUPPORTED_DTYPE, "%s: unknown pixel type %d", role, a.dtype);
  if (a.ndim != ndim)
    return fail(CLK_BAD_ARG, "%s: kernel expects a %dd image, got ndim=%d", role, ndim, (int)a.ndim);
  const int64_t d = ndim == 2 ? 1 : a.depth;
  if (a.width <= 0 || a.height <= 0 || d <= 0)
    return fail(CLK_BAD_ARG, "%s: extent must be positive (%lld x %lld x %lld)", role, (long long)a.width,
                (long long)a.height, (long long)d);
  if (ndim == 2 && a.depth > 1) return fail(CLK_BAD_ARG, "%s: 2d image with depth %lld", role, (long long)a.depth);
  if (a.width > INT32_MAX || a.height > INT32_MAX || d > INT32_MAX)
    return fail(CLK_BAD_ARG, "%s: extent too large", role);
  if (!a.ptr) return fail(CLK_BAD_ARG, "%s: null device pointer", role);
  *out = Image{a.ptr, a.dtype, ndim, (int)a.width, (int)a.height, (int)d};
  return CLK_OK;
}

clk_status parse_defines(const clk_define* defs, size_t n, Policy* p) {
  for (size_t i = 0; i < n; ++i) {
    const char* k = defs[i].name;
    const char* v = defs[i].value ? defs[i].value : "";
    if (!k) return fail(CLK_BAD_ARG, "define %zu has no name", i);
    if (!std::strcmp(k, "MAX_ARRAY_SIZE")) {
      char* end = nullptr;
      const long m = std::strtol(v, &end, 10);
      if (!*v || *end || m <= 0) return fail(CLK_BAD_ARG, "MAX_ARRAY_SIZE=%s is not a positive integer", v);
      p->max_array = m > INT32_MAX ? INT32_MAX : (int)m;
    } else if (!std::strcmp(k, "CLK_CONVERT_ROUNDING")) {
      if (!std::strcmp(v, "rtz")) p->rte = false;
      else if (!std::strcmp(v, "rte")) p->rte = true;
      else return fail(CLK_BAD_ARG, "CLK_CONVERT_ROUNDING must be rtz or rte, not %s", v);
    } else if (!std::strcmp(k, "CLK_SOBEL3D_READ")) {
      if (!std::strcmp(v, "uint")) p->sobel_narrow = false;
      else if (!std::strcmp(v, "narrow")) p->sobel_narrow = true;
      else return fail(CLK_BAD_ARG, "CLK_SOBEL3D_READ must be uint or narrow, not %s", v);
    } else if (!std::strcmp(k, "CLK_EXACT_ORDER")) {
      p->exact_order = std::strcmp(v, "0") != 0;
    }
    // any other define is accepted and ignored, as an OpenCL build would
    // ignore a macro the kernel never uses
  }
  return CLK_OK;
}

struct Bound {
  const clk_arg* a[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int ival(int i) const { return a[i]->i; }
  float fval(int i) const { return a[i]->kind == CLK_ARG_FLOAT ? a[i]->f : (float)a[i]->i; }
};

clk_status bind(const KernelInfo& k, const clk_arg* args, size_t nargs, Bound* b) {
  if (nargs && !args) return fail(CLK_BAD_ARG, "args is NULL");
  for (size_t i = 0; i < nargs; ++i) {
    const char* nm = args[i].name;
    if (!nm) return fail(CLK_BAD_ARG, "argument %zu has no name", i);
    int slot = -1;
    for (int j = 0; j < k.nparams; ++j)
      if (!std::strcmp(k.params[j].name, nm)) slot = j;
    if (slot < 0) return fail(CLK_BAD_ARG, "%s has no parameter named '%s'", k.name, nm);
    if (b->a[slot]) return fail(CLK_BAD_ARG, "%s: parameter '%s' given twice", k.name, nm);
    const int want = k.params[slot].kind, got = args[i].kind;
    const bool ok = want == got || (want == CLK_ARG_FLOAT && got == CLK_ARG_INT);
    if (!ok) return fail(CLK_BAD_ARG, "%s: parameter '%s' has the wrong kind (%d, expected %d)", k.name, nm, got, want);
    b->a[slot] = &args[i];
  }
  for (int j = 0; j < k.nparams; ++j)
    if (!b->a[j]) return fail(CLK_BAD_ARG, "%s: missing parameter '%s'", k.name, k.params[j].name);
  return CLK_OK;
}

int slot_of(const KernelInfo& k, const char* nm) {
  for (int j = 0; j < k.nparams; ++j)
    if (!std::strcmp(k.params[j].name, nm)) return j;
  return -1;
}

}  // namespace

clk_status device_ready_public() { return device_ready(); }
clk_status device_ready_no_alloc() { return device_present(); }

clk_status sep_pass(SepOp op, const Image& dst, const Image& src, int axis, const SepTaps& taps, Range r,
                    const Policy& pol, cudaStream_t st) {
  const clk_status ls = line_pass(op, dst, src, axis, taps, pol, st);
  if (ls != CLK_UNSUPPORTED_DTYPE) return ls;
  return direct_sep_pass(op, dst, src, axis, taps, r, pol, st);
}

int* wait_flag_device() { return g_wait_flag_dev; }

clk_status separable_plan(const char* kernel_name, const clk_image* dst_img, const clk_image* src_img,
                          const int32_t N[3], const float s[3], const clk_define* defines, size_t ndefines,
                          SepPlan* plan, bool may_allocate) {
  const KernelInfo* k = find_kernel(kernel_name);
  if (!k) return fail(CLK_UNKNOWN_KERNEL, "unknown kernel '%s'", kernel_name ? kernel_name : "(null)");
  if (k->fam != F_SEP) return fail(CLK_BAD_ARG, "%s is not a separable kernel", k->name);
  if (!dst_img || !src_img || !N || !s) return fail(CLK_BAD_ARG, "null argument");
  plan->pol = Policy{};
  clk_status st = parse_defines(defines, ndefines, &plan->pol);
  if (st) return st;
  if ((st = to_image(*src_img, k->ndim, "src", &plan->src))) return st;
  if ((st = to_image(*dst_img, k->ndim, "dst", &plan->dst))) return st;
  if (plan->src.w != plan->dst.w || plan->src.h != plan->dst.h || plan->src.d != plan->dst.d)
    return fail(CLK_BAD_ARG, "%s: src and dst extents differ", k->name);
  plan->op = (SepOp)k->sub;
  plan->ndim = k->ndim;
  for (int d = 0; d < 3; ++d) {
    plan->skip[d] = d >= k->ndim || N[d] <= 1 || (plan->op == SEP_GAUSS && !(s[d] > 0));
    if (plan->skip[d]) {
      box_taps(1, &plan->taps[d]);
    } else if (plan->op == SEP_GAUSS) {
      if (!gauss_taps(N[d], s[d], &plan->taps[d]))
        return fail(CLK_BAD_ARG, "%s: N[%d]=%d exceeds %d taps", k->name, d, N[d], kMaxTaps);
    } else {
      box_taps(N[d], &plan->taps[d]);
    }
  }
  return may_allocate ? device_ready() : device_present();
}

}  // namespace clk

using namespace clk;

extern "C" {

clk_status clk_execute(const char* kernel_name, const clk_arg* args, size_t nargs, const size_t* global,
                       const clk_define* defines, size_t ndefines, void* stream) {
  t_error.clear();
  TraceRange trace(kernel_name);
  const KernelInfo* k = find_kernel(kernel_name);
  if (!k) return fail(CLK_UNKNOWN_KERNEL, "unknown kernel '%s'", kernel_name ? kernel_name : "(null)");
  Bound b;
  clk_status st = bind(*k, args, nargs, &b);
  if (st) return st;
  Policy pol;
  if ((st = parse_defines(defines, ndefines, &pol))) return st;
  Image src, dst;
  const int src_slot = slot_of(*k, "src") >= 0 ? slot_of(*k, "src") : slot_of(*k, "src1");
  if ((st = to_image(b.a[src_slot]->image, k->ndim, "src", &src))) return st;
  if ((st = to_image(b.a[slot_of(*k, "dst")]->image, k->ndim, "dst", &dst))) return st;
  Range r{dst.w, dst.h, dst.d};
  if (global) {
    const size_t g2 = k->ndim == 3 ? global[2] : 1;
    if (global[0] > (size_t)dst.w || global[1] > (size_t)dst.h || g2 > (size_t)dst.d)
      return fail(CLK_BAD_ARG, "%s: global range %zu x %zu x %zu exceeds dst %d x %d x %d", k->name, global[0],
                  global[1], g2, dst.w, dst.h, dst.d);
    r = Range{(int)global[0], (int)global[1], (int)g2};
  }
  cudaStream_t s = (cudaStream_t)stream;

  switch (k->fam) {
    case F_SEP: {
      const int dim = b.ival(slot_of(*k, "dim")), N = b.ival(slot_of(*k, "N"));
      const float sg = b.fval(slot_of(*k, "s"));
      static thread_local SepTaps taps;
      if (k->sub == SEP_GAUSS) {
        if (!gauss_taps(N, sg, &taps)) return fail(CLK_BAD_ARG, "%s: N=%d exceeds %d taps", k->name, N, kMaxTaps);
      } else {
        box_taps(N, &taps);
      }
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      return direct_sep_pass((SepOp)k->sub, dst, src, dim, taps, r, pol, s);
    }
    case F_MEDIAN: {
      const bool planar = (k->sub & kPlanar) != 0;
      const int nd = planar ? 2 : k->ndim;  // dimensions of the neighbourhood
      const int Nx = b.ival(slot_of(*k, "Nx")), Ny = b.ival(slot_of(*k, "Ny"));
      const int Nz = nd == 3 ? b.ival(slot_of(*k, "Nz")) : 1;
      static thread_local MedianNbhd m;
      if (!median_nbhd((k->sub & kSphere) != 0, nd, Nx, Ny, Nz, &m, (k->sub & kNoGuard) == 0))
        return fail(CLK_BAD_ARG, "%s: neighbourhood %d x %d x %d exceeds %d elements or radius 127", k->name, Nx, Ny,
                    Nz, kMaxMedian);
      if (m.n == 0) return fail(CLK_BAD_ARG, "%s: empty neighbourhood (Nx=%d Ny=%d Nz=%d)", k->name, Nx, Ny, Nz);
      if (m.n > pol.max_array)
        return fail(CLK_BAD_ARG, "%s: neighbourhood of %d exceeds MAX_ARRAY_SIZE=%d", k->name, m.n, pol.max_array);
      if (src.dt != dst.dt)
        return fail(CLK_UNSUPPORTED_DTYPE, "%s: src and dst pixel types must match", k->name);
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      const bool full = r.x == dst.w && r.y == dst.h && r.z == dst.d && src.w == dst.w && src.h == dst.h &&
                        src.d == dst.d;
      // float windows holding both -0 and +0 (or NaN) may pick the other zero
      // on the network path; CLK_EXACT_ORDER keeps the insertion sort for them
      if (full && !(pol.exact_order && src.dt == CLK_F32)) {
        st = fast_median((k->sub & kSphere) != 0, dst, src, m, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      return direct_median(dst, src, m, r, s);
    }
    case F_MORPH: {
      const bool erode = (k->sub & 2) != 0, sphere = (k->sub & 1) != 0, planar = (k->sub & kPlanar) != 0;
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      const bool full = r.x == dst.w && r.y == dst.h && r.z == dst.d && src.w == dst.w && src.h == dst.h &&
                        src.d == dst.d;
      if (full) {
        st = fast_morph(erode, sphere, 1, dst, src, pol, s, planar);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      return direct_morph(erode, sphere, dst, src, r, pol, s, planar);
    }
    case F_RANK: {
      const RankOp op = (RankOp)(k->sub & 3);
      const RankMode mode = (RankMode)((k->sub >> 2) & 3);
      const bool planar = (k->sub & kPlanar) != 0;
      const int nd = planar ? 2 : k->ndim;
      const int Nx = b.ival(slot_of(*k, "Nx")), Ny = b.ival(slot_of(*k, "Ny"));
      const int Nz = nd == 3 ? b.ival(slot_of(*k, "Nz")) : 1;
      static thread_local MedianNbhd m;
      if (!median_nbhd(true, nd, Nx, Ny, Nz, &m))
        return fail(CLK_BAD_ARG, "%s: neighbourhood %d x %d x %d exceeds %d elements or radius 127", k->name, Nx, Ny,
                    Nz, kMaxMedian);
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      const bool full = r.x == dst.w && r.y == dst.h && r.z == dst.d && src.w == dst.w && src.h == dst.h &&
                        src.d == dst.d;
      if (full) {
        st = fast_sphere_rank(op, planar, dst, src, m, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      return direct_rank(op, mode, dst, src, m, r, pol, s);
    }
    case F_CONV: {
      Image kern;
      if ((st = to_image(b.a[slot_of(*k, "kernelImage")]->image, k->ndim, "kernelImage", &kern))) return st;
      if (kern.dt != CLK_F32) return fail(CLK_UNSUPPORTED_DTYPE, "%s: the kernel image must be float", k->name);
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      return direct_convolve(dst, src, kern, r, pol, s);
    }
    case F_STENCIL: {
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      const bool full = r.x == dst.w && r.y == dst.h && r.z == dst.d;
      if (full && k->sub <= ST_GRADIENT_Z) {
        st = fast_gradient(k->sub - ST_GRADIENT_X, dst, src, pol, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      if (full && k->sub >= ST_LAPLACE_DIAMOND_2D) {
        st = fast_laplace(k->sub, dst, src, pol, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      if (full && k->sub == ST_LAPLACE_BOX_3D) {
        st = fast_laplace_box3d(dst, src, pol, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      return direct_stencil((StencilKind)k->sub, dst, src, r, pol, s);
    }
    case F_THRESH:
    case F_COPY: {
      const bool greater = k->fam == F_THRESH;
      const float scalar = greater ? b.fval(slot_of(*k, "scalar")) : 0.f;
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      if (r.x == dst.w && r.y == dst.h && r.z == dst.d) {
        st = fast_pointwise(greater, dst, src, scalar, pol, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      return greater ? direct_greater_constant(dst, src, scalar, r, s) : direct_copy(dst, src, r, pol, s);
    }
    case F_SOBEL: {
      if (r.count() == 0) return CLK_OK;
      if ((st = device_ready())) return st;
      const bool full = r.x == dst.w && r.y == dst.h && r.z == dst.d && src.w == dst.w && src.h == dst.h &&
                        src.d == dst.d;
      if (full && !pol.exact_order) {
        st = fast_sobel(dst, src, pol, s);
        if (st != CLK_UNSUPPORTED_DTYPE) return st;
      }
      return direct_sobel(dst, src, r, pol, s);
    }
  }
  return fail(CLK_UNKNOWN_KERNEL, "unhandled kernel family");
}

clk_status clk_separable(const char* kernel_name, const clk_image* dst_img, const clk_image* src_img,
                         const int32_t N[3], const float s[3], const clk_define* defines, size_t ndefines,
                         void* stream) {
  t_error.clear();
  TraceRange trace(kernel_name);
  const KernelInfo* k = find_kernel(kernel_name);
  if (!k) return fail(CLK_UNKNOWN_KERNEL, "unknown kernel '%s'", kernel_name ? kernel_name : "(null)");
  if (k->fam != F_SEP) return fail(CLK_BAD_ARG, "%s is not a separable kernel", k->name);
  if (!dst_img || !src_img || !N || !s) return fail(CLK_BAD_ARG, "null argument");
  Policy pol;
  clk_status st = parse_defines(defines, ndefines, &pol);
  if (st) return st;
  Image src, dst;
  if ((st = to_image(*src_img, k->ndim, "src", &src))) return st;
  if ((st = to_image(*dst_img, k->ndim, "dst", &dst))) return st;
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d)
    return fail(CLK_BAD_ARG, "%s: src and dst extents differ", k->name);
  cudaStream_t stm = (cudaStream_t)stream;
  const SepOp op = (SepOp)k->sub;
  static thread_local SepTaps taps[3];
  bool skip[3] = {true, true, true};
  for (int d = 0; d < k->ndim; ++d) {
    skip[d] = N[d] <= 1 || (op == SEP_GAUSS && !(s[d] > 0));
    if (skip[d]) {
      box_taps(1, &taps[d]);
    } else if (op == SEP_GAUSS) {
      if (!gauss_taps(N[d], s[d], &taps[d]))
        return fail(CLK_BAD_ARG, "%s: N[%d]=%d exceeds %d taps", k->name, d, N[d], kMaxTaps);
    } else {
      box_taps(N[d], &taps[d]);
    }
  }
  if ((st = device_ready())) return st;
  st = fused_separable(op, dst, src, taps, skip, pol, stm);
  if (st != CLK_UNSUPPORTED_DTYPE) return st;
  st = CLK_OK;

  // Multi-pass: X, Y(, Z) with dst-typed temporaries, as three launches of
  // the reference kernels would run.
  const size_t bytes = (size_t)dst.count() * dtype_size(dst.dt);
  void* tmp[2] = {nullptr, nullptr};
  int passes = 0;
  for (int d = 0; d < k->ndim; ++d) passes += 1;
  for (int i = 0; i < 2 && i < passes - 1; ++i) {
    if (alloc_failure_injected() || cudaMallocAsync(&tmp[i], bytes, stm) != cudaSuccess) {
      cudaGetLastError();
      for (int j = 0; j < i; ++j) cudaFreeAsync(tmp[j], stm);
      return fail(CLK_OOM, "%s: cannot allocate a %zu-byte temporary", k->name, bytes);
    }
  }
  Image cur = src;
  const Range r{dst.w, dst.h, dst.d};
  for (int d = 0; d < k->ndim && st == CLK_OK; ++d) {
    const bool last = d == k->ndim - 1;
    Image out = dst;
    if (!last) out.ptr = tmp[d & 1];
    st = skip[d] ? direct_copy(out, cur, r, pol, stm) : sep_pass(op, out, cur, d, taps[d], r, pol, stm);
    cur = out;
  }
  for (int i = 0; i < 2; ++i)
    if (tmp[i]) cudaFreeAsync(tmp[i], stm);
  return st;
}

clk_status clk_morphology(const char* kernel_name, const clk_image* dst_img, const clk_image* src_img,
                          int32_t iterations, const clk_define* defines, size_t ndefines, void* stream) {
  t_error.clear();
  TraceRange trace(kernel_name);
  const KernelInfo* k = find_kernel(kernel_name);
  if (!k) return fail(CLK_UNKNOWN_KERNEL, "unknown kernel '%s'", kernel_name ? kernel_name : "(null)");
  if (k->fam != F_MORPH) return fail(CLK_BAD_ARG, "%s is not a morphology kernel", k->name);
  if (!dst_img || !src_img) return fail(CLK_BAD_ARG, "null argument");
  if (iterations < 0) return fail(CLK_BAD_ARG, "%s: iterations must be >= 0, got %d", k->name, iterations);
  Policy pol;
  clk_status st = parse_defines(defines, ndefines, &pol);
  if (st) return st;
  Image src, dst;
  if ((st = to_image(*src_img, k->ndim, "src", &src))) return st;
  if ((st = to_image(*dst_img, k->ndim, "dst", &dst))) return st;
  if (src.w != dst.w || src.h != dst.h || src.d != dst.d)
    return fail(CLK_BAD_ARG, "%s: src and dst extents differ", k->name);
  if ((st = device_ready())) return st;
  cudaStream_t stm = (cudaStream_t)stream;
  const bool erode = (k->sub & 2) != 0, sphere = (k->sub & 1) != 0, planar = (k->sub & kPlanar) != 0;
  const Range r{dst.w, dst.h, dst.d};
  if (iterations == 0) return direct_copy(dst, src, r, pol, stm);
  // Each launch reads the previous result (dst-typed, like the orchestrator's
  // temporaries).  Pairs of iterations run fused where the pixel types and
  // layout allow; the chain of steps ping-pongs between a temporary and dst
  // so that the last step writes dst and no step reads what it writes.
  const bool fuse = !planar && fast_morph_fusable(dst, src);
  const int nsteps = fuse ? (iterations + 1) / 2 : iterations;
  void* tmp = nullptr;
  if (nsteps > 1) {
    const size_t bytes = (size_t)dst.count() * dtype_size(dst.dt);
    if (alloc_failure_injected() || cudaMallocAsync(&tmp, bytes, stm) != cudaSuccess) {
      cudaGetLastError();
      return fail(CLK_OOM, "%s: cannot allocate a %zu-byte temporary", k->name, bytes);
    }
  }
  Image cur = src;
  int left = iterations;
  for (int i = 0; i < nsteps && st == CLK_OK; ++i) {
    Image out = dst;
    if (i != nsteps - 1) out.ptr = ((nsteps - 1 - i) % 2 == 1) ? tmp : dst.ptr;
    const int take = (fuse && left >= 2) ? 2 : 1;
    st = fast_morph(erode, sphere, take, out, cur, pol, stm, planar);
    if (st == CLK_UNSUPPORTED_DTYPE && take == 1) st = direct_morph(erode, sphere, out, cur, r, pol, stm, planar);
    left -= take;
    cur = out;
  }
  if (tmp) cudaFreeAsync(tmp, stm);
  return st;
}

int clk_supported(const char* kernel_name, int32_t src_dtype, int32_t dst_dtype, int32_t ndim) {
  const KernelInfo* k = find_kernel(kernel_name);
  if (!k || k->ndim != ndim) return 0;
  if (src_dtype < CLK_U8 || src_dtype > CLK_F32 || dst_dtype < CLK_U8 || dst_dtype > CLK_F32) return 0;
  if (k->fam == F_MEDIAN && src_dtype != dst_dtype) return 0;
  if (k->fam == F_RANK && ((k->sub >> 2) & 3) == RANK_CAST && src_dtype == CLK_F32 && dst_dtype != CLK_F32) return 0;
  return 1;
}

clk_status clk_host_image_pointer(const void* host_ptr, void** device_ptr) {
  t_error.clear();
  if (!host_ptr || !device_ptr) return fail(CLK_BAD_ARG, "clk_host_image_pointer: null pointer");
  *device_ptr = nullptr;
  if (const clk_status st = device_ready(); st != CLK_OK) return st;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, host_ptr) != cudaSuccess) {
    cudaGetLastError();
    return fail(CLK_BAD_ARG, "clk_host_image_pointer: %p is not memory known to CUDA", host_ptr);
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer)
    return fail(CLK_BAD_ARG, "clk_host_image_pointer: %p is not page-locked host memory", host_ptr);
  *device_ptr = a.devicePointer;
  return CLK_OK;
}

const char* clk_last_error_string(void) { return t_error.c_str(); }

const char* clk_version(void) {
  static char v[64];
  std::snprintf(v, sizeof v, "%d.%d (sm_103a)", CLK_VERSION_MAJOR, CLK_VERSION_MINOR);
  return v;
}

int clk_kernel_count(void) { return kRegistrySize; }

const char* clk_kernel_name(int i) { return i >= 0 && i < kRegistrySize ? kRegistry[i].name : nullptr; }

uint64_t clk_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

}  // extern "C"
