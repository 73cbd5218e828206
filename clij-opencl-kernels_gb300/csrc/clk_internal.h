// clk_internal.h - host-side interface between the C-ABI dispatcher
// (clk_api.cpp) and the CUDA launchers (*.cu).  Not installed.
#pragma once
#include <cuda_runtime_api.h>
#include <stdint.h>

#include <vector>

#include "clk.h"

#ifdef __CUDACC__
#define CLK_HD __host__ __device__
#else
#define CLK_HD
#endif

namespace clk {

constexpr int kMaxTaps = 1001;        // separable window 2c+1 (kernel params)
constexpr int kMaxMedian = 1000;      // median neighbourhood size (kernel params)
constexpr int kDefaultMaxArray = 1024;

struct Image {
  void* ptr;
  int dt;    // clk_dtype
  int ndim;  // 2 or 3
  int w, h, d;
  CLK_HD int64_t count() const { return (int64_t)w * h * d; }
};

struct Range {
  int x, y, z;
  CLK_HD int64_t count() const { return (int64_t)x * y * z; }
};

// Host-side policies the reference leaves to its preamble / host (each one
// is a define of clk_execute, include/clk.h).
struct Policy {
  bool rte = false;           // CONVERT rounding half-to-even instead of toward zero
  bool sobel_narrow = false;  // sobel_3d reads unsigned pixels as int, not uint
  bool exact_order = false;   // reference-order float sums for float outputs too
  int max_array = kDefaultMaxArray;
};

enum SepOp { SEP_GAUSS = 0, SEP_MEAN = 1, SEP_MIN = 2, SEP_MAX = 3 };

// Taps of one separable pass: the window is v = -c..c (c = (N-1)/2 with C
// division, gaussian_blur_separable_3d_x.cl:22); for gaussian h[v+c] and
// their sequential float sum, computed exactly as the kernel does.
struct SepTaps {
  int c;
  float hsum;
  float h[kMaxTaps];
};

// Neighbourhood of a median launch in the kernel's loop order.
struct MedianNbhd {
  int n;
  int ex, ey, ez;
  char4 off[kMaxMedian];  // (dx, dy, dz, 0)
};

// error reporting (thread-local message) and launch accounting
clk_status fail(clk_status st, const char* fmt, ...);
void clear_error();  // empty the calling thread's message (start of every entry point)

// Test hook for the out-of-memory branches: while the environment variable
// CLK_INJECT_ALLOC_FAILURE is "1", every device allocation the library
// makes for temporaries reports failure (as cudaMallocAsync would when the
// device is full) and the caller sees CLK_OOM.
bool alloc_failure_injected();

// NVTX range around an entry point or a batch / server step (a named range
// on the profiler's timeline; a no-op unless a tool is attached).
struct TraceRange {
  explicit TraceRange(const char* name);
  ~TraceRange();
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};
clk_status check_launch(const char* what);
void count_launch(int n = 1);
void uncount_launches(uint64_t n);  // launches recorded while capturing a graph
clk_status device_ready_public();   // CLK_NO_DEVICE (with message) if no GPU
// The same check without the one-time mapping of the wait flag (a pinned host
// allocation): for the entry point that must allocate nothing.  Until some
// other call has mapped the flag, kernels that need it are not chosen.
clk_status device_ready_no_alloc();
// Device pointer of a host-mapped word that kernels set to 1 when one of
// their bounded waits runs out (nullptr if it could not be mapped).  The next
// entry-point call reports that as CLK_TIMEOUT and clears the word.
int* wait_flag_device();

int dtype_size(int dt);
bool gauss_taps(int N, float s, SepTaps* t);  // false: window too large
void box_taps(int N, SepTaps* t);
// guard = false reproduces median_slice_by_slice_sphere_3d_x.cl:39-45, which
// omits the FLT_MIN guard (a zero semi-axis leaves the neighbourhood empty)
bool median_nbhd(bool sphere, int ndim, int Nx, int Ny, int Nz, MedianNbhd* m, bool guard = true);
enum RankOp { RANK_MIN = 0, RANK_MAX = 1, RANK_MEAN = 2 };
enum RankMode { RANK_FLOAT = 0, RANK_CONVERT = 1, RANK_CAST = 2 };

// The validated inputs of a whole separable filter (the checks of
// clk_separable): kernel, images, policy, per-axis taps and skipped axes.
struct SepPlan {
  SepOp op;
  int ndim;
  Image dst, src;
  Policy pol;
  bool skip[3];
  SepTaps taps[3];
};
clk_status separable_plan(const char* kernel_name, const clk_image* dst, const clk_image* src, const int32_t N[3],
                          const float s[3], const clk_define* defines, size_t ndefines, SepPlan* plan,
                          bool may_allocate = true);

// z-chunks per tile for a kernel whose CTAs each stream one tile through a
// z-chunk: the count c (1..maxc) that minimises waves(c) x (planes per chunk
// + halo), waves = ceil(tiles x chunks / slots) and slots = resident CTAs of
// the whole GPU; chunks are whole multiples of `step` planes.  (A last wave
// that fills a fraction of the GPU costs as much as a full one.)
inline int wave_chunks(int64_t tiles, int depth, int halo, int64_t slots, int step = 1, int maxc = 16) {
  int best = 1;
  double best_cost = 0;
  for (int c = 1; c <= maxc; ++c) {
    int zc = (depth + c - 1) / c;
    zc = (zc + step - 1) / step * step;
    const int n = (depth + zc - 1) / zc;  // chunks actually launched
    if (c > 1 && n < c) break;
    const double waves = (double)((tiles * n + slots - 1) / slots);
    const double cost = waves * (zc + halo);
    if (c == 1 || cost < best_cost * 0.99) best = c, best_cost = cost;
  }
  return best;
}

// ---- generic ("direct") kernels: one thread per output voxel, every
// pixel-type pair, the reference's own evaluation order (bit-exact).
clk_status direct_sep_pass(SepOp op, const Image& dst, const Image& src, int dim, const SepTaps& taps, Range r,
                           const Policy& p, cudaStream_t st);
clk_status direct_copy(const Image& dst, const Image& src, Range r, const Policy& p, cudaStream_t st);
clk_status direct_median(const Image& dst, const Image& src, const MedianNbhd& m, Range r, cudaStream_t st);
clk_status direct_rank(RankOp op, RankMode mode, const Image& dst, const Image& src, const MedianNbhd& m, Range r,
                       const Policy& p, cudaStream_t st);
clk_status direct_greater_constant(const Image& dst, const Image& src, float scalar, Range r, cudaStream_t st);
enum StencilKind {
  ST_GRADIENT_X, ST_GRADIENT_Y, ST_GRADIENT_Z,
  ST_LAPLACE_DIAMOND_2D, ST_LAPLACE_DIAMOND_3D, ST_LAPLACE_BOX_2D, ST_LAPLACE_BOX_3D
};
clk_status direct_stencil(StencilKind kind, const Image& dst, const Image& src, Range r, const Policy& p,
                          cudaStream_t st);
clk_status direct_convolve(const Image& dst, const Image& src, const Image& kern, Range r, const Policy& p,
                           cudaStream_t st);
// min / max / mean over the radius-1 and radius-2 spheres (disks when planar
// or 2-D) for 8/16-bit pixels, src type = dst type (clk_sphere_rank.cu)
clk_status fast_sphere_rank(RankOp op, bool planar, const Image& dst, const Image& src, const MedianNbhd& m,
                            cudaStream_t st);
// whole-image copy (greater = false) or greater_constant, vectorised
// (clk_pointwise.cu); CLK_UNSUPPORTED_DTYPE where extents or alignment differ
clk_status fast_pointwise(bool greater, const Image& dst, const Image& src, float scalar, const Policy& p,
                          cudaStream_t st);
// gradient along axis 0/1/2 over whole rows (width a multiple of 8, aligned)
clk_status fast_gradient(int axis, const Image& dst, const Image& src, const Policy& p, cudaStream_t st);
// laplace_diamond_{2d,3d} / laplace_box_2d (integer pixels) and laplace_box_3d
// (signed integer pixels) over whole images, row-vectorised
clk_status fast_laplace(int kind, const Image& dst, const Image& src, const Policy& p, cudaStream_t st);
// laplace_box_3d over whole images, every pixel type, in the reference's order
clk_status fast_laplace_box3d(const Image& dst, const Image& src, const Policy& p, cudaStream_t st);
clk_status direct_morph(bool erode, bool sphere, const Image& dst, const Image& src, Range r, const Policy& p,
                        cudaStream_t st, bool planar = false);
clk_status direct_sobel(const Image& dst, const Image& src, Range r, const Policy& p, cudaStream_t st);

// ---- fused / tiled fast paths.  Return CLK_UNSUPPORTED_DTYPE (without
// setting an error) when the case is not covered, so the caller falls back.
// One separable pass along `axis` by the line kernels (clk_line.cu):
// min/max of any pixel type (src type == dst type), mean of integer pixels,
// Gaussian to float; radius 1..127.  CLK_UNSUPPORTED_DTYPE otherwise.
bool line_eligible(SepOp op, const Image& dst, const Image& src, const Policy& pol);
clk_status line_pass(SepOp op, const Image& dst, const Image& src, int axis, const SepTaps& taps, const Policy& pol,
                     cudaStream_t st);
// Whole-filter routing shared by clk_separable and the batch planner: a
// filter the register-window kernels cannot take runs as line passes (one
// launch per axis) rather than the generic fused kernel once a radius
// exceeds this.
constexpr int kLineMinR = 12;
inline bool prefer_line(SepOp op, const Image& dst, const Image& src, const int c[3], const Policy& pol) {
  const int m = c[0] > c[1] ? (c[0] > c[2] ? c[0] : c[2]) : (c[1] > c[2] ? c[1] : c[2]);
  return m > kLineMinR && line_eligible(op, dst, src, pol);
}
// the separable pass the multi-pass orchestration runs for one axis: a
// line pass where eligible, else the reference-order generic kernel
clk_status sep_pass(SepOp op, const Image& dst, const Image& src, int axis, const SepTaps& taps, Range r,
                    const Policy& pol, cudaStream_t st);
clk_status fused_separable(SepOp op, const Image& dst, const Image& src, const SepTaps taps[3], const bool skip[3],
                           const Policy& p, cudaStream_t st);
clk_status fast_morph(bool erode, bool sphere, int iterations, const Image& dst, const Image& src, const Policy& p,
                      cudaStream_t st, bool planar = false);
bool fast_morph_fusable(const Image& dst, const Image& src);  // fast_morph takes iterations = 2
// the bit-word kernels (clk_morph_bits.cu): 8-bit 3-D images with rows of
// whole 32-voxel words, one or two iterations; CLK_UNSUPPORTED_DTYPE where
// they do not apply
clk_status morph_bits(bool erode, bool sphere, int iterations, const Image& dst, const Image& src, cudaStream_t st);
clk_status fast_sobel(const Image& dst, const Image& src, const Policy& p, cudaStream_t st);
clk_status fast_median(bool sphere, const Image& dst, const Image& src, const MedianNbhd& m, cudaStream_t st);

}  // namespace clk
