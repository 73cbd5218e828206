/*
 * clk.h - C ABI of the GB300-native neighbourhood-filter library.
 *
 * The reference (clEsperanto/clij-opencl-kernels) ships OpenCL C kernels only.
 * A host orchestrator (CLIc, clij-clearcl, pyclesperanto) calls each kernel by
 * its __kernel name with an ordered list of named arguments (images "src" and
 * "dst" with a per-image pixel type, int/float scalars such as "dim", "N",
 * "s", "Nx"), a global range equal to the dst extent and compile-time defines
 * such as MAX_ARRAY_SIZE (README.md:16-141).  This header is the drop-in for
 * that call: the same kernel names, the same argument names and meanings,
 * arguments bound by NAME (the reference's argument order differs between
 * families, e.g. (dst, src, ...) in median_box_3d_x.cl:24-30 but (src, dst)
 * in erode_box_3d_x.cl:3-6).
 *
 * Images are caller-owned device buffers laid out x-fastest,
 * idx = x + w*(y + h*z), exactly like the reference's buffer storage.  The
 * library never frees them.  Every entry point is stream-ordered on the
 * stream passed in (a cudaStream_t given as void*, NULL = legacy default
 * stream) and returns a status; nothing throws across the ABI.  A per-thread
 * message describes the last error.
 */
#ifndef CLK_H
#define CLK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CLK_VERSION_MAJOR 0
#define CLK_VERSION_MINOR 1

typedef enum clk_status {
  CLK_OK = 0,
  CLK_UNKNOWN_KERNEL = 1,    /* kernel name not in the registry            */
  CLK_BAD_ARG = 2,           /* missing/extra/mistyped argument, bad range */
  CLK_UNSUPPORTED_DTYPE = 3, /* pixel-type combination not provided        */
  CLK_OOM = 4,               /* a temporary could not be allocated         */
  CLK_LAUNCH_FAILED = 5,     /* CUDA reported an error                     */
  CLK_TIMEOUT = 6,           /* a bounded device wait ran out              */
  CLK_NO_DEVICE = 7,         /* no usable CUDA device                      */
  CLK_BUSY = 8               /* admission refused (budget / slots)         */
} clk_status;

/* Pixel types of README.md:64-72 (char, uchar, short, ushort, float). */
typedef enum clk_dtype {
  CLK_U8 = 0,
  CLK_I8 = 1,
  CLK_U16 = 2,
  CLK_I16 = 3,
  CLK_F32 = 4
} clk_dtype;

typedef enum clk_arg_kind {
  CLK_ARG_IMAGE = 0,
  CLK_ARG_INT = 1,
  CLK_ARG_FLOAT = 2
} clk_arg_kind;

/* One image: a device pointer plus its pixel type and extent.  For a 2-D
 * image depth is 1 (ndim = 2); ndim must match the kernel's _2d/_3d suffix. */
typedef struct clk_image {
  void* ptr;
  int32_t dtype; /* clk_dtype */
  int32_t ndim;  /* 2 or 3 */
  int64_t width, height, depth;
} clk_image;

/* One named argument.  name is the parameter name of the .cl kernel
 * ("src", "dst", "dim", "N", "s", "Nx", "Ny", "Nz"). */
typedef struct clk_arg {
  const char* name;
  int32_t kind; /* clk_arg_kind */
  int32_t i;    /* CLK_ARG_INT   */
  float f;      /* CLK_ARG_FLOAT */
  clk_image image;
} clk_arg;

/* A compile-time define of the reference's host (name = value).  Honoured:
 *   MAX_ARRAY_SIZE      capacity of the median's neighbourhood array
 *                       (median_box_3d_x.cl:36); a larger neighbourhood is
 *                       rejected with CLK_BAD_ARG instead of overflowing.
 *   CLK_CONVERT_ROUNDING "rtz" (default) or "rte": float->integer rounding
 *                       of CONVERT_dst_PIXEL_TYPE (saturating in both).
 *   CLK_SOBEL3D_READ    "uint" (default) or "narrow": value type of the
 *                       unsigned reads that sobel_3d multiplies by its int
 *                       coefficients (sobel_3d_x.cl:47-49).
 *   CLK_EXACT_ORDER     "1": float accumulations in the reference's own
 *                       order (v = -c..c, separate multiply and add) for
 *                       float outputs too; integer outputs always use it. */
typedef struct clk_define {
  const char* name;
  const char* value;
} clk_define;

/* ---------------------------------------------------------------------
 * Plain path: one kernel launch, the drop-in for enqueueing one .cl kernel.
 * kernel_name: one of
 *   gaussian_blur_separable_{2d,3d}  (dst, src, int dim, int N, float s)
 *                                    gaussian_blur_separable_3d_x.cl:6-12
 *   mean_separable_{2d,3d}           (dst, src, int dim, int N, float s)
 *                                    mean_separable_3d_x.cl:3-10
 *   minimum_separable_{2d,3d}        (dst, src, int dim, int N, float s)
 *                                    minimum_separable_3d_x.cl:3-10
 *   maximum_separable_{2d,3d}        (dst, src, int dim, int N, float s)
 *                                    maximum_separable_3d_x.cl:3-10
 *   median_box_2d, median_sphere_2d  (dst, src, int Nx, int Ny)
 *                                    median_box_2d_x.cl:22-28
 *   median_box_3d, median_sphere_3d  (dst, src, int Nx, int Ny, int Nz)
 *                                    median_sphere_3d_x.cl:22-29
 *   erode_box_{2d,3d}, erode_sphere_{2d,3d},
 *   dilate_box_{2d,3d}, dilate_sphere_{2d,3d}   (src, dst)
 *                                    erode_box_3d_x.cl:3-6
 *   sobel_{2d,3d}                    (dst, src)   sobel_3d_x.cl:3-7
 * global: the global work size; voxels [0,global[0]) x [0,global[1]) x
 *   [0,global[2]) of dst are written (the reference's NDRange); it must not
 *   exceed dst's extent.  NULL means "dst's extent".  Reads of src are
 *   clamped to src's own extent (CLK_ADDRESS_CLAMP_TO_EDGE).
 * Replaces: clEnqueueNDRangeKernel of the named .cl kernel as CLIc /
 *   clij-clearcl issue it (README.md:16-26).
 * ------------------------------------------------------------------- */
clk_status clk_execute(const char* kernel_name, const clk_arg* args,
                       size_t nargs, const size_t* global,
                       const clk_define* defines, size_t ndefines,
                       void* stream);

/* ---------------------------------------------------------------------
 * Orchestrator convenience: the whole separable filter X -> Y -> Z for one
 * of gaussian_blur_separable_{2d,3d}, mean/minimum/maximum_separable_{2d,3d}.
 * N[d], s[d] are the per-axis "N" and "s" arguments of the passes; an axis
 * with N[d] <= 1 (gaussian: also s[d] <= 0) is skipped (converting copy).
 * Results equal three launches through clk_execute with dst-typed
 * temporaries in X, Y, Z order; the library fuses the passes into one HBM
 * round trip where the pixel types allow it.
 * Replaces: the host orchestrator's separable driver (CLIc
 *   execute_separable), which is not part of the reference repository.
 * ------------------------------------------------------------------- */
clk_status clk_separable(const char* kernel_name, const clk_image* dst,
                         const clk_image* src, const int32_t N[3],
                         const float s[3], const clk_define* defines,
                         size_t ndefines, void* stream);

/* ---------------------------------------------------------------------
 * clk_separable for callers that cannot let the library allocate device
 * memory: a host application that owns the whole device-memory budget and
 * forbids allocations it does not make itself, a loop that must not stall
 * or fail with out-of-memory halfway through, or a plugin whose host
 * manages all GPU memory.  This entry point has no counterpart in the
 * reference.
 * Same arguments, results and errors as clk_separable, computed pass by
 * pass; the two temporaries come from one fixed array in device memory
 * (64 MiB, held by every GPU that loads the library until the process
 * exits), so a call allocates nothing.  Limit: dst voxels x dst pixel size
 * must be at most 32 MiB, else CLK_BAD_ARG.  The first call on each device
 * looks up the array's device address (make it outside any stream
 * capture).  Calls share the array: calls that overlap on the GPU race.
 * ------------------------------------------------------------------- */
clk_status clk_separable_noalloc(const char* kernel_name, const clk_image* dst,
                                 const clk_image* src, const int32_t N[3],
                                 const float s[3], const clk_define* defines,
                                 size_t ndefines, void* stream);

/* ---------------------------------------------------------------------
 * Orchestrator convenience: `iterations` successive launches of one of the
 * r=1 morphology kernels erode/dilate_{box,sphere}_{2d,3d} (which have no
 * radius parameter, erode_sphere_3d_x.cl:3-6) -- the radius-r request of
 * the orchestrator.  The result equals that many clk_execute launches, each
 * reading the previous result with clamp-to-edge; for byte images two
 * iterations run fused in one pass.  iterations = 0 is a converting copy.
 * Replaces: the host loop over the r=1 kernel (not in the reference).
 * ------------------------------------------------------------------- */
clk_status clk_morphology(const char* kernel_name, const clk_image* dst,
                          const clk_image* src, int32_t iterations,
                          const clk_define* defines, size_t ndefines,
                          void* stream);

/* Is kernel_name available for this (src, dst) pixel-type pair and ndim?
 * Returns 1 if yes, 0 if no. */
int clk_supported(const char* kernel_name, int32_t src_dtype,
                  int32_t dst_dtype, int32_t ndim);

/* Message of the calling thread's last non-OK status ("" if none). */
const char* clk_last_error_string(void);

/* "major.minor (sm_103a)" */
const char* clk_version(void);

/* Number of kernel names in the registry and the i-th name (NULL if out of
 * range); lets a binding enumerate the drop-in surface. */
int clk_kernel_count(void);
const char* clk_kernel_name(int i);

/* Number of CUDA kernels this library launched since load (all threads).
 * Used by benchmarks to count launches inside a timed region. */
uint64_t clk_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* CLK_H */
