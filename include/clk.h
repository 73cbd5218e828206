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
  CLK_BUSY = 8,              /* admission refused (budget / slots)         */
  CLK_CANCELLED = 9          /* a served request was cancelled             */
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
 *   and the neighbourhood filters either side of them:
 *   minimum_sphere_{2d,3d}, maximum_sphere_{2d,3d}, mean_sphere_{2d,3d}
 *                                    (dst, src, int Nx, int Ny[, int Nz])
 *                                    minimum_sphere_3d_x.cl:3-10
 *   minimum/maximum/mean_slice_by_slice_sphere_3d,
 *   median_slice_by_slice_box_3d, median_slice_by_slice_sphere_3d
 *                                    (dst, src, int Nx, int Ny)
 *                                    minimum_slice_by_slice_sphere_3d_x.cl:3-9
 *   erode/dilate_box/sphere_slice_by_slice_3d   (src, dst)
 *   greater_constant_{2d,3d}         (src1, float scalar, dst)
 *                                    greater_constant_3d_x.cl:3-7
 *   copy_{2d,3d}                     (dst, src)   copy_3d_x.cl:3-6
 *   gradient_x_2d, gradient_y_2d, gradient_{x,y,z}_3d   (dst, src)
 *   laplace_box_{2d,3d}, laplace_diamond_{2d,3d}        (dst, src)
 *   convolve_{2d,3d}                 (src, kernelImage, dst); the kernel
 *                                    image is float   convolve_3d_x.cl:1-5
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
 * clk_separable for callers that cannot let the library allocate memory:
 * a host application that owns the whole device-memory budget and forbids
 * allocations it does not make itself, a loop that must not stall or fail
 * with out-of-memory halfway through, or a plugin whose host manages all
 * GPU memory.  This entry point has no counterpart in the reference.
 * Same arguments, errors and results as clk_separable, bit for bit: it
 * runs the same fused kernel where one applies (no temporaries at all), and
 * otherwise the same passes, with the two temporaries in one fixed array in
 * device memory (64 MiB, held by every GPU that loads the library until the
 * process exits) instead of the stream-ordered allocator.  A call allocates
 * nothing: no device memory, and not the pinned host word the other entry
 * points map on their first call.  Limit, for the pass-by-pass form only:
 * dst voxels x dst pixel size at most 32 MiB, else CLK_BAD_ARG.  The first
 * call in each CUDA context looks up the array's device address (make it
 * outside any stream capture).  Calls share the array: calls that overlap
 * on the GPU race.
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

/* ---------------------------------------------------------------------
 * Batched form: the same pipeline of filters over many independent images
 * of uneven shape and pixel type.  Each step runs as ONE persistent launch
 * over a work list of tiles of all images (pixel type dispatched per tile),
 * the pipeline is captured once as a CUDA graph, and the z-depth of a work
 * item and, for integer-output separable steps, the tile body (64x32
 * register-window or 64x16 generic tiles) are picked by an autotuner whose
 * choices persist in a JSON cache (env CLK_AUTOTUNE_CACHE, default
 * $HOME/.cache/clk_gb300/autotune.json).
 * Results equal per-image plain calls bit for bit.
 * Replaces: the host loop that enqueues every kernel per image (CLIc /
 *   pyclesperanto), which the reference leaves to its callers.
 * ------------------------------------------------------------------- */
typedef enum clk_op_kind {
  CLK_OP_SEPARABLE = 0,  /* whole separable filter, as clk_separable       */
  CLK_OP_KERNEL = 1,     /* one kernel launch, as clk_execute (median, sobel) */
  CLK_OP_MORPHOLOGY = 2  /* r=1 kernel applied `iterations` times           */
} clk_op_kind;

/* One step, applied to every image.  kernel: a reference kernel name
 * WITHOUT its _2d/_3d suffix (picked per image), e.g.
 * "gaussian_blur_separable" (SEPARABLE: N[3], s[3] as clk_separable),
 * "median_box" / "median_sphere" (KERNEL: N = Nx, Ny, Nz), "sobel",
 * "erode_sphere" (MORPHOLOGY: iterations). */
typedef struct clk_op {
  const char* kernel;
  int32_t kind; /* clk_op_kind */
  int32_t N[3];
  float s[3];
  int32_t iterations;
} clk_op;

typedef struct clk_batch clk_batch;

/* Plan a pipeline over images src[i] -> dst[i] (same extent; the steps'
 * results and temporaries carry dst[i]'s pixel type).  Allocates the
 * temporaries and work lists, autotunes (running the pipeline on the given
 * images), and captures the CUDA graph.  The image buffers must stay valid
 * until clk_batch_destroy. */
clk_status clk_batch_create(const clk_op* ops, int32_t nops, const clk_image* src, const clk_image* dst,
                            int32_t nimages, const clk_define* defines, size_t ndefines, void* stream,
                            clk_batch** out);
/* Run the pipeline (one graph launch) on the stream. */
clk_status clk_batch_run(clk_batch* batch, void* stream);
/* Run the same pipeline image by image with plain calls (no batching, no
 * graph): the per-call baseline the batched form is measured against. */
clk_status clk_batch_run_plain(clk_batch* batch, void* stream);
/* The same pipeline as the reference's callers launch it: every kernel of
 * every image by itself through clk_execute (a separable filter = one
 * launch per axis with dst-typed temporaries, the orchestrator's pattern). */
clk_status clk_batch_run_per_kernel(clk_batch* batch, void* stream);
/* Kernel launches per clk_batch_run (nodes of the graph). */
int32_t clk_batch_launches(const clk_batch* batch);
void clk_batch_destroy(clk_batch* batch);

/* ---------------------------------------------------------------------
 * Served form: a request loop with continuous admission.  Each request is
 * one image and a pipeline of steps (clk_op, suffix picked per image).  A
 * scheduler thread admits queued requests in arrival order as soon as a
 * slot (a CUDA stream) and HBM budget (the request's device temporaries)
 * are free, so requests that arrive while others run start at once and
 * their kernels overlap on the device.  Temporaries stay on the device;
 * optional host buffers are copied in before and out after the pipeline on
 * the request's stream.  Latency = submit -> completion of its last copy.
 * Replaces: the per-request host loop of a serving application (not in the
 * reference).
 * ------------------------------------------------------------------- */
typedef struct clk_server clk_server;

typedef struct clk_server_stats {
  uint64_t submitted, completed, failed;
  int64_t bytes_in_use, bytes_peak;  /* admitted temporaries vs budget */
  int32_t inflight, queued;
  double p50_ms, p99_ms, mean_ms;    /* over completed requests */
  double voxel_steps;                /* sum over completed of voxels x steps */
  double busy_s;                     /* first submit -> last completion */
  uint64_t cancelled;                /* requests cancelled before they ran */
} clk_server_stats;

/* slots: concurrent requests (streams), 1..64; hbm_budget_bytes: limit on
 * the admitted requests' temporaries (0 = no limit). */
clk_status clk_server_create(int32_t slots, int64_t hbm_budget_bytes, clk_server** out);
/* Queue a request; src/dst are device images (same extent), host_in /
 * host_out optional host buffers of src's / dst's size (pinned memory makes
 * the copies asynchronous).  CLK_BUSY if the queue is full; CLK_BAD_ARG if
 * the request alone exceeds the budget. */
clk_status clk_server_submit(clk_server* server, const clk_op* ops, int32_t nops, const clk_image* src,
                             const clk_image* dst, const void* host_in, void* host_out, uint64_t* ticket);
/* Wait (at most timeout_ms) for a request; CLK_TIMEOUT if it has not
 * finished; its latency in ms. */
clk_status clk_server_wait(clk_server* server, uint64_t ticket, int32_t timeout_ms, double* latency_ms);
/* Cancel a request that is still queued: it never runs, and waiting for
 * its ticket returns CLK_CANCELLED.  A request already running on the
 * device cannot be stopped (CLK_BUSY; wait for it instead); CLK_BAD_ARG for
 * an unknown or already waited-for ticket. */
clk_status clk_server_cancel(clk_server* server, uint64_t ticket);
/* Wait (at most timeout_ms) until nothing is queued or in flight. */
clk_status clk_server_drain(clk_server* server, int32_t timeout_ms);
clk_status clk_server_get_stats(clk_server* server, clk_server_stats* out);
void clk_server_destroy(clk_server* server);

/* The address under which kernels reach a page-locked host buffer (memory
 * from cudaHostAlloc / cudaMallocHost or registered with cudaHostRegister,
 * e.g. a pinned torch tensor), for use as a clk_image ptr.  A kernel given
 * it as dst stores its output straight into host memory over the host link
 * (zero-copy: no device copy of the output and no separate device->host
 * transfer); as src every read crosses the link, so inputs of neighbourhood
 * filters are better copied to the device first.  CLK_BAD_ARG if host_ptr is
 * not page-locked host memory.  Replaces the pull of a result image
 * (CLIc's pull / clij's pull of a device buffer to a host array) for
 * callers that keep results on the host. */
clk_status clk_host_image_pointer(const void* host_ptr, void** device_ptr);

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
