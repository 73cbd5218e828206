// ref_loop.h - TEST INFRASTRUCTURE ONLY (oracle).  The host-side NDRange
// loop that drives the reference's kernels compiled as C++ (oracle/_ref): it
// plays the OpenCL runtime, setting get_global_id() for every work-item of
// the global range, with OpenMP threads over (z, y).
#pragma once
#include <omp.h>

#include "cl_shim.h"

extern "C" {
// Arguments of one kernel call.  ia/fa hold the kernel's int and float
// parameters in declaration order (e.g. dim, N then s for the separable
// kernels, gaussian_blur_separable_3d_x.cl:8-11).
struct clkref_call {
  void* src;
  int sw, sh, sd;
  void* dst;
  int dw, dh, dd;
  int gx, gy, gz;
  int ia[4];
  float fa[4];
  int nthreads;
  void* kimg;  // convolve: the float kernel image
  int kw, kh, kd;
};
}

template <class F>
static void clkref_loop(const clkref_call* c, F body) {
  const int nt = c->nthreads > 0 ? c->nthreads : omp_get_max_threads();
  const long planes = (long)c->gz * c->gy;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (long zy = 0; zy < planes; ++zy) {
    clkcl::clk_gid[2] = (int)(zy / c->gy);
    clkcl::clk_gid[1] = (int)(zy % c->gy);
    for (int x = 0; x < c->gx; ++x) {
      clkcl::clk_gid[0] = x;
      body();
    }
  }
}
