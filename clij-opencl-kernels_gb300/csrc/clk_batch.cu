// clk_batch.cu - the batch engine behind clk_batch_* (include/clk.h).
//
// A pipeline of steps over N images.  For every step the engine picks, per
// image, the tile body the plain path would run (so results are identical),
// collects the tiles of all images that share a kernel (step x pixel type)
// into one work list, and launches ONE persistent kernel per list; the lists
// of a step run as concurrent graph nodes.  Images or steps without a
// batched body (morphology, sobel, unusual radii or layouts) run their plain
// calls inside the same graph.  The z-depth of a work item (zchunk) trades
// load balance against halo re-reads, and integer-output separable images
// can run on either tile body (register-window 64x32 or generic 64x16,
// bit-identical); the autotuner times the depths (x bodies) per step on the
// real images and remembers the winners in a JSON cache.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "clk_batch.cuh"

namespace clk {
namespace batch {

const void* batch_sep_kernel(int op, int R, int dt) {
  switch (op) {
    case SEP_GAUSS: return batch_sep_kernel_op<SEP_GAUSS>(R, dt);
    case SEP_MEAN: return batch_sep_kernel_op<SEP_MEAN>(R, dt);
    case SEP_MIN: return batch_sep_kernel_op<SEP_MIN>(R, dt);
    case SEP_MAX: return batch_sep_kernel_op<SEP_MAX>(R, dt);
  }
  return nullptr;
}

const void* batch_sep2_kernel(int op, int R, int dt) {
  switch (op) {
    case SEP_GAUSS: return batch_sep2_kernel_op<SEP_GAUSS>(R, dt);
    case SEP_MEAN: return batch_sep2_kernel_op<SEP_MEAN>(R, dt);
    case SEP_MIN: return batch_sep2_kernel_op<SEP_MIN>(R, dt);
    case SEP_MAX: return batch_sep2_kernel_op<SEP_MAX>(R, dt);
  }
  return nullptr;
}

namespace {
template <class T> const void* median_kernel_t(int algo) {
  switch (algo) {
    case A_MED27: return (const void*)k_batch_median<T, A_MED27>;
    case A_MED9: return (const void*)k_batch_median<T, A_MED9>;
    case A_MED33: return (const void*)k_batch_median<T, A_MED33>;
  }
  if constexpr (sizeof(T) <= 2) {
    if (algo == A_MED27Y) return (const void*)k_batch_median<T, A_MED27Y>;
    if (algo == A_MED33P) return (const void*)k_batch_median<T, A_MED33P>;
  }
  if constexpr (sizeof(T) == 2) {
    if (algo == A_MED27S) return (const void*)k_batch_median<T, A_MED27S>;
    if (algo == A_MED33S) return (const void*)k_batch_median<T, A_MED33S>;
  }
  if constexpr (sizeof(T) == 4) {
    if (algo == A_MED33F) return (const void*)k_batch_median<T, A_MED33F>;
  }
  return nullptr;
}
}  // namespace

const void* batch_median_kernel(int dt, int algo) {
  switch (dt) {
    case CLK_U8: return median_kernel_t<uint8_t>(algo);
    case CLK_U16: return median_kernel_t<uint16_t>(algo);
    case CLK_I16: return median_kernel_t<int16_t>(algo);
    case CLK_F32: return median_kernel_t<float>(algo);
  }
  return nullptr;
}

namespace {

bool batch_type(int dt) { return dt == CLK_U8 || dt == CLK_U16 || dt == CLK_I16 || dt == CLK_F32; }
bool batch_radius(int R) {
  for (int r : kBatchRadii)
    if (r == R) return true;
  return false;
}

// shared memory of a sep2 tile body (host side of sep2::Geo)
template <class T, int OP, int R> size_t sep2_smem_t(int cz) { return sep2::Geo<T, S2OpT<OP, T>::v, R>::smem(cz); }
template <int OP, int R> size_t sep2_smem_r(int dt, int cz) {
  if constexpr (OP == SEP_GAUSS) {  // float: the FMA Gaussian; 8/16-bit: the exact-order one
    switch (dt) {
      case CLK_F32: return sep2_smem_t<float, OP, R>(cz);
      case CLK_U8: return sep2_smem_t<uint8_t, OP, R>(cz);
      case CLK_U16: return sep2_smem_t<uint16_t, OP, R>(cz);
      case CLK_I16: return sep2_smem_t<int16_t, OP, R>(cz);
    }
    return 0;
  } else {  // min/max/mean: 8/16-bit pixels; min/max: float too
    if (dt == CLK_F32) {
      if constexpr (OP == SEP_MIN || OP == SEP_MAX) return sep2_smem_t<float, OP, R>(cz);
      return 0;
    }
    switch (dt) {
      case CLK_U8: return sep2_smem_t<uint8_t, OP, R>(cz);
      case CLK_U16: return sep2_smem_t<uint16_t, OP, R>(cz);
      case CLK_I16: return sep2_smem_t<int16_t, OP, R>(cz);
    }
    return 0;
  }
}
template <int OP> size_t sep2_smem_op(int R, int dt, int cz) {
  switch (R) {
    case 2: return sep2_smem_r<OP, 2>(dt, cz);
    case 3: return sep2_smem_r<OP, 3>(dt, cz);
    case 4: return sep2_smem_r<OP, 4>(dt, cz);
    case 5: return sep2_smem_r<OP, 5>(dt, cz);
    case 6: return sep2_smem_r<OP, 6>(dt, cz);
  }
  return 0;
}
size_t sep2_smem(int op, int R, int dt, int cz) {
  switch (op) {
    case SEP_GAUSS: return sep2_smem_op<SEP_GAUSS>(R, dt, cz);
    case SEP_MEAN: return sep2_smem_op<SEP_MEAN>(R, dt, cz);
    case SEP_MIN: return sep2_smem_op<SEP_MIN>(R, dt, cz);
    case SEP_MAX: return sep2_smem_op<SEP_MAX>(R, dt, cz);
  }
  return 0;
}


// ---------------------------------------------------------------- tuning cache
class TuneCache {
 public:
  bool get(const std::string& k, int* v) {
    std::lock_guard<std::mutex> l(mu_);
    load();
    auto it = m_.find(k);
    if (it == m_.end()) return false;
    *v = it->second;
    return true;
  }
  void put(const std::string& k, int v) {
    std::lock_guard<std::mutex> l(mu_);
    load();
    m_[k] = v;
    const std::string p = path();
    for (size_t q = 1; q < p.size(); ++q)  // create the directories (an unwritable path is not an error)
      if (p[q] == '/') mkdir(p.substr(0, q).c_str(), 0755);
    std::ofstream f(p);
    if (!f) return;
    f << "{\n";
    size_t n = 0;
    for (const auto& kv : m_) f << "  \"" << kv.first << "\": " << kv.second << (++n < m_.size() ? ",\n" : "\n");
    f << "}\n";
  }

 private:
  static std::string path() {
    if (const char* p = std::getenv("CLK_AUTOTUNE_CACHE")) return p;
    const char* home = std::getenv("HOME");
    return std::string(home ? home : "/tmp") + "/.cache/clk_gb300/autotune.json";
  }
  void load() {
    if (loaded_) return;
    loaded_ = true;
    std::ifstream f(path());
    if (!f) return;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string s = ss.str();
    size_t i = 0;
    while ((i = s.find('"', i)) != std::string::npos) {
      const size_t j = s.find('"', i + 1);
      const size_t c = j == std::string::npos ? j : s.find(':', j);
      if (c == std::string::npos) break;
      m_[s.substr(i + 1, j - i - 1)] = std::atoi(s.c_str() + c + 1);
      i = s.find_first_of(",}", c);
      if (i == std::string::npos) break;
    }
  }
  std::mutex mu_;
  std::map<std::string, int> m_;
  bool loaded_ = false;
};
TuneCache g_tune;

// ---------------------------------------------------------------- plan
struct Group {  // one persistent launch: a kernel and its work list
  const void* kernel = nullptr;
  bool median = false;
  int dt = 0;
  std::vector<int> imgs;  // images of this group
  std::vector<WorkItem> items;
  WorkItem* d_items = nullptr;
  size_t cap = 0;  // allocated items
  size_t smem = 0;
  int grid = 0;
};

struct ImgStep {  // how one image runs one step
  int algo = 0;   // 0: plain call; else Algo
  int tx = 0, ty = 0;  // tile size of the body
  int R = 0;           // batch kernel radius (separable)
};

}  // namespace
}  // namespace batch
}  // namespace clk

struct clk_batch {
  std::vector<clk_op> ops;
  std::vector<std::string> names;  // op kernel bases (ops[].kernel points here)
  std::vector<clk::Image> src, dst;
  clk::Policy pol;
  std::vector<clk_define> defs;
  std::vector<std::string> def_store;
  void* scratch = nullptr;                 // intermediates of all images
  std::vector<std::array<void*, 2>> tmp;  // per image ping-pong
  void* pk_scratch = nullptr;              // per-kernel mode: pass temporaries
  std::vector<std::array<void*, 2>> pk_tmp;
  // per step
  std::vector<std::vector<clk::batch::ImgStep>> how;
  std::vector<std::vector<clk::batch::Group>> groups;
  std::vector<clk::batch::SepDesc*> d_sep;
  std::vector<clk::batch::MedDesc*> d_med;
  std::vector<int> zchunk;
  std::vector<char> generic;  // per step: integer-output separables on the 64x16 generic tiles
  cudaStream_t streams[4] = {};
  cudaEvent_t events[8] = {};
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int launches = 0;
};

namespace clk {
namespace batch {
namespace {

clk::Image in_of(const clk_batch* b, int s, int i) {
  clk::Image im = s == 0 ? b->src[i] : b->dst[i];
  if (s > 0) im.ptr = b->tmp[i][(s - 1) % 2];
  return im;
}
clk::Image out_of(const clk_batch* b, int s, int i) {
  clk::Image im = b->dst[i];
  if (s != (int)b->ops.size() - 1) im.ptr = b->tmp[i][s % 2];
  return im;
}
clk_image to_abi(const clk::Image& im) {
  clk_image c;
  c.ptr = im.ptr;
  c.dtype = im.dt;
  c.ndim = im.ndim;
  c.width = im.w;
  c.height = im.h;
  c.depth = im.d;
  return c;
}
std::string kname(const clk_batch* b, int s, int i) {
  return b->names[s] + (b->src[i].ndim == 2 ? "_2d" : "_3d");
}

// The plain call of step s on image i (the public entry points themselves).
clk_status plain_step(clk_batch* b, int s, int i, cudaStream_t st) {
  const clk_op& op = b->ops[s];
  const clk::Image in = in_of(b, s, i), out = out_of(b, s, i);
  clk_image ci = to_abi(in), co = to_abi(out);
  const std::string k = kname(b, s, i);
  const clk_define* d = b->defs.empty() ? nullptr : b->defs.data();
  const size_t nd = b->defs.size();
  if (op.kind == CLK_OP_SEPARABLE) return clk_separable(k.c_str(), &co, &ci, op.N, op.s, d, nd, st);
  if (op.kind == CLK_OP_MORPHOLOGY) return clk_morphology(k.c_str(), &co, &ci, op.iterations, d, nd, st);
  clk_arg a[5];
  int na = 0;
  a[na++] = clk_arg{"src", CLK_ARG_IMAGE, 0, 0.f, ci};
  a[na++] = clk_arg{"dst", CLK_ARG_IMAGE, 0, 0.f, co};
  if (b->names[s].rfind("median", 0) == 0) {
    a[na++] = clk_arg{"Nx", CLK_ARG_INT, op.N[0], 0.f, clk_image{}};
    a[na++] = clk_arg{"Ny", CLK_ARG_INT, op.N[1], 0.f, clk_image{}};
    if (in.ndim == 3) a[na++] = clk_arg{"Nz", CLK_ARG_INT, op.N[2], 0.f, clk_image{}};
  }
  return clk_execute(k.c_str(), a, na, nullptr, d, nd, st);
}

int sep_op_of(const std::string& base) {
  if (base == "gaussian_blur_separable") return SEP_GAUSS;
  if (base == "mean_separable") return SEP_MEAN;
  if (base == "minimum_separable") return SEP_MIN;
  if (base == "maximum_separable") return SEP_MAX;
  return -1;
}

// Decide how image i runs separable step s and fill its descriptor; mirrors
// fused_separable's choice (clk_sep_fused.cu) so results equal plain calls.
ImgStep plan_sep(clk_batch* b, int s, int i, SepDesc* d) {
  ImgStep h;
  const clk_op& op = b->ops[s];
  const clk::Image in = in_of(b, s, i), out = out_of(b, s, i);
  if (in.dt != out.dt || !batch_type(in.dt)) return h;
  const std::string k = kname(b, s, i);
  clk_image ci = to_abi(in), co = to_abi(out);
  static thread_local SepPlan plan;
  if (separable_plan(k.c_str(), &co, &ci, op.N, op.s, b->defs.empty() ? nullptr : b->defs.data(), b->defs.size(),
                     &plan) != CLK_OK)
    return h;
  const int opn = plan.op;
  const bool fast = opn == SEP_GAUSS && out.dt == CLK_F32 && !plan.pol.exact_order;
  fused::FusedTaps ft{};
  for (int a = 0; a < 3; ++a) {
    const bool sk = plan.skip[a] || (a == 2 && in.ndim == 2);
    const int c = sk ? 0 : plan.taps[a].c;
    if (c < 0 || c > fused::kFusedMaxR) return h;
    ft.c[a] = c;
    if (sk || opn != SEP_GAUSS) {
      ft.h[a][0] = 1.0f;
      ft.hsum[a] = 1.0f;
    } else if (fast) {
      double sum = 0;
      for (int v = 0; v <= 2 * c; ++v) sum += plan.taps[a].h[v];
      for (int v = 0; v <= 2 * c; ++v) ft.h[a][v] = (float)(plan.taps[a].h[v] / sum);
      ft.hsum[a] = 1.0f;
    } else {
      for (int v = 0; v <= 2 * c; ++v) ft.h[a][v] = plan.taps[a].h[v];
      ft.hsum[a] = plan.taps[a].hsum;
    }
  }
  const int cx = ft.c[0], cy = ft.c[1], cz = ft.c[2];
  const bool ints = in.dt != CLK_F32;
  const bool even = ((uintptr_t)out.ptr % (2 * dtype_size(out.dt))) == 0 &&
                    ((uintptr_t)in.ptr % dtype_size(in.dt)) == 0;
  *d = SepDesc{};
  d->src = in.ptr;
  d->dst = out.ptr;
  d->W = in.w, d->H = in.h, d->D = in.d;
  d->dt = in.dt;
  d->rte = plan.pol.rte;
  d->ft = ft;
  // the register-window kernel, where the plain path takes it
  if (cx == cy && cx >= 1 && even && cz <= sep2::kMaxCz) {
    const int R = cx;
    const bool s2_int = ints && opn != SEP_GAUSS && R <= 8;
    const bool s2_gauss = fast && R <= 12;
    const bool s2_gx = ints && opn == SEP_GAUSS && R <= 8 && in.dt == out.dt;  // exact order, as the plain path
    const bool s2_mmf = !ints && out.dt == CLK_F32 && (opn == SEP_MIN || opn == SEP_MAX) && R <= 8;
    // integer outputs are bit-identical on either body: the tuner may ask
    // for the generic 64x16 tiles instead (b->generic[s])
    const bool alt = s2_int || s2_gx;
    if ((s2_int || s2_gauss || s2_gx || s2_mmf) && !(alt && b->generic[s])) {
      if (!batch_radius(R) || sep2_smem(opn, R, in.dt, cz) > 220 * 1024) return h;  // plain call keeps parity
      d->algo = A_SEP2;
      d->p2.cz = cz;
      d->p2.mx = sep2::recip32(2 * R + 1);
      d->p2.mz = sep2::recip32(2 * cz + 1);
      if (s2_gx) {
        for (int v = 0; v <= 2 * R; ++v) d->p2.hx[v] = ft.h[0][v], d->p2.hy[v] = ft.h[1][v];
        for (int v = 0; v <= 2 * cz; ++v) d->p2.hz[v] = ft.h[2][v];
        for (int a = 0; a < 3; ++a) d->p2.hs[a] = ft.hsum[a];
        d->p2.rte = plan.pol.rte ? 1 : 0;
      }
      if (s2_gauss) {
        for (int a = 0; a < 3; ++a) {
          const int c = ft.c[a];
          double sum = 0;
          for (int v = 0; v <= 2 * c; ++v) sum += ft.h[a][v];
          float* w = a == 0 ? d->p2.wx : (a == 1 ? d->p2.wy : d->p2.wz);
          for (int q = 0; q <= c; ++q) w[q] = (float)(ft.h[a][c + q] / sum);
        }
      }
      h.algo = A_SEP2;
      h.tx = sep2::TX, h.ty = sep2::TY, h.R = R;
      return h;
    }
  }
  // the generic fused kernel (where the plain path takes line passes, a
  // plain call keeps parity)
  if (prefer_line((SepOp)opn, out, in, ft.c, plan.pol)) return h;
  if (fused::fused_smem(cx, cy, cz, dtype_size(in.dt), dtype_size(out.dt)) > 200 * 1024) return h;
  d->algo = fast ? A_FUSED_FAST : A_FUSED_EXACT;
  h.algo = d->algo;
  h.tx = fused::TX, h.ty = fused::TY;
  h.R = (cx == cy && batch_radius(cx)) ? cx : 0;
  return h;
}

ImgStep plan_median(clk_batch* b, int s, int i, MedDesc* d) {
  ImgStep h;
  const clk_op& op = b->ops[s];
  const clk::Image in = in_of(b, s, i), out = out_of(b, s, i);
  if (in.dt != out.dt || !batch_type(in.dt)) return h;
  if ((((uintptr_t)in.ptr | (uintptr_t)out.ptr) % (2 * dtype_size(in.dt))) != 0) return h;
  if (in.dt == CLK_F32 && b->pol.exact_order) return h;
  const bool sphere = b->names[s] == "median_sphere";
  static thread_local MedianNbhd m;
  if (!median_nbhd(sphere, in.ndim, op.N[0], op.N[1], in.ndim == 3 ? op.N[2] : 1, &m) || m.n == 0 ||
      m.n > b->pol.max_array)
    return h;
  int algo = 0;
  if (in.ndim == 3 && !sphere && m.ex == 1 && m.ey == 1 && m.ez == 1 && m.n == 27) algo = A_MED27;
  if (in.ndim == 3 && sphere && m.ex == 2 && m.ey == 2 && m.ez == 2 && m.n == 33) algo = A_MED33;
  if (in.ndim == 2 && m.ex == 1 && m.ey == 1 && m.n == 9) algo = A_MED9;
  if (!algo) return h;
  // even widths take the bodies the plain launcher takes (clk_median.cu)
  const int sz = dtype_size(in.dt);
  const bool even = (in.w & 1) == 0, a16 = (((uintptr_t)in.ptr | (uintptr_t)out.ptr) % 16) == 0;
  if (even && algo == A_MED27 && sz <= 2) algo = sz == 2 && in.w % 8 == 0 && a16 ? A_MED27S : A_MED27Y;
  if (even && algo == A_MED33 && sz <= 2) algo = sz == 2 && in.w % 8 == 0 && a16 ? A_MED33S : A_MED33P;
  if (even && algo == A_MED33 && in.dt == CLK_F32 && in.w % 4 == 0 && a16) algo = A_MED33F;
  *d = MedDesc{in.ptr, out.ptr, in.w, in.h, in.d, 0, in.dt, algo};
  h.algo = algo;
  h.tx = algo == A_MED33F ? med::BX : 2 * med::BX;
  h.ty = algo == A_MED27Y || algo == A_MED27S ? med::BYP : med::BY;
  return h;
}

void build_items(clk_batch* b, int s, Group& g, int zc) {
  g.items.clear();
  for (int i : g.imgs) {
    const ImgStep& h = b->how[s][i];
    const clk::Image& im = b->src[i];
    const int tx = (im.w + h.tx - 1) / h.tx, ty = (im.h + h.ty - 1) / h.ty;
    int z = std::max(1, std::min(zc, im.d));
    if (med_z_pairs(h.algo)) z += z & 1;  // these medians pair outputs along z
    const int tz = h.algo == A_MED9 ? 1 : (im.d + z - 1) / z;
    for (int bz = 0; bz < tz; ++bz)
      for (int by = 0; by < ty; ++by)
        for (int bx = 0; bx < tx; ++bx) g.items.push_back(WorkItem{i, bx, by, bz});
  }
}

clk_status upload_step(clk_batch* b, int s, int zc, cudaStream_t st) {
  // descriptors carry zchunk
  if (b->d_sep[s]) {
    std::vector<SepDesc> hd(b->src.size());
    cudaMemcpy(hd.data(), b->d_sep[s], hd.size() * sizeof(SepDesc), cudaMemcpyDeviceToHost);
    for (size_t i = 0; i < hd.size(); ++i) {
      int z = std::max(1, std::min(zc, b->src[i].d));
      hd[i].zchunk = z;
    }
    if (cudaMemcpy(b->d_sep[s], hd.data(), hd.size() * sizeof(SepDesc), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(CLK_LAUNCH_FAILED, "batch: descriptor upload failed");
  }
  if (b->d_med[s]) {
    std::vector<MedDesc> hd(b->src.size());
    cudaMemcpy(hd.data(), b->d_med[s], hd.size() * sizeof(MedDesc), cudaMemcpyDeviceToHost);
    for (size_t i = 0; i < hd.size(); ++i) {
      int z = std::max(1, std::min(zc, b->src[i].d));
      z += z & 1;
      hd[i].zchunk = z;
    }
    if (cudaMemcpy(b->d_med[s], hd.data(), hd.size() * sizeof(MedDesc), cudaMemcpyHostToDevice) != cudaSuccess)
      return fail(CLK_LAUNCH_FAILED, "batch: descriptor upload failed");
  }
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  for (Group& g : b->groups[s]) {
    build_items(b, s, g, zc);
    if (g.items.size() > g.cap) {
      if (g.d_items) cudaFree(g.d_items);
      g.d_items = nullptr;
      if (cudaMalloc(&g.d_items, g.items.size() * sizeof(WorkItem)) != cudaSuccess) {
        cudaGetLastError();
        return fail(CLK_OOM, "batch: cannot allocate a work list");
      }
      g.cap = g.items.size();
    }
    cudaMemcpyAsync(g.d_items, g.items.data(), g.items.size() * sizeof(WorkItem), cudaMemcpyHostToDevice, st);
    int occ = 0;
    if (g.smem > 48 * 1024) cudaFuncSetAttribute(g.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)g.smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, g.kernel, 256, g.smem);
    cudaGetLastError();
    g.grid = (int)std::min<size_t>(g.items.size(), (size_t)std::max(1, occ) * sms);
  }
  cudaStreamSynchronize(st);
  return check_launch("batch upload");
}

clk_status launch_group(clk_batch* b, int s, const Group& g, cudaStream_t st) {
  if (g.items.empty()) return CLK_OK;
  const int n = (int)g.items.size();
  const void* descs = g.median ? (const void*)b->d_med[s] : (const void*)b->d_sep[s];
  void* args[] = {(void*)&g.d_items, (void*)&n, (void*)&descs};
  if (cudaLaunchKernel(g.kernel, dim3(g.grid), dim3(256), args, g.smem, st) != cudaSuccess)
    return check_launch("batch step");
  count_launch();
  return CLK_OK;
}

// One step: groups and plain calls spread over the streams, joined at the end.
clk_status run_step(clk_batch* b, int s, cudaStream_t st, bool plain_only) {
  const int NS = 4;
  cudaEventRecord(b->events[0], st);
  for (int k = 0; k < NS; ++k) cudaStreamWaitEvent(b->streams[k], b->events[0], 0);
  int rr = 0;
  clk_status res = CLK_OK;
  if (!plain_only)
    for (const Group& g : b->groups[s])
      if (res == CLK_OK) res = launch_group(b, s, g, b->streams[rr++ % NS]);
  for (size_t i = 0; i < b->src.size() && res == CLK_OK; ++i)
    if (plain_only || b->how[s][i].algo == 0) res = plain_step(b, s, (int)i, b->streams[rr++ % NS]);
  for (int k = 0; k < NS; ++k) {
    cudaEventRecord(b->events[1 + k], b->streams[k]);
    cudaStreamWaitEvent(st, b->events[1 + k], 0);
  }
  return res;
}

std::string step_key(const clk_batch* b, int s) {
  std::ostringstream k;
  const clk_op& op = b->ops[s];
  int64_t vox = 0;
  int nd[5] = {0, 0, 0, 0, 0};
  for (const auto& im : b->src) {
    vox += im.count();
    nd[im.dt]++;
  }
  int lg = 0;
  while ((int64_t(1) << (lg + 1)) <= vox) ++lg;
  k << b->names[s] << "|N=" << op.N[0] << "," << op.N[1] << "," << op.N[2] << "|imgs=" << b->src.size()
    << "|vox2^" << lg << "|dt=" << nd[0] << "," << nd[1] << "," << nd[2] << "," << nd[3] << "," << nd[4];
  return k.str();
}

// Plan separable step s: every image's body (register-window or generic
// tiles per b->generic[s], or a plain call) and one group (persistent
// launch) per (radius, pixel type, body); replaces an earlier plan.
clk_status plan_sep_step(clk_batch* b, int s) {
  const int sop = sep_op_of(b->names[s]);
  const int nimages = (int)b->src.size();
  for (auto& g : b->groups[s])
    if (g.d_items) cudaFree(g.d_items);
  b->groups[s].clear();
  if (b->d_sep[s]) cudaFree(b->d_sep[s]);
  b->d_sep[s] = nullptr;
  std::vector<SepDesc> hd(nimages);
  std::map<std::tuple<int, int, bool>, int> gi;  // (R, dt, register-window body) -> group
  for (int i = 0; i < nimages; ++i) {
    b->how[s][i] = plan_sep(b, s, i, &hd[i]);
    if (!b->how[s][i].algo) continue;
    const bool s2 = b->how[s][i].algo == A_SEP2;
    const auto key = std::make_tuple(b->how[s][i].R, b->src[i].dt, s2);
    if (!gi.count(key)) {
      Group g;
      g.kernel = s2 ? batch_sep2_kernel(sop, std::get<0>(key), std::get<1>(key))
                    : batch_sep_kernel(sop, std::get<0>(key), std::get<1>(key));
      g.dt = std::get<1>(key);
      if (!g.kernel) {
        b->how[s][i].algo = 0;
        continue;
      }
      gi[key] = (int)b->groups[s].size();
      b->groups[s].push_back(g);
    }
    Group& g = b->groups[s][gi[key]];
    g.imgs.push_back(i);
    const ImgStep& h = b->how[s][i];
    const size_t need = h.algo == A_SEP2
                            ? sep2_smem(sop, h.R, b->src[i].dt, hd[i].p2.cz)
                            : fused::fused_smem(hd[i].ft.c[0], hd[i].ft.c[1], hd[i].ft.c[2],
                                                dtype_size(b->src[i].dt), dtype_size(b->dst[i].dt));
    g.smem = std::max(g.smem, need);
  }
  if (cudaMalloc(&b->d_sep[s], nimages * sizeof(SepDesc)) != cudaSuccess ||
      cudaMemcpy(b->d_sep[s], hd.data(), nimages * sizeof(SepDesc), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    return fail(CLK_OOM, "clk_batch_create: cannot allocate descriptors");
  }
  return CLK_OK;
}

// The tuner's choice per step, timed on the real images and cached under
// the step's key: the depth of a work item (zchunk) and, for steps with
// integer-output separable images, their tile body -- the register-window
// 64x32 tiles or the generic 64x16 tiles (bit-identical results; key
// "<step>|tile", 0 or 1).
clk_status tune_step(clk_batch* b, int s, cudaStream_t st) {
  if (b->groups[s].empty()) {
    b->zchunk[s] = 0;
    return CLK_OK;
  }
  const std::string key = step_key(b, s), tkey = key + "|tile";
  bool two_bodies = false;
  if (b->ops[s].kind == CLK_OP_SEPARABLE)
    for (size_t i = 0; i < b->src.size(); ++i)
      two_bodies |= b->how[s][i].algo == A_SEP2 && b->dst[i].dt != CLK_F32;
  int best = 0, tile = 0;
  if (g_tune.get(key, &best)) {
    if (two_bodies && g_tune.get(tkey, &tile) && tile != b->generic[s]) {
      b->generic[s] = (char)tile;
      if (clk_status r = plan_sep_step(b, s)) return r;
    }
    b->zchunk[s] = best;
    return upload_step(b, s, best, st);
  }
  const int cands[] = {8, 16, 32, 64, 1 << 20};
  float best_ms = 1e30f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  clk_status res = CLK_OK;
  for (int t = 0; t < (two_bodies ? 2 : 1) && res == CLK_OK; ++t) {
    if (t != b->generic[s]) {
      b->generic[s] = (char)t;
      if ((res = plan_sep_step(b, s))) break;
    }
    for (int zc : cands) {
      if ((res = upload_step(b, s, zc, st))) break;
      for (const Group& g : b->groups[s])  // warm-up
        if ((res = launch_group(b, s, g, st))) break;
      float ms_min = 1e30f;
      for (int rep = 0; rep < 3 && res == CLK_OK; ++rep) {
        cudaEventRecord(e0, st);
        for (const Group& g : b->groups[s])
          if ((res = launch_group(b, s, g, st))) break;
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_min = std::min(ms_min, ms);
      }
      if (res) break;
      if (ms_min < best_ms) best_ms = ms_min, best = zc, tile = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (res) return res;
  if (tile != b->generic[s]) {
    b->generic[s] = (char)tile;
    if ((res = plan_sep_step(b, s))) return res;
  }
  g_tune.put(key, best);
  if (two_bodies) g_tune.put(tkey, tile);
  b->zchunk[s] = best;
  return upload_step(b, s, best, st);
}

// Step s of image i as the reference's callers launch it: one clk_execute per
// kernel; a separable filter is one launch per axis (an axis with N <= 1, or
// a Gaussian with s <= 0, is launched with N = 1, s = 1: a converting copy).
clk_status per_kernel_step(clk_batch* b, int s, int i, cudaStream_t st) {
  const clk_op& op = b->ops[s];
  if (op.kind != CLK_OP_SEPARABLE) return plain_step(b, s, i, st);  // already one kernel (or r launches)
  const clk::Image in = in_of(b, s, i), out = out_of(b, s, i);
  const std::string k = kname(b, s, i);
  const int nd = in.ndim;
  const clk_define* d = b->defs.empty() ? nullptr : b->defs.data();
  clk_image cur = to_abi(in);
  clk_status r = CLK_OK;
  for (int a = 0; a < nd && r == CLK_OK; ++a) {
    clk::Image o = out;
    if (a != nd - 1) o.ptr = b->pk_tmp[i][a % 2];
    clk_image co = to_abi(o);
    const bool gauss = b->names[s] == "gaussian_blur_separable";
    const bool skip = op.N[a] <= 1 || (gauss && !(op.s[a] > 0));
    clk_arg args[5] = {{"dst", CLK_ARG_IMAGE, 0, 0.f, co},
                       {"src", CLK_ARG_IMAGE, 0, 0.f, cur},
                       {"dim", CLK_ARG_INT, a, 0.f, clk_image{}},
                       {"N", CLK_ARG_INT, skip ? 1 : op.N[a], 0.f, clk_image{}},
                       {"s", CLK_ARG_FLOAT, 0, skip ? 1.f : op.s[a], clk_image{}}};
    r = clk_execute(k.c_str(), args, 5, nullptr, d, b->defs.size(), st);
    cur = co;
  }
  return r;
}

void destroy(clk_batch* b) {
  if (!b) return;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (auto& gs : b->groups)
    for (auto& g : gs)
      if (g.d_items) cudaFree(g.d_items);
  for (auto* p : b->d_sep)
    if (p) cudaFree(p);
  for (auto* p : b->d_med)
    if (p) cudaFree(p);
  if (b->scratch) cudaFree(b->scratch);
  if (b->pk_scratch) cudaFree(b->pk_scratch);
  for (auto& s : b->streams)
    if (s) cudaStreamDestroy(s);
  for (auto& e : b->events)
    if (e) cudaEventDestroy(e);
  delete b;
}

}  // namespace
}  // namespace batch
}  // namespace clk

using namespace clk;
using namespace clk::batch;

extern "C" {

clk_status clk_batch_create(const clk_op* ops, int32_t nops, const clk_image* src, const clk_image* dst,
                            int32_t nimages, const clk_define* defines, size_t ndefines, void* stream,
                            clk_batch** out) {
  if (!out) return fail(CLK_BAD_ARG, "clk_batch_create: out is NULL");
  *out = nullptr;
  if (!ops || nops <= 0 || !src || !dst || nimages <= 0)
    return fail(CLK_BAD_ARG, "clk_batch_create: empty pipeline or image list");
  cudaStream_t st = (cudaStream_t)stream;
  clk_batch* b = new clk_batch();
  for (size_t i = 0; i < ndefines; ++i) {
    b->def_store.push_back(defines[i].name ? defines[i].name : "");
    b->def_store.push_back(defines[i].value ? defines[i].value : "");
  }
  for (size_t i = 0; i < ndefines; ++i)
    b->defs.push_back(clk_define{b->def_store[2 * i].c_str(), b->def_store[2 * i + 1].c_str()});
  // policy (for the batch-side choices; the plain calls parse the same defines)
  for (const auto& d : b->defs) {
    if (!std::strcmp(d.name, "CLK_EXACT_ORDER")) b->pol.exact_order = std::strcmp(d.value, "0") != 0;
    if (!std::strcmp(d.name, "CLK_CONVERT_ROUNDING")) b->pol.rte = !std::strcmp(d.value, "rte");
    if (!std::strcmp(d.name, "MAX_ARRAY_SIZE")) b->pol.max_array = std::atoi(d.value);
  }
  b->names.reserve(nops);
  for (int s = 0; s < nops; ++s) {
    if (!ops[s].kernel) {
      destroy(b);
      return fail(CLK_BAD_ARG, "clk_batch_create: step %d has no kernel", s);
    }
    b->names.push_back(ops[s].kernel);
    b->ops.push_back(ops[s]);
  }
  for (int s = 0; s < nops; ++s) b->ops[s].kernel = b->names[s].c_str();
  size_t scratch = 0;
  for (int i = 0; i < nimages; ++i) {
    const clk_image& a = src[i];
    const clk_image& c = dst[i];
    const int nd = a.ndim;
    if ((nd != 2 && nd != 3) || c.ndim != nd || a.width != c.width || a.height != c.height ||
        (nd == 3 && a.depth != c.depth) || a.width <= 0 || a.height <= 0 || (nd == 3 && a.depth <= 0) || !a.ptr ||
        !c.ptr || a.dtype < 0 || a.dtype > 4 || c.dtype < 0 || c.dtype > 4) {
      destroy(b);
      return fail(CLK_BAD_ARG, "clk_batch_create: image %d: bad extent, type or pointer (src and dst must match)", i);
    }
    const int d = nd == 3 ? (int)a.depth : 1;
    b->src.push_back(Image{a.ptr, a.dtype, nd, (int)a.width, (int)a.height, d});
    b->dst.push_back(Image{c.ptr, c.dtype, nd, (int)c.width, (int)c.height, d});
    if (nops > 1) scratch += 2 * (((size_t)b->dst.back().count() * dtype_size(c.dtype) + 255) & ~size_t(255));
  }
  if (device_ready_public() != CLK_OK) {
    destroy(b);
    return CLK_NO_DEVICE;
  }
  if (scratch && (alloc_failure_injected() || cudaMalloc(&b->scratch, scratch) != cudaSuccess)) {
    cudaGetLastError();
    destroy(b);
    return fail(CLK_OOM, "clk_batch_create: cannot allocate %zu bytes of intermediates", scratch);
  }
  b->tmp.resize(nimages);
  size_t off = 0;
  for (int i = 0; i < nimages; ++i) {
    const size_t bytes = ((size_t)b->dst[i].count() * dtype_size(b->dst[i].dt) + 255) & ~size_t(255);
    for (int k = 0; k < 2; ++k) {
      b->tmp[i][k] = nops > 1 ? (char*)b->scratch + off : nullptr;
      if (nops > 1) off += bytes;
    }
  }
  for (auto& s : b->streams) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  for (auto& e : b->events) cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  // plan every step
  b->how.assign(nops, std::vector<ImgStep>(nimages));
  b->groups.resize(nops);
  b->d_sep.assign(nops, nullptr);
  b->d_med.assign(nops, nullptr);
  b->zchunk.assign(nops, 0);
  b->generic.assign(nops, 0);
  clk_status res = CLK_OK;
  for (int s = 0; s < nops && res == CLK_OK; ++s) {
    const int sop = sep_op_of(b->names[s]);
    const bool med = b->names[s] == "median_box" || b->names[s] == "median_sphere";
    if (b->ops[s].kind == CLK_OP_SEPARABLE && sop >= 0) {
      res = plan_sep_step(b, s);
    } else if (b->ops[s].kind == CLK_OP_KERNEL && med) {
      std::vector<MedDesc> hd(nimages);
      std::map<int, int> gi;
      for (int i = 0; i < nimages; ++i) {
        b->how[s][i] = plan_median(b, s, i, &hd[i]);
        if (!b->how[s][i].algo) continue;
        const int dt = b->src[i].dt, key = dt * 16 + b->how[s][i].algo;  // one group per (type, body)
        if (!gi.count(key)) {
          Group g;
          g.kernel = batch_median_kernel(dt, b->how[s][i].algo);
          g.median = true;
          g.dt = dt;
          gi[key] = (int)b->groups[s].size();
          b->groups[s].push_back(g);
        }
        b->groups[s][gi[key]].imgs.push_back(i);
      }
      if (cudaMalloc(&b->d_med[s], nimages * sizeof(MedDesc)) != cudaSuccess ||
          cudaMemcpy(b->d_med[s], hd.data(), nimages * sizeof(MedDesc), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        res = fail(CLK_OOM, "clk_batch_create: cannot allocate descriptors");
      }
    }
    // other steps: plain calls per image (how[s][i].algo == 0)
  }
  // validate the plain steps once (argument errors surface here, not in the graph)
  for (int s = 0; s < nops && res == CLK_OK; ++s)
    for (int i = 0; i < nimages && res == CLK_OK; ++i)
      if (!b->how[s][i].algo) res = plain_step(b, s, i, st);
  if (res == CLK_OK) res = check_launch("batch plain steps");
  // autotune (runs the steps on the real images, in order)
  for (int s = 0; s < nops && res == CLK_OK; ++s) res = tune_step(b, s, st);
  // capture the pipeline
  if (res == CLK_OK) {
    const uint64_t before = clk_launch_count();
    cudaStream_t cs = nullptr;
    cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
      res = check_launch("batch capture");
    } else {
      for (int s = 0; s < nops && res == CLK_OK; ++s) res = run_step(b, s, cs, false);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(cs, &g);
      if (res == CLK_OK && e != cudaSuccess) res = fail(CLK_LAUNCH_FAILED, "batch capture: %s", cudaGetErrorString(e));
      b->graph = g;
      if (res == CLK_OK && cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess)
        res = check_launch("batch graph instantiate");
    }
    cudaGetLastError();
    if (cs) cudaStreamDestroy(cs);
    uncount_launches(clk_launch_count() - before);  // capture is not execution
    if (res == CLK_OK) {
      size_t n = 0;
      cudaGraphGetNodes(b->graph, nullptr, &n);
      std::vector<cudaGraphNode_t> nodes(n);
      cudaGraphGetNodes(b->graph, nodes.data(), &n);
      for (auto& nd : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nd, &t);
        if (t == cudaGraphNodeTypeKernel) b->launches++;
      }
    }
  }
  if (res != CLK_OK) {
    destroy(b);
    return res;
  }
  *out = b;
  return CLK_OK;
}

clk_status clk_batch_run(clk_batch* b, void* stream) {
  TraceRange trace("clk_batch_run");
  if (!b || !b->exec) return fail(CLK_BAD_ARG, "clk_batch_run: no batch");
  if (cudaGraphLaunch(b->exec, (cudaStream_t)stream) != cudaSuccess) return check_launch("batch graph launch");
  count_launch(b->launches);
  return CLK_OK;
}

clk_status clk_batch_run_plain(clk_batch* b, void* stream) {
  if (!b) return fail(CLK_BAD_ARG, "clk_batch_run_plain: no batch");
  cudaStream_t st = (cudaStream_t)stream;
  for (size_t s = 0; s < b->ops.size(); ++s)
    for (size_t i = 0; i < b->src.size(); ++i) {
      const clk_status r = plain_step(b, (int)s, (int)i, st);
      if (r != CLK_OK) return r;
    }
  return CLK_OK;
}

clk_status clk_batch_run_per_kernel(clk_batch* b, void* stream) {
  if (!b) return fail(CLK_BAD_ARG, "clk_batch_run_per_kernel: no batch");
  cudaStream_t st = (cudaStream_t)stream;
  if (!b->pk_scratch) {  // two pass temporaries per image, allocated on first use
    size_t total = 0;
    for (const auto& im : b->dst) total += 2 * (((size_t)im.count() * dtype_size(im.dt) + 255) & ~size_t(255));
    if (cudaMalloc(&b->pk_scratch, total) != cudaSuccess) {
      cudaGetLastError();
      b->pk_scratch = nullptr;
      return fail(CLK_OOM, "clk_batch_run_per_kernel: cannot allocate %zu bytes of pass temporaries", total);
    }
    b->pk_tmp.resize(b->dst.size());
    size_t off = 0;
    for (size_t i = 0; i < b->dst.size(); ++i) {
      const size_t bytes = ((size_t)b->dst[i].count() * dtype_size(b->dst[i].dt) + 255) & ~size_t(255);
      b->pk_tmp[i][0] = (char*)b->pk_scratch + off;
      b->pk_tmp[i][1] = (char*)b->pk_scratch + off + bytes;
      off += 2 * bytes;
    }
  }
  for (size_t s = 0; s < b->ops.size(); ++s)
    for (size_t i = 0; i < b->src.size(); ++i) {
      const clk_status r = per_kernel_step(b, (int)s, (int)i, st);
      if (r != CLK_OK) return r;
    }
  return CLK_OK;
}

int32_t clk_batch_launches(const clk_batch* b) { return b ? b->launches : 0; }

void clk_batch_destroy(clk_batch* b) { destroy(b); }

}  // extern "C"
