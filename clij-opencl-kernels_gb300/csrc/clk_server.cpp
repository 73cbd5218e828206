// clk_server.cpp - the served form behind clk_server_* (include/clk.h).
//
// Requests (one image + a pipeline of steps) queue in arrival order.  A
// scheduler thread admits the head of the queue as soon as a slot (one of
// `slots` CUDA streams) and the HBM budget for its temporaries are free, and
// enqueues its whole pipeline on that slot's stream: optional host->device
// copy, the steps as plain calls (ping-pong temporaries from the server's own
// memory pool, freed stream-ordered), optional device->host copy, and a host
// callback that stamps the completion time.  Admission never waits for a
// batch to drain: requests that arrive while others run start at once and
// their kernels overlap on the device.  No device-side wait exists; host
// waits are bounded by the caller's timeout.
#include <cuda_runtime_api.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "clk_internal.h"

namespace clk {
namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t id = 0;
  std::vector<clk_op> ops;
  std::vector<std::string> names;
  clk_image src{}, dst{};
  const void* host_in = nullptr;
  void* host_out = nullptr;
  size_t tmp_bytes = 0;  // two ping-pong temporaries when the pipeline has > 1 step
  double voxels = 0;
  Clock::time_point t_submit;
  std::atomic<int64_t> t_done_ns{0};  // stamped by the host callback
  int state = 0;                      // 0 queued, 1 in flight, 2 done, 3 failed, 4 cancelled
  clk_status status = CLK_OK;
  int slot = -1;
  void* tmp = nullptr;
  double latency_ms = 0;
};

int64_t ns_since(Clock::time_point t0) {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
}

size_t image_bytes(const clk_image& im) {
  const int64_t d = im.ndim == 3 ? im.depth : 1;
  return (size_t)(im.width * im.height * d) * (size_t)dtype_size(im.dtype);
}

}  // namespace
}  // namespace clk

struct clk_server {
  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::deque<std::shared_ptr<clk::Request>> queue;
  std::vector<std::shared_ptr<clk::Request>> inflight;
  std::map<uint64_t, std::shared_ptr<clk::Request>> live;  // queued or in flight or not yet waited
  std::vector<cudaStream_t> streams;
  std::vector<bool> busy;
  cudaMemPool_t pool = nullptr;
  int device = 0;
  int64_t budget = 0, in_use = 0, peak = 0;
  uint64_t next_id = 1, submitted = 0, completed = 0, failed = 0, cancelled = 0;
  std::vector<double> latencies;
  double voxel_steps = 0;
  clk::Clock::time_point t0;
  bool started = false;
  int64_t first_submit_ns = -1, last_done_ns = 0;
  std::atomic<bool> stop{false};
  clk::Clock::time_point t_stop;
  std::thread sched;
};

namespace clk {
namespace {

constexpr size_t kMaxQueue = 1 << 20;

void CUDART_CB on_done(void* p) {
  auto* r = static_cast<Request*>(p);
  r->t_done_ns.store(std::max<int64_t>(1, ns_since(r->t_submit)), std::memory_order_release);
}

// One step of a request as the plain call (the public entry points).
clk_status run_step(const Request& r, int k, const clk_image& in, const clk_image& out, cudaStream_t st) {
  const clk_op& op = r.ops[k];
  const std::string name = r.names[k] + (in.ndim == 2 ? "_2d" : "_3d");
  if (op.kind == CLK_OP_SEPARABLE) return clk_separable(name.c_str(), &out, &in, op.N, op.s, nullptr, 0, st);
  if (op.kind == CLK_OP_MORPHOLOGY) return clk_morphology(name.c_str(), &out, &in, op.iterations, nullptr, 0, st);
  clk_arg a[5];
  int na = 0;
  a[na++] = clk_arg{"src", CLK_ARG_IMAGE, 0, 0.f, in};
  a[na++] = clk_arg{"dst", CLK_ARG_IMAGE, 0, 0.f, out};
  if (r.names[k].rfind("median", 0) == 0) {
    a[na++] = clk_arg{"Nx", CLK_ARG_INT, op.N[0], 0.f, clk_image{}};
    a[na++] = clk_arg{"Ny", CLK_ARG_INT, op.N[1], 0.f, clk_image{}};
    if (in.ndim == 3) a[na++] = clk_arg{"Nz", CLK_ARG_INT, op.N[2], 0.f, clk_image{}};
  }
  return clk_execute(name.c_str(), a, na, nullptr, nullptr, 0, st);
}

// Enqueue a request's pipeline on its slot's stream (scheduler thread).
void launch(clk_server* s, Request& r) {
  TraceRange trace("clk_server request");
  cudaStream_t st = s->streams[r.slot];
  clk_status res = CLK_OK;
  const size_t in_bytes = image_bytes(r.src), out_bytes = image_bytes(r.dst);
  if (r.host_in && cudaMemcpyAsync(r.src.ptr, r.host_in, in_bytes, cudaMemcpyHostToDevice, st) != cudaSuccess)
    res = check_launch("server: host->device copy");
  if (res == CLK_OK && r.tmp_bytes) {
    if (alloc_failure_injected() || cudaMallocFromPoolAsync(&r.tmp, r.tmp_bytes, s->pool, st) != cudaSuccess) {
      cudaGetLastError();
      r.tmp = nullptr;
      res = fail(CLK_OOM, "server: request %llu: no memory for temporaries", (unsigned long long)r.id);
    }
  }
  const int n = (int)r.ops.size();
  const size_t half = r.tmp_bytes / 2;
  for (int k = 0; k < n && res == CLK_OK; ++k) {
    clk_image in = r.src, out = r.dst;
    in.dtype = k == 0 ? r.src.dtype : r.dst.dtype;
    if (k > 0) in.ptr = (char*)r.tmp + ((k - 1) % 2) * half;
    if (k != n - 1) out.ptr = (char*)r.tmp + (k % 2) * half;
    res = run_step(r, k, in, out, st);
  }
  if (res == CLK_OK && r.host_out &&
      cudaMemcpyAsync(r.host_out, r.dst.ptr, out_bytes, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    res = check_launch("server: device->host copy");
  if (r.tmp) cudaFreeAsync(r.tmp, st);
  r.status = res;
  if (cudaLaunchHostFunc(st, on_done, &r) != cudaSuccess) {
    cudaGetLastError();
    cudaStreamSynchronize(st);  // no callback: complete synchronously
    on_done(&r);
    if (r.status == CLK_OK) r.status = CLK_LAUNCH_FAILED;
  }
}

void scheduler(clk_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    // reap completions
    bool reaped = false;
    for (size_t i = 0; i < s->inflight.size();) {
      auto& r = s->inflight[i];
      const int64_t done = r->t_done_ns.load(std::memory_order_acquire);
      if (!done) {
        ++i;
        continue;
      }
      r->latency_ms = done * 1e-6;
      r->state = r->status == CLK_OK ? 2 : 3;
      s->busy[r->slot] = false;
      s->in_use -= (int64_t)r->tmp_bytes;
      if (r->state == 2) {
        s->completed++;
        s->latencies.push_back(r->latency_ms);
        s->voxel_steps += r->voxels * (double)r->ops.size();
      } else {
        s->failed++;
      }
      s->last_done_ns = std::max(s->last_done_ns, ns_since(s->t0));
      s->inflight.erase(s->inflight.begin() + i);
      reaped = true;
    }
    if (reaped) s->cv_done.notify_all();
    // admit in arrival order while a slot and the budget allow
    while (!s->queue.empty()) {
      auto& r = s->queue.front();
      int slot = -1;
      for (size_t k = 0; k < s->busy.size(); ++k)
        if (!s->busy[k]) {
          slot = (int)k;
          break;
        }
      if (slot < 0) break;
      if (s->budget > 0 && s->in_use + (int64_t)r->tmp_bytes > s->budget) break;
      s->busy[slot] = true;
      s->in_use += (int64_t)r->tmp_bytes;
      s->peak = std::max(s->peak, s->in_use);
      r->slot = slot;
      r->state = 1;
      s->inflight.push_back(r);
      auto req = r;
      s->queue.pop_front();
      launch(s, *req);
    }
    if (s->stop.load() && s->queue.empty() && s->inflight.empty()) break;
    if (s->stop.load() && ns_since(s->t_stop) > 60LL * 1000000000LL) break;  // never hang the caller's exit
    // in-flight work completes without notifying us: poll at a short period
    s->cv_sched.wait_for(lk, std::chrono::microseconds(s->inflight.empty() ? 2000 : 20));
  }
}

}  // namespace
}  // namespace clk

using namespace clk;

extern "C" {

clk_status clk_server_create(int32_t slots, int64_t hbm_budget_bytes, clk_server** out) {
  if (!out) return fail(CLK_BAD_ARG, "clk_server_create: out is NULL");
  *out = nullptr;
  if (slots < 1 || slots > 64) return fail(CLK_BAD_ARG, "clk_server_create: slots must be 1..64, got %d", slots);
  if (hbm_budget_bytes < 0) return fail(CLK_BAD_ARG, "clk_server_create: negative budget");
  clk_status st = device_ready_public();
  if (st) return st;
  auto* s = new clk_server();
  cudaGetDevice(&s->device);
  s->budget = hbm_budget_bytes;
  s->streams.resize(slots);
  s->busy.assign(slots, false);
  for (auto& x : s->streams) cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking);
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = s->device;
  if (cudaMemPoolCreate(&s->pool, &props) != cudaSuccess) {
    cudaGetLastError();
    for (auto& x : s->streams) cudaStreamDestroy(x);
    delete s;
    return fail(CLK_OOM, "clk_server_create: cannot create a memory pool");
  }
  uint64_t keep = hbm_budget_bytes > 0 ? (uint64_t)hbm_budget_bytes : UINT64_MAX;
  cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);  // reuse, do not return to the OS
  s->t0 = Clock::now();
  s->sched = std::thread(scheduler, s);
  *out = s;
  return CLK_OK;
}

clk_status clk_server_submit(clk_server* s, const clk_op* ops, int32_t nops, const clk_image* src,
                             const clk_image* dst, const void* host_in, void* host_out, uint64_t* ticket) {
  if (!s || !ops || nops <= 0 || !src || !dst || !ticket) return fail(CLK_BAD_ARG, "clk_server_submit: null argument");
  if (src->ndim != dst->ndim || src->width != dst->width || src->height != dst->height ||
      (src->ndim == 3 && src->depth != dst->depth) || !src->ptr || !dst->ptr || dtype_size(src->dtype) == 0 ||
      dtype_size(dst->dtype) == 0)
    return fail(CLK_BAD_ARG, "clk_server_submit: src and dst must be device images of the same extent");
  auto r = std::make_shared<Request>();
  for (int k = 0; k < nops; ++k) {
    if (!ops[k].kernel) return fail(CLK_BAD_ARG, "clk_server_submit: step %d has no kernel", k);
    r->names.push_back(ops[k].kernel);
    r->ops.push_back(ops[k]);
  }
  for (int k = 0; k < nops; ++k) r->ops[k].kernel = r->names[k].c_str();
  r->src = *src;
  r->dst = *dst;
  if (src->ndim == 2) r->src.depth = r->dst.depth = 1;
  r->host_in = host_in;
  r->host_out = host_out;
  const size_t half = (image_bytes(*dst) + 255) & ~size_t(255);
  r->tmp_bytes = nops > 1 ? 2 * half : 0;
  r->voxels = (double)src->width * (double)src->height * (double)(src->ndim == 3 ? src->depth : 1);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->budget > 0 && (int64_t)r->tmp_bytes > s->budget)
    return fail(CLK_BAD_ARG, "clk_server_submit: request needs %zu bytes of temporaries, budget is %lld",
                r->tmp_bytes, (long long)s->budget);
  if (s->queue.size() >= kMaxQueue) return fail(CLK_BUSY, "clk_server_submit: queue full");
  r->id = s->next_id++;
  r->t_submit = Clock::now();
  if (s->first_submit_ns < 0) s->first_submit_ns = ns_since(s->t0);
  s->queue.push_back(r);
  s->live[r->id] = r;
  s->submitted++;
  *ticket = r->id;
  s->cv_sched.notify_one();
  return CLK_OK;
}

clk_status clk_server_wait(clk_server* s, uint64_t ticket, int32_t timeout_ms, double* latency_ms) {
  if (!s) return fail(CLK_BAD_ARG, "clk_server_wait: no server");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end()) return fail(CLK_BAD_ARG, "clk_server_wait: unknown ticket %llu", (unsigned long long)ticket);
  auto r = it->second;
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)), [&] { return r->state >= 2; }))
    return fail(CLK_TIMEOUT, "clk_server_wait: request %llu not finished after %d ms", (unsigned long long)ticket,
                timeout_ms);
  if (latency_ms) *latency_ms = r->latency_ms;
  s->live.erase(ticket);
  return r->status;
}

clk_status clk_server_cancel(clk_server* s, uint64_t ticket) {
  if (!s) return fail(CLK_BAD_ARG, "clk_server_cancel: no server");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->live.find(ticket);
  if (it == s->live.end())
    return fail(CLK_BAD_ARG, "clk_server_cancel: unknown ticket %llu", (unsigned long long)ticket);
  auto r = it->second;
  if (r->state != 0)
    return fail(CLK_BUSY, "clk_server_cancel: request %llu is %s", (unsigned long long)ticket,
                r->state == 1 ? "already running on the device" : "already finished");
  for (auto q = s->queue.begin(); q != s->queue.end(); ++q)
    if (q->get() == r.get()) {
      s->queue.erase(q);
      break;
    }
  r->state = 4;
  r->status = fail(CLK_CANCELLED, "request %llu was cancelled before it started", (unsigned long long)ticket);
  s->cancelled++;
  s->cv_done.notify_all();
  s->cv_sched.notify_one();
  return CLK_OK;
}

clk_status clk_server_drain(clk_server* s, int32_t timeout_ms) {
  if (!s) return fail(CLK_BAD_ARG, "clk_server_drain: no server");
  std::unique_lock<std::mutex> lk(s->mu);
  if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(std::max(0, timeout_ms)),
                           [&] { return s->queue.empty() && s->inflight.empty(); }))
    return fail(CLK_TIMEOUT, "clk_server_drain: %zu queued, %zu in flight after %d ms", s->queue.size(),
                s->inflight.size(), timeout_ms);
  return CLK_OK;
}

clk_status clk_server_get_stats(clk_server* s, clk_server_stats* out) {
  if (!s || !out) return fail(CLK_BAD_ARG, "clk_server_get_stats: null argument");
  std::lock_guard<std::mutex> lk(s->mu);
  clk_server_stats st{};
  st.submitted = s->submitted;
  st.completed = s->completed;
  st.failed = s->failed;
  st.cancelled = s->cancelled;
  st.bytes_in_use = s->in_use;
  st.bytes_peak = s->peak;
  st.inflight = (int32_t)s->inflight.size();
  st.queued = (int32_t)s->queue.size();
  if (!s->latencies.empty()) {
    std::vector<double> l = s->latencies;
    std::sort(l.begin(), l.end());
    auto q = [&](double p) { return l[std::min(l.size() - 1, (size_t)(p * (double)(l.size() - 1) + 0.5))]; };
    st.p50_ms = q(0.50);
    st.p99_ms = q(0.99);
    double sum = 0;
    for (double v : l) sum += v;
    st.mean_ms = sum / (double)l.size();
  }
  st.voxel_steps = s->voxel_steps;
  st.busy_s = s->first_submit_ns < 0 ? 0 : (s->last_done_ns - s->first_submit_ns) * 1e-9;
  *out = st;
  return CLK_OK;
}

void clk_server_destroy(clk_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->t_stop = Clock::now();
  }
  s->stop.store(true);
  s->cv_sched.notify_all();
  if (s->sched.joinable()) s->sched.join();
  for (auto& x : s->streams) {
    cudaStreamSynchronize(x);
    cudaStreamDestroy(x);
  }
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
}

}  // extern "C"
