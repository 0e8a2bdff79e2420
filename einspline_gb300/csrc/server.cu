// Request server: continuous batching of walker-shaped requests over one
// table.  The reference has no serving layer; its batched entry evaluates
// one fixed set of walker positions per synchronous call
// (src/multi_bspline_cuda_s_impl.h:542-563, driven from src/cuda_walker.cu:69-95).
//
// Design:
//  * submit() copies a request's positions and queues it (FIFO);
//  * a worker thread admits queued requests while their outputs fit in a
//    device-memory arena (first-fit free list), packs admitted requests into
//    a batch of at most max_batch_points and launches it on one of
//    max_inflight slots, each with its own stream, pinned staging buffer and
//    instantiated CUDA graph (copy-in -> evaluation kernel -> event record);
//  * a completion thread polls the in-flight batches' events, stamps
//    completion times and frees the slot, so new requests join the next
//    batch while earlier batches are still running; it sleeps when nothing
//    is in flight, and the worker spins ~100 us before it sleeps: the two
//    thread wake-ups a request would otherwise wait for cost tens of
//    microseconds each, more than the evaluation of a walker;
//  * release() returns a request's outputs to the arena and wakes admission.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>

#include "eg_internal.h"

namespace eg {

static double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, size) with coalescing.
class Arena {
 public:
  void reset(size_t size) { free_.clear(); if (size) free_[0] = size; used_ = peak_ = 0; size_ = size; }
  bool alloc(size_t bytes, size_t *off) {
    bytes = align_up_sz(bytes, 256);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes;
        const size_t noff = it->first + bytes;
        free_.erase(it);
        if (rest) free_[noff] = rest;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = align_up_sz(bytes, 256);
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
    }
  }
  size_t size() const { return size_; }
  size_t peak() const { return peak_; }

 private:
  std::map<size_t, size_t> free_;
  size_t used_ = 0, peak_ = 0, size_ = 0;
};

struct Request {
  int npts = 0;
  std::vector<char> pos;
  size_t off = 0, bytes = 0;
  double t_submit = 0, t_done = 0;
  int state = 0;  // 0 queued, 1 admitted, 2 running, 3 done
};

struct Server;

struct Slot {
  Server *srv = nullptr;
  cudaStream_t stream = nullptr;
  char *stage_h = nullptr, *stage_d = nullptr;
  void *sort_d = nullptr;      // counting-sort scratch (sort option)
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphNode_t n_copy = nullptr, n_kernel = nullptr, n_event = nullptr;
  cudaEvent_t done = nullptr;  // recorded after the batch's kernel
  bool busy = false;
  bool launched = false;       // the batch (and its event record) is enqueued
  std::vector<int64_t> reqs;
  int64_t points = 0;
};

}  // namespace eg

struct einspline_gb300_server {
  uint32_t magic = eg::kMagic;
  eg::Server *impl = nullptr;
};

namespace eg {

struct Server {
  Table *t = nullptr;
  einspline_gb300_server_opts o;
  int out_reals_per_pt = 0;  // vals + grads + hess reals per point
  size_t rb = 4;             // output real bytes
  size_t pos_b = 24;         // bytes per position
  char *arena_d = nullptr;
  Arena arena;
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_poll;
  // bumped, under mu, whenever the worker may have something new to do (a
  // submit, a finished batch, released memory): the worker spins on it
  // briefly before it blocks
  std::atomic<uint64_t> epoch{0};
  int device = 0;
  int launched = 0;            // slots launched and not yet seen complete
  bool stop_poll = false;
  std::thread poller;
  std::deque<int64_t> queue, admitted;
  std::unordered_map<int64_t, Request> reqs;
  std::vector<Slot> slots;
  std::thread worker;
  bool stop = false;
  int64_t next_id = 0;
  einspline_gb300_server_stats st;
  int inflight = 0;
  double t_first = -1, t_last = 0;
  int tx = 0, ty = 0, pb = 0;
  const void *func = nullptr;
  std::string worker_error;

  size_t stage_bytes() const { return (size_t)o.max_batch_points * (24 + pos_b); }
};

// Marks a batch's requests done (under the server lock).
static void complete_locked(Server *v, Slot &s, double t) {
  for (int64_t id : s.reqs) {
    auto it = v->reqs.find(id);
    if (it != v->reqs.end()) { it->second.state = 3; it->second.t_done = t; }
  }
  v->st.completed += (int64_t)s.reqs.size();
  s.reqs.clear();
  s.busy = false;
  s.launched = false;
  v->launched--;
  v->inflight--;
  v->t_last = t;
}

// Completion thread: while batches are in flight it polls their events
// (a few microseconds from the GPU finishing to the requests being marked
// done, against a host-callback thread's wake-up); with nothing in flight it
// sleeps.  It leaves only when stopped and every launched batch is done.
static void poller_loop(Server *v) {
  cudaSetDevice(v->device);
  std::vector<Slot *> live;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(v->mu);
      v->cv_poll.wait(lk, [&] { return v->launched > 0 || v->stop_poll; });
      if (v->launched == 0) return;  // stopped and drained
      live.clear();
      for (auto &sl : v->slots)
        if (sl.busy && sl.launched) live.push_back(&sl);
    }
    bool any = false;
    for (Slot *sl : live) {
      const cudaError_t e = cudaEventQuery(sl->done);
      if (e == cudaErrorNotReady) continue;
      const double t = now_s();
      {
        std::lock_guard<std::mutex> g(v->mu);
        if (e != cudaSuccess && v->worker_error.empty()) v->worker_error = cudaGetErrorString(e);
        complete_locked(v, *sl, t);
        v->epoch.fetch_add(1);
      }
      any = true;
    }
    if (any) {
      v->cv_done.notify_all();
      v->cv_work.notify_one();
    } else {
      std::this_thread::yield();
    }
  }
}

// Packed staging of a batch of n points: vals_pp[n], grads_pp[n], hess_pp[n],
// then n positions.
static void fill_args(Server *v, Slot &s, EvalArgs &a, int64_t n) {
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(v->t, a);
  a.pos_f64 = v->o.pos_f64;
  a.rule = v->o.rule;
  a.layout = 0;
  a.npts = n;
  void **pp = (void **)s.stage_d;
  a.vals_pp = pp;
  a.grads_pp = pp + n;
  a.hess_pp = pp + 2 * n;
  a.pos = s.stage_d + 24 * n;
}

static int build_graph(Server *v, Slot &s) {
  EvalArgs a;
  fill_args(v, s, a, 1);
  const void *func;
  dim3 grid, block;
  size_t smem;
  if (int r = prepare_eval(v->t, a, v->o.vgh != 0, v->tx, v->ty, v->pb, &func, &grid, &block, &smem)) return r;
  EG_CUDA(cudaGraphCreate(&s.graph, 0));
  EG_CUDA(cudaGraphAddMemcpyNode1D(&s.n_copy, s.graph, nullptr, 0, s.stage_d, s.stage_h, 64, cudaMemcpyHostToDevice));
  cudaKernelNodeParams kp;
  memset(&kp, 0, sizeof(kp));
  void *args[] = {&a};
  kp.func = (void *)func;
  kp.gridDim = grid;
  kp.blockDim = block;
  kp.sharedMemBytes = (unsigned)smem;
  kp.kernelParams = args;
  EG_CUDA(cudaGraphAddKernelNode(&s.n_kernel, s.graph, &s.n_copy, 1, &kp));
  EG_CUDA(cudaGraphAddEventRecordNode(&s.n_event, s.graph, &s.n_kernel, 1, s.done));
  EG_CUDA(cudaGraphInstantiate(&s.exec, s.graph, 0));
  v->func = func;
  return 0;
}

static int launch_batch(Server *v, Slot &s) {
  const int64_t n = s.points;
  EvalArgs a;
  fill_args(v, s, a, n);
  const size_t bytes = (size_t)n * (24 + v->pos_b);
  if (v->o.use_graphs) {
    const void *func;
    dim3 grid, block;
    size_t smem;
    if (int r = prepare_eval(v->t, a, v->o.vgh != 0, v->tx, v->ty, v->pb, &func, &grid, &block, &smem)) return r;
    cudaKernelNodeParams kp;
    memset(&kp, 0, sizeof(kp));
    void *args[] = {&a};
    kp.func = (void *)func;
    kp.gridDim = grid;
    kp.blockDim = block;
    kp.sharedMemBytes = (unsigned)smem;
    kp.kernelParams = args;
    EG_CUDA(cudaGraphExecMemcpyNodeSetParams1D(s.exec, s.n_copy, s.stage_d, s.stage_h, bytes, cudaMemcpyHostToDevice));
    EG_CUDA(cudaGraphExecKernelNodeSetParams(s.exec, s.n_kernel, &kp));
    EG_CUDA(cudaGraphLaunch(s.exec, s.stream));
    count_launch();
  } else {
    EG_CUDA(cudaMemcpyAsync(s.stage_d, s.stage_h, bytes, cudaMemcpyHostToDevice, s.stream));
    if (v->o.sort && n > 1) {
      int *perm = nullptr;
      if (int r = small_sort_into(a, s.sort_d, &perm, s.stream)) return r;
      a.perm = perm;
    }
    if (int r = launch_eval(v->t, a, v->o.vgh != 0, s.stream, v->tx, v->ty, v->pb)) return r;
    EG_CUDA(cudaEventRecord(s.done, s.stream));
  }
  return 0;
}

// Spin budget of the worker before it blocks on its condition variable.
constexpr double kSpinSeconds = 100e-6;

static void worker_loop(Server *v) {
  cudaSetDevice(v->device);
  const size_t ncol = v->t->ncol;
  for (;;) {
    Slot *slot = nullptr;
    {
      std::unique_lock<std::mutex> lk(v->mu);
      for (;;) {
        if (v->stop && v->queue.empty() && v->admitted.empty()) return;
        // admission by device memory, in arrival order
        while (!v->queue.empty()) {
          Request &r = v->reqs[v->queue.front()];
          size_t off;
          if (!v->arena.alloc(r.bytes, &off)) break;
          r.off = off;
          r.state = 1;
          v->admitted.push_back(v->queue.front());
          v->queue.pop_front();
        }
        slot = nullptr;
        if (!v->admitted.empty())
          for (auto &s : v->slots)
            if (!s.busy) { slot = &s; break; }
        if (slot) break;
        // nothing to launch: spin briefly on the epoch (a thread wake-up
        // costs tens of microseconds), then block
        const uint64_t seen = v->epoch.load();
        lk.unlock();
        const double t_spin = now_s() + kSpinSeconds;
        while (v->epoch.load() == seen && now_s() < t_spin) std::this_thread::yield();
        lk.lock();
        if (v->epoch.load() == seen && !v->stop)
          v->cv_work.wait_for(lk, std::chrono::milliseconds(50), [&] { return v->epoch.load() != seen || v->stop; });
      }
      // form a batch from admitted requests
      slot->reqs.clear();
      slot->points = 0;
      while (!v->admitted.empty()) {
        Request &r = v->reqs[v->admitted.front()];
        if (slot->points + r.npts > v->o.max_batch_points && slot->points > 0) break;
        slot->reqs.push_back(v->admitted.front());
        slot->points += r.npts;
        r.state = 2;
        v->admitted.pop_front();
      }
      slot->busy = true;
      v->inflight++;
      v->st.peak_inflight = std::max(v->st.peak_inflight, v->inflight);
      v->st.batches++;
      if (v->t_first < 0) v->t_first = now_s();
      // host staging (the requests' positions stay put while running)
      const int64_t n = slot->points;
      void **pp = (void **)slot->stage_h;
      char *posb = slot->stage_h + 24 * n;
      int64_t j = 0;
      for (int64_t id : slot->reqs) {
        Request &r = v->reqs[id];
        char *base = v->arena_d + r.off;
        const size_t vb = ncol * v->rb;
        for (int k = 0; k < r.npts; k++, j++) {
          pp[j] = base + (size_t)k * vb;
          pp[n + j] = base + (size_t)r.npts * vb + (size_t)k * 3 * vb;
          pp[2 * n + j] = base + (size_t)r.npts * 4 * vb + (size_t)k * 6 * vb;
        }
        memcpy(posb + (j - r.npts) * v->pos_b, r.pos.data(), (size_t)r.npts * v->pos_b);
        v->st.evals += (int64_t)r.npts * v->t->num_splines;
      }
    }
    if (launch_batch(v, *slot)) {
      std::lock_guard<std::mutex> g(v->mu);
      v->worker_error = einspline_gb300_last_error_message();
      for (int64_t id : slot->reqs) v->reqs[id].state = 3;
      slot->busy = false;
      v->inflight--;
      v->cv_done.notify_all();
    } else {
      {
        std::lock_guard<std::mutex> g(v->mu);
        slot->launched = true;
        v->launched++;
      }
      v->cv_poll.notify_one();
    }
  }
}

void destroy_server(Server *v);

static Server *srv_of(einspline_gb300_server *s) {
  if (!s || s->magic != kMagic || !s->impl) {
    fail(EINSPLINE_GB300_EINVAL, "bad server handle");
    return nullptr;
  }
  return s->impl;
}

}  // namespace eg

using namespace eg;

extern "C" {

einspline_gb300_server *einspline_gb300_server_create(einspline_gb300_table *t, const einspline_gb300_server_opts *opts) {
  clear();
  if (!table3_ok(t)) { fail(EINSPLINE_GB300_EINVAL, "bad table handle"); return nullptr; }
  if (table_flush(t)) return nullptr;
  Server *v = new Server();
  v->t = t;
  memset(&v->o, 0, sizeof(v->o));
  if (opts) v->o = *opts; else { v->o.vgh = 1; v->o.pos_f64 = 1; v->o.use_graphs = 1; }
  if (v->o.max_inflight <= 0) v->o.max_inflight = 3;
  v->o.max_inflight = std::min(v->o.max_inflight, 8);
  if (v->o.max_batch_points <= 0) v->o.max_batch_points = 16384;
  if (v->o.sort) {
    if (v->o.max_batch_points > kSmallSort) {
      delete v;
      fail(EINSPLINE_GB300_EINVAL, "server: sort takes max_batch_points <= %lld", (long long)kSmallSort);
      return nullptr;
    }
    v->o.use_graphs = 0;  // the per-batch sort is launched directly
  }
  v->rb = t->storage == ST_F64 ? 8 : 4;
  v->pos_b = v->o.pos_f64 ? 24 : 12;
  v->out_reals_per_pt = (v->o.vgh ? 10 : 1) * t->ncol;
  memset(&v->st, 0, sizeof(v->st));
  size_t budget = v->o.hbm_budget_bytes;
  if (!budget) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    budget = std::min<size_t>(4ull << 30, fr / 2);
  }
  auto bail = [&](const char *what) -> einspline_gb300_server * {
    const int code = einspline_gb300_last_error();
    std::string msg = einspline_gb300_last_error_message();
    destroy_server(v);
    if (code) fail(code, "%s: %s", what, msg.c_str());
    else cuda_check(cudaGetLastError(), what);
    return nullptr;
  };
  cudaGetDevice(&v->device);
  if (cudaMalloc(&v->arena_d, budget) != cudaSuccess) return bail("server arena");
  v->arena.reset(budget);
  v->st.budget_bytes = budget;
  pick_tile(t, v->o.vgh != 0, v->o.max_batch_points, v->tx, v->ty, v->pb, v->o.sort != 0);
  v->slots.resize(v->o.max_inflight);
  for (auto &s : v->slots) {
    s.srv = v;
    if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMallocHost(&s.stage_h, v->stage_bytes()) != cudaSuccess ||
        cudaMalloc(&s.stage_d, v->stage_bytes()) != cudaSuccess ||
        cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess ||
        (v->o.sort && cudaMalloc(&s.sort_d, small_sort_bytes(v->o.max_batch_points)) != cudaSuccess))
      return bail("server slot");
    if (v->o.use_graphs && build_graph(v, s)) return bail("server graph");
  }
  {
    std::lock_guard<std::mutex> g(t->mu);
    t->servers++;
  }
  v->poller = std::thread(poller_loop, v);
  v->worker = std::thread(worker_loop, v);
  auto *h = new einspline_gb300_server();
  h->impl = v;
  return h;
}

int einspline_gb300_server_destroy(einspline_gb300_server *s) {
  clear();
  Server *v = srv_of(s);
  if (!v) return EINSPLINE_GB300_EINVAL;
  {
    std::lock_guard<std::mutex> g(v->t->mu);
    v->t->servers--;
  }
  destroy_server(v);
  s->magic = 0;
  s->impl = nullptr;
  delete s;
  return 0;
}

}  // extern "C"

namespace eg {

void destroy_server(Server *v) {
  {
    std::lock_guard<std::mutex> g(v->mu);
    v->stop = true;
    // requests that were never admitted are dropped
    for (int64_t id : v->queue) v->reqs.erase(id);
    v->queue.clear();
  }
  v->cv_work.notify_all();
  if (v->worker.joinable()) v->worker.join();
  {
    // the poller drains the launched batches, then leaves
    std::lock_guard<std::mutex> g(v->mu);
    v->stop_poll = true;
  }
  v->cv_poll.notify_all();
  if (v->poller.joinable()) v->poller.join();
  for (auto &sl : v->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.exec) cudaGraphExecDestroy(sl.exec);
    if (sl.graph) cudaGraphDestroy(sl.graph);
    if (sl.stage_h) cudaFreeHost(sl.stage_h);
    if (sl.stage_d) cudaFree(sl.stage_d);
    if (sl.sort_d) cudaFree(sl.sort_d);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  cudaFree(v->arena_d);
  cudaGetLastError();
  delete v;
}

}  // namespace eg

extern "C" {

int64_t einspline_gb300_server_submit(einspline_gb300_server *s, const void *pos_host, int npts) {
  clear();
  Server *v = srv_of(s);
  if (!v) return -1;
  if (npts < 1 || !pos_host) { fail(EINSPLINE_GB300_EINVAL, "submit: npts must be >= 1 with positions"); return -1; }
  if (npts > v->o.max_batch_points) {
    fail(EINSPLINE_GB300_ESIZE, "submit: %d points exceed max_batch_points %d", npts, v->o.max_batch_points);
    return -1;
  }
  const size_t bytes = (size_t)npts * v->out_reals_per_pt * v->rb;
  if (align_up_sz(bytes, 256) > v->arena.size()) {
    fail(EINSPLINE_GB300_ESIZE, "submit: outputs (%zu bytes) exceed the memory budget", bytes);
    return -1;
  }
  Request r;
  r.npts = npts;
  r.bytes = bytes;
  r.pos.assign((const char *)pos_host, (const char *)pos_host + (size_t)npts * v->pos_b);
  r.t_submit = now_s();
  int64_t id;
  {
    std::lock_guard<std::mutex> g(v->mu);
    id = v->next_id++;
    v->reqs.emplace(id, std::move(r));
    v->queue.push_back(id);
    v->st.submitted++;
    v->epoch.fetch_add(1);  // under the lock: the worker's wait cannot miss it
  }
  v->cv_work.notify_one();
  return id;
}

int einspline_gb300_server_wait(einspline_gb300_server *s, int64_t id, double timeout_s) {
  clear();
  Server *v = srv_of(s);
  if (!v) return EINSPLINE_GB300_EINVAL;
  std::unique_lock<std::mutex> lk(v->mu);
  auto done = [&] {
    auto it = v->reqs.find(id);
    return it == v->reqs.end() || it->second.state == 3;
  };
  if (v->reqs.find(id) == v->reqs.end()) return fail(EINSPLINE_GB300_EINVAL, "wait: unknown request %lld", (long long)id);
  if (!v->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), done))
    return fail(EINSPLINE_GB300_ETIMEOUT, "wait: request %lld not done after %.3f s", (long long)id, timeout_s);
  if (!v->worker_error.empty()) return fail(EINSPLINE_GB300_ECUDA, "server: %s", v->worker_error.c_str());
  return 0;
}

int einspline_gb300_server_result(einspline_gb300_server *s, int64_t id, void **vals_d, void **grads_d, void **hess_d,
                                  double *latency_s) {
  clear();
  Server *v = srv_of(s);
  if (!v) return EINSPLINE_GB300_EINVAL;
  std::lock_guard<std::mutex> g(v->mu);
  auto it = v->reqs.find(id);
  if (it == v->reqs.end() || it->second.state != 3) return fail(EINSPLINE_GB300_EINVAL, "result: request not done");
  const Request &r = it->second;
  const size_t vb = v->t->ncol * v->rb;
  char *base = v->arena_d + r.off;
  if (vals_d) *vals_d = base;
  if (grads_d) *grads_d = base + (size_t)r.npts * vb;
  if (hess_d) *hess_d = base + (size_t)r.npts * 4 * vb;
  if (latency_s) *latency_s = r.t_done - r.t_submit;
  return 0;
}

int einspline_gb300_server_copy_result(einspline_gb300_server *s, int64_t id, void *vals_h, void *grads_h,
                                       void *hess_h) {
  void *vd, *gd, *hd;
  if (int r = einspline_gb300_server_result(s, id, &vd, &gd, &hd, nullptr)) return r;
  Server *v = s->impl;
  int npts;
  {
    std::lock_guard<std::mutex> g(v->mu);
    npts = v->reqs[id].npts;
  }
  const size_t vb = (size_t)npts * v->t->ncol * v->rb;
  if (vals_h) EG_CUDA(cudaMemcpy(vals_h, vd, vb, cudaMemcpyDeviceToHost));
  if (v->o.vgh && grads_h) EG_CUDA(cudaMemcpy(grads_h, gd, 3 * vb, cudaMemcpyDeviceToHost));
  if (v->o.vgh && hess_h) EG_CUDA(cudaMemcpy(hess_h, hd, 6 * vb, cudaMemcpyDeviceToHost));
  return 0;
}

int einspline_gb300_server_release(einspline_gb300_server *s, int64_t id) {
  clear();
  Server *v = srv_of(s);
  if (!v) return EINSPLINE_GB300_EINVAL;
  {
    std::lock_guard<std::mutex> g(v->mu);
    auto it = v->reqs.find(id);
    if (it == v->reqs.end()) return fail(EINSPLINE_GB300_EINVAL, "release: unknown request %lld", (long long)id);
    if (it->second.state != 3) return fail(EINSPLINE_GB300_EINVAL, "release: request %lld is not done", (long long)id);
    v->arena.release(it->second.off, it->second.bytes);
    v->reqs.erase(it);
    v->st.released++;
    v->epoch.fetch_add(1);
  }
  v->cv_work.notify_one();
  return 0;
}

int einspline_gb300_server_get_stats(einspline_gb300_server *s, einspline_gb300_server_stats *out) {
  clear();
  Server *v = srv_of(s);
  if (!v || !out) return fail(EINSPLINE_GB300_EINVAL, "bad argument");
  std::lock_guard<std::mutex> g(v->mu);
  *out = v->st;
  out->peak_bytes_in_use = v->arena.peak();
  out->busy_seconds = v->t_first < 0 ? 0.0 : v->t_last - v->t_first;
  return 0;
}

int einspline_gb300_server_replay(einspline_gb300_server *s, int nreq, const double *arrival_s, const int *npts,
                                  const int64_t *offsets, const void *pos_host, double *latency_s, double *wall_s) {
  clear();
  Server *v = srv_of(s);
  if (!v) return EINSPLINE_GB300_EINVAL;
  if (nreq < 0 || (nreq && (!arrival_s || !npts || !offsets || !pos_host || !latency_s)))
    return fail(EINSPLINE_GB300_EINVAL, "replay: bad argument");
  std::vector<int64_t> ids(nreq, -1);
  std::mutex m;
  std::condition_variable cv;
  int submitted = 0;
  int err = 0;
  const double t0 = now_s();
  // collector: release requests in submission order as they complete
  std::thread collector([&] {
    for (int i = 0; i < nreq; i++) {
      int64_t id;
      {
        std::unique_lock<std::mutex> lk(m);
        cv.wait(lk, [&] { return submitted > i || err; });
        if (ids[i] < 0) { latency_s[i] = -1; continue; }
        id = ids[i];
      }
      if (einspline_gb300_server_wait(s, id, 600.0)) { latency_s[i] = -1; continue; }
      einspline_gb300_server_result(s, id, nullptr, nullptr, nullptr, &latency_s[i]);
      einspline_gb300_server_release(s, id);
    }
  });
  for (int i = 0; i < nreq; i++) {
    const double due = t0 + arrival_s[i];
    double dt = due - now_s();
    if (dt > 0) std::this_thread::sleep_for(std::chrono::duration<double>(dt));
    const int64_t id = einspline_gb300_server_submit(
        s, (const char *)pos_host + offsets[i] * (int64_t)v->pos_b, npts[i]);
    {
      std::lock_guard<std::mutex> g(m);
      ids[i] = id;
      submitted = i + 1;
      if (id < 0) err = 1;
    }
    cv.notify_all();
  }
  collector.join();
  if (wall_s) *wall_s = now_s() - t0;
  return err ? fail(EINSPLINE_GB300_EINVAL, "replay: a request was refused") : 0;
}

}  // extern "C"
