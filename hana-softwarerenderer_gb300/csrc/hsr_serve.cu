// hsr_serve.cu — replayable plans (CUDA graphs) and the continuous-batching server.
//
// The reference renders one frame at a time on one thread (main.cpp:87-155); every frame
// is DrawModel::draw (scene.h:53-99): an optional shadow pass, then the main pass.  Here a
// frame is a pair of draws in a batch, and many frames share one launch sequence:
//   - a plan records the launch sequence of a fixed batch into a CUDA graph once and
//     replays it; uniforms (cameras, lights) change between replays through the pinned
//     staging the graph's upload node reads at launch time;
//   - a server turns independently arriving requests into batches: a scheduler thread
//     admits queued requests while the framebuffer pool has room, packs everything admitted
//     into one launch sequence on a free slot, and completes requests as their batch's event
//     fires.  A slot is one batch in flight: launch sequences run one after another on the
//     server's compute stream (two launch sequences sharing the SMs finish later than the same
//     two in turn), while the host forms the next batch and each slot's copy stream brings its
//     results back under the next batch's kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "hsr_internal.h"
#include "hsr_runtime.h"

namespace hsr {

// ============================================================================================
// plans
// ============================================================================================
struct PlanObj {
  Plan p;
  std::vector<hsr_draw_desc> descs;
  std::vector<hsr_shader_data> uniforms;
  char* dev = nullptr;
  size_t dev_cap = 0;
  char* host = nullptr;
  size_t host_cap = 0;
  cudaGraphExec_t exec = nullptr;
  bool in_flight = false;
  ~PlanObj() {
    if (exec) cudaGraphExecDestroy(exec);
    if (dev) cudaFree(dev);
    if (host) cudaFreeHost(host);
  }
};

static std::unordered_map<uint64_t, PlanObj*> g_plans;

static int plan_bind_and_record(Runtime* rt, PlanObj* po) {
  Plan& p = po->p;
  p.layout();
  if (p.dev_bytes > po->dev_cap) {
    if (po->dev) cudaFree(po->dev);
    po->dev = nullptr;
    po->dev_cap = 0;
    cudaError_t e = cudaMalloc(&po->dev, p.dev_bytes);
    if (e != cudaSuccess) { cudaGetLastError(); return fail(HSR_ERR_OUT_OF_MEMORY, "plan: scratch allocation failed"); }
    po->dev_cap = p.dev_bytes;
  }
  if (p.stage_bytes > po->host_cap) {
    if (po->host) cudaFreeHost(po->host);
    po->host = nullptr;
    po->host_cap = 0;
    cudaError_t e = cudaMallocHost(&po->host, p.stage_bytes);
    if (e != cudaSuccess) { cudaGetLastError(); return fail(HSR_ERR_OUT_OF_MEMORY, "plan: staging allocation failed"); }
    po->host_cap = p.stage_bytes;
  }
  p.bind(po->dev, po->host);
  if (po->exec) {
    cudaGraphExecDestroy(po->exec);
    po->exec = nullptr;
  }
  cudaError_t e = cudaStreamBeginCapture(rt->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(e, "plan: begin capture");
  int rc = p.enqueue(rt->stream, rt->num_sms, rt->tuning, nullptr);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(rt->stream, &graph);
  if (rc != HSR_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "plan: end capture");
  e = cudaGraphInstantiate(&po->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda_fail(e, "plan: graph instantiate");
  return HSR_OK;
}

// Refresh draw k's descriptor in the staging from its uniforms (camera*model etc.).
static void plan_refresh_view(PlanObj* po, int k) {
  Plan& p = po->p;
  DView& v = p.views[k];
  const hsr_draw_desc& d = po->descs[p.order[k]];
  v.u = *d.uniforms;
  mat_mul_ref(d.shader == HSR_SHADER_SHADOW ? v.u.light_vp_matrix : v.u.camera_vp_matrix, v.u.model_matrix, v.mvp);
  std::memcpy(p.host + p.o_views + sizeof(DView) * (size_t)k, &v, sizeof(DView));
}

static int plan_wait(Runtime* rt, PlanObj* po) {
  for (int attempt = 0; attempt < 6; attempt++) {
    if (!po->in_flight) return HSR_OK;
    cudaError_t e = cudaStreamSynchronize(rt->stream);
    po->in_flight = false;
    if (e != cudaSuccess) return cuda_fail(e, "plan: wait");
    const Ctl c = *(const Ctl*)(po->p.host + po->p.host_bytes);
    if (po->p.grow(c)) {  // overflow: nothing was drawn; larger scratch, record again, re-run
      rt->stats.retries++;
      rt->learn_caps(po->p);
      int rc = plan_bind_and_record(rt, po);
      if (rc != HSR_OK) return rc;
      e = cudaGraphLaunch(po->exec, rt->stream);
      if (e != cudaSuccess) return cuda_fail(e, "plan: relaunch");
      po->in_flight = true;
      continue;
    }
    if (c.error & (kErrWaitTimeout | kErrScanTimeout)) return fail(HSR_ERR_TIMEOUT, "plan: a bounded device wait gave up");
    rt->record_result(po->p, c);
    return HSR_OK;
  }
  return fail(HSR_ERR_BIN_OVERFLOW, "plan: scratch overflow persisted after retries");
}

// ============================================================================================
// server
// ============================================================================================
struct SrvReq {
  hsr_request r;
  hsr_request_status st;
  size_t bytes = 0;           // pool bytes of its targets
  char* mem = nullptr;        // one pool allocation: main planes then shadow planes
  uint64_t h_main = 0, h_shadow = 0;
  int idle_alloc_failures = 0;  // failed allocations while no batch was in flight
};
// A request whose targets cannot be allocated while no batch is in flight (so no memory of
// this server will free up) is failed after this many attempts.
constexpr int kMaxIdleAllocFailures = 8;

struct Slot {
  cudaStream_t stream = nullptr;  // copies of results, after the batch's kernels
  cudaEvent_t kdone = nullptr;    // the batch's kernels are done (on the compute stream)
  cudaEvent_t done = nullptr;     // its results are copied (on the slot's stream)
  char* host = nullptr;           // the batch's descriptors and control block
  size_t host_cap = 0;
  Plan plan;
  std::vector<hsr_draw_desc> descs;
  std::vector<SrvReq*> reqs;
  bool busy = false;
  uint32_t batch = 0;
};

struct ServerObj {
  hsr_server_config cfg;
  int device = 0;
  int num_sms = 1;
  hsr_tuning tuning;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<SrvReq*> pending;
  std::unordered_map<uint64_t, SrvReq*> reqs;
  std::vector<Slot> slots;
  cudaStream_t compute = nullptr;  // every batch's launch sequence, in batch order
  char* dev = nullptr;             // scratch of every batch (they run in turn on `compute`)
  size_t dev_cap = 0;
  uint64_t pool_used = 0;
  uint64_t next_ticket = 1;
  uint32_t next_batch = 1;
  int inject_alloc_failures = 0;  // hsr_server_inject_alloc_failures (guarded by mu)
  bool stop = false;
  std::thread th;
  std::chrono::steady_clock::time_point t0;
  double now() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

static std::unordered_map<uint64_t, ServerObj*> g_servers;
static uint64_t g_next_obj = 1;

// A target is three 256-byte aligned planes (colour, depth, prim ids) in one block.
static size_t plane_bytes(int w, int h) { return ((size_t)w * (size_t)h * 4 + 255) / 256 * 256; }

static size_t req_bytes(const hsr_request& r) {
  return 3 * plane_bytes(r.width, r.height) + (r.shadow_size > 0 ? 3 * plane_bytes(r.shadow_size, r.shadow_size) : 0);
}

// Grow the scratch and a slot's staging geometrically (x1.5), so a run of slightly larger
// batches does not reallocate on every batch (each new block of scratch is memory the pool maps
// while batches run).  Batches run in turn on the compute stream, so
// one device scratch serves them all (the next batch's counter reset follows the previous
// batch's control-block read in stream order); it comes from the stream-ordered pool on that
// stream, so replacing it waits only for the batches before it (cudaMalloc / cudaFree would
// synchronise the whole device).  Staging stays per slot: the host fills the next batch's
// descriptors while the previous batch may still be reading its own.
static int slot_reserve(ServerObj* so, Slot& s, const Plan& p) {
  if (p.dev_bytes > so->dev_cap) {
    // headroom over this batch as well: the next batches of a stream are seldom much larger
    const size_t want = std::max(p.dev_bytes + p.dev_bytes / 2, so->dev_cap + so->dev_cap / 2);
    if (so->dev) cudaFreeAsync(so->dev, so->compute);
    so->dev = nullptr;
    so->dev_cap = 0;
    if (cudaMallocAsync(reinterpret_cast<void**>(&so->dev), want, so->compute) != cudaSuccess) {
      cudaGetLastError();
      so->dev = nullptr;
      return HSR_ERR_OUT_OF_MEMORY;
    }
    so->dev_cap = want;
  }
  if (p.stage_bytes > s.host_cap) {
    const size_t want = std::max(p.stage_bytes, s.host_cap + s.host_cap / 2);
    if (s.host) cudaFreeHost(s.host);  // the slot is idle: nothing in flight reads it
    s.host = nullptr;
    s.host_cap = 0;
    if (cudaMallocHost(&s.host, want) != cudaSuccess) { cudaGetLastError(); return HSR_ERR_OUT_OF_MEMORY; }
    s.host_cap = want;
  }
  return HSR_OK;
}

// Enqueue the slot's plan on the compute stream and the copies of every request's results on
// the slot's stream after it.
static int slot_enqueue(ServerObj* so, Slot& s) {
  s.plan.layout();
  int rc = slot_reserve(so, s, s.plan);
  if (rc != HSR_OK) return rc;
  s.plan.bind(so->dev, s.host);
  rc = s.plan.enqueue(so->compute, so->num_sms, so->tuning, nullptr);
  if (rc != HSR_OK) return rc;
  cudaError_t e = cudaEventRecord(s.kdone, so->compute);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s.stream, s.kdone, 0);
  if (e != cudaSuccess) return cuda_fail(e, "server: order copies after the batch");
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (g_rt) g_rt->launches += (uint64_t)s.plan.kernel_count();
  }
  for (SrvReq* q : s.reqs) {
    const size_t n = (size_t)q->r.width * (size_t)q->r.height, pl = plane_bytes(q->r.width, q->r.height);
    const char* base = q->mem;
    if (q->r.out_rgba) cudaMemcpyAsync(q->r.out_rgba, base, 4 * n, cudaMemcpyDeviceToHost, s.stream);
    if (q->r.out_depth) cudaMemcpyAsync(q->r.out_depth, base + pl, 4 * n, cudaMemcpyDeviceToHost, s.stream);
    if (q->r.out_prim) cudaMemcpyAsync(q->r.out_prim, base + 2 * pl, 4 * n, cudaMemcpyDeviceToHost, s.stream);
  }
  e = cudaEventRecord(s.done, s.stream);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "server: event record");
}

static TargetObj* make_pooled_target(char* mem, int w, int h) {
  TargetObj* t = new TargetObj();
  const size_t pl = plane_bytes(w, h);
  t->color = reinterpret_cast<uint32_t*>(mem);
  t->depth = reinterpret_cast<float*>(mem + pl);
  t->prim = reinterpret_cast<uint32_t*>(mem + 2 * pl);
  t->w = w;
  t->h = h;
  t->pooled = true;
  return t;
}

static void finish(ServerObj* so, Slot& s, int status) {
  const double t = so->now();
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (SrvReq* q : s.reqs) {
      for (uint64_t h : {q->h_main, q->h_shadow}) {
        if (!g_rt || !h) continue;
        auto it = g_rt->targets.find(h);
        if (it != g_rt->targets.end()) {
          delete it->second;
          g_rt->targets.erase(it);
        }
      }
      q->h_main = q->h_shadow = 0;
    }
  }
  std::lock_guard<std::mutex> lk(so->mu);
  for (SrvReq* q : s.reqs) {
    if (q->mem) cudaFreeAsync(q->mem, s.stream);
    q->mem = nullptr;
    so->pool_used -= q->bytes;
    q->st.done_ms = t;
    q->st.status = status;
  }
  s.reqs.clear();
  s.busy = false;
  so->cv_done.notify_all();
}

// Form and launch one batch on a free slot; returns true if something was launched.
static bool try_launch(ServerObj* so, Slot& s) {
  std::vector<SrvReq*> batch;
  {
    std::lock_guard<std::mutex> lk(so->mu);
    while (!so->pending.empty() && (int)batch.size() < so->cfg.max_batch) {
      SrvReq* q = so->pending.front();
      if (q->bytes > so->cfg.pool_bytes) {  // can never be admitted
        so->pending.pop_front();
        q->st.status = HSR_ERR_OUT_OF_MEMORY;
        q->st.done_ms = so->now();
        so->cv_done.notify_all();
        continue;
      }
      if (so->pool_used + q->bytes > so->cfg.pool_bytes) break;  // wait for memory (arrival order kept)
      so->pending.pop_front();
      so->pool_used += q->bytes;
      batch.push_back(q);
    }
  }
  if (batch.empty()) return false;
  // targets from the stream-ordered pool; from the first request whose allocation fails on,
  // the requests go back to the head of the queue in arrival order (deferred, not failed)
  size_t got = 0;
  for (; got < batch.size(); got++) {
    SrvReq* q = batch[got];
    bool injected = false;
    {
      std::lock_guard<std::mutex> lk(so->mu);
      if (so->inject_alloc_failures > 0) {
        so->inject_alloc_failures--;
        injected = true;
      }
    }
    if (injected || cudaMallocAsync(reinterpret_cast<void**>(&q->mem), q->bytes, so->compute) != cudaSuccess) {
      if (!injected) cudaGetLastError();
      q->mem = nullptr;
      break;
    }
  }
  if (got < batch.size()) {
    bool any_busy = false;
    for (const Slot& o : so->slots) any_busy |= o.busy;
    std::lock_guard<std::mutex> lk(so->mu);
    for (size_t k = batch.size(); k-- > got;) {
      SrvReq* q = batch[k];
      so->pool_used -= q->bytes;
      q->st.deferred++;
      so->pending.push_front(q);
    }
    batch.resize(got);
    if (batch.empty()) {
      SrvReq* head = so->pending.front();
      if (!any_busy && ++head->idle_alloc_failures >= kMaxIdleAllocFailures) {
        so->pending.pop_front();
        head->st.status = HSR_ERR_OUT_OF_MEMORY;
        head->st.done_ms = so->now();
        so->cv_done.notify_all();
        return true;
      }
      return false;  // retried when a batch completes or after the scheduler's poll interval
    }
  }
  s.reqs = batch;
  s.batch = so->next_batch++;
  const double t = so->now();
  s.descs.clear();
  int rc = HSR_OK;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_rt) rc = HSR_ERR_NOT_INITIALIZED;
    for (SrvReq* q : batch) {
      if (rc != HSR_OK) break;
      if (!q->mem) { rc = HSR_ERR_OUT_OF_MEMORY; break; }
      const size_t main_bytes = 3 * plane_bytes(q->r.width, q->r.height);
      TargetObj* tm = make_pooled_target(q->mem, q->r.width, q->r.height);
      q->h_main = g_rt->next_handle++;
      g_rt->targets[q->h_main] = tm;
      hsr_target shadow = 0;
      if (q->r.shadow_size > 0) {
        TargetObj* ts = make_pooled_target(q->mem + main_bytes, q->r.shadow_size, q->r.shadow_size);
        q->h_shadow = g_rt->next_handle++;
        g_rt->targets[q->h_shadow] = ts;
        shadow = q->h_shadow;
        hsr_draw_desc d;
        std::memset(&d, 0, sizeof(d));
        d.mesh = q->r.mesh;
        d.shader = HSR_SHADER_SHADOW;
        d.flags = HSR_DRAW_CLEAR;
        d.diffuse = q->r.diffuse;
        d.normal = q->r.normal;
        d.target = shadow;
        d.uniforms = &q->r.uniforms;
        d.clear_depth = q->r.shadow_clear_depth;
        std::memcpy(d.clear_rgba, q->r.shadow_clear_rgba, 4);
        s.descs.push_back(d);
      }
      hsr_draw_desc d;
      std::memset(&d, 0, sizeof(d));
      d.mesh = q->r.mesh;
      d.shader = q->r.shader;
      d.flags = HSR_DRAW_CLEAR;
      d.diffuse = q->r.diffuse;
      d.normal = q->r.normal;
      d.target = q->h_main;
      d.shadow_map = shadow;
      d.uniforms = &q->r.uniforms;
      d.clear_depth = q->r.clear_depth;
      std::memcpy(d.clear_rgba, q->r.clear_rgba, 4);
      s.descs.push_back(d);
    }
    if (rc == HSR_OK) rc = g_rt->plan_build(s.descs.data(), (int)s.descs.size(), s.plan);
  }
  for (SrvReq* q : batch) {
    q->st.launch_ms = t;
    q->st.batch = s.batch;
    q->st.batch_requests = (uint32_t)batch.size();
  }
  s.busy = true;
  if (rc == HSR_OK) rc = slot_enqueue(so, s);
  if (rc != HSR_OK) {
    cudaStreamSynchronize(so->compute);
    cudaStreamSynchronize(s.stream);
    finish(so, s, rc);
  }
  return true;
}

static void complete_if_done(ServerObj* so, Slot& s) {
  if (!s.busy || cudaEventQuery(s.done) != cudaSuccess) return;
  const Ctl c = *(const Ctl*)(s.plan.host + s.plan.host_bytes);
  if (s.plan.grow(c)) {  // nothing was drawn: re-run the same batch with larger scratch
    {
      std::lock_guard<std::mutex> lk(g_mu);
      if (g_rt) {
        g_rt->stats.retries++;
        g_rt->learn_caps(s.plan);  // later batches start from these capacities
      }
    }
    int rc = slot_enqueue(so, s);
    if (rc != HSR_OK) {
      cudaStreamSynchronize(so->compute);
      cudaStreamSynchronize(s.stream);
      finish(so, s, rc);
    }
    return;
  }
  finish(so, s, (c.error & (kErrWaitTimeout | kErrScanTimeout)) ? HSR_ERR_TIMEOUT : HSR_OK);
}

static void scheduler(ServerObj* so) {
  cudaSetDevice(so->device);
  for (;;) {
    bool progress = false;
    for (Slot& s : so->slots) {
      const bool was = s.busy;
      complete_if_done(so, s);
      progress |= was && !s.busy;
    }
    for (Slot& s : so->slots)
      if (!s.busy) progress |= try_launch(so, s);
    std::unique_lock<std::mutex> lk(so->mu);
    bool any_busy = false;
    for (Slot& s : so->slots) any_busy |= s.busy;
    if (so->stop && !any_busy) break;
    if (!progress) {
      // nothing changed: sleep until a submission arrives or a short poll interval passes
      so->cv_work.wait_for(lk, std::chrono::microseconds(any_busy ? 20 : 2000));
    }
  }
}

}  // namespace hsr

using namespace hsr;

#define RT_LOCK()                                                                   \
  std::lock_guard<std::mutex> lock_(g_mu);                                          \
  if (!g_rt) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init() has not succeeded")

extern "C" {

int hsr_plan_create(const hsr_draw_desc* descs, int32_t n, hsr_plan* out) {
  RT_LOCK();
  if (!descs || n <= 0 || !out) return fail(HSR_ERR_INVALID_ARG, "plan_create: bad arguments");
  if (first_reclear(descs, n) < n)
    return fail(HSR_ERR_INVALID_ARG, "plan_create: a draw clears a target an earlier draw of the plan writes "
                                     "(one plan is one launch sequence: make two plans)");
  PlanObj* po = new PlanObj();
  po->descs.assign(descs, descs + n);
  po->uniforms.resize(n);
  for (int i = 0; i < n; i++) {
    if (!descs[i].uniforms) { delete po; return fail(HSR_ERR_INVALID_ARG, "plan_create: uniforms is null"); }
    po->uniforms[i] = *descs[i].uniforms;
    po->descs[i].uniforms = &po->uniforms[i];
  }
  int rc = g_rt->plan_build(po->descs.data(), n, po->p);
  if (rc == HSR_OK) rc = plan_bind_and_record(g_rt, po);
  if (rc != HSR_OK) { delete po; return rc; }
  const uint64_t h = g_next_obj++;
  g_plans[h] = po;
  *out = h;
  return HSR_OK;
}

int hsr_plan_set_uniforms(hsr_plan plan, int32_t draw, const hsr_shader_data* u) {
  RT_LOCK();
  auto it = g_plans.find(plan);
  if (it == g_plans.end()) return fail(HSR_ERR_BAD_HANDLE, "plan_set_uniforms: unknown plan");
  PlanObj* po = it->second;
  if (!u || draw < 0 || draw >= (int)po->descs.size()) return fail(HSR_ERR_INVALID_ARG, "plan_set_uniforms: bad draw");
  int rc = plan_wait(g_rt, po);  // the staging must not change under a running replay
  if (rc != HSR_OK) return rc;
  po->uniforms[draw] = *u;
  for (int k = 0; k < po->p.n; k++)
    if (po->p.order[k] == draw) plan_refresh_view(po, k);
  return HSR_OK;
}

int hsr_plan_launch(hsr_plan plan) {
  RT_LOCK();
  auto it = g_plans.find(plan);
  if (it == g_plans.end()) return fail(HSR_ERR_BAD_HANDLE, "plan_launch: unknown plan");
  PlanObj* po = it->second;
  for (const hsr_draw_desc& d : po->descs)  // meshes, textures and targets must outlive the plan
    if (g_rt->validate(d) != HSR_OK) return fail(HSR_ERR_BAD_HANDLE, "plan_launch: a handle of the plan was released");
  int rc = plan_wait(g_rt, po);
  if (rc != HSR_OK) return rc;
  cudaError_t e = cudaGraphLaunch(po->exec, g_rt->stream);
  if (e != cudaSuccess) return cuda_fail(e, "plan_launch");
  po->in_flight = true;
  g_rt->launches += (uint64_t)po->p.kernel_count();
  return HSR_OK;
}

int hsr_plan_wait(hsr_plan plan) {
  RT_LOCK();
  auto it = g_plans.find(plan);
  if (it == g_plans.end()) return fail(HSR_ERR_BAD_HANDLE, "plan_wait: unknown plan");
  return plan_wait(g_rt, it->second);
}

int hsr_plan_release(hsr_plan plan) {
  RT_LOCK();
  auto it = g_plans.find(plan);
  if (it == g_plans.end()) return fail(HSR_ERR_BAD_HANDLE, "plan_release: unknown plan");
  cudaStreamSynchronize(g_rt->stream);
  delete it->second;
  g_plans.erase(it);
  return HSR_OK;
}

int hsr_server_create(const hsr_server_config* cfg, hsr_server* out) {
  ServerObj* so = nullptr;
  {
    RT_LOCK();
    if (!cfg || !out || cfg->max_batch < 1 || cfg->slots < 1 || cfg->slots > 16 || cfg->pool_bytes == 0)
      return fail(HSR_ERR_INVALID_ARG, "server_create: bad configuration");
    so = new ServerObj();
    so->cfg = *cfg;
    so->device = g_rt->device;
    so->num_sms = g_rt->num_sms;
    so->tuning = g_rt->tuning;
    so->t0 = std::chrono::steady_clock::now();
    so->slots.resize(cfg->slots);
    bool ok = cudaStreamCreateWithFlags(&so->compute, cudaStreamNonBlocking) == cudaSuccess;
    for (Slot& s : so->slots)
      ok = ok && cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) == cudaSuccess &&
           cudaEventCreateWithFlags(&s.kdone, cudaEventDisableTiming) == cudaSuccess &&
           cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      for (Slot& s : so->slots) {
        if (s.done) cudaEventDestroy(s.done);
        if (s.kdone) cudaEventDestroy(s.kdone);
        if (s.stream) cudaStreamDestroy(s.stream);
      }
      if (so->compute) cudaStreamDestroy(so->compute);
      delete so;
      return fail(HSR_ERR_CUDA, "server_create: stream / event creation failed");
    }
    const uint64_t h = g_next_obj++;
    g_servers[h] = so;
    *out = h;
  }
  so->th = std::thread(scheduler, so);
  return HSR_OK;
}

static ServerObj* server_of(hsr_server s) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_servers.find(s);
  return it == g_servers.end() ? nullptr : it->second;
}

int hsr_server_submit(hsr_server s, const hsr_request* req, uint64_t* ticket) {
  ServerObj* so = server_of(s);
  if (!so) return fail(HSR_ERR_BAD_HANDLE, "server_submit: unknown server");
  if (!req || !ticket) return fail(HSR_ERR_INVALID_ARG, "server_submit: null argument");
  if (req->width <= 0 || req->height <= 0 || req->width > 32768 || req->height > 32768 || req->shadow_size < 0 ||
      req->shadow_size > 32768)
    return fail(HSR_ERR_INVALID_ARG, "server_submit: bad target size");
  if (req->shader < 0 || req->shader >= HSR_SHADER_COUNT) return fail(HSR_ERR_UNKNOWN_SHADER, "server_submit: unknown shader");
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_rt || !g_rt->mesh(req->mesh)) return fail(HSR_ERR_BAD_HANDLE, "server_submit: unknown mesh");
    if ((req->diffuse && !g_rt->tex(req->diffuse)) || (req->normal && !g_rt->tex(req->normal)))
      return fail(HSR_ERR_BAD_HANDLE, "server_submit: unknown texture");
  }
  SrvReq* q = new SrvReq();
  q->r = *req;
  q->bytes = req_bytes(*req);
  std::memset(&q->st, 0, sizeof(q->st));
  q->st.status = HSR_ERR_BUSY;
  {
    std::lock_guard<std::mutex> lk(so->mu);
    if (so->stop) {
      delete q;
      return fail(HSR_ERR_INVALID_ARG, "server_submit: server is shutting down");
    }
    q->st.submit_ms = so->now();
    *ticket = so->next_ticket++;
    so->reqs[*ticket] = q;
    so->pending.push_back(q);
  }
  so->cv_work.notify_one();
  return HSR_OK;
}

int hsr_server_poll(hsr_server s, uint64_t ticket, hsr_request_status* out) {
  ServerObj* so = server_of(s);
  if (!so) return fail(HSR_ERR_BAD_HANDLE, "server_poll: unknown server");
  std::lock_guard<std::mutex> lk(so->mu);
  auto it = so->reqs.find(ticket);
  if (it == so->reqs.end()) return fail(HSR_ERR_BAD_HANDLE, "server_poll: unknown ticket");
  if (out) *out = it->second->st;
  return it->second->st.status == HSR_ERR_BUSY ? HSR_ERR_BUSY : HSR_OK;
}

int hsr_server_wait(hsr_server s, uint64_t ticket, int32_t timeout_ms, hsr_request_status* out) {
  ServerObj* so = server_of(s);
  if (!so) return fail(HSR_ERR_BAD_HANDLE, "server_wait: unknown server");
  std::unique_lock<std::mutex> lk(so->mu);
  auto it = so->reqs.find(ticket);
  if (it == so->reqs.end()) return fail(HSR_ERR_BAD_HANDLE, "server_wait: unknown ticket");
  SrvReq* q = it->second;
  const bool ok = so->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                       [&] { return q->st.status != HSR_ERR_BUSY; });
  if (out) *out = q->st;
  if (!ok) return fail(HSR_ERR_TIMEOUT, "server_wait: timed out");
  return HSR_OK;
}

int hsr_server_inject_alloc_failures(hsr_server s, int32_t n) {
  ServerObj* so = server_of(s);
  if (!so) return fail(HSR_ERR_BAD_HANDLE, "server_inject_alloc_failures: unknown server");
  if (n < 0) return fail(HSR_ERR_INVALID_ARG, "server_inject_alloc_failures: n must be >= 0");
  std::lock_guard<std::mutex> lk(so->mu);
  so->inject_alloc_failures = n;
  return HSR_OK;
}

int hsr_server_now_ms(hsr_server s, double* out) {
  ServerObj* so = server_of(s);
  if (!so || !out) return fail(HSR_ERR_BAD_HANDLE, "server_now_ms: unknown server");
  *out = so->now();
  return HSR_OK;
}

int hsr_server_destroy(hsr_server s) {
  ServerObj* so = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_servers.find(s);
    if (it == g_servers.end()) return fail(HSR_ERR_BAD_HANDLE, "server_destroy: unknown server");
    so = it->second;
    g_servers.erase(it);
  }
  {
    std::lock_guard<std::mutex> lk(so->mu);
    so->stop = true;
    for (SrvReq* q : so->pending) {  // queued, never launched
      q->st.status = HSR_ERR_INVALID_ARG;
      q->st.done_ms = so->now();
    }
    so->pending.clear();
  }
  so->cv_work.notify_all();
  if (so->th.joinable()) so->th.join();
  if (so->dev) cudaFreeAsync(so->dev, so->compute);  // back to the stream-ordered pool
  for (Slot& sl : so->slots) {
    cudaStreamSynchronize(sl.stream);
    if (sl.host) cudaFreeHost(sl.host);
    cudaEventDestroy(sl.done);
    cudaEventDestroy(sl.kdone);
    cudaStreamDestroy(sl.stream);
  }
  cudaStreamSynchronize(so->compute);
  cudaStreamDestroy(so->compute);
  for (auto& kv : so->reqs) delete kv.second;
  delete so;
  return HSR_OK;
}

}  // extern "C"

namespace hsr {
// Called by hsr_shutdown before it takes the runtime lock: servers join their scheduler
// threads (which take that lock), plans free their graphs and scratch.
void serve_shutdown() {
  std::vector<uint64_t> hs;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& kv : g_servers) hs.push_back(kv.first);
  }
  for (uint64_t h : hs) hsr_server_destroy(h);
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_rt) cudaStreamSynchronize(g_rt->stream);
  for (auto& kv : g_plans) delete kv.second;
  g_plans.clear();
}
}  // namespace hsr
