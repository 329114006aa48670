// hsr_runtime.cu — host runtime and C ABI (include/hsr.h).
//
// Replaces graphics_draw_triangle(DrawData*) (graphics.h:15, graphics.cpp:378-407) by
// handle-based calls.  Meshes, textures and targets live in device memory; hsr_draw_batch
// turns a list of draws into one launch sequence of eight kernels (vertex, cull, emit, clip,
// split, scan, scatter, raster) over all of them, or into several in array order where a draw
// clears a target an earlier draw of the list writes.  Scratch is a grow-only arena; an
// overflow detected on the device
// leaves the targets untouched (the raster checks the error word first) and the batch is
// re-run with larger capacity.  No CPU fallback exists: without a device every call
// fails with a status code.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "hsr_internal.h"
#include "hsr_runtime.h"

namespace hsr {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return HSR_ERR_CUDA;
}

Runtime* g_rt = nullptr;
std::mutex g_mu;

// ---- small helpers --------------------------------------------------------------------
static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Matrix product in the reference's order: out[i][j] = a[i] . col_j(b), accumulated from
// index 3 down (matrix.h:118-123, vector.h:69-73).  Host code is built without FP
// contraction, so these are plain IEEE single-precision operations.
void mat_mul_ref(const float* a, const float* b, float* out) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      float r = 0.f;
      for (int k = 3; k >= 0; k--) {
        float p = a[i * 4 + k] * b[k * 4 + j];
        r = r + p;
      }
      out[i * 4 + j] = r;
    }
}

// ---- device buffers ---------------------------------------------------------------------
static int dalloc(void** p, size_t bytes, const char* what) {
  *p = nullptr;
  if (bytes == 0) return HSR_OK;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(HSR_ERR_OUT_OF_MEMORY, std::string("cudaMalloc failed for ") + what + ": " + cudaGetErrorString(e));
  }
  return HSR_OK;
}

MeshObj::~MeshObj() {
  for (void* p : {(void*)px, (void*)py, (void*)pz, (void*)nx, (void*)ny, (void*)nz, (void*)p4, (void*)n4, (void*)pk,
                  (void*)uv, (void*)fv, (void*)fvt, (void*)fvn})
    if (p) cudaFree(p);
}
TexObj::~TexObj() {
  if (words) cudaFree(words);
}
TargetObj::~TargetObj() {
  if (pooled || !block) return;
  cudaFreeAsync(block, stream);
}

int Arena::reserve(size_t bytes) {
  if (bytes <= cap) return HSR_OK;
  const size_t want = std::max(bytes, cap + cap / 2);
  if (base) cudaFree(base);
  base = nullptr;
  cap = 0;
  int rc = dalloc((void**)&base, want, "scratch arena");
  if (rc != HSR_OK) return rc;
  cap = want;
  return HSR_OK;
}

int Pinned::reserve(size_t bytes) {
  if (bytes <= cap) return HSR_OK;
  const size_t want = std::max({bytes, cap + cap / 2, (size_t)1 << 16});
  if (base) cudaFreeHost(base);
  base = nullptr;
  cap = 0;
  cudaError_t e = cudaMallocHost((void**)&base, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(HSR_ERR_OUT_OF_MEMORY, "cudaMallocHost failed");
  }
  cap = want;
  return HSR_OK;
}

template <class T> T* Runtime::get(std::unordered_map<uint64_t, T*>& m, uint64_t h) {
  auto it = m.find(h);
  return it == m.end() ? nullptr : it->second;
}

MeshObj* Runtime::mesh(uint64_t h) { return get(meshes, h); }
TexObj* Runtime::tex(uint64_t h) { return get(textures, h); }
TargetObj* Runtime::target(uint64_t h) { return get(targets, h); }

// ---- batch planning -----------------------------------------------------------------------
int Runtime::validate(const hsr_draw_desc& d) {
  if (!d.uniforms) return fail(HSR_ERR_INVALID_ARG, "draw: uniforms is null");
  if (d.shader < 0 || d.shader >= HSR_SHADER_COUNT) return fail(HSR_ERR_UNKNOWN_SHADER, "draw: unknown shader kind");
  if (!mesh(d.mesh)) return fail(HSR_ERR_BAD_HANDLE, "draw: unknown mesh handle");
  if (!target(d.target)) return fail(HSR_ERR_BAD_HANDLE, "draw: unknown target handle");
  if (d.diffuse && !tex(d.diffuse)) return fail(HSR_ERR_BAD_HANDLE, "draw: unknown diffuse texture handle");
  if (d.normal && !tex(d.normal)) return fail(HSR_ERR_BAD_HANDLE, "draw: unknown normal texture handle");
  if (d.shadow_map && !target(d.shadow_map)) return fail(HSR_ERR_BAD_HANDLE, "draw: unknown shadow_map handle");
  if (d.shadow_map && d.shadow_map == d.target) return fail(HSR_ERR_INVALID_ARG, "draw: shadow_map is the target itself");
  return HSR_OK;
}

// Order the draws: a consumer of a shadow map waits for the draw that renders it; draws into
// one target keep their array order.  Returns levels via topological order.
int Runtime::plan_order(const hsr_draw_desc* d, int n, std::vector<int>& order, std::vector<int>& dep0,
                        std::vector<int>& dep1) {
  dep0.assign(n, -1);
  dep1.assign(n, -1);
  for (int i = 0; i < n; i++) {
    if (d[i].shadow_map) {
      for (int j = n - 1; j >= 0; j--)
        if (j != i && d[j].target == d[i].shadow_map) { dep0[i] = j; break; }
    }
    for (int j = i - 1; j >= 0; j--)
      if (d[j].target == d[i].target) { dep1[i] = j; break; }
  }
  std::vector<int> level(n, -1);
  // longest-path levels with cycle detection (n is small)
  for (int iter = 0; iter <= n; iter++) {
    bool changed = false;
    for (int i = 0; i < n; i++) {
      int l = 0;
      for (int dp : {dep0[i], dep1[i]})
        if (dp >= 0) l = std::max(l, level[dp] < 0 ? 1 : level[dp] + 1);
      if (l != level[i]) { level[i] = l; changed = true; }
    }
    if (!changed) break;
    if (iter == n) return fail(HSR_ERR_INVALID_ARG, "draw batch: circular shadow-map / target dependencies");
  }
  order.resize(n);
  for (int i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return level[a] < level[b]; });
  return HSR_OK;
}

int Runtime::plan_build(const hsr_draw_desc* descs, int n, Plan& p) {
  for (int i = 0; i < n; i++) {
    int rc = validate(descs[i]);
    if (rc != HSR_OK) return rc;
  }
  std::vector<int> order, dep0, dep1;
  int rc = plan_order(descs, n, order, dep0, dep1);
  if (rc != HSR_OK) return rc;
  std::vector<int> pos(n);
  for (int k = 0; k < n; k++) pos[order[k]] = k;

  const int T = tuning.tile;
  p = Plan();
  p.n = n;
  p.tile = T;
  p.stash_warps = T >= 16 ? (uint32_t)num_sms * kStashWarpsPerSm : 0u;  // 8x8 tiles keep theirs in shared memory
  p.views.resize(n);
  p.offs.resize(n);
  p.order = order;
  size_t bytes = 0;
  for (int k = 0; k < n; k++) {
    const hsr_draw_desc& d = descs[order[k]];
    MeshObj* m = mesh(d.mesh);
    TargetObj* tg = target(d.target);
    DView& v = p.views[k];
    std::memset(&v, 0, sizeof(v));
    v.px = m->px; v.py = m->py; v.pz = m->pz;
    v.nx = m->nx; v.ny = m->ny; v.nz = m->nz;
    v.p4 = m->p4; v.n4 = m->n4; v.pk = m->pk;
    v.world = world_attrs(d.shader);
    v.uv = m->uv;
    v.fv = m->fv; v.fvt = m->fvt; v.fvn = m->fvn;
    v.npos = m->npos; v.nnrm = m->nnrm; v.nuv = m->nuv; v.nfaces = m->nfaces;
    v.unified = m->unified ? 1 : 0;
    v.shader = d.shader;
    v.flags = d.flags;
    v.u = *d.uniforms;
    mat_mul_ref(d.shader == HSR_SHADER_SHADOW ? v.u.light_vp_matrix : v.u.camera_vp_matrix, v.u.model_matrix, v.mvp);
    if (d.diffuse) {
      TexObj* t = tex(d.diffuse);
      v.diffuse = t->words; v.dw = t->w; v.dh = t->h; v.dbpp = t->bpp;
    }
    if (d.normal) {
      TexObj* t = tex(d.normal);
      v.normal = t->words; v.nw = t->w; v.nh = t->h; v.nbpp = t->bpp;
    }
    v.color = tg->color; v.depth = tg->depth; v.prim = tg->prim; v.W = tg->w; v.H = tg->h;
    if (d.shadow_map) {
      TargetObj* sm = target(d.shadow_map);
      v.sm_color = sm->color; v.smW = sm->w; v.smH = sm->h;
    }
    v.dep0 = dep0[order[k]] >= 0 ? pos[dep0[order[k]]] : -1;
    v.dep1 = dep1[order[k]] >= 0 ? pos[dep1[order[k]]] : -1;
    v.tiles_x = (tg->w + T - 1) / T;
    v.tiles_y = (tg->h + T - 1) / T;
    v.ntiles = v.tiles_x * v.tiles_y;
    v.tile_base = (int32_t)p.total_tiles;
    v.prim_base = d.prim_base;
    v.clear_depth = d.clear_depth;
    std::memcpy(&v.clear_rgba, d.clear_rgba, 4);
    p.total_tiles += (size_t)v.ntiles;
    p.total_faces += (size_t)m->nfaces;
    p.total_pos += (size_t)m->npos;
    p.total_pixels += (size_t)tg->w * (size_t)tg->h;
    Plan::Off& o = p.offs[k];
    o.clip = bytes; bytes = align_up(bytes + sizeof(float4) * (size_t)std::max(m->npos, 1), 256);
    v.vch_base = p.nvch;
    v.vch_npos = (m->npos + kVertexChunk - 1) / kVertexChunk;
    v.vch_count = v.vch_npos;
    v.sch_base = p.nsch;
    v.cch_base = p.ncch;
    p.nvch += v.vch_count;
    p.nsch += (m->nfaces + kSetupChunk - 1) / kSetupChunk;
    if (d.flags & HSR_DRAW_CLEAR) p.ncch += (int)(((size_t)tg->w * (size_t)tg->h + kClearChunk - 1) / kClearChunk);
  }
  for (int k = 0; k < n; k++) {
    if (p.views[k].dep0 >= 0) p.views[p.views[k].dep0].has_dependents = 1;
    if (p.views[k].dep1 >= 0) p.views[p.views[k].dep1].has_dependents = 1;
  }
  if (p.total_tiles >= (size_t)kMaxBatchTiles)
    return fail(HSR_ERR_INVALID_ARG, "draw batch: too many tiles for one launch sequence (2^26)");
  p.view_bytes = bytes;
  p.rec_cap = std::max<size_t>(cap_rec_hint, p.total_faces + p.total_faces / 4 + 1024);
  p.clip_cap = std::max<size_t>(cap_clip_hint, p.total_faces / 16 + 256);
  p.big_cap = std::max<size_t>(cap_big_hint, p.total_faces / 64 + 256);
  p.bin_cap = std::max<size_t>(cap_bin_hint,
                               (size_t)(tuning.bin_factor * (double)(p.total_faces + p.total_tiles)) + 4096);
  return HSR_OK;
}

void Plan::layout() {
  rec_cap = std::min<size_t>(rec_cap, 0xfffff000u);
  clip_cap = std::min<size_t>(clip_cap, 0xfffff000u);
  big_cap = std::min<size_t>(big_cap, 0xfffff000u);
  bin_cap = std::min<size_t>(bin_cap, 0xfffff000u);
  nscan = scan_blocks((int)total_tiles);
  // [views | chunks | per-view vertex outputs | ctl | view_done | tile_count | tile_fill |
  //  scan_status | tile_off | ne_off | tile_list | recs | clipbuf | bins]; the zeroed part is one memset
  size_t off = 0;
  o_views = off; off = align_up(off + sizeof(DView) * n, 256);
  host_bytes = off;
  o_vout = off; off = align_up(off + view_bytes, 256);
  o_zero = off;
  o_ctl = off; off = align_up(off + sizeof(Ctl), 256);
  o_done = off; off = align_up(off + sizeof(uint32_t) * n, 256);
  o_cnt = off; off = align_up(off + sizeof(uint32_t) * total_tiles, 256);
  o_fill = off; off = align_up(off + sizeof(uint32_t) * total_tiles, 256);
  o_stat = off; off = align_up(off + sizeof(unsigned long long) * std::max(nscan, 1), 256);
  zero_bytes = off - o_zero;
  o_toff = off; off = align_up(off + sizeof(uint32_t) * total_tiles, 256);
  o_neoff = off; off = align_up(off + sizeof(uint32_t) * (total_tiles + 1), 256);
  o_list = off; off = align_up(off + sizeof(uint32_t) * total_tiles, 256);
  o_recs = off; off = align_up(off + sizeof(RasterRec) * rec_cap, 256);
  o_pay = off; off = align_up(off + sizeof(Payload) * rec_cap, 256);
  o_clip = off; off = align_up(off + sizeof(int2) * clip_cap, 256);
  o_big = off; off = align_up(off + sizeof(BigItem) * big_cap, 256);
  o_bins = off; off = align_up(off + sizeof(uint32_t) * bin_cap, 256);
  o_stash = off; off = align_up(off + sizeof(float) * (size_t)stash_floats(tile) * (size_t)stash_warps, 256);
  dev_bytes = off;
  stage_bytes = host_bytes + sizeof(Ctl);
}

void Plan::bind(char* dev_base, char* host_base) {
  dev = dev_base;
  host = host_base;
  for (int k = 0; k < n; k++) {
    DView& v = views[k];
    v.sv = (float4*)(dev + o_vout + offs[k].clip);
  }
  std::memcpy(host + o_views, views.data(), sizeof(DView) * n);
  sc.ctl = (Ctl*)(dev + o_ctl);
  sc.view_done = (uint32_t*)(dev + o_done);
  sc.recs = (RasterRec*)(dev + o_recs); sc.rec_cap = (uint32_t)rec_cap;
  sc.pay = (Payload*)(dev + o_pay);
  sc.clipq = (int2*)(dev + o_clip); sc.clip_cap = (uint32_t)clip_cap;
  sc.bigq = (BigItem*)(dev + o_big); sc.big_cap = (uint32_t)big_cap;
  sc.tile_count = (uint32_t*)(dev + o_cnt);
  sc.tile_fill = (uint32_t*)(dev + o_fill);
  sc.tile_off = (uint32_t*)(dev + o_toff);
  sc.ne_off = (uint32_t*)(dev + o_neoff);
  sc.tile_list = (uint32_t*)(dev + o_list);
  sc.scan_status = (unsigned long long*)(dev + o_stat);
  sc.bins = (uint32_t*)(dev + o_bins); sc.bin_cap = (uint32_t)bin_cap;
  sc.ntiles = (int32_t)total_tiles;
  sc.nviews = n;
  sc.stash = stash_warps ? (float*)(dev + o_stash) : nullptr;
  sc.stash_warps = stash_warps;
}

// Upload of the view descriptors, one memset, the kernels, read-back of the control
// block: everything stream-ordered, nothing synchronous (capturable into a CUDA graph).
// `ev` (may be null) holds Runtime::kEvents events: [0] before the upload and [kEvents-1]
// after the raster are recorded whenever `ev` is given; [1] after the memset and [2+k]
// after kernel k only where non-null (profiling).
int Plan::enqueue(cudaStream_t s, int num_sms, const hsr_tuning& tu, cudaEvent_t* ev) {
  const DView* dviews = (const DView*)(dev + o_views);
  auto mark = [&](int k) {
    if (ev && ev[k]) cudaEventRecord(ev[k], s);
  };
  mark(0);
  cudaError_t e = cudaMemcpyAsync(dev, host, host_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "upload views");
  e = cudaMemsetAsync(dev + o_zero, 0, zero_bytes, s);
  if (e != cudaSuccess) return cuda_fail(e, "clear scratch");
  mark(1);
  int kr = launch_vertex(dviews, n, nvch, num_sms * 8, s);
  if (kr) return cuda_fail((cudaError_t)kr, "vertex kernel");
  mark(2);
  kr = launch_setup(dviews, n, nsch, sc, num_sms * 8, s);
  if (kr) return cuda_fail((cudaError_t)kr, "setup kernel");
  mark(3);
  kr = launch_emit(dviews, tile, sc, num_sms * 8, s);
  if (kr) return cuda_fail((cudaError_t)kr, "emit kernel");
  mark(4);
  kr = launch_post(dviews, tile, sc, num_sms * 4, s);
  if (kr) return cuda_fail((cudaError_t)kr, "post kernel");
  mark(5);
  kr = launch_big(dviews, tile, sc, num_sms * 2, s);
  if (kr) return cuda_fail((cudaError_t)kr, "big-triangle kernel");
  mark(6);
  kr = launch_scan(sc, s);
  if (kr) return cuda_fail((cudaError_t)kr, "scan kernel");
  mark(7);
  // grid-stride over the records: one full wave of 256-thread blocks (fewer when there are
  // few records and nothing to clear), not one sized by the capacity (which can be far
  // above this batch's record count)
  const size_t want = ncch ? (size_t)num_sms * 8 : std::min<size_t>((rec_cap + 255) / 256, (size_t)num_sms * 8);
  kr = launch_scatter(dviews, tile, sc, (int)std::max<size_t>(want, 1), ncch, s);
  if (kr) return cuda_fail((cudaError_t)kr, "scatter kernel");
  mark(8);
  kr = launch_raster(dviews, tile, sc, num_sms * tu.ctas_per_sm, tu.warps_per_cta, s);
  if (kr) return cuda_fail((cudaError_t)kr, "raster kernel");
  mark(9);
  e = cudaMemcpyAsync(host + host_bytes, sc.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return cuda_fail(e, "read control block");
  return HSR_OK;
}

int Plan::kernel_count() const {
  return (nvch ? 1 : 0) + (nsch ? 1 : 0) + 3 + (nscan > 0 ? 1 : 0) + 2;
}

// Grow the capacity an overflow reported; returns false if nothing overflowed.
bool Plan::grow(const Ctl& c) {
  if (!(c.error & kErrCapacity)) return false;
  if (c.error & kErrBigOverflow) big_cap = std::max<size_t>(big_cap * 2, (size_t)c.big_count + 256);
  if (c.error & kErrRecOverflow) rec_cap = std::max<size_t>(rec_cap * 2, (size_t)c.rec_count + 1024);
  if (c.error & kErrClipOverflow) clip_cap = std::max<size_t>(clip_cap * 2, (size_t)c.clip_count + 256);
  if (c.error & kErrBinOverflow) bin_cap = std::max<size_t>(bin_cap * 2, (size_t)c.bin_total + 4096);
  return true;
}

void Runtime::learn_caps(const Plan& p) {
  cap_rec_hint = std::max(cap_rec_hint, p.rec_cap);
  cap_clip_hint = std::max(cap_clip_hint, p.clip_cap);
  cap_bin_hint = std::max(cap_bin_hint, p.bin_cap);
  cap_big_hint = std::max(cap_big_hint, p.big_cap);
}

void Runtime::record_result(const Plan& p, const Ctl& c) {
  stats.records = c.rec_count;
  stats.clipped_faces = c.clip_count;
  stats.bin_pairs = c.bin_total;
  stats.tiles = p.total_tiles;
  timing.records = c.rec_count;
  timing.bin_pairs = c.bin_total;
  timing.shaded_pixels = c.shaded_px;
  timing.fragments = c.frag_px;
  timing.raster_pixels = std::min<uint64_t>((uint64_t)c.ne_tiles * (uint64_t)p.tile * (uint64_t)p.tile, p.total_pixels);
  timing.pixels = p.total_pixels;
  timing.faces = p.total_faces;
  timing.vertices = p.total_pos;
  timing.normals = p.total_nrm;
  timing.clipped_faces = c.clip_count;
  timing.launches = (uint32_t)p.kernel_count();
  timing.h2d_bytes = p.host_bytes;
  timing.d2h_bytes = sizeof(Ctl);
  timing.views = (uint32_t)p.n;
  timing.tiles = p.total_tiles;
  timing.split_triangles = c.big_count;
  timing.payload_bytes = c.pay_bytes;
}

// Index of the first draw that clears a target an earlier draw of the batch writes (n if none).
// Within one launch sequence the fused clears of all views land before any view is rasterised
// (empty tiles in the scatter grid), so such a clear cannot follow the earlier draw's pixels there.
int first_reclear(const hsr_draw_desc* d, int n) {
  for (int i = 1; i < n; i++)
    if (d[i].flags & HSR_DRAW_CLEAR)
      for (int j = 0; j < i; j++)
        if (d[j].target == d[i].target) return i;
  return n;
}

// A batch runs as one launch sequence, or as several in array order where a draw clears a
// target that an earlier draw of the batch writes (the sequential semantics of the calls).
int Runtime::run_batch(const hsr_draw_desc* descs, int n) {
  while (n > 0) {
    const int k = first_reclear(descs, n);
    const int rc = run_sequence(descs, k);
    if (rc != HSR_OK) return rc;
    descs += k;
    n -= k;
  }
  return HSR_OK;
}

int Runtime::run_sequence(const hsr_draw_desc* descs, int n) {
  if (n <= 0) return HSR_OK;
  Plan p;
  int rc = plan_build(descs, n, p);
  if (rc != HSR_OK) return rc;
  for (int attempt = 0; attempt < 6; attempt++) {
    p.layout();
    rc = arena.reserve(p.dev_bytes);
    if (rc != HSR_OK) return rc;
    rc = staging.reserve(p.stage_bytes);
    if (rc != HSR_OK) return rc;
    p.bind(arena.base, staging.base);
    p.sc.faults = faults;
    p.sc.poll_limit = poll_limit;
    cudaEvent_t evs[kEvents];
    for (int k = 0; k < kEvents; k++) evs[k] = (k == 0 || k == kEvents - 1 || profiling) ? ev[k] : nullptr;
    rc = p.enqueue(stream, num_sms, tuning, evs);
    if (rc != HSR_OK) return rc;
    launches += (uint64_t)p.kernel_count();
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "draw batch");
    const Ctl c = *(const Ctl*)(p.host + p.host_bytes);
    if (p.grow(c)) {
      stats.retries++;
      learn_caps(p);
      continue;
    }
    if (c.error & (kErrWaitTimeout | kErrScanTimeout))
      return fail(HSR_ERR_TIMEOUT, "draw batch: a bounded device wait gave up");
    record_result(p, c);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[kEvents - 1]);
    timing.batch_ms = ms;
    for (int k = 0; k < HSR_KERNEL_COUNT; k++) {
      float km = 0.f;
      if (profiling) cudaEventElapsedTime(&km, ev[k + 1], ev[k + 2]);
      timing.kernel_ms[k] = km;
    }
    return HSR_OK;
  }
  return fail(HSR_ERR_BIN_OVERFLOW, "draw batch: scratch overflow persisted after retries");
}

// The packed vertex of a mesh whose corners index positions, normals and uvs alike: vertex i
// as (x, y, z, nx), (ny, nz, u, v) from the position, normal and uv arrays (zeros where an
// array is shorter), so a corner's attributes are one 32-byte sector.
__global__ void k_pack_vertices(float4* __restrict__ pk, const float4* __restrict__ p4, const float4* __restrict__ n4,
                                const float2* __restrict__ uv, int npos, int nnrm, int nuv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npos; i += gridDim.x * blockDim.x) {
    const float4 p = p4[i];
    const float4 n = i < nnrm ? n4[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 t = i < nuv ? uv[i] : make_float2(0.f, 0.f);
    pk[2 * i] = make_float4(p.x, p.y, p.z, n.x);
    pk[2 * i + 1] = make_float4(n.y, n.z, t.x, t.y);
  }
}

int launch_pack_vertices(float4* pk, const float4* p4, const float4* n4, const float2* uv, int npos, int nnrm, int nuv,
                         cudaStream_t s) {
  if (npos <= 0) return 0;
  k_pack_vertices<<<std::min((npos + 255) / 256, 4096), 256, 0, s>>>(pk, p4, n4, uv, npos, nnrm, nuv);
  return (int)cudaGetLastError();
}

// renderbuffer_clear_color / renderbuffer_clear_depth (renderbuffer.cpp:59-75) with the
// colour given as bytes; prim ids -> 0.
__global__ void k_clear(uint32_t* __restrict__ color, float* __restrict__ depth, uint32_t* __restrict__ prim,
                        size_t n, uint32_t rgba, float d) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    color[i] = rgba;
    depth[i] = d;
    if (prim) prim[i] = 0u;
  }
}

int launch_clear(uint32_t* color, float* depth, uint32_t* prim, size_t n, uint32_t rgba, float d, cudaStream_t s) {
  const int grid = (int)std::min<size_t>((n + 255) / 256, 4096);
  k_clear<<<std::max(grid, 1), 256, 0, s>>>(color, depth, prim, n, rgba, d);
  return (int)cudaGetLastError();
}

int Runtime::clear_target(TargetObj* t, const uint8_t rgba[4], float depth) {
  uint32_t word;
  std::memcpy(&word, rgba, 4);
  int kr = launch_clear(t->color, t->depth, t->prim, (size_t)t->w * (size_t)t->h, word, depth, stream);
  if (kr) return cuda_fail((cudaError_t)kr, "clear kernel");
  launches++;
  cudaError_t e = cudaStreamSynchronize(stream);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "clear");
}

}  // namespace hsr

using namespace hsr;

#define RT_OR_FAIL()                                                                \
  std::lock_guard<std::mutex> lock_(g_mu);                                          \
  if (!g_rt) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init() has not succeeded")

extern "C" {

int hsr_abi_version(void) { return HSR_ABI_VERSION; }

const char* hsr_last_error(void) { return g_last_error.c_str(); }

int hsr_init(int device) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_rt) return HSR_OK;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) {
    cudaGetLastError();
    return fail(HSR_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
  }
  if (device < 0 || device >= count) return fail(HSR_ERR_INVALID_ARG, "hsr_init: device index out of range");
  e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  Runtime* rt = new Runtime();
  rt->device = device;
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, device);
  if (e != cudaSuccess) { delete rt; return cuda_fail(e, "cudaGetDeviceProperties"); }
  rt->num_sms = prop.multiProcessorCount;
  // keep memory freed into the device's stream-ordered pool cached instead of returning it
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  e = cudaStreamCreateWithFlags(&rt->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete rt; return cuda_fail(e, "cudaStreamCreate"); }
  for (int k = 0; k < Runtime::kEvents; k++) {
    e = cudaEventCreate(&rt->ev[k]);
    if (e != cudaSuccess) { delete rt; return cuda_fail(e, "cudaEventCreate"); }
  }
  g_rt = rt;
  return HSR_OK;
}

int hsr_shutdown(void) {
  serve_shutdown();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_rt) return HSR_OK;
  cudaStreamSynchronize(g_rt->stream);
  for (auto& kv : g_rt->meshes) delete kv.second;
  for (auto& kv : g_rt->textures) delete kv.second;
  for (auto& kv : g_rt->targets) delete kv.second;
  if (g_rt->arena.base) cudaFree(g_rt->arena.base);
  if (g_rt->staging.base) cudaFreeHost(g_rt->staging.base);
  for (int k = 0; k < Runtime::kEvents; k++) cudaEventDestroy(g_rt->ev[k]);
  cudaStreamDestroy(g_rt->stream);
  delete g_rt;
  g_rt = nullptr;
  return HSR_OK;
}

// (x, y, z, 0) per item of an xyz array into a device array of max(n, 1) float4s.
static int write_xyz0(const float* src, int32_t n, float4* dst) {
  std::vector<float4> tmp((size_t)std::max(n, 1), make_float4(0.f, 0.f, 0.f, 0.f));
  for (int32_t i = 0; i < n; i++) tmp[i] = make_float4(src[(size_t)i * 3], src[(size_t)i * 3 + 1], src[(size_t)i * 3 + 2], 0.f);
  cudaError_t e = cudaMemcpy(dst, tmp.data(), sizeof(float4) * tmp.size(), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "mesh upload");
}
static int upload_xyz0(const float* src, int32_t n, float4** dst) {
  int rc = dalloc((void**)dst, sizeof(float4) * (size_t)std::max(n, 1), "mesh");
  return rc == HSR_OK ? write_xyz0(src, n, *dst) : rc;
}

int hsr_mesh_upload(const float* pos, int32_t npos, const float* nrm, int32_t nnrm, const float* uv, int32_t nuv,
                    const int32_t* faces, int32_t nfaces, hsr_mesh* out) {
  RT_OR_FAIL();
  if (!out || npos < 0 || nnrm < 0 || nuv < 0 || nfaces < 0) return fail(HSR_ERR_INVALID_ARG, "mesh: bad arguments");
  if (nfaces > (1 << 27)) return fail(HSR_ERR_INVALID_ARG, "mesh: more than 2^27 faces");
  if ((npos && !pos) || (nnrm && !nrm) || (nuv && !uv) || (nfaces && !faces))
    return fail(HSR_ERR_INVALID_ARG, "mesh: null array with nonzero count");
  for (int64_t i = 0; i < (int64_t)nfaces * 3; i++) {
    const int32_t* c = faces + i * 3;
    if (c[0] < 0 || c[0] >= npos || c[1] < 0 || c[1] >= nuv || c[2] < 0 || c[2] >= nnrm)
      return fail(HSR_ERR_INVALID_ARG, "mesh: face index out of range (face " + std::to_string(i / 3) + ")");
  }
  MeshObj* m = new MeshObj();
  m->npos = npos; m->nnrm = nnrm; m->nuv = nuv; m->nfaces = nfaces;
  const size_t P = align_up((size_t)std::max(npos, 1), 4), N = align_up((size_t)std::max(nnrm, 1), 4);
  std::vector<float> tmp(std::max(P, N), 0.f);
  int rc = HSR_OK;
  auto up_soa = [&](const float* src, int cnt, int comp, size_t padded, float** dst) -> int {
    int r = dalloc((void**)dst, sizeof(float) * padded, "mesh");
    if (r != HSR_OK) return r;
    std::fill(tmp.begin(), tmp.begin() + padded, 0.f);
    for (int i = 0; i < cnt; i++) tmp[i] = src[(size_t)i * 3 + comp];
    cudaError_t e = cudaMemcpy(*dst, tmp.data(), sizeof(float) * padded, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? HSR_OK : cuda_fail(e, "mesh upload");
  };
  for (int c = 0; c < 3 && rc == HSR_OK; c++) rc = up_soa(pos, npos, c, P, c == 0 ? &m->px : (c == 1 ? &m->py : &m->pz));
  for (int c = 0; c < 3 && rc == HSR_OK; c++) rc = up_soa(nrm, nnrm, c, N, c == 0 ? &m->nx : (c == 1 ? &m->ny : &m->nz));
  if (rc == HSR_OK) rc = upload_xyz0(pos, npos, &m->p4);
  if (rc == HSR_OK) rc = upload_xyz0(nrm, nnrm, &m->n4);
  if (rc == HSR_OK) rc = dalloc((void**)&m->uv, sizeof(float2) * (size_t)std::max(nuv, 1), "mesh uv");
  if (rc == HSR_OK && nuv) {
    cudaError_t e = cudaMemcpy(m->uv, uv, sizeof(float2) * (size_t)nuv, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(e, "mesh uv upload");
  }
  if (rc == HSR_OK) {
    const size_t F = (size_t)std::max(nfaces, 1);
    std::vector<int4> fv(F), ft(F), fn(F);
    bool unified = true;
    for (int i = 0; i < nfaces; i++) {
      const int32_t* f = faces + (size_t)i * 9;
      fv[i] = make_int4(f[0], f[3], f[6], 0);
      ft[i] = make_int4(f[1], f[4], f[7], 0);
      fn[i] = make_int4(f[2], f[5], f[8], 0);
      for (int k = 0; k < 9; k += 3) unified = unified && f[k] == f[k + 1] && f[k] == f[k + 2];
    }
    m->unified = unified;
    if (unified && npos > 0 && rc == HSR_OK) {
      rc = dalloc((void**)&m->pk, sizeof(float4) * 2 * (size_t)npos, "packed vertices");
      if (rc == HSR_OK) {
        int kr = launch_pack_vertices(m->pk, m->p4, m->n4, m->uv, npos, nnrm, nuv, g_rt->stream);
        cudaError_t e = kr ? (cudaError_t)kr : cudaStreamSynchronize(g_rt->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "pack vertices");
      }
    }
    int4** dsts[3] = {&m->fv, &m->fvt, &m->fvn};
    std::vector<int4>* srcs[3] = {&fv, &ft, &fn};
    for (int k = 0; k < 3 && rc == HSR_OK; k++) {
      rc = dalloc((void**)dsts[k], sizeof(int4) * F, "mesh faces");
      if (rc == HSR_OK) {
        cudaError_t e = cudaMemcpy(*dsts[k], srcs[k]->data(), sizeof(int4) * F, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) rc = cuda_fail(e, "mesh faces upload");
      }
    }
  }
  if (rc != HSR_OK) { delete m; return rc; }
  const uint64_t h = g_rt->next_handle++;
  g_rt->meshes[h] = m;
  *out = h;
  return HSR_OK;
}

int hsr_mesh_update_normals(hsr_mesh mh, const float* nrm, int32_t nnrm) {
  RT_OR_FAIL();
  MeshObj* m = g_rt->mesh(mh);
  if (!m) return fail(HSR_ERR_BAD_HANDLE, "mesh_update_normals: unknown mesh");
  if (nnrm != m->nnrm || (nnrm && !nrm)) return fail(HSR_ERR_INVALID_ARG, "mesh_update_normals: count mismatch");
  cudaStreamSynchronize(g_rt->stream);
  const size_t N = align_up((size_t)std::max(nnrm, 1), 4);
  std::vector<float> tmp(N, 0.f);
  float* dst[3] = {m->nx, m->ny, m->nz};
  for (int c = 0; c < 3; c++) {
    for (int i = 0; i < nnrm; i++) tmp[i] = nrm[(size_t)i * 3 + c];
    cudaError_t e = cudaMemcpy(dst[c], tmp.data(), sizeof(float) * N, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "normal upload");
  }
  int rc = write_xyz0(nrm, nnrm, m->n4);
  if (rc == HSR_OK && m->pk) {  // the packed vertices carry the normals too
    int kr = launch_pack_vertices(m->pk, m->p4, m->n4, m->uv, m->npos, m->nnrm, m->nuv, g_rt->stream);
    cudaError_t e = kr ? (cudaError_t)kr : cudaStreamSynchronize(g_rt->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "pack vertices");
  }
  return rc;
}

int hsr_mesh_release(hsr_mesh mh) {
  RT_OR_FAIL();
  auto it = g_rt->meshes.find(mh);
  if (it == g_rt->meshes.end()) return fail(HSR_ERR_BAD_HANDLE, "mesh_release: unknown mesh");
  cudaStreamSynchronize(g_rt->stream);
  delete it->second;
  g_rt->meshes.erase(it);
  return HSR_OK;
}

int hsr_texture_upload(const uint8_t* data, int32_t w, int32_t h, int32_t bytespp, hsr_texture* out) {
  RT_OR_FAIL();
  if (!out || !data || w <= 0 || h <= 0 || (bytespp != 1 && bytespp != 3 && bytespp != 4))
    return fail(HSR_ERR_INVALID_ARG, "texture: bad arguments (bytespp must be 1, 3 or 4)");
  const size_t n = (size_t)w * (size_t)h;
  std::vector<uint32_t> words(n);
  for (size_t i = 0; i < n; i++) {
    uint32_t wv = 0;
    for (int k = 0; k < bytespp; k++) wv |= (uint32_t)data[i * bytespp + k] << (8 * k);
    words[i] = wv;
  }
  TexObj* t = new TexObj();
  t->w = w; t->h = h; t->bpp = bytespp;
  int rc = dalloc((void**)&t->words, sizeof(uint32_t) * n, "texture");
  if (rc == HSR_OK) {
    cudaError_t e = cudaMemcpy(t->words, words.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda_fail(e, "texture upload");
  }
  if (rc != HSR_OK) { delete t; return rc; }
  const uint64_t hd = g_rt->next_handle++;
  g_rt->textures[hd] = t;
  *out = hd;
  return HSR_OK;
}

int hsr_texture_release(hsr_texture th) {
  RT_OR_FAIL();
  auto it = g_rt->textures.find(th);
  if (it == g_rt->textures.end()) return fail(HSR_ERR_BAD_HANDLE, "texture_release: unknown texture");
  cudaStreamSynchronize(g_rt->stream);
  delete it->second;
  g_rt->textures.erase(it);
  return HSR_OK;
}

int hsr_target_create(int32_t w, int32_t h, hsr_target* out) {
  RT_OR_FAIL();
  if (!out || w <= 0 || h <= 0 || w > 32768 || h > 32768)
    return fail(HSR_ERR_INVALID_ARG, "target: size must be in [1, 32768]");
  TargetObj* t = new TargetObj();
  t->w = w; t->h = h;
  const size_t n = (size_t)w * (size_t)h;
  // the three planes in one block from the device's stream-ordered pool (freed blocks stay
  // cached in the pool, so creating and releasing targets of varying size stays cheap)
  const size_t plane = align_up(4 * n, 256);
  cudaError_t e = cudaMallocAsync((void**)&t->block, 3 * plane, g_rt->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    t->block = nullptr;
    delete t;
    return fail(HSR_ERR_OUT_OF_MEMORY, "target: device allocation of " + std::to_string(3 * plane) + " bytes failed");
  }
  t->stream = g_rt->stream;
  t->color = reinterpret_cast<uint32_t*>(t->block);
  t->depth = reinterpret_cast<float*>(t->block + plane);
  t->prim = reinterpret_cast<uint32_t*>(t->block + 2 * plane);
  // RenderBuffer's constructor clears to colour (0,0,0,1) -> bytes (0,0,0,255) and depth 1
  // (renderbuffer.cpp:3-18)
  const uint8_t rgba[4] = {0, 0, 0, 255};
  const uint64_t hd = g_rt->next_handle++;
  g_rt->targets[hd] = t;
  *out = hd;
  return g_rt->clear_target(t, rgba, 1.0f);
}

int hsr_target_release(hsr_target th) {
  RT_OR_FAIL();
  auto it = g_rt->targets.find(th);
  if (it == g_rt->targets.end()) return fail(HSR_ERR_BAD_HANDLE, "target_release: unknown target");
  cudaStreamSynchronize(g_rt->stream);
  delete it->second;
  g_rt->targets.erase(it);
  return HSR_OK;
}

int hsr_target_clear(hsr_target th, const uint8_t rgba[4], float depth) {
  RT_OR_FAIL();
  TargetObj* t = g_rt->target(th);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "target_clear: unknown target");
  if (!rgba) return fail(HSR_ERR_INVALID_ARG, "target_clear: rgba is null");
  return g_rt->clear_target(t, rgba, depth);
}

int hsr_target_upload(hsr_target th, const uint8_t* rgba, const float* depth, const uint32_t* prim) {
  RT_OR_FAIL();
  TargetObj* t = g_rt->target(th);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "target_upload: unknown target");
  const size_t n = (size_t)t->w * (size_t)t->h;
  cudaError_t e = cudaSuccess;
  if (rgba && e == cudaSuccess) e = cudaMemcpyAsync(t->color, rgba, 4 * n, cudaMemcpyHostToDevice, g_rt->stream);
  if (depth && e == cudaSuccess) e = cudaMemcpyAsync(t->depth, depth, 4 * n, cudaMemcpyHostToDevice, g_rt->stream);
  if (prim && e == cudaSuccess) e = cudaMemcpyAsync(t->prim, prim, 4 * n, cudaMemcpyHostToDevice, g_rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_rt->stream);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "target upload");
}

int hsr_target_download(hsr_target th, uint8_t* rgba, float* depth, uint32_t* prim) {
  RT_OR_FAIL();
  TargetObj* t = g_rt->target(th);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "target_download: unknown target");
  const size_t n = (size_t)t->w * (size_t)t->h;
  cudaError_t e = cudaSuccess;
  if (rgba && e == cudaSuccess) e = cudaMemcpyAsync(rgba, t->color, 4 * n, cudaMemcpyDeviceToHost, g_rt->stream);
  if (depth && e == cudaSuccess) e = cudaMemcpyAsync(depth, t->depth, 4 * n, cudaMemcpyDeviceToHost, g_rt->stream);
  if (prim && e == cudaSuccess) e = cudaMemcpyAsync(prim, t->prim, 4 * n, cudaMemcpyDeviceToHost, g_rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_rt->stream);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "target download");
}

int hsr_draw(const hsr_draw_desc* desc) {
  RT_OR_FAIL();
  if (!desc) return fail(HSR_ERR_INVALID_ARG, "draw: desc is null");
  return g_rt->run_batch(desc, 1);
}

int hsr_draw_batch(const hsr_draw_desc* descs, int32_t n) {
  RT_OR_FAIL();
  if (n < 0 || (n > 0 && !descs)) return fail(HSR_ERR_INVALID_ARG, "draw_batch: bad arguments");
  return g_rt->run_batch(descs, n);
}

int hsr_synchronize(void) {
  RT_OR_FAIL();
  cudaError_t e = cudaStreamSynchronize(g_rt->stream);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "synchronize");
}

int hsr_get_tuning(hsr_tuning* out) {
  RT_OR_FAIL();
  if (!out) return fail(HSR_ERR_INVALID_ARG, "get_tuning: null");
  *out = g_rt->tuning;
  return HSR_OK;
}

int hsr_set_tuning(const hsr_tuning* in) {
  RT_OR_FAIL();
  if (!in) return fail(HSR_ERR_INVALID_ARG, "set_tuning: null");
  if (in->tile != 8 && in->tile != 16 && in->tile != 32)
    return fail(HSR_ERR_INVALID_ARG, "set_tuning: tile must be 8, 16 or 32");
  if (in->warps_per_cta != 4 && in->warps_per_cta != 8) return fail(HSR_ERR_INVALID_ARG, "set_tuning: warps_per_cta must be 4 or 8");
  if (in->tile >= 16 && in->warps_per_cta != 4)
    return fail(HSR_ERR_INVALID_ARG, "set_tuning: tiles of 16 and 32 run 4 warps per CTA");
  if (in->ctas_per_sm < 1 || in->ctas_per_sm > 16) return fail(HSR_ERR_INVALID_ARG, "set_tuning: ctas_per_sm in [1,16]");
  if (!(in->bin_factor >= 0.5f && in->bin_factor <= 64.f)) return fail(HSR_ERR_INVALID_ARG, "set_tuning: bin_factor in [0.5,64]");
  g_rt->tuning = *in;
  return HSR_OK;
}

int hsr_set_fault_injection(uint32_t faults, int32_t poll_limit) {
  RT_OR_FAIL();
  if (faults & ~(uint32_t)(HSR_FAULT_DEPENDENCY_STALL | HSR_FAULT_SCAN_STALL))
    return fail(HSR_ERR_INVALID_ARG, "set_fault_injection: unknown fault bit");
  if (poll_limit < 0) return fail(HSR_ERR_INVALID_ARG, "set_fault_injection: poll_limit must be >= 0");
  g_rt->faults = faults;
  g_rt->poll_limit = poll_limit;
  return HSR_OK;
}

int hsr_set_profiling(int on) {
  RT_OR_FAIL();
  g_rt->profiling = on != 0;
  return HSR_OK;
}

int hsr_last_timing(hsr_timing* out) {
  RT_OR_FAIL();
  if (!out) return fail(HSR_ERR_INVALID_ARG, "last_timing: null");
  *out = g_rt->timing;
  return HSR_OK;
}

int hsr_host_alloc(size_t bytes, void** out) {
  if (!out) return fail(HSR_ERR_INVALID_ARG, "host_alloc: null");
  *out = nullptr;
  cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(HSR_ERR_OUT_OF_MEMORY, "host_alloc: cudaMallocHost failed");
  }
  return HSR_OK;
}

int hsr_host_free(void* p) {
  if (!p) return HSR_OK;
  cudaError_t e = cudaFreeHost(p);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "host_free");
}

// Autotuner: renders the batch with each launch shape (tile 8 / 16 / 32, warps per CTA 4 / 8,
// CTAs per SM 1..8), keeps the fastest median device time, then searches the bin capacity:
// the smallest factor of a ladder with which the batch runs without a bin overflow (capacity
// hints learnt from earlier overflows set aside during the search), plus a quarter of headroom
// for the next batches of a stream, and at least 1 (a bin entry per triangle and tile).  The batch's targets receive the renders.
int hsr_autotune(const hsr_draw_desc* descs, int32_t n, int32_t reps, hsr_tuning* out) {
  RT_OR_FAIL();
  if (!descs || n <= 0 || reps <= 0) return fail(HSR_ERR_INVALID_ARG, "autotune: bad arguments");
  const hsr_tuning saved = g_rt->tuning;
  const bool saved_prof = g_rt->profiling;
  g_rt->profiling = false;
  auto restore = [&](int rc) {
    g_rt->tuning = saved;
    g_rt->profiling = saved_prof;
    return rc;
  };
  hsr_tuning best = saved;
  float best_ms = 1e30f;
  const int tiles[3] = {8, 16, 32}, warps[2] = {4, 8}, ctas[4] = {1, 2, 4, 8};
  for (int ti : tiles)
    for (int wi : warps)
      for (int ci : ctas) {
        if (ci * wi > 32) continue;          // beyond one SM's warp slots for these kernels
        if (ti >= 16 && wi != 4) continue;   // shared-memory budget of the 16x16 and 32x32 tiles
        hsr_tuning cand = saved;
        cand.tile = ti;
        cand.warps_per_cta = wi;
        cand.ctas_per_sm = ci;
        g_rt->tuning = cand;
        std::vector<float> ms;
        for (int r = 0; r < reps + 1; r++) {
          int rc = g_rt->run_batch(descs, n);
          if (rc != HSR_OK) return restore(rc);
          if (r > 0) ms.push_back(g_rt->timing.batch_ms);  // first run warms up
        }
        std::sort(ms.begin(), ms.end());
        const float med = ms[ms.size() / 2];
        if (med < best_ms) {
          best_ms = med;
          best = cand;
        }
      }
  // bin capacity = factor * (faces + tiles) + 4096 pairs
  const float ladder[] = {0.5f, 0.75f, 1.f, 1.5f, 2.f, 3.f, 4.f, 6.f, 8.f, 12.f, 16.f, 24.f, 32.f, 48.f, 64.f};
  const size_t saved_hint = g_rt->cap_bin_hint;
  float fits = 64.f;
  for (float f : ladder) {
    hsr_tuning cand = best;
    cand.bin_factor = f;
    g_rt->tuning = cand;
    g_rt->cap_bin_hint = 0;
    const uint64_t retries = g_rt->stats.retries;
    int rc = g_rt->run_batch(descs, n);
    if (rc != HSR_OK) {
      g_rt->cap_bin_hint = saved_hint;
      return restore(rc);
    }
    if (g_rt->stats.retries == retries) {
      fits = f;
      break;
    }
  }
  g_rt->cap_bin_hint = saved_hint;
  best.bin_factor = std::min(64.f, std::max(1.f, fits * 1.25f));
  g_rt->tuning = best;
  g_rt->profiling = saved_prof;
  if (out) *out = best;
  return HSR_OK;
}

int hsr_get_stats(hsr_stats* out) {
  RT_OR_FAIL();
  if (!out) return fail(HSR_ERR_INVALID_ARG, "get_stats: null");
  *out = g_rt->stats;
  out->kernel_launches = g_rt->launches;
  return HSR_OK;
}

}  // extern "C"
