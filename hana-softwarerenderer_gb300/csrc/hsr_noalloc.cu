// hsr_noalloc.cu — a draw call that allocates nothing.
//
// hsr_draw() sizes its scratch (view descriptors, transformed vertices, triangle records,
// tile lists) per call and grows a device arena and a page-locked staging buffer with
// cudaMalloc / cudaMallocHost when a draw needs more.  Some callers cannot allow that: render
// loops with a frame deadline (allocating or freeing device memory can synchronise the whole
// device), processes held to a fixed device-memory budget that must not grow once running
// (a GPU shared with other services, where a late allocation can fail mid-frame), and host
// applications that forbid allocation inside their per-frame callbacks.  hsr_draw_noalloc()
// renders the same draw with the same kernels, but its scratch is one file-scope __device__
// array of kStaticScratchBytes (128 MiB) and its host-side staging is a file-scope host
// array: it calls no cudaMalloc, cudaFree, cudaMallocHost or other allocating routine.
//
// Limits and sharing:
//   - the success path allocates nothing on the device or the host (a failing call only
//     writes its message into the library's error string);
//   - a draw whose scratch does not fit in 128 MiB is rejected with HSR_ERR_INVALID_ARG
//     (roughly 400k faces into a 1920x1080 target); one that overflows it on the device
//     (more clipped or large triangles than the fixed split allows) returns
//     HSR_ERR_BIN_OVERFLOW and leaves the target untouched;
//   - the call is synchronous: it runs on the library's stream and waits for its own result;
//   - every GPU that loads libhsr holds the array until the process exits;
//   - all calls share the array, which keeps the last call's contents; each call clears the
//     counters it needs, but two calls whose work overlaps on the GPU race on the array: run
//     them one after another;
//   - the first call on a device looks up the array's device address (cudaGetSymbolAddress)
//     for that device, with that device current; make that first call before any stream
//     capture begins.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "hsr_internal.h"
#include "hsr_runtime.h"

namespace hsr {

constexpr size_t kStaticScratchBytes = size_t(128) << 20;
constexpr size_t kStaticHostBytes = 4096;
constexpr int kMaxDevices = 64;

// The scratch every call uses.  In host code this name is only a host-side stand-in for
// the device array: its device address comes from cudaGetSymbolAddress, per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kStaticScratchBytes];

static unsigned char g_noalloc_host[kStaticHostBytes];  // view descriptor and control block
static_assert(((sizeof(DView) + 255) / 256 * 256) + sizeof(Ctl) <= kStaticHostBytes, "host staging too small");
static void* g_noalloc_dev[kMaxDevices];

static size_t nal(size_t x) { return (x + 255) / 256 * 256; }

static int noalloc_draw(Runtime* rt, const hsr_draw_desc& d) {
  int rc = rt->validate(d);
  if (rc != HSR_OK) return rc;
  if (rt->device < 0 || rt->device >= kMaxDevices) return fail(HSR_ERR_INVALID_ARG, "draw_noalloc: device ordinal");
  cudaError_t se = cudaSetDevice(rt->device);  // make the library's device current on this thread
  if (se != cudaSuccess) return cuda_fail(se, "draw_noalloc: cudaSetDevice");
  // one-time set-up for this device, with that device current
  if (!g_noalloc_dev[rt->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(e, "draw_noalloc: cudaGetSymbolAddress");
    g_noalloc_dev[rt->device] = p;
  }
  char* dev = static_cast<char*>(g_noalloc_dev[rt->device]);

  MeshObj* m = rt->mesh(d.mesh);
  TargetObj* tg = rt->target(d.target);
  const int T = rt->tuning.tile;

  // ---- the single view ------------------------------------------------------------------
  DView v;
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
    TexObj* t = rt->tex(d.diffuse);
    v.diffuse = t->words; v.dw = t->w; v.dh = t->h; v.dbpp = t->bpp;
  }
  if (d.normal) {
    TexObj* t = rt->tex(d.normal);
    v.normal = t->words; v.nw = t->w; v.nh = t->h; v.nbpp = t->bpp;
  }
  v.color = tg->color; v.depth = tg->depth; v.prim = tg->prim; v.W = tg->w; v.H = tg->h;
  if (d.shadow_map) {
    TargetObj* sm = rt->target(d.shadow_map);
    v.sm_color = sm->color; v.smW = sm->w; v.smH = sm->h;
  }
  v.dep0 = v.dep1 = -1;
  v.tiles_x = (tg->w + T - 1) / T;
  v.tiles_y = (tg->h + T - 1) / T;
  v.ntiles = v.tiles_x * v.tiles_y;
  v.tile_base = 0;
  v.prim_base = d.prim_base;
  v.clear_depth = d.clear_depth;
  std::memcpy(&v.clear_rgba, d.clear_rgba, 4);
  v.has_dependents = 0;

  // ---- work chunks and the fixed layout of the static array ------------------------------
  v.vch_base = 0;
  v.vch_npos = (m->npos + kVertexChunk - 1) / kVertexChunk;
  v.vch_count = v.vch_npos;
  v.sch_base = 0;
  v.cch_base = 0;
  const int nvch = v.vch_count;
  const int ncch = (d.flags & HSR_DRAW_CLEAR) ? (int)(((size_t)tg->w * (size_t)tg->h + kClearChunk - 1) / kClearChunk) : 0;
  const int nsch = (m->nfaces + kSetupChunk - 1) / kSetupChunk;
  const size_t faces = (size_t)m->nfaces, tiles = (size_t)v.ntiles;
  const size_t rec_cap = faces + faces / 4 + 1024, clip_cap = faces / 16 + 256, big_cap = faces / 64 + 256;
  const size_t bin_cap = (size_t)(rt->tuning.bin_factor * (double)(faces + tiles)) + 4096;
  const int nscan = scan_blocks((int)tiles);
  size_t off = 0;
  const size_t o_view = off; off = nal(off + sizeof(DView));
  const size_t host_bytes = off;
  const size_t o_clip = off; off = nal(off + sizeof(float4) * (size_t)std::max(m->npos, 1));
  const size_t o_zero = off;
  const size_t o_ctl = off; off = nal(off + sizeof(Ctl));
  const size_t o_done = off; off = nal(off + sizeof(uint32_t));
  const size_t o_cnt = off; off = nal(off + sizeof(uint32_t) * tiles);
  const size_t o_fill = off; off = nal(off + sizeof(uint32_t) * tiles);
  const size_t o_stat = off; off = nal(off + sizeof(unsigned long long) * (size_t)std::max(nscan, 1));
  const size_t zero_bytes = off - o_zero;
  const size_t o_toff = off; off = nal(off + sizeof(uint32_t) * tiles);
  const size_t o_neoff = off; off = nal(off + sizeof(uint32_t) * (tiles + 1));
  const size_t o_list = off; off = nal(off + sizeof(uint32_t) * tiles);
  const size_t o_recs = off; off = nal(off + sizeof(RasterRec) * rec_cap);
  const size_t o_pay = off; off = nal(off + sizeof(Payload) * rec_cap);
  const size_t o_clipq = off; off = nal(off + sizeof(int2) * clip_cap);
  const size_t o_big = off; off = nal(off + sizeof(BigItem) * big_cap);
  const size_t o_bins = off; off = nal(off + sizeof(uint32_t) * bin_cap);
  if (off > kStaticScratchBytes)
    return fail(HSR_ERR_INVALID_ARG, "draw_noalloc: the draw needs more scratch than the 128 MiB the allocation-free path holds");

  v.sv = (float4*)(dev + o_clip);

  unsigned char* h = g_noalloc_host;
  std::memcpy(h + o_view, &v, sizeof(DView));

  Scratch sc;
  std::memset(&sc, 0, sizeof(sc));
  sc.ctl = (Ctl*)(dev + o_ctl);
  sc.view_done = (uint32_t*)(dev + o_done);
  sc.recs = (RasterRec*)(dev + o_recs); sc.rec_cap = (uint32_t)rec_cap;
  sc.pay = (Payload*)(dev + o_pay);
  sc.clipq = (int2*)(dev + o_clipq); sc.clip_cap = (uint32_t)clip_cap;
  sc.bigq = (BigItem*)(dev + o_big); sc.big_cap = (uint32_t)big_cap;
  sc.tile_count = (uint32_t*)(dev + o_cnt);
  sc.tile_fill = (uint32_t*)(dev + o_fill);
  sc.tile_off = (uint32_t*)(dev + o_toff);
  sc.ne_off = (uint32_t*)(dev + o_neoff);
  sc.tile_list = (uint32_t*)(dev + o_list);
  sc.scan_status = (unsigned long long*)(dev + o_stat);
  sc.bins = (uint32_t*)(dev + o_bins); sc.bin_cap = (uint32_t)bin_cap;
  sc.ntiles = (int32_t)tiles;
  sc.nviews = 1;

  // ---- the launch sequence of hsr_draw on the static scratch ------------------------------
  cudaStream_t s = rt->stream;
  const DView* dview = (const DView*)(dev + o_view);
  cudaError_t e = cudaMemcpyAsync(dev, h, host_bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "draw_noalloc: upload");
  e = cudaMemsetAsync(dev + o_zero, 0, zero_bytes, s);  // counters start at zero every call
  if (e != cudaSuccess) return cuda_fail(e, "draw_noalloc: clear counters");
  int kr = launch_vertex(dview, 1, nvch, rt->num_sms * 8, s);
  if (!kr) kr = launch_setup(dview, 1, nsch, sc, rt->num_sms * 8, s);
  if (!kr) kr = launch_emit(dview, T, sc, rt->num_sms * 8, s);
  if (!kr) kr = launch_post(dview, T, sc, rt->num_sms * 4, s);
  if (!kr) kr = launch_big(dview, T, sc, rt->num_sms * 2, s);
  if (!kr) kr = launch_scan(sc, s);
  if (!kr) kr = launch_scatter(dview, T, sc, rt->num_sms * 8, ncch, s);
  if (!kr) kr = launch_raster(dview, T, sc, rt->num_sms * rt->tuning.ctas_per_sm, rt->tuning.warps_per_cta, s);
  if (kr) return cuda_fail((cudaError_t)kr, "draw_noalloc: kernel launch");
  rt->launches += 8;
  Ctl* hc = reinterpret_cast<Ctl*>(h + host_bytes);
  e = cudaMemcpyAsync(hc, sc.ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "draw_noalloc");
  if (hc->error & kErrCapacity)
    return fail(HSR_ERR_BIN_OVERFLOW, "draw_noalloc: the draw overflowed the fixed scratch split (target untouched)");
  if (hc->error & (kErrWaitTimeout | kErrScanTimeout))
    return fail(HSR_ERR_TIMEOUT, "draw_noalloc: a bounded device wait gave up");
  return HSR_OK;
}

}  // namespace hsr

extern "C" int hsr_draw_noalloc(const hsr_draw_desc* desc) {
  std::lock_guard<std::mutex> lock(hsr::g_mu);
  if (!hsr::g_rt) return hsr::fail(HSR_ERR_NOT_INITIALIZED, "hsr_init() has not succeeded");
  if (!desc) return hsr::fail(HSR_ERR_INVALID_ARG, "draw_noalloc: desc is null");
  return hsr::noalloc_draw(hsr::g_rt, *desc);
}
