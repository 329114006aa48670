// kernels_geom.cu — vertex transform and triangle setup (sm_103a).
//
// k_vertex replaces the per-corner IShader::vertex calls of graphics.cpp:380-387.  The
// vertex shader is a pure function of its a2v inputs, and each output stream depends on
// one attribute stream only (clip and world position on `v`, world normal and light
// intensity on `vn`, uv passes through), so every corner gets the same bits whether an
// output is computed once per vertex or once per corner.  The clip position and the
// per-corner work of rasterize_triangle that depends on one vertex alone — the visibility
// test of clip_triangle's fast accept (graphics.cpp:132-134, 140-142) and, for a visible
// vertex, the perspective divide and 1/w (:320-337) — is done here once per vertex (the
// screen vertex, see screen_vertex), so setup divides nothing on the fast path.  World
// position and normal are needed only for the corners of the one triangle in five that
// survives setup: k_emit (and the clipper) transform them per corner (world_pos_of,
// world_normal_of) instead of this pass writing and re-reading them for every vertex.
//
// k_setup (the cull pass) follows graphics.cpp:136-161 (clip) and :314-347 (cull, viewport,
// bounding box) for every face that passes the fast accept and stores one RasterRec per
// surviving triangle; faces that need the clipper are queued.  k_emit writes the surviving
// records' shading payloads and tile counts on dense warps; k_post clips the queued faces (two
// per warp: lane k of a half-warp carries varying k of the polygon through Sutherland-Hodgman)
// and emits their fan triangles; k_big splits triangles that touch more than kMaxRecordTiles
// tiles into sub-records.
#include <float.h>

#include <algorithm>

#include "hsr_device.cuh"

namespace hsr {

constexpr unsigned kFull = 0xffffffffu;

// ---------------------------------------------------------------------------------------
// clip-space helpers
// ---------------------------------------------------------------------------------------
enum { PW, PX, NX, PY, NY, PZ, NZ };

// is_inside_plane (graphics.cpp:29-49) on clip coordinates c[0..3]
__device__ __forceinline__ bool inside_plane(const float* c, int plane) {
  switch (plane) {
    case PW: return c[3] >= 1e-5f;
    case PX: return c[0] <= c[3];
    case NX: return c[0] >= -c[3];
    case PY: return c[1] <= c[3];
    case NY: return c[1] >= -c[3];
    case PZ: return c[2] <= c[3];
    default: return c[2] >= -c[3];
  }
}
// get_intersect_ratio (graphics.cpp:51-71)
__device__ __forceinline__ float intersect_ratio(const float* p, const float* q, int plane) {
  switch (plane) {
    case PW: return fd(fs(p[3], 1e-5f), fs(p[3], q[3]));
    case PX: return fd(fs(p[3], p[0]), fs(fs(p[3], p[0]), fs(q[3], q[0])));
    case NX: return fd(fa(p[3], p[0]), fs(fa(p[3], p[0]), fa(q[3], q[0])));
    case PY: return fd(fs(p[3], p[1]), fs(fs(p[3], p[1]), fs(q[3], q[1])));
    case NY: return fd(fa(p[3], p[1]), fs(fa(p[3], p[1]), fa(q[3], q[1])));
    case PZ: return fd(fs(p[3], p[2]), fs(fs(p[3], p[2]), fs(q[3], q[2])));
    default: return fd(fa(p[3], p[2]), fs(fa(p[3], p[2]), fa(q[3], q[2])));
  }
}
__device__ __forceinline__ bool vertex_visible(float4 c) {  // is_vertex_visible (:132-134)
  return fabsf(c.x) <= c.w && fabsf(c.y) <= c.w && fabsf(c.z) <= c.w;
}

// Clip position of vertex i of a view: ObjectToClipPos (IShader.h:55-61), the bits k_vertex
// computed for it.
__device__ __forceinline__ float4 clip_of(const DView& v, int i) {
  return mat_vec(v.mvp, __ldg(v.px + i), __ldg(v.py + i), __ldg(v.pz + i), 1.f);
}

// Screen vertex of one clip position.  A vertex that is visible (is_vertex_visible,
// graphics.cpp:132-134) with w >= 1e-5 stores what rasterize_triangle derives from it
// alone: (x/w, y/w, z/w, 1/w) (graphics.cpp:321-323, 335-337); its |x/w| is <= 1 or NaN.
// Any other vertex stores (kSvSpecial, mask, 0, 0), bit p of the mask being
// is_inside_plane for plane p in the clipper's order (W, +X, -X, +Y, -Y, +Z, -Z) and bit 7
// is_vertex_visible.  A normal screen vertex is inside every plane (|x|,|y|,|z| <= w and
// w >= 1e-5), so its mask is 0xff.
constexpr float kSvSpecial = 4.0f;
__device__ __forceinline__ float4 screen_vertex(float4 c) {
  const bool vis = vertex_visible(c);
  if (vis && c.w >= 1e-5f) return make_float4(fd(c.x, c.w), fd(c.y, c.w), fd(c.z, c.w), fd(1.f, c.w));
  const float a[4] = {c.x, c.y, c.z, c.w};
  uint32_t m = vis ? 0x80u : 0u;
#pragma unroll
  for (int p = PW; p <= NZ; p++)
    if (inside_plane(a, p)) m |= 1u << p;
  return make_float4(kSvSpecial, __uint_as_float(m), 0.f, 0.f);
}
__device__ __forceinline__ bool sv_normal(float4 s) { return !(fabsf(s.x) > 1.f); }

// ObjectToWorldPos (IShader.h:63-65) of an object-space position.
__device__ __forceinline__ float4 world_pos(const DView& v, float x, float y, float z) {
  const float4 w = mat_vec(v.u.model_matrix, x, y, z, 1.f);
  return make_float4(w.x, w.y, w.z, 0.f);
}
__device__ __forceinline__ float4 world_pos_of(const DView& v, int i) {
  const float4 p = __ldg(v.p4 + i);
  return world_pos(v, p.x, p.y, p.z);
}
// ObjectToWorldNormal (IShader.h:71-75) = [n, 1] * model_I of an object-space normal, with the
// intensity of Ground / Toon, saturate(worldN . light_dir) (IShader.cpp:8, :26), in w.
__device__ __forceinline__ float4 world_normal(const DView& v, float nx, float ny, float nz) {
  const float* m = v.u.model_matrix_I;
  F3 wn;
  wn.x = dot4(nx, ny, nz, 1.f, m[0], m[4], m[8], m[12]);
  wn.y = dot4(nx, ny, nz, 1.f, m[1], m[5], m[9], m[13]);
  wn.z = dot4(nx, ny, nz, 1.f, m[2], m[6], m[10], m[14]);
  const F3 L = {v.u.light_dir[0], v.u.light_dir[1], v.u.light_dir[2]};
  return make_float4(wn.x, wn.y, wn.z, saturate(dot3(wn, L)));
}
__device__ __forceinline__ float4 world_normal_of(const DView& v, int i) {
  const float4 n = __ldg(v.n4 + i);
  return world_normal(v, n.x, n.y, n.z);
}
__device__ __forceinline__ uint32_t sv_mask(float4 s) { return sv_normal(s) ? 0xffu : __float_as_uint(s.y); }

// ---------------------------------------------------------------------------------------
// work chunks
// ---------------------------------------------------------------------------------------
// The chunk bases of all views in shared memory (nviews <= kSharedViews), read with
// `base_of` (field selector); every thread of the block calls this (ends with a barrier).
template <class F>
__device__ __forceinline__ const int32_t* share_bases(const DView* views, int nviews, int32_t* s_base, F base_of) {
  if (nviews > kSharedViews) return nullptr;
  for (int i = threadIdx.x; i < nviews; i += blockDim.x) s_base[i] = base_of(views[i]);
  __syncthreads();
  return s_base;
}
// View of chunk c: the last view whose base is <= c (views with no chunks share the next
// view's base and are never returned for a chunk they do not hold).  A block visits its
// chunks in increasing order, so the search walks forward from the view of its previous
// chunk (`hint`), usually zero or one step.
template <class F>
__device__ __forceinline__ int chunk_view(const DView* views, const int32_t* s_base, int nviews, int c, F base_of,
                                          int hint) {
  int k = hint;
  while (k + 1 < nviews && (s_base ? s_base[k + 1] : base_of(views[k + 1])) <= c) k++;
  return k;
}
// The same by binary search, for a block that starts cold.
template <class F>
__device__ __forceinline__ int chunk_view_search(const DView* views, const int32_t* s_base, int nviews, int c,
                                                 F base_of) {
  int lo = 0, hi = nviews - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((s_base ? s_base[mid] : base_of(views[mid])) <= c) lo = mid; else hi = mid - 1;
  }
  return lo;
}
struct VchBase { __device__ int32_t operator()(const DView& v) const { return v.vch_base; } };
struct SchBase { __device__ int32_t operator()(const DView& v) const { return v.sch_base; } };

// Chunk c of the vertex stage: view and position range.
__device__ __forceinline__ Chunk vertex_chunk(const DView* views, const int32_t* s_base, int nviews, int c) {
  const int k = chunk_view_search(views, s_base, nviews, c, VchBase());
  const DView& v = views[k];
  Chunk ch;
  ch.view = k;
  ch.begin = (c - v.vch_base) * kVertexChunk;
  ch.end = min(v.npos, ch.begin + kVertexChunk);
  return ch;
}
// Chunk c of the setup stage: view and face range.
__device__ __forceinline__ Chunk setup_chunk(const DView* views, const int32_t* s_base, int nviews, int c, int hint) {
  const int k = chunk_view(views, s_base, nviews, c, SchBase(), hint);
  const DView& v = views[k];
  Chunk ch;
  ch.view = k;
  ch.begin = (c - v.sch_base) * kSetupChunk;
  ch.end = min(v.nfaces, ch.begin + kSetupChunk);
  return ch;
}

// ---------------------------------------------------------------------------------------
// vertex stage
// ---------------------------------------------------------------------------------------
// One vertex chunk (kVertexChunk positions, 8 per thread, 256 threads): ObjectToClipPos /
// ObjectToViewPos (IShader.h:55-61) -> screen vertex.
__device__ __forceinline__ void vertex_chunk_work(const DView& v, const Chunk& ch) {
  // item i = begin + threadIdx.x + 256 k: consecutive threads read consecutive floats and
  // write consecutive float4s, so every load and store instruction of a warp is one
  // contiguous span; the loads of a thread are issued before any is used
  constexpr int kPer = kVertexChunk / 256;
  const int i0 = ch.begin + (int)threadIdx.x;
  float xs[kPer], ys[kPer], zs[kPer];
#pragma unroll
  for (int k = 0; k < kPer; k++) {
    const int i = i0 + 256 * k;
    const bool in = i < ch.end;
    xs[k] = in ? __ldg(v.px + i) : 0.f;
    ys[k] = in ? __ldg(v.py + i) : 0.f;
    zs[k] = in ? __ldg(v.pz + i) : 0.f;
  }
#pragma unroll
  for (int k = 0; k < kPer; k++) {
    const int i = i0 + 256 * k;
    if (i >= ch.end) break;
    v.sv[i] = screen_vertex(mat_vec(v.mvp, xs[k], ys[k], zs[k], 1.f));
  }
}

// One block per chunk (the blocks are short and many: their prologues overlap others' work).
__global__ void __launch_bounds__(256) k_vertex(const DView* __restrict__ views, int nviews) {
  __shared__ int32_t s_base[kSharedViews];
  const int32_t* base = share_bases(views, nviews, s_base, VchBase());
  const Chunk ch = vertex_chunk(views, base, nviews, (int)blockIdx.x);
  vertex_chunk_work(views[ch.view], ch);
}

int launch_vertex(const DView* views, int nviews, int nchunks, int grid, cudaStream_t s) {
  (void)grid;
  if (nchunks <= 0) return 0;
  k_vertex<<<nchunks, 256, 0, s>>>(views, nviews);
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// setup stage
// ---------------------------------------------------------------------------------------
constexpr int kSetupCoverPixels = 12;  // pixel ranges up to this size are tested in setup

__device__ __forceinline__ bool coord_ok(float c) {
  // |c| == 0 or 2^-8 <= |c| <= 2^20, on the bits of |c| (NaN and inf are above the range)
  const uint32_t b = __float_as_uint(c) & 0x7fffffffu;
  return b == 0u || b - 0x3b800000u <= 0x49800000u - 0x3b800000u;
}

// Perspective divide of rasterize_triangle (graphics.cpp:321-323): clip / w per component.
__device__ __forceinline__ F3 ndc_of(float4 c) { return {fd(c.x, c.w), fd(c.y, c.w), fd(c.z, c.w)}; }

// Cull, viewport, bounding box of one fan triangle from its corners' NDC coordinates
// (graphics.cpp:324-347).
__device__ __forceinline__ bool build_rec(const DView& v, F3 n0, F3 n1, F3 n2, uint32_t seq, uint32_t view,
                                          RasterRec& r) {
  // is_back_facing (:172-180), evaluated left to right
  float sa = fs(fm(n0.x, n1.y), fm(n0.y, n1.x));
  sa = fa(sa, fm(n1.x, n2.y));
  sa = fs(sa, fm(n1.y, n2.x));
  sa = fa(sa, fm(n2.x, n0.y));
  sa = fs(sa, fm(n2.y, n0.x));
  if (sa <= 0.f) return false;
  const F3 s0 = viewport(v.W, v.H, n0), s1 = viewport(v.W, v.H, n1), s2 = viewport(v.W, v.H, n2);
  // bounding box with std::min / std::max (:339-347)
  float bminx, bminy, bmaxx, bmaxy;
  const float clampx = (float)(v.W - 1), clampy = (float)(v.H - 1);
  const float sx[3] = {s0.x, s1.x, s2.x}, sy[3] = {s0.y, s1.y, s2.y};
  if (!(sx[0] != sx[0] || sx[1] != sx[1] || sx[2] != sx[2] || sy[0] != sy[0] || sy[1] != sy[1] || sy[2] != sy[2])) {
    // no NaN: the chains below reduce to min / max (a signed zero only reaches the (int)
    // conversions and the < 0 tests, which treat -0 and +0 alike)
    bminx = fmaxf(0.f, fminf(fminf(sx[0], sx[1]), sx[2]));
    bmaxx = fminf(clampx, fmaxf(fmaxf(sx[0], sx[1]), sx[2]));
    bminy = fmaxf(0.f, fminf(fminf(sy[0], sy[1]), sy[2]));
    bmaxy = fminf(clampy, fmaxf(fmaxf(sy[0], sy[1]), sy[2]));
  } else {
    bminx = FLT_MAX; bminy = FLT_MAX; bmaxx = -FLT_MAX; bmaxy = -FLT_MAX;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      bminx = std_max(0.f, std_min(bminx, sx[i]));
      bmaxx = std_min(clampx, std_max(bmaxx, sx[i]));
      bminy = std_max(0.f, std_min(bminy, sy[i]));
      bmaxy = std_min(clampy, std_max(bmaxy, sy[i]));
    }
  }
  // pixels visited: x from (int)bboxmin.x while x <= bboxmax.x (:350-351)
  const int32_t x0 = cvt_i32(bminx), y0 = cvt_i32(bminy);
  if (x0 < 0 || y0 < 0 || bmaxx < 0.f || bmaxy < 0.f) return false;
  const int32_t x1 = (int32_t)floorf(bmaxx), y1 = (int32_t)floorf(bmaxy);
  if (x0 > x1 || y0 > y1) return false;
  // barycentric() constants (:222-233): u.z = (C.x-A.x)(B.y-A.y) - (B.x-A.x)(C.y-A.y)
  const float e1x = fs(s1.x, s0.x), e1y = fs(s1.y, s0.y);
  const float e2x = fs(s2.x, s0.x), e2y = fs(s2.y, s0.y);
  const float uz = fs(fm(e2x, e1y), fm(e1x, e2y));
  if (!(fabsf(uz) > 0.01f)) return false;  // degenerate: every pixel gets (-1,1,1)
  const bool ok = coord_ok(s0.x) && coord_ok(s0.y) && coord_ok(s1.x) && coord_ok(s1.y) &&
                  coord_ok(s2.x) && coord_ok(s2.y) && fabsf(uz) <= 0x1p30f;
  // a small pixel range is tested here with the raster's own coverage test: a triangle
  // that covers none of its pixels would only be visited and rejected pixel by pixel
  if ((x1 - x0 + 1) * (y1 - y0 + 1) <= kSetupCoverPixels) {
    bool any = false;
    for (int32_t y = y0; y <= y1 && !any; y++)
      for (int32_t x = x0; x <= x1 && !any; x++) {
        float b0, b1, b2;
        any = cover_test(s0.x, s0.y, e1x, e1y, e2x, e2y, uz, !ok, (float)x, (float)y, b0, b1, b2);
      }
    if (!any) return false;
  }
  r.ax = s0.x; r.ay = s0.y; r.e1x = e1x; r.e1y = e1y;
  r.e2x = e2x; r.e2y = e2y; r.uz = uz; r.d0 = s0.z;
  r.d1 = s1.z; r.d2 = s2.z;
  r.seq = seq;
  r.xr = (uint32_t)x0 | ((uint32_t)x1 << 16);
  r.yr = (uint32_t)y0 | ((uint32_t)y1 << 16);
  r.view = view | ((ok ? 0u : kRecExact) << kRecFlagShift);
  r.rsv = 0u;
  r.pad = 0u;
  return true;
}

__device__ __forceinline__ void store_rec(RasterRec* dst, const RasterRec& r) {
  const float4* s = reinterpret_cast<const float4*>(&r);
  st_v8(dst, s[0], s[1]);
  st_v8(reinterpret_cast<char*>(dst) + 32, s[2], s[3]);
}

// Payload floats a shader reads, rounded up to whole float4s (see the Payload layout).
__device__ __forceinline__ int payload_f4(int shader) {
  switch (shader) {
    case HSR_SHADER_FLAT: return 0;
    case HSR_SHADER_SHADOW: case HSR_SHADER_GROUND: case HSR_SHADER_TOON: return 2;
    case HSR_SHADER_TEXTURE: return 3;
    case HSR_SHADER_TEXTURE_WITH_LIGHT: return 6;
    default: return 8;
  }
}

// Corner varyings c[k] in shader_struct_v2f order (13 floats) -> payload.
__device__ __forceinline__ void make_payload(int shader, const float* c0, const float* c1, const float* c2,
                                             Payload& p) {
  const float* c[3] = {c0, c1, c2};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    p.f[k] = fd(1.f, c[k][3]);                                   // recip_w (graphics.cpp:333-337)
    p.f[3 + k] = shader == HSR_SHADER_SHADOW ? c[k][2] : c[k][12];
    p.f[6 + 2 * k] = c[k][10];
    p.f[7 + 2 * k] = c[k][11];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      p.f[12 + 3 * k + q] = c[k][7 + q];
      p.f[21 + 3 * k + q] = c[k][4 + q];
    }
  }
  p.f[30] = 0.f;
  p.f[31] = 0.f;
}

__device__ __forceinline__ void store_payload(Payload* dst, const Payload& p, int nf4) {
  float4* d = reinterpret_cast<float4*>(dst);
  const float4* s = reinterpret_cast<const float4*>(&p);
#pragma unroll
  for (int q = 0; q < 8; q += 2) {
    if (q + 1 < nf4) st_v8(d + q, s[q], s[q + 1]);
    else if (q < nf4) d[q] = s[q];
  }
}

// Tile rectangle of a record; T is a power of two (8 or 16).
__device__ __forceinline__ void rec_tiles(const RasterRec& r, int T, int& tx0, int& ty0, int& ntw, int& nt) {
  const int ts = __ffs(T) - 1;
  const int x0 = (int)(r.xr & 0xffffu), x1 = (int)(r.xr >> 16);
  const int y0 = (int)(r.yr & 0xffffu), y1 = (int)(r.yr >> 16);
  tx0 = x0 >> ts;
  ty0 = y0 >> ts;
  ntw = (x1 >> ts) - tx0 + 1;
  nt = ntw * ((y1 >> ts) - ty0 + 1);
}

// Slot of this lane's item when `want`, one atomicAdd per warp (~0u otherwise).
__device__ __forceinline__ uint32_t warp_reserve(bool want, uint32_t* counter) {
  const int lane = threadIdx.x & 31;
  const unsigned m = __ballot_sync(kFull, want);
  if (!m) return ~0u;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
  base = __shfl_sync(kFull, base, leader);
  return want ? base + (uint32_t)__popc(m & ((1u << lane) - 1u)) : ~0u;
}

// Slot of this thread's item when `want`, one atomicAdd per block (~0u otherwise).  Every
// thread of the block calls this.  All warps of the grid append to one counter, and a
// returning atomic on a single address is served one at a time: reserving per block
// instead of per warp divides those atomics by the warps of a block.
template <int THREADS>
__device__ __forceinline__ uint32_t block_reserve(bool want, uint32_t* counter) {
  __shared__ uint32_t s_count[THREADS / 32];
  __shared__ uint32_t s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(kFull, want);
  if (lane == 0) s_count[warp] = (uint32_t)__popc(m);
  __syncthreads();
  if (warp == 0) {
    const uint32_t c = lane < THREADS / 32 ? s_count[lane] : 0u;
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < THREADS / 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(kFull, incl, THREADS / 32 - 1);
    if (lane < THREADS / 32) s_count[lane] = incl - c;
    if (lane == 0) s_base = total ? atomicAdd(counter, total) : 0u;
  }
  __syncthreads();
  return want ? s_base + s_count[warp] + (uint32_t)__popc(m & ((1u << lane) - 1u)) : ~0u;
}

// Store the records of a warp at their slots (at most one per lane, each touching
// <= kMaxRecordTiles tiles) with their payloads, and count the tiles they touch,
// aggregating equal tiles across lanes.  All 32 lanes call this.
// With `in_place`, the record is already stored (the emit pass): only its payload (at the
// record's own index) and its tile counts are written.
__device__ void append_counts(bool valid, uint32_t slot, const RasterRec& r, const Payload& pl, int nf4, const DView& v,
                              int T, const Scratch& sc, bool in_place = false) {
  const int lane = threadIdx.x & 31;
  int tx0 = 0, ty0 = 0, ntw = 1, nt = 0;
  if (valid) {
    if (!in_place) store_rec(&sc.recs[slot], r);
    store_payload(&sc.pay[slot], pl, nf4);
    rec_tiles(r, T, tx0, ty0, ntw, nt);
  }
  const int maxn = __reduce_max_sync(kFull, nt);
  int kx = 0, ky = 0;  // tile k of the rectangle = (kx, ky), row-major
  for (int k = 0; k < maxn; k++) {
    const int tile = (k < nt) ? v.tile_base + (ty0 + ky) * v.tiles_x + tx0 + kx : -1;
    const unsigned grp = __match_any_sync(kFull, tile);
    if (tile >= 0 && lane == __ffs(grp) - 1) atomicAdd(&sc.tile_count[tile], (uint32_t)__popc(grp));
    if (++kx == ntw) { kx = 0; ky++; }
  }
}

// append_counts at slots reserved by the caller, checked against the record capacity.
__device__ void append_small(bool valid, uint32_t slot, RasterRec r, const Payload& pl, int nf4, const DView& v,
                             int T, const Scratch& sc) {
  const bool ok = valid && slot < sc.rec_cap;
  if (valid && !ok) atomicOr(&sc.ctl->error, kErrRecOverflow);
  append_counts(ok, slot, r, pl, nf4, v, T, sc);
}

// True when the reference's clipper returns 0 vertices for this face without creating any
// new vertex: Sutherland-Hodgman copies a polygon whose vertices are all inside a plane
// unchanged, so if the three corners pass every plane before some plane (in the order
// W, +X, -X, +Y, -Y, +Z, -Z of graphics.cpp:152-158) and all fail that plane, that stage
// emits nothing and the face is dropped (CLIP_IN2OUT / CLIP_OUT2IN return 0).  Faces whose
// corners straddle a plane first go to the full clipper.  m0..m2 are the corners' plane
// masks (see screen_vertex).
__device__ __forceinline__ bool clip_trivially_empty(uint32_t m0, uint32_t m1, uint32_t m2) {
#pragma unroll
  for (int plane = PW; plane <= NZ; plane++) {
    const uint32_t all = (m0 & m1 & m2) >> plane & 1u, any = (m0 | m1 | m2) >> plane & 1u;
    if (!any) return true;
    if (!all) return false;
  }
  return false;
}

constexpr int kSetupThreads = kSetupChunk;  // one face per thread; a block's barriers span 4 warps
constexpr int kEmitThreads = 256;
constexpr int kPolyStride = kVaryings;  // floats per polygon vertex in shared memory


// Cull pass, one thread per face: fast accept, cull, viewport, bounding box and the
// coverage check of small ranges; a surviving triangle's 64-byte record is stored at a
// block-reserved slot (its payload and tile counts are still to come: k_emit), and
// faces that need the clipper are queued.  Four in five faces of the serving batches die
// here, so the per-record work runs in k_emit on dense warps instead of on the few lanes
// that survive in each warp of this pass.
//
// Persistent: block b takes chunks b, b + grid, ... (kSetupChunk faces each) and loads the face
// indices of its next chunk while it culls the current one, so the index stream from HBM
// overlaps the gathers and arithmetic instead of waiting at the head of every chunk.
__device__ __forceinline__ void cull_face(const DView& v, int f, uint32_t view, int4 iv, bool& valid,
                                          bool& needs_clip, RasterRec& r) {
  const int pi[3] = {iv.x, iv.y, iv.z};
  float4 sv[3];
#pragma unroll
  for (int k = 0; k < 3; k++) sv[k] = __ldg(&v.sv[pi[k]]);
  bool accept = sv_normal(sv[0]) && sv_normal(sv[1]) && sv_normal(sv[2]);
  if (!accept) {
    const uint32_t m0 = sv_mask(sv[0]), m1 = sv_mask(sv[1]), m2 = sv_mask(sv[2]);
    if (m0 & m1 & m2 & 0x80u) {
      // all three visible, one with w < 1e-5: fast accept (graphics.cpp:140-148), divide here
      accept = true;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const F3 n = ndc_of(clip_of(v, pi[k]));
        sv[k] = make_float4(n.x, n.y, n.z, 0.f);
      }
    } else {
      needs_clip = !clip_trivially_empty(m0, m1, m2);
    }
  }
  if (accept)
    valid = build_rec(v, {sv[0].x, sv[0].y, sv[0].z}, {sv[1].x, sv[1].y, sv[1].z}, {sv[2].x, sv[2].y, sv[2].z},
                      (uint32_t)f << 4, view, r);
}

__global__ void __launch_bounds__(kSetupThreads, 8) k_setup(const DView* __restrict__ views, int nviews,
                                                         int nchunks, Scratch sc) {
  __shared__ int32_t s_base[kSharedViews];
  const int32_t* base = share_bases(views, nviews, s_base, SchBase());
  int c = (int)blockIdx.x;
  const int c_end = nchunks;
  if (c >= c_end) return;
  Chunk ch = setup_chunk(views, base, nviews, c, 0);
  int4 iv = make_int4(0, 0, 0, 0);
  if (ch.begin + (int)threadIdx.x < ch.end) iv = __ldg(&views[ch.view].fv[ch.begin + (int)threadIdx.x]);
  for (;;) {
    // the next chunk's face indices: issued now, consumed next iteration
    const bool more = c + (int)gridDim.x < c_end;
    Chunk chn = ch;
    int4 ivn = make_int4(0, 0, 0, 0);
    if (more) {
      chn = setup_chunk(views, base, nviews, c + (int)gridDim.x, ch.view);
      if (chn.begin + (int)threadIdx.x < chn.end) ivn = __ldg(&views[chn.view].fv[chn.begin + (int)threadIdx.x]);
    }
    const DView& v = views[ch.view];
    const int f = ch.begin + (int)threadIdx.x;
    bool needs_clip = false, valid = false;
    RasterRec r;
    if (f < ch.end) cull_face(v, f, (uint32_t)ch.view, iv, valid, needs_clip, r);
    const uint32_t slot = block_reserve<kSetupThreads>(valid, &sc.ctl->rec_count);
    if (valid) {
      if (slot < sc.rec_cap) {
        store_rec(&sc.recs[slot], r);
      } else {
        atomicOr(&sc.ctl->error, kErrRecOverflow);
      }
    }
    const uint32_t cslot = warp_reserve(needs_clip, &sc.ctl->clip_count);
    if (needs_clip) {
      if (cslot < sc.clip_cap) sc.clipq[cslot] = make_int2(ch.view, f);
      else atomicOr(&sc.ctl->error, kErrClipOverflow);
    }
    if (!more) break;
    c += (int)gridDim.x;
    ch = chn;
    iv = ivn;
  }
}

// Payload of an unclipped face (Payload layout): the corner varyings of its three vertex()
// calls and their 1/w.  A mesh whose corners index positions, normals and uvs alike gives each
// corner's attributes in one 32-byte sector (DView::pk), and the corner's 1/w is computed from
// its position with the operations k_vertex used for the screen vertex (clip = mvp * [p, 1],
// 1 / clip.w; graphics.cpp:333-337), so no screen vertex is gathered again.
__device__ __forceinline__ void face_payload(const DView& v, int f, int nf4, int4 iv, Payload& pl) {
  int4 it = iv, in = iv;  // meshes whose v, vt and vn indices agree skip two loads
  if (!v.unified) {
    if (v.uv && nf4 >= 3) it = __ldg(&v.fvt[f]);
    if (v.world & kWorldNormal) in = __ldg(&v.fvn[f]);
  }
  const int pi[3] = {iv.x, iv.y, iv.z}, ti[3] = {it.x, it.y, it.z}, ni[3] = {in.x, in.y, in.z};
  const bool shadow = v.shader == HSR_SHADER_SHADOW;
  const bool need_nrm = (v.world & kWorldNormal) != 0u;
  const bool need_uv = v.uv && nf4 >= 3;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float px, py, pz, nx = 0.f, ny = 0.f, nz = 0.f;
    float2 t = make_float2(0.f, 0.f);
    if (v.pk) {
      const float4 a = __ldg(&v.pk[2 * pi[k]]);
      px = a.x; py = a.y; pz = a.z; nx = a.w;
      if (need_nrm || need_uv) {
        const float4 b = __ldg(&v.pk[2 * pi[k] + 1]);
        ny = b.x; nz = b.y; t = make_float2(b.z, b.w);
      }
    } else {
      const float4 p = __ldg(v.p4 + pi[k]);
      px = p.x; py = p.y; pz = p.z;
      if (need_nrm) {
        const float4 n = __ldg(v.n4 + ni[k]);
        nx = n.x; ny = n.y; nz = n.z;
      }
      if (need_uv) t = __ldg(&v.uv[ti[k]]);
    }
    const float4 c = mat_vec(v.mvp, px, py, pz, 1.f);  // ObjectToClipPos (IShader.h:55-61)
    const float4 wp = (v.world & kWorldPos) ? world_pos(v, px, py, pz) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 wn = need_nrm ? world_normal(v, nx, ny, nz) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (!need_uv) t = make_float2(0.f, 0.f);
    pl.f[k] = fd(1.f, c.w);  // recip_w
    // ShadowShader's interpolated clip z (ObjectToViewPos, IShader.cpp:170-174), else intensity
    pl.f[3 + k] = shadow ? c.z : wn.w;
    pl.f[6 + 2 * k] = t.x;
    pl.f[7 + 2 * k] = t.y;
    pl.f[12 + 3 * k] = wn.x; pl.f[13 + 3 * k] = wn.y; pl.f[14 + 3 * k] = wn.z;
    pl.f[21 + 3 * k] = wp.x; pl.f[22 + 3 * k] = wp.y; pl.f[23 + 3 * k] = wp.z;
  }
  pl.f[30] = 0.f;
  pl.f[31] = 0.f;
}

// Emit pass over the records of k_setup (dense: one thread per surviving triangle): the
// shading payload, the tile counts, and the hand-over of huge triangles to k_big (their
// slot becomes a hole the binning skips).  Grid-stride with warp-uniform trip counts, so
// the warp collectives of append_small see every lane.
__global__ void __launch_bounds__(kEmitThreads, 4) k_emit(const DView* __restrict__ views, int T, Scratch sc) {
  const int lane = threadIdx.x & 31;
  if (sc.ctl->error & kErrCapacity) return;
  const uint32_t nrec = min(sc.ctl->rec_count, sc.rec_cap);
  const uint32_t stride = gridDim.x * blockDim.x;
  uint32_t pay_bytes = 0;  // payload bytes this lane wrote for the raster (big ones: k_big)
  for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < nrec; i0 += stride) {
    const uint32_t i = i0 + (uint32_t)lane;
    bool valid = false;
    RasterRec r;
    Payload pl;
    int nf4 = 0;
    const DView* v = views;
    if (i < nrec) {
      // the words this pass needs (seq, view, pixel range: the record's last 16 bytes); the
      // whole record only for a huge triangle.  Every record below the count is the cull
      // pass's: the clipper and k_big append theirs after this pass.
      const uint4 a = *reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(&sc.recs[i]) + 48);
      r.seq = a.x; r.view = a.y; r.xr = a.z; r.yr = a.w;
      valid = true;
      v = views + (r.view & kRecViewMask);
      nf4 = payload_f4(v->shader);
      if (nf4 > 0) {
        const int f = (int)(r.seq >> 4);
        face_payload(*v, f, nf4, __ldg(&v->fv[f]), pl);
      }
    }
    int tx0, ty0, ntw, nt = 0;
    if (valid) rec_tiles(r, T, tx0, ty0, ntw, nt);
    const bool big = valid && nt > kMaxRecordTiles;
    const bool small = valid && !big;
    if (small) {
      pay_bytes += 16u * (uint32_t)nf4;
    }
    append_counts(small, i, r, pl, nf4, *v, T, sc, true);
    const uint32_t bslot = warp_reserve(big, &sc.ctl->big_count);
    if (big) {
      r = sc.recs[i];
      sc.recs[i].view = r.view | (kRecHole << kRecFlagShift);
      if (bslot < sc.big_cap) {
        store_rec(&sc.bigq[bslot].rec, r);
        store_payload(&sc.bigq[bslot].pay, pl, nf4);
      } else {
        atomicOr(&sc.ctl->error, kErrBigOverflow);
      }
    }
  }
  pay_bytes = __reduce_add_sync(kFull, pay_bytes);
  if (lane == 0 && pay_bytes) atomicAdd(&sc.ctl->pay_bytes, (unsigned long long)pay_bytes);
}

int launch_emit(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s) {
  k_emit<<<grid, kEmitThreads, 0, s>>>(views, tile, sc);
  return (int)cudaGetLastError();
}

// Homogeneous clipping (graphics.cpp:73-161), two faces per warp: each half-warp clips its own
// face (`active`), lane k of the half carrying varying k of the polygon through
// Sutherland-Hodgman while every lane evaluates the plane tests on the clip coordinates; lanes
// j < n-2 of the half then build the fan triangles (:394-405).  The halves run the same
// instructions, each masked to its own polygon; every __syncwarp is reached by all 32 lanes.
__device__ void clip_face(bool active, const DView& v, int view, int face, int T, const Scratch& sc, float* A,
                          float* B) {
  const int lane = threadIdx.x & 31, hl = lane & 15;
  if (active && hl < 3) {
    const int4 iv = __ldg(&v.fv[face]), it = __ldg(&v.fvt[face]), in = __ldg(&v.fvn[face]);
    const int pi = hl == 0 ? iv.x : (hl == 1 ? iv.y : iv.z);
    const int ti = hl == 0 ? it.x : (hl == 1 ? it.y : it.z);
    const int ni = hl == 0 ? in.x : (hl == 1 ? in.y : in.z);
    float* o = A + hl * kPolyStride;
    const float4 c = clip_of(v, pi);
    o[0] = c.x; o[1] = c.y; o[2] = c.z; o[3] = c.w;
    const float4 wp = (v.world & kWorldPos) ? world_pos_of(v, pi) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 wn = (v.world & kWorldNormal) ? world_normal_of(v, ni) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 t = v.uv ? __ldg(&v.uv[ti]) : make_float2(0.f, 0.f);
    o[4] = wp.x; o[5] = wp.y; o[6] = wp.z;
    o[7] = wn.x; o[8] = wn.y; o[9] = wn.z;
    o[10] = t.x; o[11] = t.y; o[12] = wn.w;
  }
  __syncwarp();
  int n = active ? 3 : 0;
  float* src = A;
  float* dst = B;
#pragma unroll
  for (int plane = PW; plane <= NZ; plane++) {
    // a polygon with fewer than 3 vertices is dropped (its later planes are skipped)
    int m = 0;
    if (n >= 3) {
      for (int i = 0; i < n; i++) {
        const float* prev = src + (i == 0 ? n - 1 : i - 1) * kPolyStride;
        const float* curr = src + i * kPolyStride;
        const bool pin = inside_plane(prev, plane), cin = inside_plane(curr, plane);
        if (pin != cin) {
          const float t = intersect_ratio(prev, curr, plane);
          if (hl < kVaryings) dst[m * kPolyStride + hl] = fa(prev[hl], fm(fs(curr[hl], prev[hl]), t));
          m++;
        }
        if (cin) {
          if (hl < kVaryings) dst[m * kPolyStride + hl] = curr[hl];
          m++;
        }
      }
      n = m;
    }
    __syncwarp();
    float* tmp = src; src = dst; dst = tmp;
  }
  bool valid = false;
  RasterRec r;
  Payload pl;
  if (n >= 3 && hl < n - 2) {
    const float* p0 = src;
    const float* p1 = src + (hl + 1) * kPolyStride;
    const float* p2 = src + (hl + 2) * kPolyStride;
    valid = build_rec(v, ndc_of(make_float4(p0[0], p0[1], p0[2], p0[3])), ndc_of(make_float4(p1[0], p1[1], p1[2], p1[3])),
                      ndc_of(make_float4(p2[0], p2[1], p2[2], p2[3])), ((uint32_t)face << 4) | ((uint32_t)hl << 1) | 1u,
                      (uint32_t)view, r);
    if (valid) make_payload(v.shader, p0, p1, p2, pl);
  }
  int tx0, ty0, ntw, nt = 0;
  if (valid) rec_tiles(r, T, tx0, ty0, ntw, nt);
  const bool big = valid && nt > kMaxRecordTiles;
  const int nf4 = payload_f4(v.shader);
  const uint32_t slot = warp_reserve(valid && !big, &sc.ctl->rec_count);
  append_small(valid && !big, slot, r, pl, nf4, v, T, sc);
  const uint32_t pb = __reduce_add_sync(kFull, (valid && !big && slot < sc.rec_cap) ? 16u * (uint32_t)nf4 : 0u);
  if (lane == 0 && pb) atomicAdd(&sc.ctl->pay_bytes, (unsigned long long)pb);
  const uint32_t bslot = warp_reserve(big, &sc.ctl->big_count);
  if (big) {
    if (bslot < sc.big_cap) {
      store_rec(&sc.bigq[bslot].rec, r);
      store_payload(&sc.bigq[bslot].pay, pl, nf4);
    } else {
      atomicOr(&sc.ctl->error, kErrBigOverflow);
    }
  }
  __syncwarp();
}

constexpr int kPostThreads = 256;

// Drains the clip queue of k_setup, two faces per warp.  Face pairs are claimed one ahead, so
// the claim's round trip overlaps the current pair; the grid fills every SM (the queue is short
// and each face is a chain of dependent loads, so resident warps set the throughput).
__global__ void __launch_bounds__(kPostThreads, 3) k_post(const DView* __restrict__ views, int T, Scratch sc) {
  __shared__ float poly[kPostThreads / 32][2][2][16 * kPolyStride];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, half = lane >> 4;
  if (sc.ctl->error & kErrCapacity) return;
  const uint32_t nclip = min(sc.ctl->clip_count, sc.clip_cap);
  uint32_t item = 0, ahead = 0;
  if (lane == 0) {
    item = atomicAdd(&sc.ctl->post_next, 2u);
    ahead = item < nclip ? atomicAdd(&sc.ctl->post_next, 2u) : nclip;
  }
  item = __shfl_sync(kFull, item, 0);
  for (;;) {
    if (item >= nclip) break;
    const uint32_t next = __shfl_sync(kFull, ahead, 0);
    if (lane == 0) ahead = next < nclip ? atomicAdd(&sc.ctl->post_next, 2u) : nclip;
    const uint32_t mine = item + (uint32_t)half;
    const bool active = mine < nclip;
    const int2 vf = active ? sc.clipq[mine] : make_int2(0, 0);
    clip_face(active, views[vf.x], vf.x, vf.y, T, sc, poly[warp][half][0], poly[warp][half][1]);
    item = next;
  }
}

int launch_post(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s) {
  k_post<<<grid, kPostThreads, 0, s>>>(views, tile, sc);
  return (int)cudaGetLastError();
}

constexpr int kBigThreads = 512;

// Expands each queued huge triangle with a whole CTA: its tile rectangle splits into
// sub-records over blocks of kSubTilesX x kSubTilesY tiles (same triangle constants and
// seq, pixel range clipped to the block, one shared payload at the first sub-record's
// slot), and every tile of the rectangle is counted once.  The sub-ranges partition the
// triangle's pixel range, so each pixel is still tested exactly once.
__global__ void __launch_bounds__(kBigThreads) k_big(const DView* __restrict__ views, int T, Scratch sc) {
  __shared__ uint32_t s_base;
  if (sc.ctl->error & kErrCapacity) return;
  const uint32_t nbig = min(sc.ctl->big_count, sc.big_cap);
  for (uint32_t item = blockIdx.x; item < nbig; item += gridDim.x) {
    const BigItem& bi = sc.bigq[item];
    const RasterRec b = bi.rec;
    const DView& v = views[b.view & kRecViewMask];
    int tx0, ty0, ntw, nt;
    rec_tiles(b, T, tx0, ty0, ntw, nt);
    const int nth = nt / ntw;
    const int nbx = (ntw + kSubTilesX - 1) / kSubTilesX, nby = (nth + kSubTilesY - 1) / kSubTilesY;
    const int nsub = nbx * nby;
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint32_t base = atomicAdd(&sc.ctl->rec_count, (uint32_t)nsub);
      s_base = base;
      if ((uint64_t)base + (uint64_t)nsub > (uint64_t)sc.rec_cap) atomicOr(&sc.ctl->error, kErrRecOverflow);
    }
    __syncthreads();
    const uint32_t base = s_base;
    if ((uint64_t)base + (uint64_t)nsub > (uint64_t)sc.rec_cap) continue;
    // every sub-record carries its own copy of the payload, so that a record's payload index is
    // its own index (the raster loads the payload from the record index in shared memory)
    const int nf4 = payload_f4(v.shader);
    for (int k = threadIdx.x; k < nsub * nf4; k += kBigThreads)
      reinterpret_cast<float4*>(&sc.pay[base + (uint32_t)(k / nf4)])[k % nf4] =
          reinterpret_cast<const float4*>(&bi.pay)[k % nf4];
    if (threadIdx.x == 0 && nf4) atomicAdd(&sc.ctl->pay_bytes, 16ull * (unsigned long long)(nf4 * nsub));
    const int x0 = (int)(b.xr & 0xffffu), x1 = (int)(b.xr >> 16);
    const int y0 = (int)(b.yr & 0xffffu), y1 = (int)(b.yr >> 16);
    for (int sidx = threadIdx.x; sidx < nsub; sidx += kBigThreads) {
      const int bx = sidx % nbx, by = sidx / nbx;
      const int stx0 = tx0 + bx * kSubTilesX, stx1 = min(tx0 + ntw - 1, stx0 + kSubTilesX - 1);
      const int sty0 = ty0 + by * kSubTilesY, sty1 = min(ty0 + nth - 1, sty0 + kSubTilesY - 1);
      RasterRec w = b;
      w.xr = (uint32_t)max(x0, stx0 * T) | ((uint32_t)min(x1, stx1 * T + T - 1) << 16);
      w.yr = (uint32_t)max(y0, sty0 * T) | ((uint32_t)min(y1, sty1 * T + T - 1) << 16);
      w.pad = 0u;
      store_rec(&sc.recs[base + (uint32_t)sidx], w);
    }
    for (int k = threadIdx.x; k < nt; k += kBigThreads)
      atomicAdd(&sc.tile_count[v.tile_base + (ty0 + k / ntw) * v.tiles_x + tx0 + k % ntw], 1u);
  }
}

int launch_big(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s) {
  k_big<<<grid, kBigThreads, 0, s>>>(views, tile, sc);
  return (int)cudaGetLastError();
}

int launch_setup(const DView* views, int nviews, int nchunks, Scratch sc, int grid, cudaStream_t s) {
  if (nchunks <= 0) return 0;
  k_setup<<<std::max(1, std::min(grid, nchunks)), kSetupThreads, 0, s>>>(views, nviews, nchunks, sc);
  return (int)cudaGetLastError();
}

}  // namespace hsr
