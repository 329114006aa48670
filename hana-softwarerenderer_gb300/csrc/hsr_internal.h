// hsr_internal.h — data layout shared by the host runtime and the sm_103a kernels.
//
// Pipeline of one launch sequence (a batch of views = draws):
//   k_vertex  : SoA positions -> screen vertex per view (world attributes are transformed per
//               corner where a triangle survives: k_emit, and the clipper)
//   k_setup   : per face: fast accept or homogeneous clip (graphics.cpp:132-161), then per
//               fan triangle divide / cull / viewport / bbox (graphics.cpp:314-347) -> one
//               64-byte RasterRec, plus per-tile counts (warp-aggregated atomics)
//   k_scan    : exclusive prefix sums of the per-tile counts and of the non-empty tiles
//               (decoupled look-back), and the list of non-empty tiles in tile order
//   k_scatter : (record, tile) pairs into per-tile lists; beside it, in the same grid, the
//               fused clear of the tiles no triangle touches, streamed row by row
//   k_raster  : persistent over the non-empty tiles; one warp owns one screen tile,
//               resolves visibility per pixel as min over (depth, later-submitted) — the
//               sequential loop's result — then shades the winners and writes colour /
//               depth / prim id once.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/hsr.h"

namespace hsr {

constexpr int kMaxPoly = 10;              // 3 vertices + one per clip plane (7 planes)
constexpr int kVaryings = 13;             // floats in shader_struct_v2f (IShader.h:41-47)
constexpr int kMaxRecordTiles = 32;       // records never touch more tiles (big ones are split)
constexpr int kSubTilesX = 8, kSubTilesY = 4;  // tile block of one sub-record
constexpr int kPayloadFloats = 32;        // per-record shading payload (see Payload layout)

// Error bits in Ctl::error.
enum : uint32_t {
  kErrRecOverflow = 1u,
  kErrClipOverflow = 2u,
  kErrBinOverflow = 4u,
  kErrWaitTimeout = 8u,
  kErrScanTimeout = 16u,
  kErrBigOverflow = 32u,
};
constexpr uint32_t kErrCapacity = kErrRecOverflow | kErrClipOverflow | kErrBinOverflow | kErrBigOverflow;
// A sequence with one of these draws nothing: the binning and the raster return before
// writing (an overflow is re-run with larger scratch; a scan that gave up has no tile lists).
constexpr uint32_t kErrNoDraw = kErrCapacity | kErrScanTimeout;
// Default poll limits of the bounded waits (Scratch::poll_limit overrides both).
constexpr long kDepWaitPolls = 1L << 23;   // raster: a shadow map's tiles (~1-2 s)
constexpr long kScanWaitPolls = 1L << 22;  // scan: a predecessor block's prefix

// Record flags.
enum : uint32_t {
  kRecExact = 1u,  // coordinates outside the range where the division-free coverage test is
                   // exact: the raster evaluates the reference's divisions instead
  kRecHole = 2u,   // slot of a huge triangle handed to k_big: binned nowhere
};

// One triangle that reached the raster (64 bytes).  A, B-A, C-A are the per-triangle
// constants of barycentric() (graphics.cpp:222-233); uz is u.z, constant per triangle.  The
// last 16 bytes are the words the emit pass and the scatter read (one 16-byte load each); a
// record's payload is at the record's own index.
struct __align__(16) RasterRec {
  float ax, ay, e1x, e1y;   // A; e1 = B - A
  float e2x, e2y, uz, d0;   // e2 = C - A; u.z; screen depth of A
  float d1, d2;             // screen depths of B, C
  uint32_t rsv, pad;        // reserved (zero)
  uint32_t seq;             // (face << 4) | (fan << 1) | clipped — submission order
  uint32_t view;            // index of the view in the batch | flags << 28 (kRec*)
  uint32_t xr, yr;          // inclusive pixel range: x0 | x1 << 16, y0 | y1 << 16
};
static_assert(offsetof(RasterRec, seq) == 48 && offsetof(RasterRec, yr) == 60, "binning words in the last 16 bytes");
constexpr uint32_t kRecViewMask = 0x0fffffffu;
constexpr int kRecFlagShift = 28;

// Per-record shading payload (kPayloadFloats floats, same index as the record): the
// reciprocal w of each corner (graphics.cpp:333-337) and the corner varyings the shader
// reads, so that shading a pixel needs the record and this payload only.
//   [0..2] 1/w of corners 0..2, [3] unused,
//   corner k at 4 + 9k: world_pos[3], world_normal[3], uv[2], scalar
//   (scalar = clip_pos.z for ShadowShader, intensity for Ground/Toon).
struct __align__(16) Payload {
  float f[kPayloadFloats];
};
static_assert(sizeof(RasterRec) == 64, "RasterRec must stay 64 bytes");

// Per-draw descriptor on the device.  The fields every raster tile reads come first, in
// one 128-byte line (the struct is 128-byte aligned); the rest is read by the vertex and
// setup stages and by the shading of tiles that hold fragments.
struct __align__(128) DView {
  // target and tiles (read per raster tile)
  uint32_t* color; float* depth; uint32_t* prim; int32_t W, H;
  int32_t tile_base, tiles_x, tiles_y, ntiles;
  int32_t shader;
  uint32_t flags;       // HSR_DRAW_*
  float clear_depth;
  uint32_t clear_rgba;
  // ordering inside the batch: views this one waits for (-1 = none)
  int32_t dep0, dep1;
  int32_t has_dependents;  // another view of the batch waits for this one's tiles
  uint32_t prim_base;
  // mesh (device)
  const float* px; const float* py; const float* pz;   // positions, SoA, padded to 4
  const float* nx; const float* ny; const float* nz;   // normals, SoA, padded to 4
  const float2* uv;
  const int4* fv; const int4* fvt; const int4* fvn;    // per-face corner indices (+pad)
  int32_t npos, nnrm, nuv, nfaces;
  int32_t unified;  // every face corner has equal v, vt and vn indices (fvt, fvn unused)
  // the mesh's positions and normals as (x, y, z, 0), gathered per corner for the world
  // attributes, and which of those the view's shader reads (kWorld*)
  const float4* p4; const float4* n4;
  const float4* pk;  // unified meshes: position, normal and uv of a vertex in one sector (else null)
  uint32_t world;
  // vertex outputs (scratch)
  float4* sv;     // [npos] screen vertex: (x/w, y/w, z/w, 1/w) or plane mask (k_vertex)
  // shading
  float mvp[16];        // camera_vp*model (light_vp*model for SHADOW), host-computed
  hsr_shader_data u;
  const uint32_t* diffuse; int32_t dw, dh, dbpp;
  const uint32_t* normal;  int32_t nw, nh, nbpp;
  // shadow map (colour plane of another target), null when ShaderData::shadow_map is null
  const uint32_t* sm_color; int32_t smW, smH;
  // this view's work chunks in the batch's chunk spaces (a kernel finds the view of chunk c
  // as the last view whose base is <= c): vertex chunks of kVertexChunk positions, setup
  // chunks of kSetupChunk faces, clear chunks of kClearChunk pixels (none for a view drawn
  // without the fused clear)
  int32_t vch_base, vch_npos, vch_count;
  int32_t sch_base;
  int32_t cch_base;
};
constexpr int kVertexChunk = 2048;  // positions per vertex-stage chunk
constexpr uint32_t kWorldPos = 1u, kWorldNormal = 2u;  // DView::world
// The world attributes a shader's fragment() reads (IShader.cpp): the world position for the
// view vector and the shadow lookup, the world normal for lighting (and the intensity of
// Ground / Toon, which rides in its w).
__host__ __device__ inline uint32_t world_attrs(int shader) {
  const bool pos = shader == HSR_SHADER_BLINN || shader == HSR_SHADER_NORMALMAP;
  const bool nrm = shader == HSR_SHADER_GROUND || shader == HSR_SHADER_TOON || shader == HSR_SHADER_TEXTURE_WITH_LIGHT ||
                   shader == HSR_SHADER_BLINN || shader == HSR_SHADER_NORMALMAP;
  return (pos ? kWorldPos : 0u) | (nrm ? kWorldNormal : 0u);
}
constexpr int kSetupChunk = 128;    // faces per setup chunk (one per thread of a block)
constexpr int kClearChunk = 1024;   // pixels per clear chunk (32 per lane of a warp)
constexpr int64_t kMaxBatchTiles = (int64_t)1 << 26;  // tiles of one launch sequence (scan word)
static_assert(offsetof(DView, prim_base) + sizeof(uint32_t) <= 128, "per-tile fields must share one line");

struct Ctl {
  uint32_t rec_count;
  uint32_t clip_count;
  uint32_t tile_next;
  uint32_t scan_ticket;
  uint32_t error;
  uint32_t bin_total;
  uint32_t big_count;      // triangles queued for sub-record expansion
  uint32_t post_next;      // work counter of k_post
  unsigned long long shaded_px;  // pixels whose winner was shaded by the raster
  unsigned long long frag_px;    // covered (pixel, triangle) pairs the raster depth-tested
  uint32_t ne_tiles;             // tiles with at least one record (k_scan)
  uint32_t ctl_pad;
  unsigned long long pay_bytes;  // shading payload bytes written (k_emit, k_post, k_big)
};
static_assert(sizeof(Ctl) == 64, "Ctl is read back whole: keep it one 64-byte block");

// A triangle whose bounding box touches more than kMaxRecordTiles tiles, queued by setup
// and expanded into sub-records by k_post.
struct __align__(16) BigItem {
  RasterRec rec;
  Payload pay;
};

// Work chunk for the vertex and setup kernels: items [begin, end) of one view.
struct Chunk {
  int32_t view;
  int32_t begin;
  int32_t end;
};
constexpr int kSharedViews = 256;  // views whose chunk / tile bases kernels copy to shared memory

// Scratch of one launch sequence (device pointers, sized by the host).
struct Scratch {
  Ctl* ctl;
  uint32_t* view_done;      // [nviews] tiles finished per view
  RasterRec* recs;  uint32_t rec_cap;
  Payload* pay;             // [rec_cap]
  int2* clipq;      uint32_t clip_cap;   // (view, face) of faces that need clipping
  BigItem* bigq;    uint32_t big_cap;
  uint32_t* tile_count;     // [ntiles]
  uint32_t* tile_fill;      // [ntiles]
  uint32_t* tile_off;       // [ntiles]
  uint32_t* ne_off;         // [ntiles + 1] non-empty tiles before each tile
  uint32_t* tile_list;      // [ntiles] the non-empty tiles in tile order (ne_tiles of them)
  unsigned long long* scan_status;  // [scan blocks]
  uint32_t* bins;   uint32_t bin_cap;
  int32_t ntiles;
  int32_t nviews;
  float* stash;             // [stash_warps][stash_floats(tile)] per raster warp (may be null)
  uint32_t stash_warps;
  uint32_t faults;          // HSR_FAULT_* injected by the host (tests of the failure paths)
  int32_t poll_limit;       // polls before a bounded wait gives up (0: the defaults above)
};
// Per raster warp of a 16x16 or 32x32 tile, per pixel: the winner's weights b0, b1, b2 as one
// 16-byte entry — what shading would otherwise re-derive from the record.  (The winner's record
// index, which is also its payload index, and its submission word are in the tile's shared state.)
__host__ __device__ constexpr int stash_floats(int tile) { return 4 * tile * tile; }
constexpr int kStashWarpsPerSm = 32;  // raster warps resident per SM at most

// Kernel launchers (kernels_*.cu).  All return cudaError_t as int.
int launch_vertex(const DView* views, int nviews, int nchunks, int grid, cudaStream_t s);
int launch_setup(const DView* views, int nviews, int nchunks, Scratch sc, int grid, cudaStream_t s);
int launch_emit(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s);
int launch_post(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s);
int launch_big(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s);
int launch_scan(Scratch sc, cudaStream_t s);
int launch_scatter(const DView* views, int tile, Scratch sc, int grid, int clear_chunks, cudaStream_t s);
int launch_raster(const DView* views, int tile, Scratch sc, int grid, int warps, cudaStream_t s);
int scan_blocks(int ntiles);

}  // namespace hsr
