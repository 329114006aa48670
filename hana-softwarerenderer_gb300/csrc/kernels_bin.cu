// kernels_bin.cu — tile binning (sm_103a).  The reference has no binning: it loops over
// each triangle's bounding box (graphics.cpp:349-375).  Here the (record, tile) pairs are
// laid out per tile so that one warp can own a tile in the raster.
//
// k_scan    exclusive prefix sums of the per-tile counts and of the non-empty tiles, single
//           pass with decoupled look-back, and the list of non-empty tiles in tile order;
//           block order comes from a ticket so a block only waits on blocks that already
//           run, and every wait is bounded (error bit + give up, never a hang).
// k_scatter writes record indices into the per-tile lists with warp-aggregated atomics;
//           a record touches at most kMaxRecordTiles tiles (k_big splits larger ones).
//           The same grid clears the tiles no record touches, streamed in row order.
#include "hsr_device.cuh"

namespace hsr {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // tiles per scan block
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPre = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

__host__ __device__ __forceinline__ int scan_blocks_hd(int ntiles) { return (ntiles + kScanTile - 1) / kScanTile; }
int scan_blocks(int ntiles) { return scan_blocks_hd(ntiles); }

__device__ __forceinline__ unsigned long long ld_volatile64(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// Scan word: bits 0-35 the count prefix, bits 36-61 the non-empty tile prefix, 62-63 the
// look-back flags.  Neither field can carry into the next: a batch has fewer than 2^26
// tiles (kMaxBatchTiles), and 2^36 (record, tile) pairs would need more records than the
// device memory holds (each record touches at most kMaxRecordTiles tiles).
constexpr int kCntBits = 36;
constexpr unsigned long long kCntMask = (1ull << kCntBits) - 1;
constexpr unsigned long long kOneTile = 1ull << kCntBits;

__device__ __forceinline__ unsigned long long scan_item(uint32_t count) {
  return (unsigned long long)count + (count ? kOneTile : 0ull);
}

__global__ void __launch_bounds__(kScanThreads) k_scan(Scratch sc) {
  __shared__ unsigned long long warp_sums[kScanThreads / 32];
  __shared__ unsigned long long s_prefix;
  __shared__ uint32_t s_block;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_block = atomicAdd(&sc.ctl->scan_ticket, 1u);
  __syncthreads();
  const uint32_t blk = s_block;
  const int base = (int)blk * kScanTile + (int)threadIdx.x * kScanItems;
  uint32_t vals[kScanItems];
  unsigned long long local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    vals[k] = (base + k < sc.ntiles) ? sc.tile_count[base + k] : 0u;
    local += scan_item(vals[k]);
  }
  // block-wide exclusive scan of the thread sums
  unsigned long long incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    const unsigned long long w = lane < kScanThreads / 32 ? warp_sums[lane] : 0ull;
    unsigned long long wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned long long y = __shfl_up_sync(kFull, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = wi - w;  // exclusive per warp
    if (lane == kScanThreads / 32 - 1) {
      // lane 7 holds the block aggregate; publish and look back
      const unsigned long long agg = wi;
      unsigned long long* st = sc.scan_status;
      unsigned long long prefix = 0;
      const long limit = sc.poll_limit > 0 ? (long)sc.poll_limit : kScanWaitPolls;
      if (blk == 0 && (sc.faults & HSR_FAULT_SCAN_STALL)) {
        // injected stall: withhold the prefix and wait on a word nothing sets (its own)
        long spins = 0;
        while ((ld_volatile64(&st[0]) >> 62) == 0) {
          if (++spins > limit) {
            atomicOr(&sc.ctl->error, kErrScanTimeout);
            break;
          }
          __nanosleep(64);
        }
      } else if (blk == 0) {
        atomicExch(&st[0], kFlagPre | agg);
      } else {
        atomicExch(&st[blk], kFlagAgg | agg);
        unsigned long long acc = 0;
        int p = (int)blk - 1;
        long spins = 0;
        while (p >= 0) {
          const unsigned long long s = ld_volatile64(&st[p]);
          if ((s >> 62) == 0) {
            if (++spins > limit) {
              atomicOr(&sc.ctl->error, kErrScanTimeout);
              break;
            }
            __nanosleep(64);
            continue;
          }
          acc += s & kValMask;
          if ((s >> 62) == 2) break;
          p--;
        }
        prefix = acc;
        atomicExch(&st[blk], kFlagPre | (acc + agg));
      }
      s_prefix = prefix;
      if ((int)blk == scan_blocks_hd(sc.ntiles) - 1) {
        const unsigned long long total = prefix + agg;
        const unsigned long long pairs = total & kCntMask;
        const uint32_t ne = (uint32_t)(total >> kCntBits);
        sc.ctl->bin_total = (uint32_t)min(pairs, 0xffffffffull);
        if (pairs > sc.bin_cap) atomicOr(&sc.ctl->error, kErrBinOverflow);
        sc.ctl->ne_tiles = ne;
        sc.ne_off[sc.ntiles] = ne;
      }
    }
  }
  __syncthreads();
  unsigned long long run = s_prefix + warp_sums[warp] + (incl - local);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    const int t = base + k;
    if (t < sc.ntiles) {
      const uint32_t ne = (uint32_t)(run >> kCntBits);
      sc.tile_off[t] = (uint32_t)(run & kCntMask);  // below bin_cap unless the batch overflows
      sc.ne_off[t] = ne;
      if (vals[k]) sc.tile_list[ne] = (uint32_t)t;
    }
    run += scan_item(vals[k]);
  }
}

int launch_scan(Scratch sc, cudaStream_t s) {
  const int nb = scan_blocks(sc.ntiles);
  if (nb <= 0) return 0;
  k_scan<<<nb, kScanThreads, 0, s>>>(sc);
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
// (record, tile) pairs into the per-tile lists, records [first block's, nrec) in steps of
// `nblocks` blocks.
__device__ __forceinline__ void scatter_records(const DView* __restrict__ views, int T, const Scratch& sc, uint32_t block,
                                                uint32_t nblocks) {
  const int lane = threadIdx.x & 31;
  const uint32_t nrec = min(sc.ctl->rec_count, sc.rec_cap);
  if (sc.ctl->error & kErrNoDraw) return;
  const uint32_t stride = nblocks * blockDim.x;
  const int ts = __ffs(T) - 1;  // T is a power of two
  // warp-uniform trip count so every lane takes part in the warp-level collectives
  for (uint32_t i0 = block * blockDim.x + (threadIdx.x & ~31u); i0 < nrec; i0 += stride) {
    const uint32_t i = i0 + (uint32_t)lane;
    const bool ok = i < nrec;
    int tx0 = 0, ty0 = 0, ntw = 0, nt = 0, tbase = 0, tiles_x = 0;
    // the record's view and pixel range: its last 16 bytes (seq, view, xr, yr) in one load
    const uint4 w = ok ? *reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(&sc.recs[i]) + 48)
                       : make_uint4(0u, kRecHole << kRecFlagShift, 0u, 0u);
    if (ok && !((w.y >> kRecFlagShift) & kRecHole)) {  // holes: huge triangles split by k_big
      const uint32_t xr = w.z, yr = w.w;
      const DView& v = views[w.y & kRecViewMask];
      tbase = v.tile_base;
      tiles_x = v.tiles_x;
      tx0 = (int)(xr & 0xffffu) >> ts;
      ty0 = (int)(yr & 0xffffu) >> ts;
      ntw = ((int)(xr >> 16) >> ts) - tx0 + 1;
      nt = ntw * (((int)(yr >> 16) >> ts) - ty0 + 1);
    }
    const int my_n = min(nt, kMaxRecordTiles);
    const int maxn = __reduce_max_sync(kFull, my_n);
    int kx = 0, ky = 0;  // tile k of the rectangle, row-major
    for (int k = 0; k < maxn; k++) {
      const int tile = (k < my_n) ? tbase + (ty0 + ky) * tiles_x + tx0 + kx : -1;
      if (++kx == ntw) { kx = 0; ky++; }
      const unsigned grp = __match_any_sync(kFull, tile);
      const int leader = __ffs(grp) - 1;
      uint32_t b = 0;
      if (tile >= 0 && lane == leader) b = atomicAdd(&sc.tile_fill[tile], (uint32_t)__popc(grp));
      b = __shfl_sync(kFull, b, leader);
      if (tile >= 0) {
        const uint32_t pos = sc.tile_off[tile] + b + (uint32_t)__popc(grp & ((1u << lane) - 1u));
        if (pos < sc.bin_cap) sc.bins[pos] = i;
      }
    }
  }
}

// The fused clear (renderbuffer_clear_color / renderbuffer_clear_depth, renderbuffer.cpp:59-75,
// prim ids -> 0) of the pixels whose tile holds no record: the raster visits only the
// non-empty tiles and writes every pixel of those.  A chunk is kClearChunk consecutive pixels
// of one view in row-major order, so a warp's stores form one contiguous run per plane (16 bytes
// a lane where four neighbours are all cleared); the pixel's tile count (the same word for up
// to T neighbours) decides whether it is written.
// Block `block` of the `nblocks` clearing blocks takes chunks warp by warp; `cbase` holds the
// views' chunk bases when the batch has at most kSharedViews views (else null).
__device__ __forceinline__ void clear_empty_tiles(const DView* __restrict__ views, int T, int nchunks, const Scratch& sc,
                                                  int block, int nblocks, const int32_t* cbase) {
  if (sc.ctl->error & kErrNoDraw) return;  // an overflowing or stalled sequence draws nothing
  const int ts = __ffs(T) - 1;
  const int nv = sc.nviews;
  const int lane = (int)threadIdx.x & 31, wpb = (int)blockDim.x >> 5;
  // one chunk per warp at a time: each warp's view lookup and tile counts are an independent
  // chain of loads, so a block keeps several chunks in flight
  for (int c = block * wpb + ((int)threadIdx.x >> 5); c < nchunks; c += nblocks * wpb) {
    // the view of chunk c: the last view whose base is <= c (views without chunks share
    // their successor's base and are never the last such view)
    int lo = 0, hi = nv - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((cbase ? cbase[mid] : views[mid].cch_base) <= c) lo = mid; else hi = mid - 1;
    }
    const DView& v = views[lo];
    const int W = v.W, npx = v.W * v.H;  // below 2^30 (targets are at most 32768 x 32768)
    const int cbeg = (c - v.cch_base) * kClearChunk, cend = min(cbeg + kClearChunk, npx);
    const int32_t tb = v.tile_base, tx = v.tiles_x;
    // groups of 4 consecutive pixels (a group may run on into the next row): lane l takes the
    // groups starting at cbeg + 4l + 128k, k < kGroups; all of a lane's tile counts are in
    // flight before its stores
    constexpr int kGroups = kClearChunk / 128;
    const int g0 = cbeg + 4 * lane;
    int y = g0 / W, x = g0 - y * W;
    const int qy = 128 / W, qx = 128 - qy * W;  // the step of 128 pixels in rows and columns
    uint32_t empty = 0;  // bit 4k + d: pixel g0 + 128k + d is in the chunk and its tile has no record
#pragma unroll
    for (int k = 0; k < kGroups; k++) {
#pragma unroll
      for (int d = 0; d < 4; d++) {
        int xx = x + d, yy = y;
        if (xx >= W) {  // the group runs on into the next row(s)
          yy += xx / W;
          xx -= (xx / W) * W;
        }
        if (g0 + 128 * k + d < cend && sc.tile_count[tb + (yy >> ts) * tx + (xx >> ts)] == 0u)
          empty |= 1u << (4 * k + d);
      }
      x += qx;
      y += qy;
      if (x >= W) { x -= W; y++; }
    }
    if (!__any_sync(0xffffffffu, empty != 0u)) continue;
    const uint32_t rgba = v.clear_rgba;
    const float depth = v.clear_depth;
    uint32_t* const prim = v.prim;
    // a group starts at a multiple of 4 pixels, so with 16-byte aligned planes (the library
    // allocates them 256-byte aligned) a full group is one 16-byte store per plane
    const bool vec = ((reinterpret_cast<uintptr_t>(v.color) | reinterpret_cast<uintptr_t>(v.depth) |
                       reinterpret_cast<uintptr_t>(prim)) & 15u) == 0u;
#pragma unroll
    for (int k = 0; k < kGroups; k++) {
      const uint32_t m = (empty >> (4 * k)) & 15u;
      if (!m) continue;
      const int i = g0 + 128 * k;
      if (m == 15u && vec) {
        *reinterpret_cast<uint4*>(v.color + i) = make_uint4(rgba, rgba, rgba, rgba);
        *reinterpret_cast<float4*>(v.depth + i) = make_float4(depth, depth, depth, depth);
        if (prim) *reinterpret_cast<uint4*>(prim + i) = make_uint4(0u, 0u, 0u, 0u);
      } else {
#pragma unroll
        for (int d = 0; d < 4; d++) {
          if (m >> d & 1u) {
            v.color[i + d] = rgba;
            v.depth[i + d] = depth;
            if (prim) prim[i + d] = 0u;
          }
        }
      }
    }
  }
}

// Scatter and clear in one grid: every kClearEvery-th block clears (when the batch has clear
// chunks), the others scatter, so the store-bound clear runs beside the atomic-bound scatter
// instead of after it.
constexpr int kClearEvery = 2;

__global__ void __launch_bounds__(256) k_scatter(const DView* __restrict__ views, int T, Scratch sc, int nchunks) {
  __shared__ int32_t s_cbase[kSharedViews];
  const uint32_t b = blockIdx.x, g = gridDim.x;
  if (nchunks > 0 && b % kClearEvery == kClearEvery - 1) {  // block-uniform
    const bool in_shared = sc.nviews <= kSharedViews;
    if (in_shared)
      for (int i = threadIdx.x; i < sc.nviews; i += blockDim.x) s_cbase[i] = views[i].cch_base;
    __syncthreads();
    clear_empty_tiles(views, T, nchunks, sc, (int)(b / kClearEvery), (int)(g / kClearEvery), in_shared ? s_cbase : nullptr);
  } else if (nchunks > 0) {
    scatter_records(views, T, sc, b - b / kClearEvery, g - g / kClearEvery);
  } else {
    scatter_records(views, T, sc, b, g);
  }
}

// `grid` blocks of 256 threads (at least kClearEvery when the batch clears, so both parts
// have blocks).
int launch_scatter(const DView* views, int tile, Scratch sc, int grid, int nchunks, cudaStream_t s) {
  if (nchunks > 0 && grid < kClearEvery) grid = kClearEvery;
  k_scatter<<<grid > 0 ? grid : 1, 256, 0, s>>>(views, tile, sc, nchunks);
  return (int)cudaGetLastError();
}

}  // namespace hsr
