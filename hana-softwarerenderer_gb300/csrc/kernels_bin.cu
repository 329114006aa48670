// kernels_bin.cu — tile binning (sm_103a).  The reference has no binning: it loops over
// each triangle's bounding box (graphics.cpp:349-375).  Here the (record, tile) pairs are
// laid out per tile so that one warp can own a tile in the raster.
//
// k_scan    exclusive prefix sum of per-tile counts, single pass with decoupled look-back;
//           block order comes from a ticket so a block only waits on blocks that already
//           run, and every wait is bounded (error bit + give up, never a hang).
// k_scatter writes record indices into the per-tile lists with warp-aggregated atomics;
//           a record touches at most kMaxRecordTiles tiles (setup splits larger ones).
#include "hsr_device.cuh"

namespace hsr {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;  // tiles per scan block
constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPre = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;
constexpr long kSpinLimit = 1L << 22;

__host__ __device__ __forceinline__ int scan_blocks_hd(int ntiles) { return (ntiles + kScanTile - 1) / kScanTile; }
int scan_blocks(int ntiles) { return scan_blocks_hd(ntiles); }

__device__ __forceinline__ unsigned long long ld_volatile64(const unsigned long long* p) {
  return *reinterpret_cast<const volatile unsigned long long*>(p);
}

__global__ void __launch_bounds__(kScanThreads) k_scan(Scratch sc) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  __shared__ uint32_t s_block, s_prefix;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_block = atomicAdd(&sc.ctl->scan_ticket, 1u);
  __syncthreads();
  const uint32_t blk = s_block;
  const int base = (int)blk * kScanTile + (int)threadIdx.x * kScanItems;
  uint32_t vals[kScanItems];
  uint32_t local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    vals[k] = (base + k < sc.ntiles) ? sc.tile_count[base + k] : 0u;
    local += vals[k];
  }
  // block-wide exclusive scan of the thread sums
  uint32_t incl = local;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0u;
    uint32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = wi - w;  // exclusive per warp
    if (lane == kScanThreads / 32 - 1) {
      // lane 7 holds the block aggregate; publish and look back
      const unsigned long long agg = wi;
      unsigned long long* st = sc.scan_status;
      uint32_t prefix = 0;
      if (blk == 0) {
        atomicExch(&st[0], kFlagPre | agg);
      } else {
        atomicExch(&st[blk], kFlagAgg | agg);
        unsigned long long acc = 0;
        int p = (int)blk - 1;
        long spins = 0;
        while (p >= 0) {
          unsigned long long s = ld_volatile64(&st[p]);
          if ((s >> 62) == 0) {
            if (++spins > kSpinLimit) {
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
        prefix = (uint32_t)acc;
        atomicExch(&st[blk], kFlagPre | (acc + agg));
      }
      s_prefix = prefix;
      if ((int)blk == scan_blocks_hd(sc.ntiles) - 1) {
        const uint32_t total = prefix + (uint32_t)agg;
        sc.ctl->bin_total = total;
        if (total > sc.bin_cap) atomicOr(&sc.ctl->error, kErrBinOverflow);
      }
    }
  }
  __syncthreads();
  uint32_t run = s_prefix + warp_sums[warp] + (incl - local);
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < sc.ntiles) sc.tile_off[base + k] = run;
    run += vals[k];
  }
}

int launch_scan(Scratch sc, cudaStream_t s) {
  const int nb = scan_blocks(sc.ntiles);
  if (nb <= 0) return 0;
  k_scan<<<nb, kScanThreads, 0, s>>>(sc);
  return (int)cudaGetLastError();
}

// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_scatter(const DView* __restrict__ views, int T, Scratch sc) {
  const int lane = threadIdx.x & 31;
  const uint32_t nrec = min(sc.ctl->rec_count, sc.rec_cap);
  if (sc.ctl->error & (kErrBinOverflow | kErrRecOverflow | kErrClipOverflow | kErrScanTimeout)) return;
  const uint32_t stride = gridDim.x * blockDim.x;
  const int ts = __ffs(T) - 1;  // T is a power of two
  // warp-uniform trip count so every lane takes part in the warp-level collectives
  for (uint32_t i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); i0 < nrec; i0 += stride) {
    const uint32_t i = i0 + (uint32_t)lane;
    const bool ok = i < nrec;
    int tx0 = 0, ty0 = 0, ntw = 0, nt = 0, tbase = 0, tiles_x = 0;
    if (ok && !((sc.recs[i].view >> kRecFlagShift) & kRecHole)) {  // holes: huge triangles split by k_big
      const RasterRec& r = sc.recs[i];
      const uint32_t xr = r.xr, yr = r.yr;
      const DView& v = views[r.view & kRecViewMask];
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

int launch_scatter(const DView* views, int tile, Scratch sc, int grid, cudaStream_t s) {
  k_scatter<<<grid, 256, 0, s>>>(views, tile, sc);
  return (int)cudaGetLastError();
}

}  // namespace hsr
