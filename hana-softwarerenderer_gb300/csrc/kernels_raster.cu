// kernels_raster.cu — persistent per-tile raster + resolve + shade (sm_103a).
//
// Reference: rasterize_triangle (graphics.cpp:314-376).  The reference walks triangles in
// submission order and, per pixel of the bounding box, keeps a fragment when
// `!(frag_depth > depth)`.  With finite depths that sequential loop leaves, per pixel, the
// fragment of minimum depth, and among equal minima the LAST submitted one; a previous
// buffer depth equal to that minimum loses.  Fragment depths are never -0 or NaN
// (interpolate_depth starts from +0), so the order-independent rule
//     min over (depth, later-submitted)
// with the buffer's depth as the weakest entry reproduces the loop exactly, whatever
// order the tile lists hold.  All shaders return `discard = false` and have no side
// effects (IShader.cpp:14,38,56,76,108,161,179), so shading only the winner equals
// shading every passing fragment in order.
//
// Coverage.  barycentric() (graphics.cpp:222-233) divides by u.z three times per pixel.
// With u = (ux, uy, uz) and s = ux + uy (all rounded exactly as there),
//     1 - s/uz < 0  <=>  s/uz rounds above 1  <=>  s > uz (uz > 0) or s < uz (uz < 0),
//     uy/uz < 0     <=>  uy != 0 with the opposite sign of uz (no underflow to -0),
// so the test needs no division.  The equivalence holds when nonzero |ux|, |uy| cannot
// underflow after the division; setup marks records outside that range (kRecExact) and
// those evaluate the reference's divisions literally.  Covered pixels then compute the
// three IEEE quotients for the depth.
#include <float.h>

#include "hsr_device.cuh"

namespace hsr {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kNone = 0xffffffffu;

// View owning tile t: the last view whose first tile is <= t (views hold consecutive tile
// ranges in batch order).  `tbase` is the shared copy when the batch has at most
// kSharedViews views, else null and the descriptors are searched in global memory.
__device__ __forceinline__ int find_view(const DView* views, const int32_t* tbase, int nviews, int t) {
  int lo = 0, hi = nviews - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((tbase ? tbase[mid] : views[mid].tile_base) <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Wait until every non-empty tile of view `dep` is done (its empty tiles were cleared in the
// scatter grid, which runs before the raster).  Bounded: after the poll limit the wait sets
// kErrWaitTimeout and returns, and once any wait of the sequence has given up the others
// stop waiting (so a dependency that never completes costs one limit, not one per tile).
// HSR_FAULT_DEPENDENCY_STALL makes the wait ask for one tile more than the view has.
__device__ __forceinline__ void wait_view(const Scratch& sc, const DView* views, int dep) {
  if (dep < 0) return;
  const int tb = views[dep].tile_base;
  const uint32_t need = sc.ne_off[tb + views[dep].ntiles] - sc.ne_off[tb] +
                        ((sc.faults & HSR_FAULT_DEPENDENCY_STALL) ? 1u : 0u);
  const long limit = sc.poll_limit > 0 ? (long)sc.poll_limit : kDepWaitPolls;
  long spins = 0;
  while (*reinterpret_cast<volatile uint32_t*>(&sc.view_done[dep]) < need) {
    if (++spins > limit || (*reinterpret_cast<volatile uint32_t*>(&sc.ctl->error) & kErrWaitTimeout)) {
      atomicOr(&sc.ctl->error, kErrWaitTimeout);
      return;
    }
    __nanosleep(128);
  }
  __threadfence();
}

// Ordered bits of a float: unsigned order equals float order (-inf < ... < -0 < +0 < ... < +inf).
__device__ __forceinline__ uint32_t ord_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float from_ord(uint32_t o) {
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
// Key of the depth already in the buffer: it loses every tie (low word above any fragment's),
// -0 compares equal to +0 as `frag_depth > depth` does, NaN admits every fragment.
__device__ __forceinline__ unsigned long long buffer_key(float d) {
  if (d == 0.f) d = 0.f;
  if (d != d) d = __int_as_float(0x7f800000);
  return ((unsigned long long)ord_bits(d) << 32) | 0xffffffffull;
}

// q / d for q < 1024 and 1 <= d <= 32 by multiply-shift: ceil(65536 / d).
__constant__ uint32_t kDivMagic[33] = {0,     65536, 32768, 21846, 16384, 13108, 10923, 9363, 8192, 7282, 6554,
                                       5958,  5462,  5042,  4682,  4370,  4096,  3856,  3641, 3450, 3277, 3121,
                                       2979,  2850,  2731,  2622,  2521,  2428,  2341,  2260, 2185, 2115, 2048};

// The non-empty records of one batch of a tile list, compacted.  The coverage constants a
// candidate reads are two arrays of float4 and one of uint2 (three shared loads per candidate;
// consecutive records are consecutive 16-byte entries, so a quarter-warp's loads of different
// records fall in different banks); the fields resolve reads are one array each.
struct __align__(16) BatchRecs {
  float4 a4[32];       // ax, ay, e1x, e1y
  float4 b4[32];       // e2x, e2y, uz, box (x0 | y0 << 8 | width << 16, bit 31 = kRecExact)
  uint2 c2[32];        // first candidate of the record's run, ceil(65536 / width)
  float4 d4[32];       // screen depths d0, d1, d2 of the corners, submission order (bits)
  uint32_t ri[32];     // record index (also the index of its payload)
};

// Covered candidates waiting for their weights, depth and visibility update (a ring of 64 per
// warp): the cross products (u.x, u.y) of barycentric() and the run | pixel << 8.  The
// coverage pass fills it at the rate candidates are tested; the weights' three divisions and
// the depth test then run on full warps of covered candidates.
struct CandQueue {
  float2 u[64];
  uint32_t jp[64];
};

// Per-warp tile state in shared memory: per pixel the key (ordered depth | submission) and
// the index of the record that holds it, which is also the index of its payload.  8x8 tiles
// also keep the winner's barycentric weights (24 bytes a pixel in all), so shading reads no
// record; 16x16 and 32x32 tiles keep 12 bytes a pixel and the weights in the warp's stash.
template <int NPIX>
struct TileState {
  static constexpr bool kKeep = NPIX <= 64;
  unsigned long long key[NPIX];
  uint32_t rec[NPIX];
  float b0[kKeep ? NPIX : 1], b1[kKeep ? NPIX : 1], b2[kKeep ? NPIX : 1];
};

// Everything one raster CTA keeps in shared memory, in one dynamically sized block (a 32x32
// tile needs more than the 48 KB of static shared memory; the launch opts in above that).
template <int T, int WARPS>
struct RasterSmem {
  TileState<T * T> st[WARPS];
  BatchRecs br[WARPS];
  CandQueue cq[WARPS];
  float u8f[256], u8n[256];
  int32_t tbase[kSharedViews];
};

// Shade the winners of one tile and write colour, depth and prim id (fused clear writes the
// clear values where nothing won).  S is the shader, known at compile time.  Without kept
// weights (16x16 and 32x32 tiles) the winner's weights come from the warp's stash in global
// memory (written by the visibility pass, read back from L2), or, with no stash, are evaluated
// again from its record: the same operations on the same values as in the visibility pass
// either way, so the same bits.
template <int T, int S>
__device__ __forceinline__ uint32_t shade_tile(const DView& v, const Scratch& sc, const TileState<T * T>& st, int ox,
                                               int oy, bool clear, const ByteTables& bt, const float* stash) {
  constexpr int PPL = T * T / 32;
  constexpr int NF4 = payload_f4_of<S>();
  const int lane = threadIdx.x & 31;
  uint32_t shaded = 0;
#pragma unroll 1
  for (int q = 0; q < PPL; q++) {
    const int p = lane + 32 * q;
    const int x = ox + p % T, y = oy + p / T;
    if (x >= v.W || y >= v.H) continue;
    const size_t idx = (size_t)y * v.W + x;
    const uint32_t ri = st.rec[p];
    if (ri != kNone) {
      shaded++;
      float b0, b1, b2;
      uint32_t pay, seq;
      // a record's payload index is its own index, and the winner's submission is the low word of
      // its key: the payload's loads wait for nothing but the record index
      if constexpr (TileState<T * T>::kKeep) {
        b0 = st.b0[p]; b1 = st.b1[p]; b2 = st.b2[p];
        pay = ri;
        seq = 0xfffffffeu - (uint32_t)st.key[p];
      } else if (stash) {
        pay = ri;
        seq = 0xfffffffeu - (uint32_t)st.key[p];
        const float4 w = __ldcg(reinterpret_cast<const float4*>(stash) + p);
        b0 = w.x; b1 = w.y; b2 = w.z;
      } else {
        const RasterRec r = sc.recs[ri];
        cover_test(r.ax, r.ay, r.e1x, r.e1y, r.e2x, r.e2y, r.uz, ((r.view >> kRecFlagShift) & kRecExact) != 0u,
                   (float)x, (float)y, b0, b1, b2);
        pay = ri;
        seq = r.seq;
      }
      float P[NF4 > 0 ? NF4 * 4 : 4];
      if constexpr (NF4 > 0) {
        const float4* src = reinterpret_cast<const float4*>(&sc.pay[pay]);
#pragma unroll
        for (int k = 0; k < NF4; k++) reinterpret_cast<float4*>(P)[k] = src[k];
      }
      const uint32_t prim = v.prim_base + (seq >> 4) + 1u;
      const uint32_t alpha = clear ? v.clear_rgba : __ldcg(&v.color[idx]);
      v.color[idx] = pack_rgb(fragment_s<S>(v, P, b0, b1, b2, prim, bt), alpha);
      v.depth[idx] = from_ord((uint32_t)(st.key[p] >> 32));
      if (v.prim) v.prim[idx] = prim;
    } else if (clear) {
      v.color[idx] = v.clear_rgba;
      v.depth[idx] = v.clear_depth;
      if (v.prim) v.prim[idx] = 0u;
    }
  }
  return shaded;
}

// One warp per non-empty screen tile (k_scan lists them in tile order; the scatter grid has
// cleared the others).  For each batch of 32 records of the tile list, every record's
// bounding-box pixels inside the tile form a run of candidates; the non-empty runs are
// compacted and laid end to end (warp prefix sum) and the lanes walk the candidates 32 at
// a time, so the work is proportional to the pixels the triangles can touch rather than
// to records x 32 lanes.  The run owning a candidate is found from a ballot of the runs
// starting in the current window of 32 candidates.  A covered candidate resolves
// visibility with a 64-bit atomicMin on
//     (ordered depth << 32) | (0xfffffffe - seq)
// in shared memory: smallest depth first, and among equal depths the later submission.
// The lane whose key is still the minimum after the warp's atomics records the winner's
// record (two lanes of one step never hold the same key: one triangle covers a pixel
// once).  Shading then runs once per pixel with a winner.
// Four-warp CTAs are compiled for 7 per SM (72 registers a thread, fewer spills than at 8 per
// SM's 64: measured faster on the serving batches, 1.72 -> 1.65 ms).
template <int T, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, WARPS == 4 ? 7 : 32 / WARPS) k_raster(const DView* __restrict__ views, Scratch sc) {
  constexpr int NPIX = T * T;
  constexpr int PPL = NPIX / 32;
  extern __shared__ __align__(16) unsigned char raster_smem[];
  RasterSmem<T, WARPS>& sm = *reinterpret_cast<RasterSmem<T, WARPS>*>(raster_smem);
  build_byte_tables(sm.u8f, sm.u8n);
  const int32_t* tbase = sc.nviews <= kSharedViews ? sm.tbase : nullptr;
  if (tbase)
    for (int i = threadIdx.x; i < sc.nviews; i += blockDim.x) sm.tbase[i] = views[i].tile_base;
  __syncthreads();
  const ByteTables bt{sm.u8f, sm.u8n};
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  TileState<NPIX>& st = sm.st[warp];
  BatchRecs& br = sm.br[warp];
  CandQueue& cq = sm.cq[warp];
  float* stash = nullptr;
  if constexpr (!TileState<NPIX>::kKeep) {
    const uint32_t gw = blockIdx.x * (uint32_t)WARPS + (uint32_t)warp;
    if (sc.stash && gw < sc.stash_warps) stash = sc.stash + (size_t)gw * (size_t)stash_floats(T);
  }
  if (sc.ctl->error & kErrNoDraw) return;
  const uint32_t nrec = min(sc.ctl->rec_count, sc.rec_cap);

  // The non-empty tiles are handed out by one counter over their list, two ahead: while a
  // tile is rasterised, the next tile's list bounds are already loading and the one after it
  // is being claimed, so neither the counter's round trip nor the list lookup waits on the
  // critical path (the list is in tile order and dependencies only point to lower tile
  // indices, so holding later tiles never blocks).
  const uint32_t nlist = min(sc.ctl->ne_tiles, (uint32_t)sc.ntiles);
  const uint32_t ntiles = (uint32_t)sc.ntiles;
  uint32_t li = 0, li_ahead = 0;  // positions in the list
  if (lane == 0) {
    li = atomicAdd(&sc.ctl->tile_next, 1u);
    li_ahead = atomicAdd(&sc.ctl->tile_next, 1u);
  }
  li = __shfl_sync(kFull, li, 0);
  uint32_t t = li < nlist ? sc.tile_list[li] : ntiles;
  uint32_t n = 0, off = 0;
  if (t < ntiles) {
    n = sc.tile_count[t];
    off = sc.tile_off[t];
  }
  // views of a warp's tiles only move forward: after the first, search on from the last one
  int vi = t < ntiles ? find_view(views, tbase, sc.nviews, (int)t) : 0;
  for (;;) {
    if (t >= ntiles) break;
    const uint32_t li_next = __shfl_sync(kFull, li_ahead, 0);
    if (lane == 0) li_ahead = li_next < nlist ? atomicAdd(&sc.ctl->tile_next, 1u) : nlist;
    const uint32_t t_next = li_next < nlist ? sc.tile_list[li_next] : ntiles;
    uint32_t n_next = 0, off_next = 0;
    if (t_next < ntiles) {
      n_next = sc.tile_count[t_next];
      off_next = sc.tile_off[t_next];
    }
    if (t_next < ntiles) {  // warm L1 with the next tile's view descriptor line
      const DView* vn = views + find_view(views, tbase, sc.nviews, (int)t_next);
      asm volatile("prefetch.global.L1 [%0];" ::"l"(vn));
    }
    if (tbase) {
      while (vi + 1 < sc.nviews && tbase[vi + 1] <= (int)t) vi++;
    } else {
      vi = find_view(views, tbase, sc.nviews, (int)t);
    }
    const DView& v = views[vi];
    if (lane == 0) {
      wait_view(sc, views, v.dep0);
      wait_view(sc, views, v.dep1);
    }
    __syncwarp();
    const int lt = (int)t - v.tile_base;
    const int tx = lt % v.tiles_x, ty = lt / v.tiles_x;
    const int ox = tx * T, oy = ty * T;
    const bool clear = (v.flags & HSR_DRAW_CLEAR) != 0u;

    if (n != 0) {  // always: the list holds the tiles with records
      if (clear) {  // every pixel starts from the clear depth
        const unsigned long long k0 = buffer_key(v.clear_depth);
#pragma unroll 8
        for (int q = 0; q < PPL; q++) {
          st.key[lane + 32 * q] = k0;
          st.rec[lane + 32 * q] = kNone;
        }
      } else {
#pragma unroll 8
        for (int q = 0; q < PPL; q++) {
          const int p = lane + 32 * q;
          const int x = ox + p % T, y = oy + p / T;
          float d = v.clear_depth;
          if (x < v.W && y < v.H) d = __ldcg(&v.depth[(size_t)y * v.W + x]);
          st.key[p] = buffer_key(d);
          st.rec[p] = kNone;
        }
      }
      uint32_t frags = 0;  // covered candidates of this lane
      for (uint32_t b = 0; b < n; b += 32) {
        const uint32_t cnt = min(32u, n - b);
        uint32_t c = 0, box = 0, ri = kNone;
        RasterRec rr;
        if ((uint32_t)lane < cnt) {
          ri = sc.bins[off + b + (uint32_t)lane];
          if (ri < nrec) {  // an index past the records never comes from a consistent bin pass
            rr = sc.recs[ri];
            const int lx0 = max((int)(rr.xr & 0xffffu) - ox, 0), lx1 = min((int)(rr.xr >> 16) - ox, T - 1);
            const int ly0 = max((int)(rr.yr & 0xffffu) - oy, 0), ly1 = min((int)(rr.yr >> 16) - oy, T - 1);
            if (lx0 <= lx1 && ly0 <= ly1) {
              c = (uint32_t)((lx1 - lx0 + 1) * (ly1 - ly0 + 1));
              box = (uint32_t)lx0 | ((uint32_t)ly0 << 8) | ((uint32_t)(lx1 - lx0 + 1) << 16);
            }
          }
        }
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t y = __shfl_up_sync(kFull, incl, o);
          if (lane >= o) incl += y;
        }
        const uint32_t W = __shfl_sync(kFull, incl, 31);
        const uint32_t start = incl - c;
        const unsigned ne = __ballot_sync(kFull, c > 0u);
        __syncwarp();
        if (c > 0u) {  // compact the non-empty runs
          const int k = __popc(ne & ((1u << lane) - 1u));
          const uint32_t bits = box | (((rr.view >> kRecFlagShift) & kRecExact) ? 0x80000000u : 0u);
          br.a4[k] = make_float4(rr.ax, rr.ay, rr.e1x, rr.e1y);
          br.b4[k] = make_float4(rr.e2x, rr.e2y, rr.uz, __uint_as_float(bits));
          br.c2[k] = make_uint2(start, kDivMagic[box >> 16]);
          br.d4[k] = make_float4(rr.d0, rr.d1, rr.d2, __uint_as_float(rr.seq));
          br.ri[k] = ri;
        }
        __syncwarp();
        // Visibility of `cnt` queued candidates from the ring head, one per lane: weights
        // (the divisions of barycentric()), depth, and a 64-bit atomicMin of the key.
        uint32_t qh = 0, qn = 0;  // ring head and queued count (warp-uniform)
        auto resolve = [&](uint32_t cnt) {
          __syncwarp();
          const bool act = (uint32_t)lane < cnt;
          unsigned long long key = 0ull, old = 0ull;
          int p = 0, j = 0;
          float b0 = 0.f, b1 = 0.f, b2 = 0.f;
          if (act) {
            const uint32_t e = (qh + (uint32_t)lane) & 63u;
            const uint32_t jp = cq.jp[e];
            j = (int)(jp & 31u);
            p = (int)(jp >> 8);
            const float2 u = cq.u[e];
            const float4 d4 = br.d4[j];
            cover_weights(u.x, u.y, br.b4[j].z, b0, b1, b2);
            // interpolate_depth (graphics.cpp:186-194)
            const float z = fa(fa(fa(0.f, fm(d4.z, b2)), fm(d4.y, b1)), fm(d4.x, b0));
            key = ((unsigned long long)ord_bits(z) << 32) | (unsigned long long)(0xfffffffeu - __float_as_uint(d4.w));
            old = atomicMin(&st.key[p], key);
          }
          __syncwarp();
          if (act && old > key && st.key[p] == key) {
            st.rec[p] = br.ri[j];
            if constexpr (TileState<NPIX>::kKeep) {
              st.b0[p] = b0;
              st.b1[p] = b1;
              st.b2[p] = b2;
            } else if (stash) {
              __stcg(reinterpret_cast<float4*>(stash) + p, make_float4(b0, b1, b2, 0.f));
            }
          }
          qh = (qh + cnt) & 63u;
          qn -= cnt;
          __syncwarp();
        };
        for (uint32_t base = 0; base < W; base += 32) {
          // runs starting before this window, and a bit per run starting inside it
          const uint32_t before = (uint32_t)__popc(__ballot_sync(kFull, c > 0u && start < base));
          const uint32_t here = __reduce_or_sync(
              kFull, (c > 0u && start >= base && start - base < 32u) ? 1u << (start - base) : 0u);
          const uint32_t i = base + (uint32_t)lane;
          bool covered = false;
          float ux = 0.f, uy = 0.f;
          int p = 0, j = 0;
          if (i < W) {
            // owner: the last run starting at or before candidate i
            j = (int)(before + (uint32_t)__popc(here & ((2u << lane) - 1u))) - 1;
            const float4 a4 = br.a4[j], b4 = br.b4[j];
            const uint2 c2 = br.c2[j];
            const uint32_t q = i - c2.x;
            const uint32_t bx = __float_as_uint(b4.w);
            const uint32_t lw = (bx >> 16) & 255u;
            const uint32_t qy = (q * c2.y) >> 16;
            const int lx = (int)(bx & 255u) + (int)(q - qy * lw);
            const int ly = (int)((bx >> 8) & 255u) + (int)qy;
            p = ly * T + lx;
            covered = cover_terms(a4.x, a4.y, a4.z, a4.w, b4.x, b4.y, b4.z, (bx >> 31) != 0u, (float)(ox + lx),
                                  (float)(oy + ly), ux, uy);
          }
          const unsigned cm = __ballot_sync(kFull, covered);
          if (covered) {  // queue behind the pending ones (at most 31 are pending here)
            frags++;
            const uint32_t e = (qh + qn + (uint32_t)__popc(cm & ((1u << lane) - 1u))) & 63u;
            cq.u[e] = make_float2(ux, uy);
            cq.jp[e] = (uint32_t)j | ((uint32_t)p << 8);
          }
          qn += (uint32_t)__popc(cm);
          if (qn >= 32u) resolve(32u);
        }
        if (qn) resolve(qn);  // before the next batch replaces the runs the queue points to
      }
      __syncwarp();
      uint32_t shaded = 0;
      switch (v.shader) {
        case HSR_SHADER_GROUND: shaded = shade_tile<T, HSR_SHADER_GROUND>(v, sc, st, ox, oy, clear, bt, stash); break;
        case HSR_SHADER_TOON: shaded = shade_tile<T, HSR_SHADER_TOON>(v, sc, st, ox, oy, clear, bt, stash); break;
        case HSR_SHADER_TEXTURE: shaded = shade_tile<T, HSR_SHADER_TEXTURE>(v, sc, st, ox, oy, clear, bt, stash); break;
        case HSR_SHADER_TEXTURE_WITH_LIGHT:
          shaded = shade_tile<T, HSR_SHADER_TEXTURE_WITH_LIGHT>(v, sc, st, ox, oy, clear, bt, stash);
          break;
        case HSR_SHADER_BLINN: shaded = shade_tile<T, HSR_SHADER_BLINN>(v, sc, st, ox, oy, clear, bt, stash); break;
        case HSR_SHADER_NORMALMAP: shaded = shade_tile<T, HSR_SHADER_NORMALMAP>(v, sc, st, ox, oy, clear, bt, stash); break;
        case HSR_SHADER_SHADOW: shaded = shade_tile<T, HSR_SHADER_SHADOW>(v, sc, st, ox, oy, clear, bt, stash); break;
        default: shaded = shade_tile<T, HSR_SHADER_FLAT>(v, sc, st, ox, oy, clear, bt, stash); break;
      }
      shaded = __reduce_add_sync(kFull, shaded);
      frags = __reduce_add_sync(kFull, frags);
      if (lane == 0) {
        if (shaded) atomicAdd(&sc.ctl->shaded_px, (unsigned long long)shaded);
        if (frags) atomicAdd(&sc.ctl->frag_px, (unsigned long long)frags);
      }
    }
    if (v.has_dependents) {
      // publish this tile's writes before counting it done (a later view reads them)
      __threadfence();
      __syncwarp();
      if (lane == 0) atomicAdd(&sc.view_done[vi], 1u);
    }
    t = t_next;
    n = n_next;
    off = off_next;
  }
}

template <int T, int WARPS>
static int launch_t(const DView* views, Scratch sc, int grid, cudaStream_t s) {
  constexpr size_t smem = sizeof(RasterSmem<T, WARPS>);
  if (smem > 48 * 1024) {  // opt in to more than the default 48 KB of dynamic shared memory
    const cudaError_t e =
        cudaFuncSetAttribute(k_raster<T, WARPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
  }
  k_raster<T, WARPS><<<grid, WARPS * 32, smem, s>>>(views, sc);
  return (int)cudaGetLastError();
}

int launch_raster(const DView* views, int tile, Scratch sc, int grid, int warps, cudaStream_t s) {
  if (warps != 4 && warps != 8) return (int)cudaErrorInvalidValue;
  switch (tile) {
    case 8: return warps == 4 ? launch_t<8, 4>(views, sc, grid, s) : launch_t<8, 8>(views, sc, grid, s);
    case 16: return warps == 4 ? launch_t<16, 4>(views, sc, grid, s) : (int)cudaErrorInvalidValue;
    case 32: return warps == 4 ? launch_t<32, 4>(views, sc, grid, s) : (int)cudaErrorInvalidValue;
    default: return (int)cudaErrorInvalidValue;
  }
}

}  // namespace hsr
