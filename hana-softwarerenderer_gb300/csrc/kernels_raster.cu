// kernels_raster.cu — persistent per-tile raster + resolve + shade (sm_103a).
//
// Reference: rasterize_triangle (graphics.cpp:314-376).  The reference walks triangles in
// submission order and, per pixel of the bounding box, keeps a fragment when
// `!(frag_depth > depth)`.  With finite depths that sequential loop leaves, per pixel, the
// fragment of minimum depth, and among equal minima the LAST submitted one; a previous
// buffer depth equal to that minimum loses.  Fragment depths are never -0 or NaN
// (interpolate_depth starts from +0), so the order-independent rule
//     new wins  <=>  z < best_z  ||  (z == best_z && seq > best_seq)
// with best initialised from the buffer (seq "-1"; NaN buffer depth -> +inf) reproduces
// the loop exactly, whatever order the tile lists hold.  All shaders return
// `discard = false` and have no side effects (IShader.cpp:14,38,56,76,108,161,179), so
// shading only the winner equals shading every passing fragment in order.
//
// Coverage.  barycentric() (graphics.cpp:222-233) divides by u.z three times per pixel.
// With u = (ux, uy, uz) and s = ux + uy (all rounded exactly as there),
//     1 - s/uz < 0  <=>  s/uz rounds above 1  <=>  s > uz (uz > 0) or s < uz (uz < 0),
//     uy/uz < 0     <=>  uy != 0 with the opposite sign of uz (no underflow to -0),
// so the test needs no division.  The equivalence holds when nonzero |ux|, |uy| cannot
// underflow after the division; setup marks records outside that range (kRecExact) and
// those evaluate the reference's divisions literally.  Covered pixels then compute the
// three quotients exactly for the depth.
#include <float.h>

#include "hsr_device.cuh"

namespace hsr {

constexpr unsigned kFull = 0xffffffffu;
constexpr long kWaitLimit = 1L << 23;  // ~1-2 s of polling before a dependency wait gives up

__device__ __forceinline__ float canon_depth(float d) {
  // the stored depth a fragment is compared with: NaN admits every fragment (z > NaN is
  // false), which an ordered compare gets from +inf
  return d != d ? __int_as_float(0x7f800000) : d;
}

// interpolate_varyings (graphics.cpp:205-220) for one float
__device__ __forceinline__ float interp(float s0, float s1, float s2, float w0, float w1, float w2, float nrm) {
  return fm(fa(fa(fm(s0, w0), fm(s1, w1)), fm(s2, w2)), nrm);
}

// Barycentric weights at integer pixel P (graphics.cpp:222-233) for a covered pixel.
__device__ __forceinline__ void bary(const RasterRec& r, float px, float py, float& b0, float& b1, float& b2) {
  const float dx = fs(r.ax, px), dy = fs(r.ay, py);
  const float ux = fs(fm(r.e1x, dy), fm(dx, r.e1y));
  const float uy = fs(fm(dx, r.e2y), fm(r.e2x, dy));
  b0 = fs(1.f, fd(fa(ux, uy), r.uz));
  b1 = fd(uy, r.uz);
  b2 = fd(ux, r.uz);
}

// Shade one pixel from its winning record and that record's payload (Payload layout in
// hsr_internal.h): perspective-correct varyings, then the fragment shader.
__device__ __forceinline__ uint32_t shade_pixel(const DView& v, const RasterRec& r, const float* P, int x, int y,
                                                uint32_t alpha_word) {
  const uint32_t prim = v.prim_base + (r.seq >> 4) + 1u;
  if (v.shader == HSR_SHADER_FLAT) return pack_rgb(fragment(v, Frag{}, prim), alpha_word);
  float b0, b1, b2;
  bary(r, (float)x, (float)y, b0, b1, b2);
  const float w0 = fm(P[0], b0), w1 = fm(P[1], b1), w2 = fm(P[2], b2);
  const float nrm = fd(1.f, fa(fa(w0, w1), w2));
  Frag f;
  const float sc = interp(P[3], P[4], P[5], w0, w1, w2, nrm);
  f.clip_z = sc;
  f.intensity = sc;
  f.u = interp(P[6], P[8], P[10], w0, w1, w2, nrm);
  f.t = interp(P[7], P[9], P[11], w0, w1, w2, nrm);
  f.wnrm = {interp(P[12], P[15], P[18], w0, w1, w2, nrm), interp(P[13], P[16], P[19], w0, w1, w2, nrm),
            interp(P[14], P[17], P[20], w0, w1, w2, nrm)};
  f.wpos = {interp(P[21], P[24], P[27], w0, w1, w2, nrm), interp(P[22], P[25], P[28], w0, w1, w2, nrm),
            interp(P[23], P[26], P[29], w0, w1, w2, nrm)};
  return pack_rgb(fragment(v, f, prim), alpha_word);
}

__device__ __forceinline__ int payload_f4_r(int shader) {
  switch (shader) {
    case HSR_SHADER_FLAT: return 0;
    case HSR_SHADER_SHADOW: case HSR_SHADER_GROUND: case HSR_SHADER_TOON: return 2;
    case HSR_SHADER_TEXTURE: return 3;
    case HSR_SHADER_TEXTURE_WITH_LIGHT: return 6;
    default: return 8;
  }
}

__device__ __forceinline__ int find_view(const DView* views, int nviews, int t) {
  int lo = 0, hi = nviews - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (views[mid].tile_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ void wait_view(const Scratch& sc, const DView* views, int dep) {
  if (dep < 0) return;
  const uint32_t need = (uint32_t)views[dep].ntiles;
  long spins = 0;
  while (*reinterpret_cast<volatile uint32_t*>(&sc.view_done[dep]) < need) {
    if (++spins > kWaitLimit) {
      atomicOr(&sc.ctl->error, kErrWaitTimeout);
      return;
    }
    __nanosleep(128);
  }
  __threadfence();
}

template <int T, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, T == 32 ? 2 : 32 / WARPS) k_raster(const DView* __restrict__ views, Scratch sc) {
  constexpr int RP = 32 / T;        // rows covered by one pass of the warp
  constexpr int PPL = T * T / 32;   // pixels per lane
  __shared__ RasterRec srec[WARPS][32];
  __shared__ uint32_t sidx[WARPS][32];
  __shared__ uint32_t swin[WARPS][T * T];
  __shared__ float sz[WARPS][T * T];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (sc.ctl->error & (kErrBinOverflow | kErrRecOverflow | kErrClipOverflow | kErrScanTimeout)) return;
  const int col = lane % T, row = lane / T;
  const uint32_t nrec = min(sc.ctl->rec_count, sc.rec_cap);

  for (;;) {
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(&sc.ctl->tile_next, 1u);
    t = __shfl_sync(kFull, t, 0);
    if ((int)t >= sc.ntiles) break;
    const int vi = find_view(views, sc.nviews, (int)t);
    const DView& v = views[vi];
    if (lane == 0) {
      wait_view(sc, views, v.dep0);
      wait_view(sc, views, v.dep1);
    }
    __syncwarp();
    const int lt = (int)t - v.tile_base;
    const int tx = lt % v.tiles_x, ty = lt / v.tiles_x;
    const int x = tx * T + col;
    const int ybase = ty * T + row;
    const bool clear = (v.flags & HSR_DRAW_CLEAR) != 0u;
    const uint32_t n = sc.tile_count[t];

    if (n == 0) {
      if (clear) {
#pragma unroll
        for (int k = 0; k < PPL; k++) {
          const int y = ybase + k * RP;
          if (x < v.W && y < v.H) {
            const size_t idx = (size_t)y * v.W + x;
            v.color[idx] = v.clear_rgba;
            v.depth[idx] = v.clear_depth;
            if (v.prim) v.prim[idx] = 0u;
          }
        }
      }
    } else {
      float cz[PPL];
      uint32_t cs[PPL], cw[PPL];
#pragma unroll
      for (int k = 0; k < PPL; k++) {
        const int y = ybase + k * RP;
        float d = v.clear_depth;
        if (!clear && x < v.W && y < v.H) d = __ldcg(&v.depth[(size_t)y * v.W + x]);
        cz[k] = canon_depth(d);
        cs[k] = 0u;
        cw[k] = 0u;
      }
      const uint32_t off = sc.tile_off[t];
      const float pxf = (float)x;
      for (uint32_t b = 0; b < n; b += 32) {
        const uint32_t cnt = min(32u, n - b);
        if ((uint32_t)lane < cnt) {
          const uint32_t ri = sc.bins[off + b + (uint32_t)lane];
          RasterRec rr;
          if (ri < nrec) {
            rr = sc.recs[ri];
          } else {        // never produced by a consistent bin pass; covers no pixel
            rr.xr = 1u;
            rr.yr = 1u;
            rr.seq = 0u;
            rr.flags = 0u;
            rr.pad = 0u;
          }
          srec[warp][lane] = rr;
          sidx[warp][lane] = ri;
        }
        __syncwarp();
        for (uint32_t j = 0; j < cnt; j++) {
          const RasterRec& r = srec[warp][j];
          const int x0 = (int)(r.xr & 0xffffu), x1 = (int)(r.xr >> 16);
          const int y0 = (int)(r.yr & 0xffffu), y1 = (int)(r.yr >> 16);
          const int r0 = max(y0 - ty * T, 0), r1 = min(y1 - ty * T, T - 1);
          const int k0 = r0 / RP, k1 = r1 / RP;
          const bool xin = x >= x0 && x <= x1;
          const uint32_t seqp1 = r.seq + 1u;
          const bool exact = (r.flags & kRecExact) != 0u;
#pragma unroll
          for (int k = 0; k < PPL; k++) {
            if (k < k0 || k > k1) continue;
            const int y = ybase + k * RP;
            if (!xin || y < y0 || y > y1) continue;
            const float pyf = (float)y;
            const float dx = fs(r.ax, pxf), dy = fs(r.ay, pyf);
            const float ux = fs(fm(r.e1x, dy), fm(dx, r.e1y));
            const float uy = fs(fm(dx, r.e2y), fm(r.e2x, dy));
            const float s = fa(ux, uy);
            bool cov;
            float b0, b1, b2;
            if (!exact) {
              cov = (r.uz < 0.f) ? (s >= r.uz && uy <= 0.f && ux <= 0.f) : (s <= r.uz && uy >= 0.f && ux >= 0.f);
              if (!cov) continue;
              b0 = fs(1.f, fd(s, r.uz));
              b1 = fd(uy, r.uz);
              b2 = fd(ux, r.uz);
            } else {
              b0 = fs(1.f, fd(s, r.uz));
              b1 = fd(uy, r.uz);
              b2 = fd(ux, r.uz);
              if (b0 < 0.f || b1 < 0.f || b2 < 0.f) continue;
            }
            // interpolate_depth (graphics.cpp:186-194)
            const float z = fa(fa(fa(0.f, fm(r.d2, b2)), fm(r.d1, b1)), fm(r.d0, b0));
            if (z < cz[k] || (z == cz[k] && seqp1 > cs[k])) {
              cz[k] = z;
              cs[k] = seqp1;
              cw[k] = sidx[warp][j];
            }
          }
        }
        __syncwarp();
      }
      // hand the winners to shared memory so the (large) shading code is not unrolled
#pragma unroll
      for (int k = 0; k < PPL; k++) {
        swin[warp][k * 32 + lane] = cs[k] ? cw[k] : 0xffffffffu;
        sz[warp][k * 32 + lane] = cz[k];
      }
      __syncwarp();
      uint32_t shaded = 0;
      const int nf4 = payload_f4_r(v.shader);
#pragma unroll 1
      for (int k = 0; k < PPL; k++) {
        const int y = ybase + k * RP;
        if (x >= v.W || y >= v.H) continue;
        const size_t idx = (size_t)y * v.W + x;
        const uint32_t w = swin[warp][k * 32 + lane];
        if (w != 0xffffffffu) {
          shaded++;
          // the payload index equals the record index except for sub-records of a split
          // triangle: load both at once, reload the payload in that rare case
          const RasterRec r = sc.recs[w];
          float P[kPayloadFloats];
          {
            float4* dst = reinterpret_cast<float4*>(P);
            const float4* src = reinterpret_cast<const float4*>(&sc.pay[w]);
#pragma unroll
            for (int q = 0; q < kPayloadFloats / 4; q++)
              dst[q] = q < nf4 ? src[q] : make_float4(0.f, 0.f, 0.f, 0.f);
            if (r.pad != w) {
              src = reinterpret_cast<const float4*>(&sc.pay[r.pad]);
#pragma unroll
              for (int q = 0; q < kPayloadFloats / 4; q++)
                dst[q] = q < nf4 ? src[q] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
          }
          const uint32_t alpha = clear ? v.clear_rgba : __ldcg(&v.color[idx]);
          v.color[idx] = shade_pixel(v, r, P, x, y, alpha);
          v.depth[idx] = sz[warp][k * 32 + lane];
          if (v.prim) v.prim[idx] = v.prim_base + (r.seq >> 4) + 1u;
        } else if (clear) {
          v.color[idx] = v.clear_rgba;
          v.depth[idx] = v.clear_depth;
          if (v.prim) v.prim[idx] = 0u;
        }
      }
      shaded = __reduce_add_sync(kFull, shaded);
      if (lane == 0 && shaded) atomicAdd(&sc.ctl->shaded_px, (unsigned long long)shaded);
      __syncwarp();
    }
    if (v.has_dependents) {
      // publish this tile's writes before counting it done (a later view reads them)
      __threadfence();
      __syncwarp();
      if (lane == 0) atomicAdd(&sc.view_done[vi], 1u);
    }
  }
}

template <int T, int WARPS>
static int launch_t(const DView* views, Scratch sc, int grid, cudaStream_t s) {
  k_raster<T, WARPS><<<grid, WARPS * 32, 0, s>>>(views, sc);
  return (int)cudaGetLastError();
}

int launch_raster(const DView* views, int tile, Scratch sc, int grid, int warps, cudaStream_t s) {
  if (warps != 4 && warps != 8) return (int)cudaErrorInvalidValue;
  switch (tile) {
    case 8: return warps == 4 ? launch_t<8, 4>(views, sc, grid, s) : launch_t<8, 8>(views, sc, grid, s);
    case 16: return warps == 4 ? launch_t<16, 4>(views, sc, grid, s) : launch_t<16, 8>(views, sc, grid, s);
    case 32: return warps == 4 ? launch_t<32, 4>(views, sc, grid, s) : (int)cudaErrorInvalidValue;
    default: return (int)cudaErrorInvalidValue;
  }
}

}  // namespace hsr
