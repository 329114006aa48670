// hsr_device.cuh — device arithmetic of the draw path.
//
// Every float operation is an explicitly rounded intrinsic (__fmul_rn, __fadd_rn, ...),
// written in the reference's evaluation order, so the compiler can neither contract into
// FMA nor reassociate: the bits equal the reference's single-precision IEEE arithmetic.
// Division and square root are the correctly rounded __fdiv_rn / __fsqrt_rn / __dsqrt_rn.
// std::min / std::max keep their ternary NaN behaviour (no fminf / fmaxf).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "hsr_internal.h"

namespace hsr {

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ float std_min(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float std_max(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float saturate(float f) { return f < 0.f ? 0.f : (f > 1.f ? 1.f : f); }  // maths.cpp:13-15

// float -> int32 with the meaning x86 cvttss2si gives (truncation; INT_MIN for NaN or
// out-of-range values), the platform the reference targets.
__device__ __forceinline__ int32_t cvt_i32(float f) {
  return (f > -2147483904.0f && f < 2147483648.0f) ? __float2int_rz(f) : (int32_t)0x80000000;
}

struct F3 { float x, y, z; };

// Vector operator* (vector.h:69-73): ret = 0; ret += a[N-1]*b[N-1]; ... ret += a[0]*b[0].
__device__ __forceinline__ float dot3(F3 a, F3 b) {
  float r = fa(0.f, fm(a.z, b.z));
  r = fa(r, fm(a.y, b.y));
  return fa(r, fm(a.x, b.x));
}
__device__ __forceinline__ float dot4(float a0, float a1, float a2, float a3,
                                      float b0, float b1, float b2, float b3) {
  float r = fa(0.f, fm(a3, b3));
  r = fa(r, fm(a2, b2));
  r = fa(r, fm(a1, b1));
  return fa(r, fm(a0, b0));
}
__device__ __forceinline__ F3 sub3(F3 a, F3 b) { return {fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z)}; }
__device__ __forceinline__ F3 add3(F3 a, F3 b) { return {fa(a.x, b.x), fa(a.y, b.y), fa(a.z, b.z)}; }
__device__ __forceinline__ F3 cross3(F3 a, F3 b) {  // vector.h:97-99
  return {fs(fm(a.y, b.z), fm(a.z, b.y)), fs(fm(a.z, b.x), fm(a.x, b.z)), fs(fm(a.x, b.y), fm(a.y, b.x))};
}
__device__ __forceinline__ F3 normalize3(F3 v) {  // vector.h:41-42
  float n = __fsqrt_rn(fa(fa(fm(v.x, v.x), fm(v.y, v.y)), fm(v.z, v.z)));
  float f = __frcp_rn(n);  // 1.f / n, correctly rounded
  return {fm(v.x, f), fm(v.y, f), fm(v.z, f)};
}
// Matrix4x4 * Vector4f row by row (matrix.h:112-116); m row-major.
__device__ __forceinline__ float4 mat_vec(const float* m, float x, float y, float z, float w) {
  return make_float4(dot4(m[0], m[1], m[2], m[3], x, y, z, w), dot4(m[4], m[5], m[6], m[7], x, y, z, w),
                     dot4(m[8], m[9], m[10], m[11], x, y, z, w), dot4(m[12], m[13], m[14], m[15], x, y, z, w));
}

// ---- Color (color.cpp:38-64) ------------------------------------------------------------
struct Col { float r, g, b, a; };
__device__ __forceinline__ Col c_add(Col a, Col b) {
  return {std_min(std_max(0.f, fa(a.r, b.r)), 1.f), std_min(std_max(0.f, fa(a.g, b.g)), 1.f),
          std_min(std_max(0.f, fa(a.b, b.b)), 1.f), std_min(std_max(0.f, fa(a.a, b.a)), 1.f)};
}
__device__ __forceinline__ Col c_mulf(Col a, float t) {
  t = (t > 1.f ? 1.f : (t < 0.f ? 0.f : t));
  return {std_min(std_max(0.f, fm(a.r, t)), 1.f), std_min(std_max(0.f, fm(a.g, t)), 1.f),
          std_min(std_max(0.f, fm(a.b, t)), 1.f), std_min(std_max(0.f, fm(a.a, t)), 1.f)};
}
__device__ __forceinline__ Col c_mulc(Col a, Col b) { return {fm(a.r, b.r), fm(a.g, b.g), fm(a.b, b.b), fm(a.a, b.a)}; }
__device__ __forceinline__ Col c_of(const float* p) { return {p[0], p[1], p[2], p[3]}; }

// ---- byte -> float tables --------------------------------------------------------------
// Colour channels and normal-map components are bytes; their float values are the IEEE
// results b/255.f (color.cpp:5, renderbuffer.cpp:46) and (b/255.f)*2.f - 1.f
// (IShader.h:97), computed once per CTA into shared memory with the same operations.
struct ByteTables {
  const float* u8f;  // b / 255.f
  const float* u8n;  // (b / 255.f) * 2.f - 1.f
};
__device__ __forceinline__ void build_byte_tables(float* u8f, float* u8n) {
  for (int i = threadIdx.x; i < 256; i += blockDim.x) {
    const float f = fd((float)i, 255.f);
    u8f[i] = f;
    u8n[i] = fs(fm(f, 2.f), 1.f);
  }
}

// ---- textures: TGAImage::get (tgaimage.cpp:248-253) on BGRA words ------------------------
// Texels are stored as 32-bit words b | g<<8 | r<<16 | a<<24 with missing bytes zero,
// which is what TGAColor(p, bytespp) holds for bytespp 1, 3 and 4.
__device__ __forceinline__ uint32_t tga_get(const uint32_t* tex, int32_t w, int32_t h, int32_t x, int32_t y) {
  if (!tex || x < 0 || y < 0 || x >= w || y >= h) return 0u;
  return __ldg(tex + (size_t)y * (size_t)w + (size_t)x);
}
// IShader::tex_diffuse (IShader.h:85-89), Color(TGAColor) (color.cpp:5)
__device__ __forceinline__ Col tex_diffuse(const DView& v, float u, float t, const ByteTables& bt) {
  uint32_t c = tga_get(v.diffuse, v.dw, v.dh, cvt_i32(fm(u, (float)v.dw)), cvt_i32(fm(t, (float)v.dh)));
  return {bt.u8f[(c >> 16) & 255u], bt.u8f[(c >> 8) & 255u], bt.u8f[c & 255u], bt.u8f[c >> 24]};
}
// IShader::tex_normal (IShader.h:91-99)
__device__ __forceinline__ F3 tex_normal(const DView& v, float u, float t, const ByteTables& bt) {
  uint32_t c = tga_get(v.normal, v.nw, v.nh, cvt_i32(fm(u, (float)v.nw)), cvt_i32(fm(t, (float)v.nh)));
  F3 r;
  r.z = bt.u8n[c & 255u];
  r.y = bt.u8n[(c >> 8) & 255u];
  r.x = bt.u8n[(c >> 16) & 255u];
  return r;
}

// barycentric() at the integer pixel (px, py) and the inside test of rasterize_triangle
// (graphics.cpp:222-233, :352-357) for a triangle with screen corner A = (ax, ay), edges
// e1 = B - A, e2 = C - A and u.z = e2.x*e1.y - e1.x*e2.y (|u.z| > 0.01).  Weights are
// (1 - (u.x+u.y)/u.z, u.y/u.z, u.x/u.z); the pixel is covered when all three are >= 0.
// `exact` selects the literal divisions; otherwise the sign test on u.x, u.y, u.x+u.y
// against u.z decides coverage without dividing (equal to the divisions' decision for
// coordinates in the range setup checks) and the weights are computed only when covered.
// The raster and the setup-side cull of pixel-less triangles share these functions, so both
// take the same decision for every pixel.
//
// The barycentric weights from the cross products (u.x = ux, u.y = uy, su = ux + uy).
__device__ __forceinline__ void cover_weights(float ux, float uy, float uz, float& b0, float& b1, float& b2) {
  b0 = fs(1.f, fd(fa(ux, uy), uz));
  b1 = fd(uy, uz);
  b2 = fd(ux, uz);
}

// The coverage decision alone, with the cross products the weights come from.
__device__ __forceinline__ bool cover_terms(float ax, float ay, float e1x, float e1y, float e2x, float e2y, float uz,
                                            bool exact, float pxf, float pyf, float& ux, float& uy) {
  const float dx = fs(ax, pxf), dy = fs(ay, pyf);
  ux = fs(fm(e1x, dy), fm(dx, e1y));
  uy = fs(fm(dx, e2y), fm(e2x, dy));
  if (!exact) {
    const float su = fa(ux, uy);
    return (uz < 0.f) ? (su >= uz && uy <= 0.f && ux <= 0.f) : (su <= uz && uy >= 0.f && ux >= 0.f);
  }
  float b0, b1, b2;
  cover_weights(ux, uy, uz, b0, b1, b2);
  return !(b0 < 0.f || b1 < 0.f || b2 < 0.f);
}

__device__ __forceinline__ bool cover_test(float ax, float ay, float e1x, float e1y, float e2x, float e2y, float uz,
                                           bool exact, float pxf, float pyf, float& b0, float& b1, float& b2) {
  float ux, uy;
  const bool covered = cover_terms(ax, ay, e1x, e1y, e2x, e2y, uz, exact, pxf, pyf, ux, uy);
  if (covered) cover_weights(ux, uy, uz, b0, b1, b2);
  return covered;
}

// (float)sqrt(1.0 - (double)s) for s = saturate(...) — the bump height of NormalMapShader
// (IShader.cpp:143), which the reference evaluates in double — in single precision (FP64 runs at
// a small fraction of the FP32 rate on this part).  For s >= 2^-29, 1 - s is exactly hi + lo
// (Fast2Sum); y = sqrtf(hi) is refined by one Newton step on the exact FMA residual hi - y*y
// (the correction step of Markstein's square root), which gives the correctly rounded square
// root of hi + lo except where it lands on a rounding midpoint.  Checked against the double
// expression for every float s in [0, 1] (tests/cuda/bump_z_check.cu): it differs only at
// s = 1 (0/0 in the correction: the answer is 0) and s = 2^-24 (1 - 2^-24 exactly; its square
// root lies 2^-51 below the midpoint 1 - 2^-25 that the float correction reaches); below 2^-29
// every s gives 1.  NaN keeps the double expression.
__device__ __forceinline__ float bump_height(float s) {
  if (!(s >= 0x1p-29f)) return s != s ? __double2float_rn(__dsqrt_rn(__dsub_rn(1.0, (double)s))) : 1.f;
  if (s == 1.f) return 0.f;
  if (s == 0x1p-24f) return 0x1.fffffep-1f;
  const float hi = __fsub_rn(1.f, s);
  const float lo = __fsub_rn(__fsub_rn(1.f, hi), s);  // exact: 1 - s = hi + lo
  const float y = __fsqrt_rn(hi);
  const float e = __fmaf_rn(-y, y, hi);              // exact residual hi - y*y
  return __fadd_rn(y, __fdiv_rn(__fadd_rn(e, lo), __fadd_rn(y, y)));
}

// viewport_transform (maths.cpp:20-25)
__device__ __forceinline__ F3 viewport(int32_t w, int32_t h, F3 ndc) {
  return {fm(fm(fa(ndc.x, 1.f), 0.5f), (float)w), fm(fm(fa(ndc.y, 1.f), 0.5f), (float)h), fm(fa(ndc.z, 1.f), 0.5f)};
}

// IShader::is_in_shadow (IShader.h:107-129).  The shadow map's colour plane was written by
// an earlier view of the batch: read it past L1 (ld.global.cg).
__device__ __forceinline__ int is_in_shadow(const DView& v, float4 dp, float n_dot_l, const ByteTables& bt) {
  if (v.u.enable_shadow && v.sm_color) {
    float widht = (float)v.smW, height = (float)v.smH;
    F3 ndc = {fd(dp.x, dp.w), fd(dp.y, dp.w), fd(dp.z, dp.w)};
    F3 pos = viewport(v.smW, v.smH, ndc);
    float depth_bias = fm(0.05f, fs(1.f, n_dot_l));
    if (depth_bias < 0.005f) depth_bias = 0.01f;
    float current_depth = fs(dp.z, depth_bias);
    if (pos.x < 0.f || pos.y < 0.f || pos.x >= widht || pos.y >= height) return 1;
    if (pos.x != pos.x || pos.y != pos.y) return 1;  // NaN: undefined in the reference; lit
    int32_t x = cvt_i32(pos.x), y = cvt_i32(pos.y);
    uint32_t word = __ldcg(v.sm_color + (size_t)y * (size_t)v.smW + (size_t)x);
    float closest_depth = bt.u8f[word & 255u];
    return current_depth < closest_depth;
  }
  return 1;
}

// ---- fragment shaders (IShader.cpp) ---------------------------------------------------------
// Perspective-correct interpolation (graphics.cpp:205-220) of the varyings a shader reads,
// from the record's payload (Payload layout in hsr_internal.h) and the pixel's barycentric
// weights, then the fragment shader.  Specialised per shader at compile time so each one
// interpolates only what it reads (every float interpolates independently, so skipping
// the others changes no bit).
__device__ __forceinline__ float interp(float s0, float s1, float s2, float w0, float w1, float w2, float nrm) {
  return fm(fa(fa(fm(s0, w0), fm(s1, w1)), fm(s2, w2)), nrm);
}

// Payload float4s a shader reads (layout in hsr_internal.h).
template <int S> __device__ __forceinline__ constexpr int payload_f4_of() {
  return S == HSR_SHADER_FLAT ? 0
       : (S == HSR_SHADER_SHADOW || S == HSR_SHADER_GROUND || S == HSR_SHADER_TOON) ? 2
       : S == HSR_SHADER_TEXTURE ? 3
       : S == HSR_SHADER_TEXTURE_WITH_LIGHT ? 6 : 8;
}

// Blinn-Phong tail shared by BlinnShader and NormalMapShader (IShader.cpp:94-109, :146-162).
__device__ __forceinline__ Col lit(const DView& v, F3 N, F3 wpos, float u, float t, const ByteTables& bt) {
  const hsr_shader_data& un = v.u;
  F3 L = {un.light_dir[0], un.light_dir[1], un.light_dir[2]};
  F3 vp = {un.view_pos[0], un.view_pos[1], un.view_pos[2]};
  Col albedo = c_mulc(tex_diffuse(v, u, t, bt), c_of(un.material_color));
  Col ambient = c_mulc(c_of(un.ambient), albedo);
  float n_dot_l = saturate(dot3(N, L));
  Col diffuse = c_mulf(c_mulc(c_of(un.light_color), albedo), n_dot_l);
  F3 view_dir = normalize3(sub3(vp, wpos));
  F3 half_dir = normalize3(add3(view_dir, L));
  Col spec = c_mulf(c_mulc(c_of(un.light_color), c_of(un.material_specular)),
                    powf(saturate(dot3(N, half_dir)), un.gloss));
  float4 depth_pos = mat_vec(un.light_vp_matrix, wpos.x, wpos.y, wpos.z, 1.f);
  int shadow = is_in_shadow(v, depth_pos, n_dot_l, bt);
  return c_add(ambient, c_mulf(c_add(diffuse, spec), (float)shadow));
}

template <int S>
__device__ __forceinline__ Col fragment_s(const DView& v, const float* P, float b0, float b1, float b2, uint32_t prim,
                                          const ByteTables& bt) {
  const Col white = {1.f, 1.f, 1.f, 255.f};
  if constexpr (S == HSR_SHADER_FLAT) {  // test shader: bytes of the prim id
    return {fd(fa((float)(prim & 255u), 0.5f), 255.f), fd(fa((float)((prim >> 8) & 255u), 0.5f), 255.f),
            fd(fa((float)((prim >> 16) & 255u), 0.5f), 255.f), 255.f};
  } else {
    const float w0 = fm(P[0], b0), w1 = fm(P[1], b1), w2 = fm(P[2], b2);
    const float nrm = __frcp_rn(fa(fa(w0, w1), w2));
    if constexpr (S == HSR_SHADER_SHADOW) {  // IShader.cpp:176-180
      return c_mulf(white, interp(P[3], P[4], P[5], w0, w1, w2, nrm));
    } else if constexpr (S == HSR_SHADER_GROUND) {  // IShader.cpp:12-15
      return c_mulf(white, interp(P[3], P[4], P[5], w0, w1, w2, nrm));
    } else if constexpr (S == HSR_SHADER_TOON) {  // IShader.cpp:30-39
      // The reference compares the float against double constants: (double)f > c holds exactly
      // when f > the largest float not above c (none of these constants is a float), so each
      // compare runs in single precision with that float.
      float intensity = interp(P[3], P[4], P[5], w0, w1, w2, nrm);
      if (intensity > 0x1.b33332p-1f) intensity = 1.f;               // .85
      else if (intensity > 0x1.333332p-1f) intensity = (float).80;   // .60
      else if (intensity > 0x1.ccccccp-2f) intensity = (float).60;   // .45
      else if (intensity > 0x1.333332p-2f) intensity = (float).45;   // .30
      else if (intensity > 0x1.333332p-3f) intensity = (float).30;   // .15
      Col base = {1.f, fd(155.f, 255.f), 0.f, 255.f};
      return c_mulf(base, intensity);
    } else {
      const float u = interp(P[6], P[8], P[10], w0, w1, w2, nrm);
      const float t = interp(P[7], P[9], P[11], w0, w1, w2, nrm);
      if constexpr (S == HSR_SHADER_TEXTURE) {  // IShader.cpp:54-57
        return tex_diffuse(v, u, t, bt);
      } else {
        const F3 wn = {interp(P[12], P[15], P[18], w0, w1, w2, nrm), interp(P[13], P[16], P[19], w0, w1, w2, nrm),
                       interp(P[14], P[17], P[20], w0, w1, w2, nrm)};
        if constexpr (S == HSR_SHADER_TEXTURE_WITH_LIGHT) {  // IShader.cpp:73-77
          F3 L = {v.u.light_dir[0], v.u.light_dir[1], v.u.light_dir[2]};
          return c_mulf(tex_diffuse(v, u, t, bt), saturate(dot3(wn, L)));
        } else {
          const F3 wp = {interp(P[21], P[24], P[27], w0, w1, w2, nrm), interp(P[22], P[25], P[28], w0, w1, w2, nrm),
                         interp(P[23], P[26], P[29], w0, w1, w2, nrm)};
          if constexpr (S == HSR_SHADER_BLINN) {  // IShader.cpp:94-109
            return lit(v, normalize3(wn), wp, u, t, bt);
          } else {  // NormalMapShader, IShader.cpp:126-162
            F3 n = wn;
            float x = n.x, y = n.y, z = n.z;
            float sq = __fsqrt_rn(fa(fm(x, x), fm(z, z)));
            F3 tg = {fd(fm(x, y), sq), sq, fd(fm(z, y), sq)};
            F3 b = cross3(n, tg);
            F3 r0 = {tg.x, b.x, n.x}, r1 = {tg.y, b.y, n.y}, r2 = {tg.z, b.z, n.z};
            F3 bump = tex_normal(v, u, t, bt);
            bump.x = fm(bump.x, v.u.bump_scale);
            bump.y = fm(bump.y, v.u.bump_scale);
            float bb = fa(fa(0.f, fm(bump.y, bump.y)), fm(bump.x, bump.x));
            bump.z = bump_height(saturate(bb));  // (float)sqrt(1.0 - saturate(bb)) in double, IShader.cpp:143
            F3 tn = {dot3(r0, bump), dot3(r1, bump), dot3(r2, bump)};
            return lit(v, normalize3(tn), wp, u, t, bt);
          }
        }
      }
    }
  }
}

// 32-byte vector global store (sm_100 and later): two float4s in one instruction, so the record
// and payload stores of the cull and emit passes take half the load/store-unit slots; the address
// must be 32-byte aligned (records are 64 bytes, payloads 128, both arrays 256-byte aligned).
__device__ __forceinline__ void st_v8(void* p, float4 a, float4 b) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"l"(p), "f"(a.x), "f"(a.y), "f"(a.z), "f"(a.w),
               "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
               : "memory");
}
// set_color (renderbuffer.cpp:38-44): R, G, B through (uchar)(c*255); alpha kept.
__device__ __forceinline__ uint32_t pack_rgb(Col c, uint32_t alpha_word) {
  uint32_t r = (uint32_t)cvt_i32(fm(c.r, 255.f)) & 255u;
  uint32_t g = (uint32_t)cvt_i32(fm(c.g, 255.f)) & 255u;
  uint32_t b = (uint32_t)cvt_i32(fm(c.b, 255.f)) & 255u;
  return r | (g << 8) | (b << 16) | (alpha_word & 0xFF000000u);
}

}  // namespace hsr
