/*
 * hsr_oracle.c — TEST INFRASTRUCTURE ONLY: CPU restatement of the reference draw path.
 *
 * Each function names the reference code it follows (file:line, relative to the
 * Hana-SoftwareRenderer source directory).  Operation order, float/double promotion and
 * the std::min/std::max ternary NaN behaviour are kept, so that with -ffp-contract=off
 * the buffers match the reference bit for bit (powf excepted where the C library
 * differs).  Undefined behaviour of the reference is given one fixed meaning here and in
 * the GPU path:
 *   - float -> int conversions follow x86 cvttss2si: truncation, INT_MIN when the value
 *     is NaN or out of range (texture coordinates, bounding-box start);
 *   - the homogeneous clipper gets ping-pong buffers large enough for 10 vertices (the
 *     reference writes the odd planes' output into a 3-element array, graphics.cpp:379
 *     with :153,:155,:157);
 *   - is_in_shadow treats a NaN light-space position as lit (the reference would index
 *     the shadow map with (int)NaN).
 */
#define _POSIX_C_SOURCE 200809L
#include "hsr_oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define EPSILON 1e-5f /* maths.h:6 */
#define NV 13         /* floats in shader_struct_v2f (IShader.h:41-47) */

typedef struct { float x, y; } v2;
typedef struct { float x, y, z; } v3;
typedef struct { float x, y, z, w; } v4;
typedef struct { float r, g, b, a; } color;

/* shader_struct_v2f as a flat float array, the view both interpolators take
 * (graphics.cpp:7-17, :205-220): [0..3] clip_pos, [4..6] world_pos, [7..9] world_normal,
 * [10..11] uv, [12] intensity. */
typedef struct { float f[NV]; } v2f;

/* ---- scalar helpers -------------------------------------------------------------- */
static float std_min(float a, float b) { return (b < a) ? b : a; }     /* std::min */
static float std_max(float a, float b) { return (a < b) ? b : a; }     /* std::max */
static float saturate(float f) { return f < 0 ? 0 : (f > 1 ? 1 : f); } /* maths.cpp:13-15 */

/* float -> int32 as x86 cvttss2si (the reference's platform). */
static int32_t cvt_i32(float f) {
  if (!(f > -2147483904.0f && f < 2147483648.0f)) return INT_MIN;
  return (int32_t)f;
}

/* Vector operator* (vector.h:69-73): accumulate from the last index down. */
static float dot3(v3 a, v3 b) {
  float r = 0.f;
  r += a.z * b.z;
  r += a.y * b.y;
  r += a.x * b.x;
  return r;
}
static float dot4(const float* a, const float* b) {
  float r = 0.f;
  r += a[3] * b[3];
  r += a[2] * b[2];
  r += a[1] * b[1];
  r += a[0] * b[0];
  return r;
}
static v3 sub3(v3 a, v3 b) { v3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static v3 add3(v3 a, v3 b) { v3 r = {a.x + b.x, a.y + b.y, a.z + b.z}; return r; }
static v3 cross3(v3 a, v3 b) { /* vector.h:97-99 */
  v3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static v3 normalize3(v3 v) { /* vector.h:41-42 */
  float n = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
  float f = 1.f / n;
  v.x *= f; v.y *= f; v.z *= f;
  return v;
}

/* Matrix product, result[i][j] = lhs[i] * rhs.getCol(j) (matrix.h:118-123). */
static void mat_mul(const float* a, const float* b, float* out) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      float col[4] = {b[0 * 4 + j], b[1 * 4 + j], b[2 * 4 + j], b[3 * 4 + j]};
      out[i * 4 + j] = dot4(&a[i * 4], col);
    }
}
/* Matrix * vector, ret[i] = lhs[i] * rhs (matrix.h:112-116). */
static v4 mat_vec(const float* m, v4 v) {
  float vv[4] = {v.x, v.y, v.z, v.w};
  v4 r = {dot4(&m[0], vv), dot4(&m[4], vv), dot4(&m[8], vv), dot4(&m[12], vv)};
  return r;
}

/* ---- Color (color.cpp:38-64) ------------------------------------------------------- */
static color c_add(color a, color b) {
  color r;
  r.r = std_min(std_max(0.f, a.r + b.r), 1.f);
  r.g = std_min(std_max(0.f, a.g + b.g), 1.f);
  r.b = std_min(std_max(0.f, a.b + b.b), 1.f);
  r.a = std_min(std_max(0.f, a.a + b.a), 1.f);
  return r;
}
static color c_mulf(color a, float t) {
  t = (t > 1.f ? 1.f : (t < 0.f ? 0.f : t));
  color r;
  r.r = std_min(std_max(0.f, a.r * t), 1.f);
  r.g = std_min(std_max(0.f, a.g * t), 1.f);
  r.b = std_min(std_max(0.f, a.b * t), 1.f);
  r.a = std_min(std_max(0.f, a.a * t), 1.f);
  return r;
}
static color c_mulc(color a, color b) {
  color r = {a.r * b.r, a.g * b.g, a.b * b.b, a.a * b.a};
  return r;
}
static color c_of(const float* p) { color c = {p[0], p[1], p[2], p[3]}; return c; }

/* ---- textures: TGAImage::get (tgaimage.cpp:248-253), Color(TGAColor) (color.cpp:5) -- */
static void tga_get(const hsro_texture* t, int32_t x, int32_t y, uint8_t bgra[4]) {
  bgra[0] = bgra[1] = bgra[2] = bgra[3] = 0;
  if (!t || !t->data || x < 0 || y < 0 || x >= t->w || y >= t->h) return;
  const uint8_t* p = t->data + ((size_t)x + (size_t)y * (size_t)t->w) * (size_t)t->bpp;
  for (int i = 0; i < t->bpp; i++) bgra[i] = p[i];
}
static int32_t tex_w(const hsro_texture* t) { return t ? t->w : 0; }
static int32_t tex_h(const hsro_texture* t) { return t ? t->h : 0; }

/* IShader::tex_diffuse (IShader.h:85-89) */
static color tex_diffuse(const hsro_texture* t, float u, float v) {
  uint8_t c[4];
  tga_get(t, cvt_i32(u * (float)tex_w(t)), cvt_i32(v * (float)tex_h(t)), c);
  color r = {c[2] / 255.f, c[1] / 255.f, c[0] / 255.f, c[3] / 255.f};
  return r;
}
/* IShader::tex_normal (IShader.h:91-99) */
static v3 tex_normal(const hsro_texture* t, float u, float v) {
  uint8_t c[4];
  tga_get(t, cvt_i32(u * (float)tex_w(t)), cvt_i32(v * (float)tex_h(t)), c);
  v3 r;
  r.z = (float)c[0] / 255.f * 2.f - 1.f;
  r.y = (float)c[1] / 255.f * 2.f - 1.f;
  r.x = (float)c[2] / 255.f * 2.f - 1.f;
  return r;
}

/* ---- draw context ------------------------------------------------------------------ */
typedef struct ctx {
  const hsr_shader_data* sd;
  int32_t shader;
  float mvp[16]; /* camera_vp*model or light_vp*model, identical to the per-corner product */
  const hsro_texture* diffuse;
  const hsro_texture* normal;
  const hsro_target* shadow_map;
  hsro_target* target;
} ctx;

/* viewport_transform (maths.cpp:20-25) */
static v3 viewport(int32_t width, int32_t height, v3 ndc) {
  v3 r;
  r.x = (ndc.x + 1) * 0.5f * (float)width;
  r.y = (ndc.y + 1) * 0.5f * (float)height;
  r.z = (ndc.z + 1) * 0.5f;
  return r;
}

/* IShader::is_in_shadow (IShader.h:107-129) */
static int is_in_shadow(const ctx* c, v4 dp, float n_dot_l) {
  if (c->sd->enable_shadow && c->shadow_map) {
    float widht = (float)c->shadow_map->w;
    float height = (float)c->shadow_map->h;
    v3 ndc = {dp.x / dp.w, dp.y / dp.w, dp.z / dp.w};
    v3 pos = viewport((int32_t)widht, (int32_t)height, ndc);
    float depth_bias = 0.05f * (1 - n_dot_l);
    if (depth_bias < 0.005f) depth_bias = 0.01f;
    float current_depth = dp.z - depth_bias;
    if (pos.x < 0 || pos.y < 0 || pos.x >= widht || pos.y >= height) return 1;
    if (pos.x != pos.x || pos.y != pos.y) return 1; /* UB in the reference, see header */
    int32_t x = cvt_i32(pos.x), y = cvt_i32(pos.y);
    float closest_depth = c->shadow_map->color[((size_t)y * c->shadow_map->w + x) * 4 + 0] / 255.f;
    return current_depth < closest_depth;
  }
  return 1;
}

/* ---- vertex shaders (IShader.cpp) ----------------------------------------------------- */
static v4 object_to(const float* mvp, const float* p) {
  v4 v = {p[0], p[1], p[2], 1.f};
  return mat_vec(mvp, v);
}
static v3 object_to_world_pos(const hsr_shader_data* sd, const float* p) { /* IShader.h:63-65 */
  v4 v = {p[0], p[1], p[2], 1.f};
  v4 r = mat_vec(sd->model_matrix, v);
  v3 o = {r.x, r.y, r.z};
  return o;
}
static v3 object_to_world_normal(const hsr_shader_data* sd, v3 n) { /* IShader.h:71-75 */
  float row[4] = {n.x, n.y, n.z, 1.f};
  const float* m = sd->model_matrix_I;
  v3 r;
  float col[4];
  col[0] = m[0]; col[1] = m[4]; col[2] = m[8]; col[3] = m[12]; r.x = dot4(row, col);
  col[0] = m[1]; col[1] = m[5]; col[2] = m[9]; col[3] = m[13]; r.y = dot4(row, col);
  col[0] = m[2]; col[1] = m[6]; col[2] = m[10]; col[3] = m[14]; r.z = dot4(row, col);
  return r;
}

static v2f vertex(const ctx* c, const float* pos, v3 nrm, const float* uv) {
  v2f o;
  memset(&o, 0, sizeof(o));
  const hsr_shader_data* sd = c->sd;
  v4 clip = object_to(c->mvp, pos);
  o.f[0] = clip.x; o.f[1] = clip.y; o.f[2] = clip.z; o.f[3] = clip.w;
  v3 ld = {sd->light_dir[0], sd->light_dir[1], sd->light_dir[2]};
  switch (c->shader) {
    case HSR_SHADER_GROUND: /* IShader.cpp:5-10 */
    case HSR_SHADER_TOON: { /* IShader.cpp:23-28 */
      o.f[12] = saturate(dot3(object_to_world_normal(sd, nrm), ld));
      break;
    }
    case HSR_SHADER_TEXTURE: /* IShader.cpp:47-52 */
      o.f[10] = uv[0]; o.f[11] = uv[1];
      break;
    case HSR_SHADER_TEXTURE_WITH_LIGHT: { /* IShader.cpp:65-71 */
      v3 wn = object_to_world_normal(sd, nrm);
      o.f[7] = wn.x; o.f[8] = wn.y; o.f[9] = wn.z;
      o.f[10] = uv[0]; o.f[11] = uv[1];
      break;
    }
    case HSR_SHADER_BLINN:       /* IShader.cpp:85-92 */
    case HSR_SHADER_NORMALMAP: { /* IShader.cpp:117-124 */
      v3 wp = object_to_world_pos(sd, pos);
      v3 wn = object_to_world_normal(sd, nrm);
      o.f[4] = wp.x; o.f[5] = wp.y; o.f[6] = wp.z;
      o.f[7] = wn.x; o.f[8] = wn.y; o.f[9] = wn.z;
      o.f[10] = uv[0]; o.f[11] = uv[1];
      break;
    }
    default: /* SHADOW (IShader.cpp:170-174) and FLAT: clip position only */
      break;
  }
  return o;
}

/* ---- fragment shaders (IShader.cpp) --------------------------------------------------- */
static color lit(const ctx* c, v3 N, const v2f* v) { /* shared tail of Blinn / NormalMap */
  const hsr_shader_data* sd = c->sd;
  v3 L = {sd->light_dir[0], sd->light_dir[1], sd->light_dir[2]};
  v3 wp = {v->f[4], v->f[5], v->f[6]};
  v3 vp = {sd->view_pos[0], sd->view_pos[1], sd->view_pos[2]};
  color albedo = c_mulc(tex_diffuse(c->diffuse, v->f[10], v->f[11]), c_of(sd->material_color));
  color ambient = c_mulc(c_of(sd->ambient), albedo);
  float n_dot_l = saturate(dot3(N, L));
  color diffuse = c_mulf(c_mulc(c_of(sd->light_color), albedo), n_dot_l);
  v3 view_dir = normalize3(sub3(vp, wp));
  v3 half_dir = normalize3(add3(view_dir, L));
  color spec = c_mulf(c_mulc(c_of(sd->light_color), c_of(sd->material_specular)),
                      powf(saturate(dot3(N, half_dir)), sd->gloss));
  v4 wp4 = {wp.x, wp.y, wp.z, 1.f};
  v4 depth_pos = mat_vec(sd->light_vp_matrix, wp4);
  int shadow = is_in_shadow(c, depth_pos, n_dot_l);
  return c_add(ambient, c_mulf(c_add(diffuse, spec), (float)shadow));
}

static color fragment(const ctx* c, const v2f* v, uint32_t prim) {
  static const color white = {1.f, 1.f, 1.f, 255.f};
  const hsr_shader_data* sd = c->sd;
  switch (c->shader) {
    case HSR_SHADER_GROUND: /* IShader.cpp:12-15 */
      return c_mulf(white, v->f[12]);
    case HSR_SHADER_TOON: { /* IShader.cpp:30-39 */
      float intensity = v->f[12];
      if ((double)intensity > .85) intensity = 1;
      else if ((double)intensity > .60) intensity = (float).80;
      else if ((double)intensity > .45) intensity = (float).60;
      else if ((double)intensity > .30) intensity = (float).45;
      else if ((double)intensity > .15) intensity = (float).30;
      color base = {1.f, 155 / 255.f, 0.f, 255.f};
      return c_mulf(base, intensity);
    }
    case HSR_SHADER_TEXTURE: /* IShader.cpp:54-57 */
      return tex_diffuse(c->diffuse, v->f[10], v->f[11]);
    case HSR_SHADER_TEXTURE_WITH_LIGHT: { /* IShader.cpp:73-77 */
      v3 wn = {v->f[7], v->f[8], v->f[9]};
      v3 L = {sd->light_dir[0], sd->light_dir[1], sd->light_dir[2]};
      float intensity = saturate(dot3(wn, L));
      return c_mulf(tex_diffuse(c->diffuse, v->f[10], v->f[11]), intensity);
    }
    case HSR_SHADER_BLINN: { /* IShader.cpp:94-109 */
      v3 wn = {v->f[7], v->f[8], v->f[9]};
      return lit(c, normalize3(wn), v);
    }
    case HSR_SHADER_NORMALMAP: { /* IShader.cpp:126-162 */
      v3 n = {v->f[7], v->f[8], v->f[9]};
      float x = n.x, y = n.y, z = n.z;
      v3 t = {x * y / sqrtf(x * x + z * z), sqrtf(x * x + z * z), z * y / sqrtf(x * x + z * z)};
      v3 b = cross3(n, t);
      v3 r0 = {t.x, b.x, n.x}, r1 = {t.y, b.y, n.y}, r2 = {t.z, b.z, n.z};
      v3 bump = tex_normal(c->normal, v->f[10], v->f[11]);
      bump.x = bump.x * sd->bump_scale;
      bump.y = bump.y * sd->bump_scale;
      float bb = 0.f;
      bb += bump.y * bump.y;
      bb += bump.x * bump.x;
      bump.z = (float)sqrt(1.0 - (double)saturate(bb));
      v3 tn = {dot3(r0, bump), dot3(r1, bump), dot3(r2, bump)};
      return lit(c, normalize3(tn), v);
    }
    case HSR_SHADER_SHADOW: /* IShader.cpp:176-180 */
      return c_mulf(white, v->f[2]);
    case HSR_SHADER_FLAT: { /* test shader: prim id bytes */
      color r = {((prim & 255u) + 0.5f) / 255.f, (((prim >> 8) & 255u) + 0.5f) / 255.f,
                 (((prim >> 16) & 255u) + 0.5f) / 255.f, 255.f};
      return r;
    }
    default: {
      color z = {0, 0, 0, 0};
      return z;
    }
  }
}

/* ---- homogeneous clipping (graphics.cpp:7-161) ----------------------------------------- */
enum { PW, PX, NX, PY, NY, PZ, NZ };

static int is_inside_plane(const float* c, int plane) { /* graphics.cpp:29-49 */
  switch (plane) {
    case PW: return c[3] >= EPSILON;
    case PX: return c[0] <= +c[3];
    case NX: return c[0] >= -c[3];
    case PY: return c[1] <= +c[3];
    case NY: return c[1] >= -c[3];
    case PZ: return c[2] <= +c[3];
    default: return c[2] >= -c[3];
  }
}
static float intersect_ratio(const float* p, const float* q, int plane) { /* :51-71 */
  switch (plane) {
    case PW: return (p[3] - EPSILON) / (p[3] - q[3]);
    case PX: return (p[3] - p[0]) / ((p[3] - p[0]) - (q[3] - q[0]));
    case NX: return (p[3] + p[0]) / ((p[3] + p[0]) - (q[3] + q[0]));
    case PY: return (p[3] - p[1]) / ((p[3] - p[1]) - (q[3] - q[1]));
    case NY: return (p[3] + p[1]) / ((p[3] + p[1]) - (q[3] + q[1]));
    case PZ: return (p[3] - p[2]) / ((p[3] - p[2]) - (q[3] - q[2]));
    default: return (p[3] + p[2]) / ((p[3] + p[2]) - (q[3] + q[2]));
  }
}
static int clip_against_plane(int plane, int n, const v2f* in, v2f* out) { /* :73-110 */
  int m = 0;
  for (int i = 0; i < n; i++) {
    int pi = (i - 1 + n) % n;
    const v2f* prev = &in[pi];
    const v2f* curr = &in[i];
    int pin = is_inside_plane(prev->f, plane);
    int cin = is_inside_plane(curr->f, plane);
    if (pin != cin) {
      float t = intersect_ratio(prev->f, curr->f, plane);
      for (int k = 0; k < NV; k++) out[m].f[k] = prev->f[k] + (curr->f[k] - prev->f[k]) * t; /* :7-17 */
      m++;
    }
    if (cin) out[m++] = *curr;
  }
  return m;
}
static int is_vertex_visible(const float* c) { /* :132-134 */
  return fabsf(c[0]) <= c[3] && fabsf(c[1]) <= c[3] && fabsf(c[2]) <= c[3];
}
/* clip_triangle (:136-161); poly receives the result, at most 10 vertices. */
static int clip_triangle(const v2f* tri, v2f* poly) {
  if (is_vertex_visible(tri[0].f) && is_vertex_visible(tri[1].f) && is_vertex_visible(tri[2].f)) {
    poly[0] = tri[0]; poly[1] = tri[1]; poly[2] = tri[2];
    return 3;
  }
  v2f a[16], b[16];
  a[0] = tri[0]; a[1] = tri[1]; a[2] = tri[2];
  int n = 3;
  static const int planes[7] = {PW, PX, NX, PY, NY, PZ, NZ};
  v2f* src = a;
  v2f* dst = b;
  for (int k = 0; k < 7; k++) {
    n = clip_against_plane(planes[k], n, src, dst);
    if (n < 3) return 0;
    v2f* t = src; src = dst; dst = t;
  }
  memcpy(poly, src, sizeof(v2f) * (size_t)n);
  return n;
}

/* ---- rasterisation (graphics.cpp:172-376) ------------------------------------------------ */
static int is_back_facing(const v3* ndc) { /* :172-180 */
  v3 a = ndc[0], b = ndc[1], c = ndc[2];
  float signed_area = a.x * b.y - a.y * b.x + b.x * c.y - b.y * c.x + c.x * a.y - c.y * a.x;
  return signed_area <= 0;
}
static v3 barycentric(v2 A, v2 B, v2 C, v2 P) { /* :222-233 */
  v3 s0, s1;
  s1.x = C.y - A.y; s1.y = B.y - A.y; s1.z = A.y - P.y; /* i = 1 */
  s0.x = C.x - A.x; s0.y = B.x - A.x; s0.z = A.x - P.x; /* i = 0 */
  v3 u = cross3(s0, s1);
  if ((double)fabsf(u.z) > 1e-2) {
    v3 r = {1.f - (u.x + u.y) / u.z, u.y / u.z, u.x / u.z};
    return r;
  }
  v3 r = {-1, 1, 1};
  return r;
}

static void set_color(hsro_target* t, size_t idx, color c) { /* renderbuffer.cpp:38-44 */
  t->color[idx * 4 + 0] = (uint8_t)cvt_i32(c.r * 255);
  t->color[idx * 4 + 1] = (uint8_t)cvt_i32(c.g * 255);
  t->color[idx * 4 + 2] = (uint8_t)cvt_i32(c.b * 255);
}

static void rasterize_triangle(const ctx* c, const v2f* v, uint32_t prim) { /* :314-376 */
  hsro_target* rb = c->target;
  v3 ndc[3];
  for (int i = 0; i < 3; i++) {
    float w = v[i].f[3];
    ndc[i].x = v[i].f[0] / w; ndc[i].y = v[i].f[1] / w; ndc[i].z = v[i].f[2] / w;
  }
  if (is_back_facing(ndc)) return;
  v2 sc[3];
  float sdepth[3];
  for (int i = 0; i < 3; i++) {
    v3 win = viewport(rb->w, rb->h, ndc[i]);
    sc[i].x = win.x; sc[i].y = win.y; sdepth[i] = win.z;
  }
  float recip_w[3];
  for (int i = 0; i < 3; i++) recip_w[i] = 1 / v[i].f[3];
  float bminx = FLT_MAX, bminy = FLT_MAX, bmaxx = -FLT_MAX, bmaxy = -FLT_MAX;
  float clampx = (float)(rb->w - 1), clampy = (float)(rb->h - 1);
  for (int i = 0; i < 3; i++) {
    bminx = std_max(0.f, std_min(bminx, sc[i].x));
    bmaxx = std_min(clampx, std_max(bmaxx, sc[i].x));
    bminy = std_max(0.f, std_min(bminy, sc[i].y));
    bmaxy = std_min(clampy, std_max(bmaxy, sc[i].y));
  }
  for (int32_t px = cvt_i32(bminx); (float)px <= bmaxx; px++) {
    for (int32_t py = cvt_i32(bminy); (float)py <= bmaxy; py++) {
      v2 P = {(float)px, (float)py};
      v3 bw = barycentric(sc[0], sc[1], sc[2], P);
      if (bw.x < 0 || bw.y < 0 || bw.z < 0) continue;
      size_t idx = (size_t)py * (size_t)rb->w + (size_t)px;
      float frag_depth = 0.f; /* interpolate_depth (:186-194) */
      frag_depth += sdepth[2] * bw.z;
      frag_depth += sdepth[1] * bw.y;
      frag_depth += sdepth[0] * bw.x;
      if (frag_depth > rb->depth[idx]) continue;
      v2f iv; /* interpolate_varyings (:205-220) */
      float w0 = recip_w[0] * bw.x, w1 = recip_w[1] * bw.y, w2 = recip_w[2] * bw.z;
      float normalizer = 1 / (w0 + w1 + w2);
      for (int k = 0; k < NV; k++) {
        float sum = v[0].f[k] * w0 + v[1].f[k] * w1 + v[2].f[k] * w2;
        iv.f[k] = sum * normalizer;
      }
      color col = fragment(c, &iv, prim);
      rb->depth[idx] = frag_depth;
      set_color(rb, idx, col);
      if (rb->prim) rb->prim[idx] = prim;
    }
  }
}

/* graphics_draw_triangle (:378-407); renormalise = Model::normal's in-place normalisation
 * on every access, or the normals used as stored (the library's hsr_mesh semantics). */
static int draw_mesh(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
                     const hsro_texture* diffuse, const hsro_texture* normal,
                     const hsro_target* shadow_map, hsro_target* target, uint32_t prim_base,
                     int renormalise) {
  if (shader < 0 || shader >= HSR_SHADER_COUNT) return -1;
  ctx c;
  c.sd = sd;
  c.shader = shader;
  c.diffuse = diffuse;
  c.normal = normal;
  c.shadow_map = shadow_map;
  c.target = target;
  /* ObjectToClipPos / ObjectToViewPos (IShader.h:55-61): the matrix product is the same
   * for every corner, so computing it once gives the same bits. */
  mat_mul(shader == HSR_SHADER_SHADOW ? sd->light_vp_matrix : sd->camera_vp_matrix,
          sd->model_matrix, c.mvp);
  v2f tri[3], poly[10];
  for (int32_t i = 0; i < mesh->nfaces; i++) {
    for (int j = 0; j < 3; j++) {
      const int32_t* corner = &mesh->faces[((size_t)i * 3 + (size_t)j) * 3];
      const float* p = &mesh->pos[(size_t)corner[0] * 3];
      const float* uv = &mesh->uv[(size_t)corner[1] * 2];
      float* np = &mesh->nrm[(size_t)corner[2] * 3];
      v3 n = {np[0], np[1], np[2]};
      if (renormalise) {
        n = normalize3(n); /* Model::normal normalises in place (model.cpp:108-111) */
        np[0] = n.x; np[1] = n.y; np[2] = n.z;
      }
      tri[j] = vertex(&c, p, n, uv);
    }
    int nv = clip_triangle(tri, poly);
    for (int j = 0; j < nv - 2; j++) {
      v2f t[3] = {poly[0], poly[j + 1], poly[j + 2]};
      rasterize_triangle(&c, t, prim_base + (uint32_t)i + 1u);
    }
  }
  return 0;
}

int hsro_draw(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
              const hsro_texture* diffuse, const hsro_texture* normal,
              const hsro_target* shadow_map, hsro_target* target, uint32_t prim_base) {
  return draw_mesh(mesh, shader, sd, diffuse, normal, shadow_map, target, prim_base, 1);
}

int hsro_draw_stored_normals(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
                             const hsro_texture* diffuse, const hsro_texture* normal,
                             const hsro_target* shadow_map, hsro_target* target, uint32_t prim_base) {
  return draw_mesh(mesh, shader, sd, diffuse, normal, shadow_map, target, prim_base, 0);
}

void hsro_clear(hsro_target* t, const uint8_t rgba[4], float depth) { /* renderbuffer.cpp:59-75 */
  size_t n = (size_t)t->w * (size_t)t->h;
  for (size_t i = 0; i < n; i++) {
    memcpy(t->color + 4 * i, rgba, 4);
    t->depth[i] = depth;
    if (t->prim) t->prim[i] = 0;
  }
}

/* ---- CPU baseline throughput --------------------------------------------------------- */
typedef struct bench_arg {
  const hsro_mesh* mesh;
  int32_t shader;
  const hsr_shader_data* sd;
  const hsro_texture* diffuse;
  const hsro_texture* normal;
  int32_t w, h, sw, shh, frames;
  int ok;
} bench_arg;

static void* bench_thread(void* p) {
  bench_arg* a = (bench_arg*)p;
  a->ok = 0;
  hsro_mesh m = *a->mesh;
  float* nrm = (float*)malloc(sizeof(float) * 3 * (size_t)(m.nnrm > 0 ? m.nnrm : 1));
  hsro_target main_t = {a->w, a->h, malloc((size_t)a->w * a->h * 4), malloc(sizeof(float) * (size_t)a->w * a->h), NULL};
  hsro_target sh_t = {a->sw, a->shh, NULL, NULL, NULL};
  if (a->sw > 0) {
    sh_t.color = malloc((size_t)a->sw * a->shh * 4);
    sh_t.depth = malloc(sizeof(float) * (size_t)a->sw * a->shh);
  }
  if (!nrm || !main_t.color || !main_t.depth || (a->sw > 0 && (!sh_t.color || !sh_t.depth))) goto done;
  memcpy(nrm, m.nrm, sizeof(float) * 3 * (size_t)m.nnrm);
  m.nrm = nrm; /* private copy: Model::normal mutates it */
  {
    const uint8_t black[4] = {0, 0, 0, 1};
    for (int f = 0; f < a->frames; f++) {
      if (a->sw > 0) {
        hsro_clear(&sh_t, black, FLT_MAX);
        hsro_draw(&m, HSR_SHADER_SHADOW, a->sd, a->diffuse, a->normal, NULL, &sh_t, 0);
      }
      hsro_clear(&main_t, black, FLT_MAX);
      hsro_draw(&m, a->shader, a->sd, a->diffuse, a->normal, a->sw > 0 ? &sh_t : NULL, &main_t, 0);
    }
  }
  a->ok = 1;
done:
  free(nrm);
  free(main_t.color); free(main_t.depth);
  free(sh_t.color); free(sh_t.depth);
  return NULL;
}

double hsro_bench_frames(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
                         const hsro_texture* diffuse, const hsro_texture* normal,
                         int32_t w, int32_t h, int32_t shadow_w, int32_t shadow_h,
                         int32_t frames_each, int32_t threads) {
  if (threads < 1 || threads > 1024) return -1.0;
  pthread_t* tid = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  bench_arg* args = (bench_arg*)calloc((size_t)threads, sizeof(bench_arg));
  if (!tid || !args) { free(tid); free(args); return -1.0; }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int i = 0; i < threads; i++) {
    bench_arg a = {mesh, shader, sd, diffuse, normal, w, h, shadow_w, shadow_h, frames_each, 0};
    args[i] = a;
    pthread_create(&tid[i], NULL, bench_thread, &args[i]);
  }
  int ok = 1;
  for (int i = 0; i < threads; i++) {
    pthread_join(tid[i], NULL);
    ok &= args[i].ok;
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  free(tid);
  free(args);
  if (!ok) return -1.0;
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

int hsro_no_contraction(void) {
  volatile float a = 1.0f + 0x1p-12f, b = 1.0f + 0x1p-12f, c = -(1.0f + 0x1p-11f);
  float r = a * b + c;
  return r == 0.0f;
}
