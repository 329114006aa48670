/*
 * hsr_host_abi.c — TEST INFRASTRUCTURE ONLY.
 *
 * A host-memory stand-in for the entry points of include/hsr.h that the drop-in shim
 * (hana-softwarerenderer_gb300/shim/hsr_graphics_shim.cpp) calls: hsr_init, mesh and
 * texture upload, hsr_mesh_update_normals, target create / upload / download / release,
 * hsr_draw and hsr_last_error.  hsr_draw is drawn by the oracle with the library's
 * semantics (normals used as stored, HSR_DRAW_CLEAR, prim ids).  Linked with the shim in
 * place of libhsr.so (oracle/Makefile, target shim-host), it lets the shim's own logic
 * run on a host without a GPU — the IShader typeid dispatch, the per-draw re-read of
 * normals through Model::normal, the RenderBuffer mirroring and the shadow-map upload —
 * and be compared with the reference's own graphics.cpp on the same jobs.  Never linked
 * into the product; the GPU library is libhsr.so.
 *
 * Handles are 1-based indices into per-kind tables; validation is what the shim's calls
 * need (null pointers, sizes, indices), with the same status codes as the library.
 */
#include <stdlib.h>
#include <string.h>

#include "hsr_oracle.h"

typedef struct host_mesh {
  float *pos, *nrm, *uv;
  int32_t *faces;
  int32_t npos, nnrm, nuv, nfaces;
} host_mesh;

typedef struct host_tex {
  uint8_t* data;
  int32_t w, h, bpp;
} host_tex;

typedef struct host_target {
  int32_t w, h;
  uint8_t* color;
  float* depth;
  uint32_t* prim;
} host_target;

static int g_init = 0;
static const char* g_err = "";
static host_mesh** g_meshes;
static host_tex** g_texs;
static host_target** g_targets;
static size_t g_nmesh, g_ntex, g_ntarget;

static int fail(int code, const char* what) {
  g_err = what;
  return code;
}

static void* dup_bytes(const void* src, size_t n) {
  void* p = malloc(n ? n : 1);
  if (p && n) memcpy(p, src, n);
  return p;
}

/* appends `obj` to a table; returns its 1-based handle, 0 when out of memory */
static uint64_t add(void*** table, size_t* n, void* obj) {
  void** t = (void**)realloc(*table, sizeof(void*) * (*n + 1));
  if (!t) return 0;
  *table = t;
  t[*n] = obj;
  return (uint64_t)++*n;
}

static void* lookup(void** table, size_t n, uint64_t h) {
  return (h >= 1 && h <= n) ? table[h - 1] : NULL;
}

const char* hsr_last_error(void) { return g_err; }

int hsr_init(int device) {
  if (device != 0) return fail(HSR_ERR_INVALID_ARG, "host stand-in: device 0 only");
  g_init = 1;
  return HSR_OK;
}

int hsr_mesh_upload(const float* pos, int32_t npos, const float* nrm, int32_t nnrm, const float* uv, int32_t nuv,
                    const int32_t* faces, int32_t nfaces, hsr_mesh* out) {
  if (!g_init) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init not called");
  if (!pos || !faces || !out || npos <= 0 || nfaces <= 0 || nnrm < 0 || nuv < 0)
    return fail(HSR_ERR_INVALID_ARG, "mesh arrays");
  for (size_t i = 0; i < (size_t)nfaces * 3; i++) {
    const int32_t* c = &faces[i * 3];
    if (c[0] < 0 || c[0] >= npos || c[1] < 0 || c[1] >= (nuv > 0 ? nuv : 1) || c[2] < 0 ||
        c[2] >= (nnrm > 0 ? nnrm : 1))
      return fail(HSR_ERR_INVALID_ARG, "face index out of range");
  }
  host_mesh* m = (host_mesh*)calloc(1, sizeof(host_mesh));
  if (!m) return fail(HSR_ERR_OUT_OF_MEMORY, "mesh");
  static const float zero3[3] = {0.f, 0.f, 0.f};
  m->npos = npos;
  m->nnrm = nnrm > 0 ? nnrm : 1;
  m->nuv = nuv > 0 ? nuv : 1;
  m->nfaces = nfaces;
  m->pos = (float*)dup_bytes(pos, sizeof(float) * 3 * (size_t)npos);
  m->nrm = (float*)dup_bytes(nnrm > 0 && nrm ? nrm : zero3, sizeof(float) * 3 * (size_t)m->nnrm);
  m->uv = (float*)dup_bytes(nuv > 0 && uv ? uv : zero3, sizeof(float) * 2 * (size_t)m->nuv);
  m->faces = (int32_t*)dup_bytes(faces, sizeof(int32_t) * 9 * (size_t)nfaces);
  uint64_t h = (m->pos && m->nrm && m->uv && m->faces) ? add((void***)&g_meshes, &g_nmesh, m) : 0;
  if (!h) return fail(HSR_ERR_OUT_OF_MEMORY, "mesh");
  *out = h;
  return HSR_OK;
}

int hsr_mesh_update_normals(hsr_mesh mesh, const float* nrm, int32_t nnrm) {
  host_mesh* m = (host_mesh*)lookup((void**)g_meshes, g_nmesh, mesh);
  if (!m || !nrm || nnrm != m->nnrm) return fail(HSR_ERR_INVALID_ARG, "mesh normals");
  memcpy(m->nrm, nrm, sizeof(float) * 3 * (size_t)nnrm);
  return HSR_OK;
}

int hsr_texture_upload(const uint8_t* data, int32_t w, int32_t h, int32_t bytespp, hsr_texture* out) {
  if (!g_init) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init not called");
  if (!data || !out || w <= 0 || h <= 0 || (bytespp != 1 && bytespp != 3 && bytespp != 4))
    return fail(HSR_ERR_INVALID_ARG, "texture");
  host_tex* t = (host_tex*)calloc(1, sizeof(host_tex));
  if (!t) return fail(HSR_ERR_OUT_OF_MEMORY, "texture");
  t->w = w;
  t->h = h;
  t->bpp = bytespp;
  t->data = (uint8_t*)dup_bytes(data, (size_t)w * (size_t)h * (size_t)bytespp);
  uint64_t hd = t->data ? add((void***)&g_texs, &g_ntex, t) : 0;
  if (!hd) return fail(HSR_ERR_OUT_OF_MEMORY, "texture");
  *out = hd;
  return HSR_OK;
}

int hsr_target_create(int32_t w, int32_t h, hsr_target* out) {
  if (!g_init) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init not called");
  if (!out || w <= 0 || h <= 0) return fail(HSR_ERR_INVALID_ARG, "target size");
  host_target* t = (host_target*)calloc(1, sizeof(host_target));
  if (!t) return fail(HSR_ERR_OUT_OF_MEMORY, "target");
  const size_t n = (size_t)w * (size_t)h;
  t->w = w;
  t->h = h;
  t->color = (uint8_t*)calloc(n * 4, 1);
  t->depth = (float*)calloc(n, sizeof(float));
  t->prim = (uint32_t*)calloc(n, sizeof(uint32_t));
  uint64_t hd = (t->color && t->depth && t->prim) ? add((void***)&g_targets, &g_ntarget, t) : 0;
  if (!hd) return fail(HSR_ERR_OUT_OF_MEMORY, "target");
  *out = hd;
  return HSR_OK;
}

int hsr_target_release(hsr_target h) {
  host_target* t = (host_target*)lookup((void**)g_targets, g_ntarget, h);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "target handle");
  free(t->color);
  free(t->depth);
  free(t->prim);
  free(t);
  g_targets[h - 1] = NULL;
  return HSR_OK;
}

int hsr_target_upload(hsr_target h, const uint8_t* rgba, const float* depth, const uint32_t* prim) {
  host_target* t = (host_target*)lookup((void**)g_targets, g_ntarget, h);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "target handle");
  const size_t n = (size_t)t->w * (size_t)t->h;
  if (rgba) memcpy(t->color, rgba, n * 4);
  if (depth) memcpy(t->depth, depth, n * sizeof(float));
  if (prim) memcpy(t->prim, prim, n * sizeof(uint32_t));
  return HSR_OK;
}

int hsr_target_download(hsr_target h, uint8_t* rgba, float* depth, uint32_t* prim) {
  host_target* t = (host_target*)lookup((void**)g_targets, g_ntarget, h);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "target handle");
  const size_t n = (size_t)t->w * (size_t)t->h;
  if (rgba) memcpy(rgba, t->color, n * 4);
  if (depth) memcpy(depth, t->depth, n * sizeof(float));
  if (prim) memcpy(prim, t->prim, n * sizeof(uint32_t));
  return HSR_OK;
}

static hsro_texture* as_tex(uint64_t h, hsro_texture* out, int* bad) {
  if (h == 0) return NULL;
  host_tex* t = (host_tex*)lookup((void**)g_texs, g_ntex, h);
  if (!t) {
    *bad = 1;
    return NULL;
  }
  out->data = t->data;
  out->w = t->w;
  out->h = t->h;
  out->bpp = t->bpp;
  return out;
}

static hsro_target as_target(const host_target* t) {
  hsro_target o;
  o.w = t->w;
  o.h = t->h;
  o.color = t->color;
  o.depth = t->depth;
  o.prim = t->prim;
  return o;
}

int hsr_draw(const hsr_draw_desc* d) {
  if (!g_init) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init not called");
  if (!d || !d->uniforms) return fail(HSR_ERR_INVALID_ARG, "draw descriptor");
  host_mesh* m = (host_mesh*)lookup((void**)g_meshes, g_nmesh, d->mesh);
  host_target* t = (host_target*)lookup((void**)g_targets, g_ntarget, d->target);
  host_target* s = d->shadow_map ? (host_target*)lookup((void**)g_targets, g_ntarget, d->shadow_map) : NULL;
  if (!m || !t || (d->shadow_map && !s)) return fail(HSR_ERR_BAD_HANDLE, "draw handle");
  if (d->shader < 0 || d->shader >= HSR_SHADER_COUNT) return fail(HSR_ERR_UNKNOWN_SHADER, "shader kind");
  int bad = 0;
  hsro_texture dt, nt;
  const hsro_texture* diffuse = as_tex(d->diffuse, &dt, &bad);
  const hsro_texture* normal = as_tex(d->normal, &nt, &bad);
  if (bad) return fail(HSR_ERR_BAD_HANDLE, "texture handle");
  hsro_mesh om;
  om.pos = m->pos;
  om.npos = m->npos;
  om.nrm = m->nrm;
  om.nnrm = m->nnrm;
  om.uv = m->uv;
  om.nuv = m->nuv;
  om.faces = m->faces;
  om.nfaces = m->nfaces;
  hsro_target ot = as_target(t);
  hsro_target os;
  if (s) os = as_target(s);
  if (d->flags & HSR_DRAW_CLEAR) hsro_clear(&ot, d->clear_rgba, d->clear_depth);
  hsro_draw_stored_normals(&om, d->shader, d->uniforms, diffuse, normal, s ? &os : NULL, &ot, d->prim_base);
  return HSR_OK;
}
