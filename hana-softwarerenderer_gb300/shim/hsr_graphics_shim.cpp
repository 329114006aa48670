// hsr_graphics_shim.cpp — drop-in replacement of the reference's graphics.cpp.
//
// Compiled inside the reference's own build instead of graphics.cpp, this file provides
//     void graphics_draw_triangle(DrawData* draw_data);     (graphics.h:15)
// for the reference's own types and renders on the GPU through include/hsr.h:
//   - the IShader's dynamic type selects the shader kind (typeid, IShader.h:132-165);
//     an IShader subclass this library does not implement is reported and not drawn
//     (there is no CPU fallback);
//   - a Model becomes a cached device mesh with one entry per face corner, filled through
//     Model::vert / uv / normal exactly as graphics.cpp:382-386 reads them; the normals are
//     re-read through Model::normal on every draw, because that accessor normalises the
//     stored normal in place (model.cpp:108-111) and the reference sees the drifted value;
//   - ShaderData (IShader.h:17-32) and Material (IShader.h:7-15) become hsr_shader_data;
//     TGAImage maps become cached device textures (keyed by image pointer: the maps are
//     loaded once and not modified afterwards);
//   - each RenderBuffer is mirrored by a device target: its host colour and depth are copied
//     in before the draw and back after it, so the caller keeps owning and reading the
//     host buffers as before (ShaderData::shadow_map is copied in the same way).
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <typeinfo>
#include <unordered_map>
#include <vector>

#include "graphics.h"
#include "hsr.h"

namespace {

struct MeshEntry {
  hsr_mesh mesh = 0;
  int nfaces = 0;
  std::vector<float> nrm;  // per corner, re-read every draw
};
struct TargetEntry {
  hsr_target target = 0;
  int w = 0, h = 0;
};

bool g_ready = false;
bool g_failed = false;
std::unordered_map<Model*, MeshEntry> g_meshes;
std::unordered_map<TGAImage*, hsr_texture> g_textures;
std::unordered_map<RenderBuffer*, TargetEntry> g_targets;

bool ready() {
  if (g_ready) return true;
  if (g_failed) return false;
  if (hsr_init(0) != HSR_OK) {
    std::fprintf(stderr, "graphics_draw_triangle: no GPU draw path: %s\n", hsr_last_error());
    g_failed = true;
    return false;
  }
  g_ready = true;
  return true;
}

int shader_kind(IShader* s) {
  const std::type_info& t = typeid(*s);
  if (t == typeid(GroundShader)) return HSR_SHADER_GROUND;
  if (t == typeid(ToonShader)) return HSR_SHADER_TOON;
  if (t == typeid(TextureShader)) return HSR_SHADER_TEXTURE;
  if (t == typeid(TextureWithLightShader)) return HSR_SHADER_TEXTURE_WITH_LIGHT;
  if (t == typeid(BlinnShader)) return HSR_SHADER_BLINN;
  if (t == typeid(NormalMapShader)) return HSR_SHADER_NORMALMAP;
  if (t == typeid(ShadowShader)) return HSR_SHADER_SHADOW;
  return -1;
}

MeshEntry* mesh_for(Model* m) {
  auto it = g_meshes.find(m);
  const int nf = m->nfaces();
  if (it == g_meshes.end()) {
    std::vector<float> pos((size_t)nf * 9), uv((size_t)nf * 6);
    std::vector<int32_t> faces((size_t)nf * 9);
    MeshEntry e;
    e.nfaces = nf;
    e.nrm.resize((size_t)nf * 9);
    for (int i = 0; i < nf; i++)
      for (int j = 0; j < 3; j++) {
        const size_t c = (size_t)i * 3 + (size_t)j;
        Vector3f p = m->vert(i, j);
        Vector2f t = m->uv(i, j);
        Vector3f n = m->normal(i, j);
        pos[c * 3 + 0] = p.x; pos[c * 3 + 1] = p.y; pos[c * 3 + 2] = p.z;
        uv[c * 2 + 0] = t.x; uv[c * 2 + 1] = t.y;
        e.nrm[c * 3 + 0] = n.x; e.nrm[c * 3 + 1] = n.y; e.nrm[c * 3 + 2] = n.z;
        faces[c * 3 + 0] = faces[c * 3 + 1] = faces[c * 3 + 2] = (int32_t)c;
      }
    const int nc = nf * 3;
    if (hsr_mesh_upload(pos.data(), nc, e.nrm.data(), nc, uv.data(), nc, faces.data(), nf, &e.mesh) != HSR_OK) {
      std::fprintf(stderr, "graphics_draw_triangle: mesh upload failed: %s\n", hsr_last_error());
      return nullptr;
    }
    return &(g_meshes[m] = e);
  }
  // the reference reads every corner's normal through Model::normal on every draw
  MeshEntry& e = it->second;
  for (int i = 0; i < nf; i++)
    for (int j = 0; j < 3; j++) {
      const size_t c = (size_t)i * 3 + (size_t)j;
      Vector3f n = m->normal(i, j);
      e.nrm[c * 3 + 0] = n.x; e.nrm[c * 3 + 1] = n.y; e.nrm[c * 3 + 2] = n.z;
    }
  if (hsr_mesh_update_normals(e.mesh, e.nrm.data(), nf * 3) != HSR_OK) return nullptr;
  return &e;
}

hsr_texture tex_for(TGAImage* img) {
  if (!img || !img->buffer() || img->get_width() <= 0) return 0;  // get() returns zero texels
  auto it = g_textures.find(img);
  if (it != g_textures.end()) return it->second;
  hsr_texture t = 0;
  if (hsr_texture_upload(img->buffer(), img->get_width(), img->get_height(), img->get_bytespp(), &t) != HSR_OK)
    return 0;
  g_textures[img] = t;
  return t;
}

TargetEntry* target_for(RenderBuffer* rb) {
  TargetEntry& e = g_targets[rb];
  if (!e.target || e.w != rb->width || e.h != rb->height) {
    if (e.target) hsr_target_release(e.target);
    e.w = rb->width;
    e.h = rb->height;
    if (hsr_target_create(e.w, e.h, &e.target) != HSR_OK) return nullptr;
  }
  return &e;
}

void copy_mat(const Matrix4x4& m, float* out) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) out[i * 4 + j] = m[i][j];
}
void copy_color(const Color& c, float* out) {
  out[0] = c.r; out[1] = c.g; out[2] = c.b; out[3] = c.a;
}

}  // namespace

void graphics_draw_triangle(DrawData* draw_data) {
  if (!ready()) return;
  IShader* sh = draw_data->shader;
  const int kind = shader_kind(sh);
  if (kind < 0) {
    std::fprintf(stderr, "graphics_draw_triangle: IShader subclass %s has no GPU implementation\n",
                 typeid(*sh).name());
    return;
  }
  ShaderData* sd = sh->shader_data;
  hsr_shader_data u;
  std::memset(&u, 0, sizeof(u));
  u.view_pos[0] = sd->view_Pos.x; u.view_pos[1] = sd->view_Pos.y; u.view_pos[2] = sd->view_Pos.z;
  u.light_dir[0] = sd->light_dir.x; u.light_dir[1] = sd->light_dir.y; u.light_dir[2] = sd->light_dir.z;
  copy_color(sd->light_color, u.light_color);
  copy_color(sd->ambient, u.ambient);
  copy_mat(sd->model_matrix, u.model_matrix);
  copy_mat(sd->model_matrix_I, u.model_matrix_I);
  copy_mat(sd->view_matrix, u.view_matrix);
  copy_mat(sd->projection_matrix, u.projection_matrix);
  copy_mat(sd->light_vp_matrix, u.light_vp_matrix);
  copy_mat(sd->camera_vp_matrix, u.camera_vp_matrix);
  u.enable_shadow = sd->enable_shadow ? 1 : 0;
  hsr_texture diffuse = 0, normal = 0;
  if (sd->matrial) {
    copy_color(sd->matrial->color, u.material_color);
    copy_color(sd->matrial->specular, u.material_specular);
    u.gloss = sd->matrial->gloss;
    u.bump_scale = sd->matrial->bump_scale;
    diffuse = tex_for(sd->matrial->diffuse_map);
    normal = tex_for(sd->matrial->normal_map);
  }
  MeshEntry* me = mesh_for(draw_data->model);
  RenderBuffer* rb = draw_data->render_buffer;
  TargetEntry* te = target_for(rb);
  if (!me || !te) return;
  hsr_target shadow = 0;
  if (sd->shadow_map && sd->shadow_map != rb) {
    TargetEntry* se = target_for(sd->shadow_map);
    if (!se) return;
    hsr_target_upload(se->target, sd->shadow_map->color_buffer, sd->shadow_map->depth_buffer, nullptr);
    shadow = se->target;
  }
  hsr_target_upload(te->target, rb->color_buffer, rb->depth_buffer, nullptr);
  hsr_draw_desc d;
  std::memset(&d, 0, sizeof(d));
  d.mesh = me->mesh;
  d.shader = kind;
  d.diffuse = diffuse;
  d.normal = normal;
  d.target = te->target;
  d.shadow_map = shadow;
  d.uniforms = &u;
  if (hsr_draw(&d) != HSR_OK) {
    std::fprintf(stderr, "graphics_draw_triangle: %s\n", hsr_last_error());
    return;
  }
  hsr_target_download(te->target, rb->color_buffer, rb->depth_buffer, nullptr);
}
