// ref_harness.cpp — TEST INFRASTRUCTURE ONLY (part of the oracle; never shipped, never
// called by the product path).
//
// Drives the reference's own graphics_draw_triangle() (graphics.cpp:378-407), compiled
// headless from the reference sources by oracle/Makefile, through the same sequence
// DrawModel::draw uses (scene.h:53-99): optional shadow pass with ShadowShader into a
// shadow RenderBuffer, shader_data->shadow_map = that buffer, then the main pass.
// Uniforms arrive as bits (no matrix is rebuilt here), textures are built in memory as
// TGAImage and meshes are loaded through Model(const char*) from an OBJ file.
//
// A second shader, PrimIdShader, is a harness IShader subclass: it writes the face id
// carried in the per-face uv (lo 12 bits in uv.x, hi bits in uv.y) as RGB bytes of id+1.
// Run on an OBJ with the same v/vn/faces and per-face vt, its coverage and depth equal
// the real shader's (same ObjectToClipPos / ObjectToViewPos), so it yields the
// primitive-id plane the reference itself does not have.
//
// Usage:
//   ref_harness draw   <job.bin> <out.bin>            one frame, writes buffers
//   ref_harness time   <job.bin> <frames>              prints ms per frame
//   ref_harness mats   <params.bin> <out.bin>          matrix builders (maths.cpp)
//   ref_harness obj    <file.obj> <out.bin>            Model's parse, per corner, first draw
//   ref_harness tga    <file.tga> <model_flip> <out.bin>   TGAImage::read_tga_file (+ flip)
//   ref_harness tgawrite <raw.bin> <rle> <out.tga>      TGAImage::write_tga_file
//   ref_harness uniforms <params.bin> <out.bin>         model matrix + DrawModel::draw uniforms
//   ref_harness camera <cases.bin> <out.bin>            Camera::update_transform
#include "camera.h"
#include "graphics.h"

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

namespace {

struct PrimIdShader : public IShader {
  bool light_space = false;
  shader_struct_v2f vertex(shader_struct_a2v* a2v) override {
    shader_struct_v2f v2f;
    v2f.clip_pos = light_space ? ObjectToViewPos(a2v->obj_pos) : ObjectToClipPos(a2v->obj_pos);
    v2f.uv = a2v->uv;
    return v2f;
  }
  bool fragment(shader_struct_v2f* v2f, Color& color) override {
    long lo = std::lround(v2f->uv.x);
    long hi = std::lround(v2f->uv.y);
    uint32_t id = (uint32_t)(hi * 4096 + lo) + 1u;
    color = Color(((id & 255u) + 0.5f) / 255.f, (((id >> 8) & 255u) + 0.5f) / 255.f,
                  (((id >> 16) & 255u) + 0.5f) / 255.f);
    return false;
  }
};

struct Reader {
  std::vector<unsigned char> buf;
  size_t off = 0;
  bool load(const char* path) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    buf.resize((size_t)n);
    size_t got = std::fread(buf.data(), 1, (size_t)n, f);
    std::fclose(f);
    return got == (size_t)n;
  }
  template <class T> T get() {
    T v;
    if (off + sizeof(T) > buf.size()) { std::fprintf(stderr, "job truncated\n"); std::exit(2); }
    std::memcpy(&v, buf.data() + off, sizeof(T));
    off += sizeof(T);
    return v;
  }
  void bytes(void* dst, size_t n) {
    if (off + n > buf.size()) { std::fprintf(stderr, "job truncated\n"); std::exit(2); }
    std::memcpy(dst, buf.data() + off, n);
    off += n;
  }
};

void read_mat(Reader& r, Matrix4x4& m) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) m[i][j] = r.get<float>();
}
void read_color(Reader& r, Color& c) {
  c.r = r.get<float>(); c.g = r.get<float>(); c.b = r.get<float>(); c.a = r.get<float>();
}
void read_vec3(Reader& r, Vector3f& v) {
  v.x = r.get<float>(); v.y = r.get<float>(); v.z = r.get<float>();
}

// Job file (little endian), written by tests/golden/make_golden.py:
//   char magic[8] = "HSRJOB1\0"
//   i32 W, H, SW, SH            (SW == 0: no shadow pass)
//   i32 shader                  (hsr_shader_kind; 7 = PrimIdShader in both passes,
//                                8 = PrimIdShader with a light-space main pass)
//   f32 clear_depth_main, clear_depth_shadow; u8 clear_rgba_main[4], clear_rgba_shadow[4]
//   hsr_shader_data fields in declaration order (include/hsr.h)
//   texture diffuse: i32 w, h, bpp, bytes[w*h*bpp]   (w == 0: none)
//   texture normal : i32 w, h, bpp, bytes
//   i32 path_len, char obj_path[path_len]
struct Job {
  int W, H, SW, SH, shader;
  float cd_main, cd_shadow;
  unsigned char cc_main[4], cc_shadow[4];
  ShaderData sd;
  Material mat;
  TGAImage* diffuse = nullptr;
  TGAImage* normal = nullptr;
  std::string obj;
};

TGAImage* read_texture(Reader& r) {
  int w = r.get<int32_t>(), h = r.get<int32_t>(), bpp = r.get<int32_t>();
  if (w <= 0) return nullptr;
  TGAImage* img = new TGAImage(w, h, bpp);
  r.bytes(img->buffer(), (size_t)w * h * bpp);
  return img;
}

bool read_job(const char* path, Job& job) {
  Reader r;
  if (!r.load(path)) return false;
  char magic[8];
  r.bytes(magic, 8);
  if (std::memcmp(magic, "HSRJOB1", 8) != 0) return false;
  job.W = r.get<int32_t>(); job.H = r.get<int32_t>();
  job.SW = r.get<int32_t>(); job.SH = r.get<int32_t>();
  job.shader = r.get<int32_t>();
  job.cd_main = r.get<float>(); job.cd_shadow = r.get<float>();
  r.bytes(job.cc_main, 4); r.bytes(job.cc_shadow, 4);
  ShaderData& sd = job.sd;
  std::memset(&sd, 0, sizeof(sd));
  read_vec3(r, sd.view_Pos);
  read_vec3(r, sd.light_dir);
  read_color(r, sd.light_color);
  read_color(r, sd.ambient);
  read_mat(r, sd.model_matrix);
  read_mat(r, sd.model_matrix_I);
  read_mat(r, sd.view_matrix);
  read_mat(r, sd.projection_matrix);
  read_mat(r, sd.light_vp_matrix);
  read_mat(r, sd.camera_vp_matrix);
  sd.enable_shadow = r.get<int32_t>() != 0;
  read_color(r, job.mat.color);
  read_color(r, job.mat.specular);
  job.mat.gloss = r.get<float>();
  job.mat.bump_scale = r.get<float>();
  job.diffuse = read_texture(r);
  job.normal = read_texture(r);
  // A missing map is an empty TGAImage: get() returns a zero texel (tgaimage.cpp:248-251).
  job.mat.diffuse_map = job.diffuse ? job.diffuse : new TGAImage();
  job.mat.normal_map = job.normal ? job.normal : new TGAImage();
  job.mat.specular_map = new TGAImage();
  int n = r.get<int32_t>();
  job.obj.resize((size_t)n);
  r.bytes(&job.obj[0], (size_t)n);
  sd.matrial = &job.mat;
  sd.shadow_map = nullptr;
  sd.targetBuffer = nullptr;
  return true;
}

IShader* make_shader(int kind) {
  switch (kind) {
    case 0: return new GroundShader();
    case 1: return new ToonShader();
    case 2: return new TextureShader();
    case 3: return new TextureWithLightShader();
    case 4: return new BlinnShader();
    case 5: return new NormalMapShader();
    case 6: return new ShadowShader();
    case 7: return new PrimIdShader();
    case 8: {
      PrimIdShader* p = new PrimIdShader();
      p->light_space = true;
      return p;
    }
    default: return nullptr;
  }
}

void fill(RenderBuffer* rb, const unsigned char rgba[4], float depth) {
  int n = rb->width * rb->height;
  for (int i = 0; i < n; i++) {
    std::memcpy(rb->color_buffer + 4 * i, rgba, 4);
    rb->depth_buffer[i] = depth;
  }
}

// One frame in DrawModel::draw order (scene.h:73-91).
void render(Job& job, Model& model, RenderBuffer* main_rb, RenderBuffer* shadow_rb) {
  fill(main_rb, job.cc_main, job.cd_main);
  job.sd.shadow_map = nullptr;
  if (shadow_rb) {
    fill(shadow_rb, job.cc_shadow, job.cd_shadow);
    IShader* ss;
    if (job.shader == 7 || job.shader == 8) {
      PrimIdShader* p = new PrimIdShader();
      p->light_space = true;
      ss = p;
    } else {
      ss = new ShadowShader();
    }
    ss->shader_data = &job.sd;
    DrawData dd;
    dd.model = &model;
    dd.shader = ss;
    dd.render_buffer = shadow_rb;
    graphics_draw_triangle(&dd);
    job.sd.shadow_map = shadow_rb;
    delete ss;
  }
  IShader* sh = make_shader(job.shader);
  sh->shader_data = &job.sd;
  DrawData dd;
  dd.model = &model;
  dd.shader = sh;
  dd.render_buffer = main_rb;
  graphics_draw_triangle(&dd);
  delete sh;
}

void write_rb(FILE* f, RenderBuffer* rb) {
  int32_t w = rb->width, h = rb->height;
  std::fwrite(&w, 4, 1, f);
  std::fwrite(&h, 4, 1, f);
  std::fwrite(rb->depth_buffer, 4, (size_t)w * h, f);
  std::fwrite(rb->color_buffer, 1, (size_t)w * h * 4, f);
}

int cmd_draw(const char* jobp, const char* outp, int frames) {
  Job job;
  if (!read_job(jobp, job)) { std::fprintf(stderr, "bad job %s\n", jobp); return 2; }
  if (!make_shader(job.shader)) { std::fprintf(stderr, "bad shader\n"); return 2; }
  Model model(job.obj.c_str());
  if (model.nfaces() == 0) { std::fprintf(stderr, "empty model %s\n", job.obj.c_str()); return 2; }
  RenderBuffer main_rb(job.W, job.H);
  RenderBuffer* shadow_rb = job.SW > 0 ? new RenderBuffer(job.SW, job.SH) : nullptr;
  if (frames <= 0) {
    render(job, model, &main_rb, shadow_rb);
    FILE* f = std::fopen(outp, "wb");
    if (!f) return 2;
    std::fwrite("HSROUT1", 1, 8, f);
    int32_t has_shadow = shadow_rb ? 1 : 0;
    std::fwrite(&has_shadow, 4, 1, f);
    write_rb(f, &main_rb);
    if (shadow_rb) write_rb(f, shadow_rb);
    std::fclose(f);
  } else {
    render(job, model, &main_rb, shadow_rb);  // warm-up
    auto t0 = std::chrono::steady_clock::now();
    for (int i = 0; i < frames; i++) render(job, model, &main_rb, shadow_rb);
    auto t1 = std::chrono::steady_clock::now();
    double ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / frames;
    std::printf("%.6f\n", ms);
  }
  delete shadow_rb;
  return 0;
}

// Matrix builders of the reference, for pinning a host-side uniform builder:
// params = f32 eye[3], target[3], up[3], fovy, aspect, near, far, light[3],
//          ortho_right, ortho_top, ortho_near, ortho_far
// out    = view, proj, camera_vp = proj*view, light_vp = ortho*lookat(light,target,up),
//          model_I of the identity model (Matrix::invert), light_dir = normalize(light-target)
int cmd_mats(const char* inp, const char* outp) {
  Reader r;
  if (!r.load(inp)) return 2;
  Vector3f eye, target, up, light;
  read_vec3(r, eye); read_vec3(r, target); read_vec3(r, up);
  float fovy = r.get<float>(), aspect = r.get<float>(), n = r.get<float>(), fa = r.get<float>();
  read_vec3(r, light);
  float orr = r.get<float>(), ot = r.get<float>(), on = r.get<float>(), of = r.get<float>();
  Matrix4x4 view = lookat(eye, target, up);
  Matrix4x4 proj = perspective(fovy, aspect, n, fa);
  Matrix4x4 cvp = proj * view;
  Matrix4x4 lvp = orthographic(orr, ot, on, of) * lookat(light, target, up);
  Matrix4x4 model = Matrix4x4::identity();
  Matrix4x4 model_I = model.invert();
  Vector3f ld = (light - target).normalize();
  FILE* f = std::fopen(outp, "wb");
  if (!f) return 2;
  Matrix4x4* ms[5] = {&view, &proj, &cvp, &lvp, &model_I};
  for (Matrix4x4* m : ms)
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) { float v = (*m)[i][j]; std::fwrite(&v, 4, 1, f); }
  float l3[3] = {ld.x, ld.y, ld.z};
  std::fwrite(l3, 4, 3, f);
  std::fclose(f);
  return 0;
}

// Model::Model's parse as the first draw reads it: per face corner (graphics.cpp:380-387),
// vert(i, j) (3 floats), uv(i, j) (2 floats), normal(i, j) (3 floats; the accessor
// normalises in place, so reading in draw order gives the first draw's values).
// out = i32 nfaces, then nfaces*3 records of 8 floats.
int cmd_obj(const char* objp, const char* outp) {
  Model m(objp);
  FILE* f = std::fopen(outp, "wb");
  if (!f) return 2;
  int32_t nf = m.nfaces();
  std::fwrite(&nf, 4, 1, f);
  for (int i = 0; i < nf; i++)
    for (int j = 0; j < 3; j++) {
      Vector3f p = m.vert(i, j);
      Vector2f t = m.uv(i, j);
      Vector3f n = m.normal(i, j);
      float rec[8] = {p.x, p.y, p.z, t.x, t.y, n.x, n.y, n.z};
      std::fwrite(rec, 4, 8, f);
    }
  std::fclose(f);
  return 0;
}

// TGAImage::read_tga_file, then (model_flip != 0) the extra flip_vertically of
// Model::load_texture.  out = i32 w, h, bytespp, then the buffer.
int cmd_tga(const char* tgap, int model_flip, const char* outp) {
  TGAImage img;
  if (!img.read_tga_file(tgap)) return 3;
  if (model_flip) img.flip_vertically();
  FILE* f = std::fopen(outp, "wb");
  if (!f) return 2;
  int32_t hdr[3] = {img.get_width(), img.get_height(), img.get_bytespp()};
  std::fwrite(hdr, 4, 3, f);
  std::fwrite(img.buffer(), 1, (size_t)hdr[0] * hdr[1] * hdr[2], f);
  std::fclose(f);
  return 0;
}

// TGAImage::write_tga_file of raw bytes: in = i32 w, h, bytespp, then the buffer.
int cmd_tgawrite(const char* inp, int rle, const char* outp) {
  Reader r;
  if (!r.load(inp)) return 2;
  int32_t w = r.get<int32_t>(), h = r.get<int32_t>(), bpp = r.get<int32_t>();
  TGAImage img(w, h, bpp);
  r.bytes(img.buffer(), (size_t)w * h * bpp);
  return img.write_tga_file(outp, rle != 0) ? 0 : 3;
}

// GameObject::GetModelMatrix (gameobject.cpp:12-17) for a transform, its inverse
// (Matrix4x4::invert) and DrawModel::draw's uniforms (scene.h:55-71) for a camera and light:
// in = f32 position[3], rotation_deg[3], scale[3], eye[3], target[3], light[3], i32 w, h
// out = model, model_I, view, proj, light_vp, camera_vp (16 floats each), light_dir (3)
int cmd_uniforms(const char* inp, const char* outp) {
  Reader r;
  if (!r.load(inp)) return 2;
  Vector3f pos, rot, scl, eye, target, light;
  read_vec3(r, pos); read_vec3(r, rot); read_vec3(r, scl);
  read_vec3(r, eye); read_vec3(r, target); read_vec3(r, light);
  int32_t w = r.get<int32_t>(), h = r.get<int32_t>();
  // the composition of GameObject::GetModelMatrix
  Matrix4x4 m_translation = translate(pos.x, pos.y, pos.z);
  Matrix4x4 m_rotate = rotate_z(TO_RADIANS(rot.z)) * rotate_x(TO_RADIANS(rot.x)) * rotate_y(TO_RADIANS(rot.y));
  Matrix4x4 m_scale = scale(scl.x, scl.y, scl.z);
  Matrix4x4 model = m_translation * m_rotate * m_scale;
  Matrix4x4 model_I = model.invert();
  // Camera::get_view_matrix / get_proj_matrix (camera.cpp:82-92), DrawModel::draw (scene.h:55-71)
  Camera cam(eye, target, (float)w / (float)h);
  Matrix4x4 view = cam.get_view_matrix();
  Matrix4x4 proj = cam.get_proj_matrix();
  float aspect = (float)w / (float)h;
  Matrix4x4 lvp = orthographic(aspect, 1, 0, 5) * lookat(light, cam.get_target_position(), Vector3f(0, 1, 0));
  Matrix4x4 cvp = proj * view;
  Vector3f ld = (light - cam.get_target_position()).normalize();
  FILE* f = std::fopen(outp, "wb");
  if (!f) return 2;
  Matrix4x4* ms[6] = {&model, &model_I, &view, &proj, &lvp, &cvp};
  for (Matrix4x4* m : ms)
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) { float v = (*m)[i][j]; std::fwrite(&v, 4, 1, f); }
  float l3[3] = {ld.x, ld.y, ld.z};
  std::fwrite(l3, 4, 3, f);
  std::fclose(f);
  return 0;
}

// Camera::update_transform (camera.cpp:63-70) for n cases:
// in = i32 n, then per case f32 position[3], target[3], orbit[2], pan[2], dolly
// out = per case the new position[3] and target[3]
// Camera keeps its target private with no getter (get_target_position returns the origin);
// the class is standard-layout (every member private), so a struct with the same members in
// the same order reads it.
struct CameraFields {
  Vector3f position;
  Vector3f target;
  float aspect;
};
static_assert(sizeof(CameraFields) == sizeof(Camera), "Camera layout");

int cmd_camera(const char* inp, const char* outp) {
  Reader r;
  if (!r.load(inp)) return 2;
  const int32_t n = r.get<int32_t>();
  FILE* f = std::fopen(outp, "wb");
  if (!f) return 2;
  for (int32_t i = 0; i < n; i++) {
    Vector3f pos, target;
    read_vec3(r, pos);
    read_vec3(r, target);
    Motion m;
    m.orbit.x = r.get<float>(); m.orbit.y = r.get<float>();
    m.pan.x = r.get<float>(); m.pan.y = r.get<float>();
    m.dolly = r.get<float>();
    Camera cam(pos, target, 1.f);
    cam.update_transform(m);
    const CameraFields* cf = reinterpret_cast<const CameraFields*>(&cam);
    const float o[6] = {cf->position.x, cf->position.y, cf->position.z, cf->target.x, cf->target.y, cf->target.z};
    std::fwrite(o, 4, 6, f);
  }
  std::fclose(f);
  return 0;
}

}  // namespace

// camera.cpp's interactive update_camera reads the Win32 input layer (win32.cpp), which is
// not built headless; the harness never calls it, so these stand-ins only satisfy the linker.
void input_query_cursor(window_t*, float* xpos, float* ypos) { *xpos = 0.f; *ypos = 0.f; }
int input_key_pressed(window_t*, keycode_t) { return 0; }
void* window_get_userdata(window_t*) { return nullptr; }
float platform_get_time(void) { return 0.f; }

int main(int argc, char** argv) {
  if (argc >= 4 && std::strcmp(argv[1], "uniforms") == 0) return cmd_uniforms(argv[2], argv[3]);
  if (argc >= 4 && std::strcmp(argv[1], "camera") == 0) return cmd_camera(argv[2], argv[3]);
  if (argc >= 4 && std::strcmp(argv[1], "obj") == 0) return cmd_obj(argv[2], argv[3]);
  if (argc >= 5 && std::strcmp(argv[1], "tga") == 0) return cmd_tga(argv[2], std::atoi(argv[3]), argv[4]);
  if (argc >= 5 && std::strcmp(argv[1], "tgawrite") == 0) return cmd_tgawrite(argv[2], std::atoi(argv[3]), argv[4]);
  if (argc >= 4 && std::strcmp(argv[1], "draw") == 0) return cmd_draw(argv[2], argv[3], 0);
  if (argc >= 4 && std::strcmp(argv[1], "time") == 0) return cmd_draw(argv[2], nullptr, std::atoi(argv[3]));
  if (argc >= 4 && std::strcmp(argv[1], "mats") == 0) return cmd_mats(argv[2], argv[3]);
  std::fprintf(stderr, "usage: ref_harness draw|time|mats|obj|tga|tgawrite|uniforms|camera ...\n");
  return 2;
}
