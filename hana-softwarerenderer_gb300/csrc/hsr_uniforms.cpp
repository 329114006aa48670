// hsr_uniforms.cpp — ShaderData the way DrawModel::draw fills it (scene.h:55-71), on the host,
// with the reference's bits.
//
// Every value is an IEEE single-precision operation in the reference's own order (this file
// is built with -ffp-contract=off):
//   - matrix product result[i][j] = lhs[i] . col_j(rhs), the dot product accumulated from
//     the last index down (matrix.h:118-123, vector.h:69-73);
//   - invert(): adjugate of cofactors (recursive determinants, first-row expansion summed
//     from the last column down), divided by the dot product of its first row with the
//     matrix's first row, transposed (matrix.h:11-109);
//   - normalize(): v * (1 / sqrt(x*x + y*y + z*z)) (vector.h:41-42);
//   - lookat / perspective / orthographic / translate / scale / rotate_x,y,z (maths.cpp:39-255)
//     with the float overloads of tan, sin and cos the reference's calls resolve to;
//   - TO_RADIANS(d) = (PI / 180) * d with PI = 3.1415927f (maths.h:6-9);
//   - GameObject::GetModelMatrix = translate * (rotate_z * rotate_x * rotate_y) * scale
//     (gameobject.cpp:12-17); the camera's FOVY 60 degrees, NEAR 0.1, FAR 10000, up (0, 1, 0)
//     (camera.cpp:11-14); light_vp = orthographic(aspect, 1, 0, 5) * lookat(light, 0, up) and
//     light_dir = normalize(light - 0) — Camera::get_target_position() returns the origin
//     (camera.cpp:94-97) — ambient and light colour constants (scene.h:8-9);
//   - Camera::update_transform (camera.cpp:31-70) with the overloads its calls resolve to:
//     the float tan / atan2 / acos / sin / cos and the double pow (its 0.95 is a double).
#include <cmath>
#include <cstring>

#include "../../include/hsr.h"

namespace {

struct M4 {
  float m[4][4];
};

M4 identity() {
  M4 r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) r.m[i][j] = (i == j) ? 1.f : 0.f;
  return r;
}

float dot_rev(const float* a, const float* b, int n) {
  float r = 0.f;
  for (int i = n - 1; i >= 0; i--) r = r + a[i] * b[i];
  return r;
}

M4 mul(const M4& a, const M4& b) {
  M4 r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      const float col[4] = {b.m[0][j], b.m[1][j], b.m[2][j], b.m[3][j]};
      r.m[i][j] = dot_rev(a.m[i], col, 4);
    }
  return r;
}

// determinant of an n x n matrix (n <= 4) stored row-major with stride 4
float det(const float* a, int n);

float cofactor(const float* a, int n, int row, int col) {
  float minor[16];
  for (int i = 0; i < n - 1; i++)
    for (int j = 0; j < n - 1; j++) minor[i * 4 + j] = a[(i < row ? i : i + 1) * 4 + (j < col ? j : j + 1)];
  return det(minor, n - 1) * (((row + col) % 2) ? -1.f : 1.f);
}

float det(const float* a, int n) {
  if (n == 1) return a[0];
  float r = 0.f;
  for (int i = n - 1; i >= 0; i--) r = r + a[i] * cofactor(a, n, 0, i);
  return r;
}

M4 invert(const M4& src) {
  const float* a = &src.m[0][0];
  M4 adj;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) adj.m[i][j] = cofactor(a, 4, i, j);
  const float tmp = dot_rev(adj.m[0], src.m[0], 4);
  M4 r;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) r.m[j][i] = adj.m[i][j] / tmp;
  return r;
}

struct V3 {
  float x, y, z;
};
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float dot(V3 a, V3 b) {
  const float u[3] = {a.x, a.y, a.z}, v[3] = {b.x, b.y, b.z};
  return dot_rev(u, v, 3);
}
V3 normalize(V3 v) {
  const float f = 1.f / std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z);
  return {v.x * f, v.y * f, v.z * f};
}
V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 scaled(V3 v, float f) { return {v.x * f, v.y * f, v.z * f}; }
float length(V3 v) { return std::sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }  // Vector3f::normal

constexpr float kPi = 3.1415927f;
float to_radians(float deg) { return (kPi / 180) * deg; }

M4 lookat(V3 eye, V3 target, V3 up) {
  const V3 z = normalize(sub(eye, target));
  const V3 x = normalize(cross(up, z));
  const V3 y = cross(z, x);
  M4 m = identity();
  const V3 axes[3] = {x, y, z};
  for (int i = 0; i < 3; i++) {
    m.m[i][0] = axes[i].x;
    m.m[i][1] = axes[i].y;
    m.m[i][2] = axes[i].z;
    m.m[i][3] = -dot(axes[i], eye);
  }
  return m;
}

M4 perspective(float fovy, float aspect, float near, float far) {
  const float z_range = far - near;
  M4 m = identity();
  // the reference calls the C library's tanf at run time; an argument the compiler could see
  // through would be folded at compile time, correctly rounded, which tanf need not be
  volatile float half = fovy / 2;
  m.m[1][1] = 1 / std::tan((float)half);
  m.m[0][0] = m.m[1][1] / aspect;
  m.m[2][2] = -(near + far) / z_range;
  m.m[2][3] = -2 * near * far / z_range;
  m.m[3][2] = -1;
  m.m[3][3] = 0;
  return m;
}

M4 orthographic(float right, float top, float near, float far) {
  const float z_range = far - near;
  M4 m = identity();
  m.m[0][0] = 1 / right;
  m.m[1][1] = 1 / top;
  m.m[2][2] = -2 / z_range;
  m.m[2][3] = -(near + far) / z_range;
  return m;
}

M4 model_matrix(const hsr_transform& t) {
  M4 tr = identity();
  tr.m[0][3] = t.position[0];
  tr.m[1][3] = t.position[1];
  tr.m[2][3] = t.position[2];
  // run-time sinf / cosf as in the reference (see perspective)
  volatile float az = to_radians(t.rotation[2]), ax = to_radians(t.rotation[0]), ay = to_radians(t.rotation[1]);
  M4 rz = identity(), rx = identity(), ry = identity();
  float c = std::cos(az), s = std::sin(az);
  rz.m[0][0] = c; rz.m[0][1] = -s; rz.m[1][0] = s; rz.m[1][1] = c;
  c = std::cos(ax); s = std::sin(ax);
  rx.m[1][1] = c; rx.m[1][2] = -s; rx.m[2][1] = s; rx.m[2][2] = c;
  c = std::cos(ay); s = std::sin(ay);
  ry.m[0][0] = c; ry.m[0][2] = s; ry.m[2][0] = -s; ry.m[2][2] = c;
  M4 sc = identity();
  sc.m[0][0] = t.scale[0];
  sc.m[1][1] = t.scale[1];
  sc.m[2][2] = t.scale[2];
  return mul(mul(tr, mul(mul(rz, rx), ry)), sc);
}

void put(const M4& a, float* out) { std::memcpy(out, &a.m[0][0], sizeof(float) * 16); }

// The camera's field of view, a constant of camera.cpp (FOVY = TO_RADIANS(60)): the reference's
// tan(FOVY / 2) has a constant argument, which the compiler evaluates at build time.
const float kFovy = (kPi / 180) * 60;

// calculate_pan (camera.cpp:31-42): the target's move for a pan of the cursor
V3 camera_pan(V3 from_camera, const hsr_camera_motion& m) {
  const V3 forward = normalize(from_camera);
  const V3 left = cross({0.f, 1.f, 0.f}, forward);
  const V3 up = cross(forward, left);
  const float distance = length(from_camera);
  const float factor = distance * std::tan(kFovy / 2) * 2;
  return add(scaled(scaled(left, m.pan[0]), factor), scaled(scaled(up, m.pan[1]), factor));
}

// calculate_offset (camera.cpp:44-61): the eye's offset from the target after dolly and orbit
V3 camera_offset(V3 from_target, const hsr_camera_motion& m) {
  float radius = length(from_target);
  float theta = std::atan2(from_target.x, from_target.z);  // azimuth
  float phi = std::acos(from_target.y / radius);           // polar
  const float factor = kPi * 2;
  radius *= (float)std::pow(0.95, (double)m.dolly);
  theta -= m.orbit[0] * factor;
  phi -= m.orbit[1] * factor;
  const float lo = 1e-5f, hi = kPi - 1e-5f;  // clamp (maths.cpp:3-5)
  phi = phi < lo ? lo : (phi > hi ? hi : phi);
  return {radius * std::sin(phi) * std::sin(theta), radius * std::cos(phi), radius * std::sin(phi) * std::cos(theta)};
}

}  // namespace

extern "C" {

int hsr_model_matrix(const hsr_transform* t, float* out) {
  if (!t || !out) return HSR_ERR_INVALID_ARG;
  put(model_matrix(*t), out);
  return HSR_OK;
}

int hsr_camera_update(const float position[3], const float target[3], const hsr_camera_motion* motion,
                      float out_position[3], float out_target[3]) {
  if (!position || !target || !motion || !out_position || !out_target) return HSR_ERR_INVALID_ARG;
  const V3 pos = {position[0], position[1], position[2]}, tgt = {target[0], target[1], target[2]};
  const V3 pan = camera_pan(sub(tgt, pos), *motion);
  const V3 offset = camera_offset(sub(pos, tgt), *motion);
  const V3 new_target = add(tgt, pan);
  const V3 new_position = add(new_target, offset);
  out_target[0] = new_target.x; out_target[1] = new_target.y; out_target[2] = new_target.z;
  out_position[0] = new_position.x; out_position[1] = new_position.y; out_position[2] = new_position.z;
  return HSR_OK;
}

int hsr_matrix_invert(const float* m, float* out) {
  if (!m || !out) return HSR_ERR_INVALID_ARG;
  M4 a;
  std::memcpy(&a.m[0][0], m, sizeof(float) * 16);
  put(invert(a), out);
  return HSR_OK;
}

int hsr_shader_data_build(const hsr_scene_params* p, hsr_shader_data* out) {
  if (!p || !out || p->width <= 0 || p->height <= 0) return HSR_ERR_INVALID_ARG;
  const V3 eye = {p->camera_position[0], p->camera_position[1], p->camera_position[2]};
  const V3 target = {p->camera_target[0], p->camera_target[1], p->camera_target[2]};
  const V3 light = {p->light_position[0], p->light_position[1], p->light_position[2]};
  const V3 up = {0.f, 1.f, 0.f}, origin = {0.f, 0.f, 0.f};
  const float aspect = (float)p->width / (float)p->height;
  const M4 view = lookat(eye, target, up);
  const M4 proj = perspective(to_radians(60), aspect, 0.1f, 10000.f);
  const M4 model = model_matrix(p->model);
  const M4 model_I = invert(model);
  std::memset(out, 0, sizeof(*out));
  out->view_pos[0] = eye.x; out->view_pos[1] = eye.y; out->view_pos[2] = eye.z;
  const V3 ld = normalize(sub(light, origin));
  out->light_dir[0] = ld.x; out->light_dir[1] = ld.y; out->light_dir[2] = ld.z;
  const float light_color[4] = {255.f / 255, 244.f / 255, 214.f / 255, 255.f};
  const float ambient[4] = {54.f / 255, 58.f / 255, 66.f / 255, 255.f};
  std::memcpy(out->light_color, light_color, sizeof light_color);
  std::memcpy(out->ambient, ambient, sizeof ambient);
  put(model, out->model_matrix);
  put(model_I, out->model_matrix_I);
  put(view, out->view_matrix);
  put(proj, out->projection_matrix);
  put(mul(orthographic(aspect, 1, 0, 5), lookat(light, origin, up)), out->light_vp_matrix);
  put(mul(proj, view), out->camera_vp_matrix);
  out->enable_shadow = p->enable_shadow ? 1 : 0;
  std::memcpy(out->material_color, p->material_color, sizeof(float) * 4);
  std::memcpy(out->material_specular, p->material_specular, sizeof(float) * 4);
  out->gloss = p->gloss;
  out->bump_scale = p->bump_scale;
  return HSR_OK;
}

}  // extern "C"
