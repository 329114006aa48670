// hsr_io.cu — the data formats on either side of the draw path: Wavefront OBJ meshes and
// TGA textures going in, and the presented frame (a top-down BGR image, optionally a TGA
// file) coming out.
//
// Reference behaviour kept:
//   - OBJ (Model::Model, model.cpp:6-48): lines starting "v ", "vt ", "vn ", "f "; floats
//     parsed as istream >> float does (strtof, correctly rounded); a face keeps its corners'
//     1-based v/vt/vn triplets, and graphics_draw_triangle draws only the first three
//     (graphics.cpp:380-387), so that is what a face becomes here.  With
//     HSR_OBJ_CORNER_NORMALS every corner gets its own normal, the value Model::normal
//     returns at that corner during a draw: the accessor normalises the stored normal in
//     place on every read (model.cpp:108-111, vector.h:41-42), and every draw reads every
//     corner once, faces in order, corners 0..2; HSR_OBJ_EARLIER_DRAWS(n) selects the draw
//     that follows n others of the same model (a frame's main pass follows its shadow pass).
//   - TGA (TGAImage::read_tga_file / load_rle_data, tgaimage.cpp:40-143): 8/24/32-bit,
//     uncompressed (2, 3) or run-length (10, 11); the image ID field is not skipped (the
//     reference reads pixel data right after the 18-byte header); rows flipped unless the
//     descriptor's top-left bit (0x20) is set, columns flipped when 0x10 is set.  With
//     HSR_TGA_MODEL_FLIP one more vertical flip follows, as Model::load_texture does
//     (model.cpp:74-83) for every texture of a model.
//   - present (window_draw_buffer, win32.cpp:348-370): row r of the bottom-up RenderBuffer
//     becomes row H-1-r of a top-down image, bytes B, G, R from the colour's R, G, B.
//   - TGA writing (TGAImage::write_tga_file / unload_rle_data, tgaimage.cpp:145-246): an
//     18-byte header with the top-left bit, raw or run-length data, then the 26-byte
//     TRUEVISION-XFILE footer; the run-length chunking follows the same rule, so the files
//     are byte-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hsr_internal.h"
#include "hsr_runtime.h"

namespace hsr {

// ---------------------------------------------------------------------------------------
// OBJ
// ---------------------------------------------------------------------------------------
struct ObjData {
  std::vector<float> pos, nrm, uv;
  std::vector<int32_t> faces;  // [nfaces][3][3], 0-based
};

static bool read_file(const char* path, std::string& out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

// istream >> float: skip white space, parse the longest float prefix.
static bool next_float(const char*& p, float& v) {
  char* end = nullptr;
  errno = 0;
  v = std::strtof(p, &end);
  if (end == p) return false;
  p = end;
  return true;
}
static bool next_int(const char*& p, int32_t& v) {
  char* end = nullptr;
  const long x = std::strtol(p, &end, 10);
  if (end == p) return false;
  v = (int32_t)x;
  p = end;
  return true;
}
// istream >> char: skip white space, take one character.
static bool next_char(const char*& p, char& c) {
  while (*p == ' ' || *p == '\t' || *p == '\r' || *p == '\v' || *p == '\f') p++;
  if (!*p) return false;
  c = *p++;
  return true;
}

static int parse_obj(const char* path, uint32_t flags, ObjData& o) {
  std::string text;
  if (!read_file(path, text)) return fail(HSR_ERR_INVALID_ARG, std::string("obj: cannot read ") + path);
  size_t start = 0;
  int64_t lineno = 0;
  while (start <= text.size()) {
    size_t end = text.find('\n', start);
    if (end == std::string::npos) end = text.size();
    std::string line = text.substr(start, end - start);
    start = end + 1;
    lineno++;
    const char* p = line.c_str();
    char trash;
    if (line.compare(0, 2, "v ") == 0) {
      next_char(p, trash);
      float v[3] = {0.f, 0.f, 0.f};
      for (int i = 0; i < 3; i++) next_float(p, v[i]);
      o.pos.insert(o.pos.end(), v, v + 3);
    } else if (line.compare(0, 3, "vn ") == 0) {
      next_char(p, trash);
      next_char(p, trash);
      float v[3] = {0.f, 0.f, 0.f};
      for (int i = 0; i < 3; i++) next_float(p, v[i]);
      o.nrm.insert(o.nrm.end(), v, v + 3);
    } else if (line.compare(0, 3, "vt ") == 0) {
      next_char(p, trash);
      next_char(p, trash);
      float v[2] = {0.f, 0.f};
      for (int i = 0; i < 2; i++) next_float(p, v[i]);
      o.uv.insert(o.uv.end(), v, v + 2);
    } else if (line.compare(0, 2, "f ") == 0) {
      next_char(p, trash);
      int32_t c[3][3];
      int n = 0;
      for (;;) {
        int32_t t[3];
        char s1, s2;
        if (!next_int(p, t[0]) || !next_char(p, s1) || !next_int(p, t[1]) || !next_char(p, s2) || !next_int(p, t[2]))
          break;
        if (n < 3)
          for (int k = 0; k < 3; k++) c[n][k] = t[k] - 1;  // OBJ indices start at 1
        n++;
      }
      if (n < 3)
        return fail(HSR_ERR_INVALID_ARG, std::string("obj: face with fewer than three v/vt/vn corners at line ") +
                                             std::to_string(lineno));
      for (int j = 0; j < 3; j++) o.faces.insert(o.faces.end(), c[j], c[j] + 3);
    }
    if (end == text.size()) break;
  }
  const int64_t npos = (int64_t)o.pos.size() / 3, nuv = (int64_t)o.uv.size() / 2, nnrm = (int64_t)o.nrm.size() / 3;
  const int64_t nfaces = (int64_t)o.faces.size() / 9;
  if (nfaces > (1 << 27)) return fail(HSR_ERR_INVALID_ARG, "obj: more than 2^27 faces");
  for (int64_t i = 0; i < nfaces * 3; i++) {
    const int32_t* c = &o.faces[(size_t)i * 3];
    if (c[0] < 0 || c[0] >= npos || c[1] < 0 || c[1] >= nuv || c[2] < 0 || c[2] >= nnrm)
      return fail(HSR_ERR_INVALID_ARG, "obj: face " + std::to_string(i / 3) + " indexes past the vertex lists");
  }
  if (flags & HSR_OBJ_CORNER_NORMALS) {
    // Model::normal(iface, nthvert) = norms_[idx].normalize(), read per corner in draw order
    const int earlier = (int)((flags >> 8) & 255u);
    std::vector<float> stored = o.nrm, corner((size_t)nfaces * 9);
    for (int d = 0; d <= earlier; d++)
      for (int64_t i = 0; i < nfaces * 3; i++) {
        float* n = &stored[(size_t)o.faces[(size_t)i * 3 + 2] * 3];
        const float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        const float f = 1.f / len;
        n[0] = n[0] * f;
        n[1] = n[1] * f;
        n[2] = n[2] * f;
        if (d == earlier) std::memcpy(&corner[(size_t)i * 3], n, 3 * sizeof(float));
      }
    for (int64_t i = 0; i < nfaces * 3; i++) o.faces[(size_t)i * 3 + 2] = (int32_t)i;
    o.nrm.swap(corner);
  }
  return HSR_OK;
}

// ---------------------------------------------------------------------------------------
// TGA
// ---------------------------------------------------------------------------------------
struct Tga {
  int32_t w = 0, h = 0, bpp = 0;
  std::vector<uint8_t> data;
};

static void flip_rows(Tga& t) {
  const size_t row = (size_t)t.w * (size_t)t.bpp;
  std::vector<uint8_t> tmp(row);
  for (int32_t y = 0; y < t.h / 2; y++) {
    uint8_t* a = &t.data[(size_t)y * row];
    uint8_t* b = &t.data[(size_t)(t.h - 1 - y) * row];
    std::memcpy(tmp.data(), a, row);
    std::memcpy(a, b, row);
    std::memcpy(b, tmp.data(), row);
  }
}
static void flip_columns(Tga& t) {
  for (int32_t y = 0; y < t.h; y++)
    for (int32_t x = 0; x < t.w / 2; x++) {
      uint8_t* a = &t.data[((size_t)y * t.w + x) * t.bpp];
      uint8_t* b = &t.data[((size_t)y * t.w + (t.w - 1 - x)) * t.bpp];
      for (int k = 0; k < t.bpp; k++) std::swap(a[k], b[k]);
    }
}

static int parse_tga(const char* path, uint32_t flags, Tga& t) {
  std::string f;
  if (!read_file(path, f)) return fail(HSR_ERR_INVALID_ARG, std::string("tga: cannot read ") + path);
  if (f.size() < 18) return fail(HSR_ERR_INVALID_ARG, "tga: truncated header");
  const uint8_t* h = reinterpret_cast<const uint8_t*>(f.data());
  const int type = h[2];
  const int16_t w = (int16_t)(h[12] | (h[13] << 8)), hh = (int16_t)(h[14] | (h[15] << 8));
  const int bpp = h[16] >> 3, desc = h[17];
  if (w <= 0 || hh <= 0 || (bpp != 1 && bpp != 3 && bpp != 4))
    return fail(HSR_ERR_INVALID_ARG, "tga: bad size or bits per pixel (8, 24 or 32 supported)");
  t.w = w;
  t.h = hh;
  t.bpp = bpp;
  const size_t nbytes = (size_t)w * (size_t)hh * (size_t)bpp, npix = (size_t)w * (size_t)hh;
  t.data.assign(nbytes, 0);
  size_t off = 18;  // the ID field is not skipped, as in the reference
  if (type == 2 || type == 3) {
    if (f.size() - off < nbytes) return fail(HSR_ERR_INVALID_ARG, "tga: truncated pixel data");
    std::memcpy(t.data.data(), f.data() + off, nbytes);
  } else if (type == 10 || type == 11) {
    size_t pix = 0, byte = 0;
    do {
      if (off >= f.size()) return fail(HSR_ERR_INVALID_ARG, "tga: truncated run-length data");
      int chunk = (uint8_t)f[off++];
      if (chunk < 128) {
        chunk++;
        for (int i = 0; i < chunk; i++) {
          if (f.size() - off < (size_t)bpp) return fail(HSR_ERR_INVALID_ARG, "tga: truncated run-length data");
          if (++pix > npix) return fail(HSR_ERR_INVALID_ARG, "tga: run-length data past the image");
          std::memcpy(&t.data[byte], f.data() + off, (size_t)bpp);
          off += (size_t)bpp;
          byte += (size_t)bpp;
        }
      } else {
        chunk -= 127;
        if (f.size() - off < (size_t)bpp) return fail(HSR_ERR_INVALID_ARG, "tga: truncated run-length data");
        for (int i = 0; i < chunk; i++) {
          if (++pix > npix) return fail(HSR_ERR_INVALID_ARG, "tga: run-length data past the image");
          std::memcpy(&t.data[byte], f.data() + off, (size_t)bpp);
          byte += (size_t)bpp;
        }
        off += (size_t)bpp;
      }
    } while (pix < npix);
  } else {
    return fail(HSR_ERR_INVALID_ARG, "tga: unsupported image type " + std::to_string(type));
  }
  if (!(desc & 0x20)) flip_rows(t);
  if (desc & 0x10) flip_columns(t);
  if (flags & HSR_TGA_MODEL_FLIP) flip_rows(t);
  return HSR_OK;
}

// TGAImage::unload_rle_data's chunking: a raw chunk ends before two equal pixels, a run
// chunk at the first differing pixel, both at 128 pixels.
static void rle_encode(const uint8_t* data, size_t npix, int bpp, std::vector<uint8_t>& out) {
  size_t cur = 0;
  while (cur < npix) {
    const size_t chunkstart = cur * (size_t)bpp;
    size_t curbyte = cur * (size_t)bpp;
    unsigned run = 1;
    bool raw = true;
    while (cur + run < npix && run < 128) {
      bool eq = true;
      for (int t = 0; eq && t < bpp; t++) eq = data[curbyte + t] == data[curbyte + t + bpp];
      curbyte += (size_t)bpp;
      if (run == 1) raw = !eq;
      if (raw && eq) {
        run--;
        break;
      }
      if (!raw && !eq) break;
      run++;
    }
    cur += run;
    out.push_back((uint8_t)(raw ? run - 1 : run + 127));
    const uint8_t* src = data + chunkstart;
    out.insert(out.end(), src, src + (raw ? run * (size_t)bpp : (size_t)bpp));
  }
}

static int write_tga(const char* path, const uint8_t* data, int32_t w, int32_t h, int bpp, bool rle) {
  std::vector<uint8_t> out(18, 0);
  out[2] = (uint8_t)(bpp == 1 ? (rle ? 11 : 3) : (rle ? 10 : 2));
  out[12] = (uint8_t)(w & 255);
  out[13] = (uint8_t)((w >> 8) & 255);
  out[14] = (uint8_t)(h & 255);
  out[15] = (uint8_t)((h >> 8) & 255);
  out[16] = (uint8_t)(bpp << 3);
  out[17] = 0x20;  // top-left origin
  const size_t npix = (size_t)w * (size_t)h;
  if (rle) rle_encode(data, npix, bpp, out);
  else out.insert(out.end(), data, data + npix * (size_t)bpp);
  const uint8_t tail[26] = {0, 0, 0, 0, 0, 0, 0, 0, 'T', 'R', 'U', 'E', 'V', 'I', 'S', 'I', 'O', 'N', '-',
                            'X', 'F', 'I', 'L', 'E', '.', 0};
  out.insert(out.end(), tail, tail + 26);
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(HSR_ERR_INVALID_ARG, std::string("tga: cannot write ") + path);
  const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
  const bool closed = std::fclose(f) == 0;
  return ok && closed ? HSR_OK : fail(HSR_ERR_INVALID_ARG, std::string("tga: write failed for ") + path);
}

// ---------------------------------------------------------------------------------------
// present
// ---------------------------------------------------------------------------------------
// window_draw_buffer: source row r (row 0 at the bottom) -> destination row H-1-r, bytes
// B, G, R; with four channels the fourth byte is 0.  One thread per destination pixel.
__global__ void __launch_bounds__(256) k_present(const uint32_t* __restrict__ color, uint8_t* __restrict__ out,
                                                 int32_t w, int32_t h, int channels) {
  const size_t n = (size_t)w * (size_t)h;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int32_t r = (int32_t)(i / (size_t)w), c = (int32_t)(i - (size_t)r * (size_t)w);
    const uint32_t px = __ldg(color + (size_t)(h - 1 - r) * (size_t)w + c);  // byte order r, g, b, a
    const uint8_t R = px & 255u, G = (px >> 8) & 255u, B = (px >> 16) & 255u;
    if (channels == 4) {
      reinterpret_cast<uint32_t*>(out)[i] = (uint32_t)B | ((uint32_t)G << 8) | ((uint32_t)R << 16);
    } else {
      out[3 * i + 0] = B;
      out[3 * i + 1] = G;
      out[3 * i + 2] = R;
    }
  }
}

static int present(uint64_t th, int channels, std::vector<uint8_t>& host, int32_t& w, int32_t& h) {
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_rt) return fail(HSR_ERR_NOT_INITIALIZED, "hsr_init() has not succeeded");
  TargetObj* t = g_rt->target(th);
  if (!t) return fail(HSR_ERR_BAD_HANDLE, "present: unknown target");
  w = t->w;
  h = t->h;
  const size_t bytes = (size_t)w * (size_t)h * (size_t)channels;
  uint8_t* dev = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&dev, bytes, g_rt->stream);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(HSR_ERR_OUT_OF_MEMORY, "present: device buffer");
  }
  const int grid = (int)std::min<size_t>(((size_t)w * (size_t)h + 255) / 256, (size_t)g_rt->num_sms * 16);
  k_present<<<grid, 256, 0, g_rt->stream>>>(t->color, dev, w, h, channels);
  e = cudaGetLastError();
  g_rt->launches++;
  host.resize(bytes);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host.data(), dev, bytes, cudaMemcpyDeviceToHost, g_rt->stream);
  cudaFreeAsync(dev, g_rt->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(g_rt->stream);
  return e == cudaSuccess ? HSR_OK : cuda_fail(e, "present");
}

}  // namespace hsr

using namespace hsr;

extern "C" {

int hsr_obj_read(const char* path, uint32_t flags, float* pos, int32_t* npos, float* nrm, int32_t* nnrm, float* uv,
                 int32_t* nuv, int32_t* faces, int32_t* nfaces) {
  if (!path || !npos || !nnrm || !nuv || !nfaces) return fail(HSR_ERR_INVALID_ARG, "obj_read: null argument");
  ObjData o;
  int rc = parse_obj(path, flags, o);
  if (rc != HSR_OK) return rc;
  const int64_t counts[4] = {(int64_t)o.pos.size() / 3, (int64_t)o.nrm.size() / 3, (int64_t)o.uv.size() / 2,
                             (int64_t)o.faces.size() / 9};
  for (int64_t c : counts)
    if (c > INT32_MAX) return fail(HSR_ERR_INVALID_ARG, "obj_read: more than 2^31 entries");
  const bool fill = pos || nrm || uv || faces;
  if (fill && (!pos || !nrm || !uv || !faces || *npos < counts[0] || *nnrm < counts[1] || *nuv < counts[2] ||
               *nfaces < counts[3]))
    return fail(HSR_ERR_INVALID_ARG, "obj_read: arrays missing or smaller than the counts");
  if (fill) {
    std::memcpy(pos, o.pos.data(), o.pos.size() * sizeof(float));
    std::memcpy(nrm, o.nrm.data(), o.nrm.size() * sizeof(float));
    std::memcpy(uv, o.uv.data(), o.uv.size() * sizeof(float));
    std::memcpy(faces, o.faces.data(), o.faces.size() * sizeof(int32_t));
  }
  *npos = (int32_t)counts[0];
  *nnrm = (int32_t)counts[1];
  *nuv = (int32_t)counts[2];
  *nfaces = (int32_t)counts[3];
  return HSR_OK;
}

int hsr_tga_read(const char* path, uint32_t flags, uint8_t* data, int32_t* w, int32_t* h, int32_t* bytespp) {
  if (!path || !w || !h || !bytespp) return fail(HSR_ERR_INVALID_ARG, "tga_read: null argument");
  Tga t;
  int rc = parse_tga(path, flags, t);
  if (rc != HSR_OK) return rc;
  if (data) {
    if ((int64_t)*w * (int64_t)*h * (int64_t)*bytespp < (int64_t)t.data.size())
      return fail(HSR_ERR_INVALID_ARG, "tga_read: buffer smaller than the image");
    std::memcpy(data, t.data.data(), t.data.size());
  }
  *w = t.w;
  *h = t.h;
  *bytespp = t.bpp;
  return HSR_OK;
}

int hsr_tga_write(const char* path, const uint8_t* data, int32_t w, int32_t h, int32_t bytespp, int32_t rle) {
  if (!path || !data || w <= 0 || h <= 0 || w > 32767 || h > 32767 || (bytespp != 1 && bytespp != 3 && bytespp != 4))
    return fail(HSR_ERR_INVALID_ARG, "tga_write: bad arguments");
  return write_tga(path, data, w, h, bytespp, rle != 0);
}

int hsr_mesh_load_obj(const char* path, uint32_t flags, hsr_mesh* out) {
  if (!path || !out) return fail(HSR_ERR_INVALID_ARG, "mesh_load_obj: null argument");
  ObjData o;
  int rc = parse_obj(path, flags, o);
  if (rc != HSR_OK) return rc;
  return hsr_mesh_upload(o.pos.data(), (int32_t)(o.pos.size() / 3), o.nrm.data(), (int32_t)(o.nrm.size() / 3),
                         o.uv.data(), (int32_t)(o.uv.size() / 2), o.faces.data(), (int32_t)(o.faces.size() / 9), out);
}

int hsr_texture_load_tga(const char* path, uint32_t flags, hsr_texture* out) {
  if (!path || !out) return fail(HSR_ERR_INVALID_ARG, "texture_load_tga: null argument");
  Tga t;
  int rc = parse_tga(path, flags, t);
  if (rc != HSR_OK) return rc;
  return hsr_texture_upload(t.data.data(), t.w, t.h, t.bpp, out);
}

int hsr_target_present(hsr_target t, uint8_t* out, int32_t channels) {
  if (!out || (channels != 3 && channels != 4)) return fail(HSR_ERR_INVALID_ARG, "present: bad arguments");
  std::vector<uint8_t> host;
  int32_t w = 0, h = 0;
  int rc = present(t, channels, host, w, h);
  if (rc != HSR_OK) return rc;
  std::memcpy(out, host.data(), host.size());
  return HSR_OK;
}

int hsr_target_write_tga(hsr_target t, const char* path, int32_t rle) {
  if (!path) return fail(HSR_ERR_INVALID_ARG, "target_write_tga: null path");
  std::vector<uint8_t> host;
  int32_t w = 0, h = 0;
  int rc = present(t, 3, host, w, h);
  if (rc != HSR_OK) return rc;
  if (w > 32767 || h > 32767) return fail(HSR_ERR_INVALID_ARG, "target_write_tga: TGA holds at most 32767 x 32767");
  return write_tga(path, host.data(), w, h, 3, rle != 0);
}

}  // extern "C"
