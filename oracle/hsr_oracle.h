/*
 * hsr_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's draw path (graphics.cpp, IShader.h/.cpp,
 * renderbuffer.cpp, color.cpp, maths.cpp, vector.h, matrix.h, model.cpp, tgaimage.cpp),
 * in plain C99, single-threaded per draw, same operation order, built with
 * -ffp-contract=off.  It is the checker of the GPU path (tests/, smoke(), and the
 * cpu_baseline leg of bench.py) and is pinned against the reference itself by the golden
 * fixtures in tests/golden/.  Nothing in the product links it.
 */
#ifndef HSR_ORACLE_H
#define HSR_ORACLE_H

#include <stdint.h>
#include "../include/hsr.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hsro_mesh {
  const float* pos; int32_t npos;    /* [npos][3]                                        */
  float* nrm; int32_t nnrm;          /* [nnrm][3]; normalised IN PLACE on every access,  */
                                     /* as Model::normal does (model.cpp:108-111)        */
  const float* uv; int32_t nuv;      /* [nuv][2]                                         */
  const int32_t* faces; int32_t nfaces; /* [nfaces][3][3] = (v, vt, vn) per corner       */
} hsro_mesh;

typedef struct hsro_texture {        /* TGAImage: texel (x,y) at (x + y*w)*bpp, B,G,R(,A) */
  const uint8_t* data; int32_t w, h, bpp;
} hsro_texture;

typedef struct hsro_target {         /* RenderBuffer + a prim-id plane (may be NULL)      */
  int32_t w, h;
  uint8_t* color;                    /* RGBA8, (y*w + x)*4                               */
  float* depth;                      /* y*w + x                                          */
  uint32_t* prim;                    /* prim_base + face + 1 where a fragment passed     */
} hsro_target;

/* One graphics_draw_triangle() call.  diffuse / normal / shadow_map may be NULL.
 * Returns 0, or -1 for an unknown shader kind. */
int hsro_draw(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
              const hsro_texture* diffuse, const hsro_texture* normal,
              const hsro_target* shadow_map, hsro_target* target, uint32_t prim_base);

/* The same draw with the normals used as stored, never normalised (the library's hsr_mesh
 * semantics: a caller that reads normals through Model::normal passes what it returned). */
int hsro_draw_stored_normals(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
                             const hsro_texture* diffuse, const hsro_texture* normal,
                             const hsro_target* shadow_map, hsro_target* target, uint32_t prim_base);

/* renderbuffer_clear_color / renderbuffer_clear_depth with explicit bytes; prim -> 0. */
void hsro_clear(hsro_target* t, const uint8_t rgba[4], float depth);

/* Throughput run for the CPU baseline: `threads` POSIX threads each render `frames_each`
 * frames (shadow pass if shadow_w > 0, then main pass) into private buffers.  Returns the
 * wall time in seconds, or a negative value on failure. */
double hsro_bench_frames(const hsro_mesh* mesh, int32_t shader, const hsr_shader_data* sd,
                         const hsro_texture* diffuse, const hsro_texture* normal,
                         int32_t w, int32_t h, int32_t shadow_w, int32_t shadow_h,
                         int32_t frames_each, int32_t threads);

/* Returns 1 if this build evaluates a*b+c with two roundings (no FMA contraction). */
int hsro_no_contraction(void);

#ifdef __cplusplus
}
#endif
#endif
