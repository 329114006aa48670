/*
 * hsr.h — C ABI of the GB300 draw path for Hana-SoftwareRenderer.
 *
 * The reference renders with one synchronous call,
 *     void graphics_draw_triangle(DrawData* draw_data);          (graphics.h:15, graphics.cpp:378-407)
 * where DrawData = {Model*, IShader*, RenderBuffer*}             (graphics.h:9-13)
 * and the shader's ShaderData / Material carry the uniforms      (IShader.h:7-32).
 *
 * This header replaces that call with plain handles, pointers and sizes so that any
 * host (C, C++, ctypes, cgo, JNI) can bind it.  Every entry point returns an int
 * status (HSR_OK == 0).  No entry point falls back to the CPU: without a usable
 * CUDA device hsr_init() fails and every other call returns HSR_ERR_NOT_INITIALIZED.
 *
 * Semantics kept from the reference (bit-exact unless noted):
 *   - vertex() runs per face corner, clip / cull / viewport / bounding box / integer
 *     pixel sampling / inclusive coverage exactly as graphics.cpp:7-376;
 *   - the depth test is `skip if frag_depth > depth` (graphics.cpp:359): equal depth
 *     passes and the later-submitted triangle wins;
 *   - colour is written R,G,B only through (uchar)(c*255) truncation (renderbuffer.cpp:38-44);
 *     alpha is never written by a draw;
 *   - RGBA8 colour is within 1 LSB of the reference (powf is not correctly rounded).
 *
 * Buffers are row-major, index y*width + x, row 0 = bottom (maths.cpp:20-25).
 */
#ifndef HSR_H
#define HSR_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define HSR_API __declspec(dllexport)
#else
#define HSR_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define HSR_ABI_VERSION 2

/* ---- status codes ---------------------------------------------------------------- */
enum {
  HSR_OK = 0,
  HSR_ERR_INVALID_ARG = 1,     /* null pointer, bad size, index out of range            */
  HSR_ERR_UNKNOWN_SHADER = 2,  /* shader kind outside hsr_shader_kind                   */
  HSR_ERR_BIN_OVERFLOW = 3,    /* scratch capacity exceeded and retries exhausted       */
  HSR_ERR_OUT_OF_MEMORY = 4,   /* device allocation failed / pool admission refused    */
  HSR_ERR_TIMEOUT = 5,         /* a bounded device wait or host wait gave up            */
  HSR_ERR_CUDA = 6,            /* CUDA runtime error (hsr_last_error() has the text)    */
  HSR_ERR_NOT_INITIALIZED = 7, /* hsr_init() not called or failed                       */
  HSR_ERR_BAD_HANDLE = 8,      /* unknown or released handle                            */
  HSR_ERR_BUSY = 9             /* request not finished yet (hsr_poll / server polling)  */
};

/* ---- shader kinds: one per IShader subclass (IShader.h:132-165) -------------------- */
typedef enum hsr_shader_kind {
  HSR_SHADER_GROUND = 0,             /* GroundShader            IShader.cpp:5-15    */
  HSR_SHADER_TOON = 1,               /* ToonShader              IShader.cpp:23-39   */
  HSR_SHADER_TEXTURE = 2,            /* TextureShader           IShader.cpp:47-57   */
  HSR_SHADER_TEXTURE_WITH_LIGHT = 3, /* TextureWithLightShader  IShader.cpp:65-77   */
  HSR_SHADER_BLINN = 4,              /* BlinnShader             IShader.cpp:85-109  */
  HSR_SHADER_NORMALMAP = 5,          /* NormalMapShader         IShader.cpp:117-162 */
  HSR_SHADER_SHADOW = 6,             /* ShadowShader            IShader.cpp:170-180 */
  HSR_SHADER_FLAT = 7,               /* test shader (no reference class): colour = bytes of
                                        prim id (face + prim_base + 1), R low byte        */
  HSR_SHADER_COUNT = 8
} hsr_shader_kind;

/* ---- uniforms: ShaderData (IShader.h:17-32) + Material scalars (IShader.h:7-15) ------
 * Matrices are row-major, m[row*4 + col], the layout of Matrix4x4 rows (matrix.h:27).
 * Colours are Color{r,g,b,a} (color.h).  The texture pointers of Material and the
 * shadow_map RenderBuffer* travel as handles in hsr_draw_desc. */
typedef struct hsr_shader_data {
  float view_pos[3];          /* ShaderData::view_Pos   */
  float light_dir[3];         /* ShaderData::light_dir  */
  float light_color[4];       /* ShaderData::light_color */
  float ambient[4];           /* ShaderData::ambient    */
  float model_matrix[16];
  float model_matrix_I[16];
  float view_matrix[16];      /* carried for completeness; the draw path does not read it */
  float projection_matrix[16];/* carried for completeness; the draw path does not read it */
  float light_vp_matrix[16];
  float camera_vp_matrix[16];
  int32_t enable_shadow;      /* ShaderData::enable_shadow */
  float material_color[4];    /* Material::color        */
  float material_specular[4]; /* Material::specular     */
  float gloss;                /* Material::gloss        */
  float bump_scale;           /* Material::bump_scale   */
} hsr_shader_data;

typedef uint64_t hsr_mesh;     /* 0 is never a valid handle */
typedef uint64_t hsr_texture;
typedef uint64_t hsr_target;

/* draw flags */
#define HSR_DRAW_CLEAR 1u        /* clear the target to clear_rgba / clear_depth / prim 0
                                    before drawing (fused: each pixel is written once) */

typedef struct hsr_draw_desc {
  hsr_mesh mesh;               /* DrawData::model                                        */
  int32_t shader;              /* hsr_shader_kind (typeid of DrawData::shader)           */
  uint32_t flags;              /* HSR_DRAW_*                                             */
  hsr_texture diffuse;         /* Material::diffuse_map, 0 = none (samples read as zero) */
  hsr_texture normal;          /* Material::normal_map,  0 = none                        */
  hsr_target target;           /* DrawData::render_buffer                                */
  hsr_target shadow_map;       /* ShaderData::shadow_map, 0 = nullptr                    */
  const hsr_shader_data* uniforms;
  uint32_t prim_base;          /* prim id written per pixel = prim_base + face + 1       */
  float clear_depth;           /* used with HSR_DRAW_CLEAR                               */
  uint8_t clear_rgba[4];       /* used with HSR_DRAW_CLEAR                               */
} hsr_draw_desc;

/* ---- lifetime ----------------------------------------------------------------------- */
HSR_API int hsr_init(int device);                 /* select device, create stream and scratch   */
HSR_API int hsr_shutdown(void);                   /* release every handle and device memory     */
HSR_API const char* hsr_last_error(void);         /* text of the last failure on this thread    */
HSR_API int hsr_abi_version(void);

/* ---- meshes: Model (model.h:8-33) --------------------------------------------------
 * pos [npos][3], nrm [nnrm][3], uv [nuv][2]; faces [nfaces][3 corners][3] holding the
 * 0-based (v, vt, vn) index of each corner, the layout of Model::faces_ (model.h:11).
 * Indices are validated on the host.  Normals are used as stored: the reference
 * normalises them in place on every access (model.cpp:108-111), which is the identity
 * for normals that are fixed points of Vector3f::normalize(). */
HSR_API int hsr_mesh_upload(const float* pos, int32_t npos, const float* nrm, int32_t nnrm,
                    const float* uv, int32_t nuv, const int32_t* faces, int32_t nfaces,
                    hsr_mesh* out);
/* Replace the normal array of a mesh (same count), e.g. per-corner normals a drop-in
 * shim extracted through Model::normal(). */
HSR_API int hsr_mesh_update_normals(hsr_mesh mesh, const float* nrm, int32_t nnrm);
HSR_API int hsr_mesh_release(hsr_mesh mesh);

/* ---- textures: TGAImage (tgaimage.h:66-98) ------------------------------------------
 * data is the TGAImage buffer: texel (x,y) at (x + y*w)*bytespp, bytes B,G,R(,A);
 * bytespp in {1,3,4}.  Sampling is TGAImage::get (tgaimage.cpp:248-253). */
HSR_API int hsr_texture_upload(const uint8_t* data, int32_t w, int32_t h, int32_t bytespp,
                       hsr_texture* out);
HSR_API int hsr_texture_release(hsr_texture tex);

/* ---- uniforms: ShaderData the way DrawModel::draw fills it (scene.h:55-71), bit for bit;
 * host only, no device needed. */
typedef struct hsr_transform {  /* GameObject::transform (gameobject.cpp:12-17) */
  float position[3];
  float rotation[3];            /* degrees about x, y, z; applied as rotate_z * rotate_x * rotate_y */
  float scale[3];
} hsr_transform;
typedef struct hsr_scene_params {
  float camera_position[3];     /* Camera::position                                          */
  float camera_target[3];       /* Camera::target (the view's look-at point)                */
  float light_position[3];      /* light->transform.position; the light looks at the origin */
  int32_t width, height;        /* frame buffer size: aspect = width / height                */
  hsr_transform model;          /* the drawn GameObject                                     */
  int32_t enable_shadow;
  float material_color[4];      /* Material (scene.cpp:81-84): White, White, 50, 1 there     */
  float material_specular[4];
  float gloss;
  float bump_scale;
} hsr_scene_params;
HSR_API int hsr_shader_data_build(const hsr_scene_params* p, hsr_shader_data* out);
HSR_API int hsr_model_matrix(const hsr_transform* t, float* out16);       /* GameObject::GetModelMatrix */
HSR_API int hsr_matrix_invert(const float* m16, float* out16);            /* Matrix4x4::invert          */
/* One step of the reference's orbital camera, Camera::update_transform (camera.cpp:31-70):
 * the target moves by the pan (in the camera's left / up plane, scaled by the distance and the
 * 60-degree field of view), then the eye is placed around the new target from the old offset's
 * radius, azimuth and polar angle, after dolly (radius * 0.95^dolly) and orbit (angles minus
 * 2*pi * orbit, polar angle clamped to [1e-5, pi - 1e-5]).  orbit and pan are cursor motions
 * in window heights and dolly is in scroll steps, accumulated as update_camera does
 * (camera.cpp:154-177).  Host only, bit for bit with the reference. */
typedef struct hsr_camera_motion {  /* Motion (camera.h:11) */
  float orbit[2];
  float pan[2];
  float dolly;
} hsr_camera_motion;
HSR_API int hsr_camera_update(const float position[3], const float target[3], const hsr_camera_motion* motion,
                              float out_position[3], float out_target[3]);

/* ---- asset files: Wavefront OBJ (Model::Model, model.cpp:6-48) and TGA
 * (TGAImage::read_tga_file, tgaimage.cpp:40-143).  The readers run on the host and need no
 * device (no hsr_init).  Call a reader with null arrays to get the counts, then again with
 * arrays at least that large (the counts in/out are the capacities). */
#define HSR_OBJ_CORNER_NORMALS 1u      /* one normal per face corner: the value Model::normal
                                          returns there during a draw (it normalises the stored
                                          normal in place on every read, model.cpp:108-111) ... */
#define HSR_OBJ_EARLIER_DRAWS(n) ((uint32_t)(n) << 8)  /* ... that follows n earlier draws of the
                                          model (0-255; a shadow pass is one: every draw reads
                                          every corner's normal once, graphics.cpp:380-387) */
#define HSR_TGA_MODEL_FLIP 1u          /* one more vertical flip after reading, as
                                          Model::load_texture does for a model's maps (model.cpp:74-83) */
/* faces: [nfaces][3 corners][v, vt, vn], 0-based, the first three corners of each face (the
 * corners graphics_draw_triangle draws, graphics.cpp:380-387). */
HSR_API int hsr_obj_read(const char* path, uint32_t flags, float* pos, int32_t* npos, float* nrm, int32_t* nnrm,
                         float* uv, int32_t* nuv, int32_t* faces, int32_t* nfaces);
/* data: w*h*bytespp bytes, the TGAImage buffer (texel (x, y) at (x + y*w)*bytespp, B,G,R(,A)). */
HSR_API int hsr_tga_read(const char* path, uint32_t flags, uint8_t* data, int32_t* w, int32_t* h, int32_t* bytespp);
/* TGAImage::write_tga_file (tgaimage.cpp:145-246): top-left origin, raw or run-length (rle != 0). */
HSR_API int hsr_tga_write(const char* path, const uint8_t* data, int32_t w, int32_t h, int32_t bytespp, int32_t rle);
/* Read and upload in one call (hsr_obj_read + hsr_mesh_upload, hsr_tga_read + hsr_texture_upload). */
HSR_API int hsr_mesh_load_obj(const char* path, uint32_t flags, hsr_mesh* out);
HSR_API int hsr_texture_load_tga(const char* path, uint32_t flags, hsr_texture* out);

/* ---- render targets: RenderBuffer (renderbuffer.h:5-22) + a prim-id plane ------------ */
HSR_API int hsr_target_create(int32_t w, int32_t h, hsr_target* out);
HSR_API int hsr_target_release(hsr_target t);
HSR_API int hsr_target_clear(hsr_target t, const uint8_t rgba[4], float depth); /* prim ids -> 0 */
/* Copy host RenderBuffer contents in (color_buffer RGBA8, depth_buffer FP32); prim may be NULL. */
HSR_API int hsr_target_upload(hsr_target t, const uint8_t* rgba, const float* depth, const uint32_t* prim);
/* Copy out; any pointer may be NULL.  Synchronises with the draws queued before it. */
HSR_API int hsr_target_download(hsr_target t, uint8_t* rgba, float* depth, uint32_t* prim);

/* Headless present, the pixels window_draw_buffer (win32.cpp:348-370) puts on screen: the
 * colour plane flipped to top-down rows, bytes B, G, R per pixel (channels 3), or B, G, R, 0
 * (channels 4; the reference never writes the fourth byte of its surface).  out holds
 * w*h*channels bytes.  hsr_target_write_tga writes the same image as a 24-bit TGA file. */
HSR_API int hsr_target_present(hsr_target t, uint8_t* out, int32_t channels);
HSR_API int hsr_target_write_tga(hsr_target t, const char* path, int32_t rle);

/* ---- drawing -------------------------------------------------------------------------
 * hsr_draw: one graphics_draw_triangle() call, queued on the library stream.
 * hsr_draw_batch: n draws in one launch sequence.  A draw whose shadow_map is the target
 * of another draw in the batch runs after it (the DrawModel::draw order, scene.h:86-91);
 * several draws into one target keep their array order.  A draw with HSR_DRAW_CLEAR into a
 * target that an earlier draw of the batch writes starts a new launch sequence, so that its
 * clear follows that draw as it would with separate calls. */
HSR_API int hsr_draw(const hsr_draw_desc* desc);
HSR_API int hsr_draw_batch(const hsr_draw_desc* descs, int32_t n);
HSR_API int hsr_synchronize(void);

/* hsr_draw_noalloc: the same draw as hsr_draw, for callers that must not allocate device or
 * page-locked host memory while they draw.  It has no counterpart in the reference.  Such
 * callers are render loops with a frame deadline (cudaMalloc and cudaFree can synchronise
 * the whole device and stall the loop for milliseconds), processes held to a fixed
 * device-memory budget that may not grow after start-up (a GPU shared with other services,
 * where a growing allocation can fail in the middle of a frame), and host applications that
 * forbid allocation inside their per-frame callbacks.  Meshes, textures and targets are the
 * caller's existing handles; the draw's own scratch is one fixed 128 MiB device array inside
 * the library, which every GPU that loads the library holds until the process exits, so the
 * call makes no cudaMalloc, cudaFree, cudaMallocHost or other allocating call.  A draw needing
 * more than 128 MiB of scratch is refused with HSR_ERR_INVALID_ARG (roughly 400k faces into
 * 1920x1080); one that overflows the fixed split on the device returns HSR_ERR_BIN_OVERFLOW
 * with the target untouched.  The call runs on the library's stream and returns when the
 * draw is complete.  Every call shares the array and it keeps the previous call's contents
 * (each call clears the counters it needs): calls whose GPU work overlaps race, so issue
 * them one after another.  The first call on a device looks up the array's address on that
 * device (cudaGetSymbolAddress); make that first call before any stream capture begins. */
HSR_API int hsr_draw_noalloc(const hsr_draw_desc* desc);

/* ---- tuning ------------------------------------------------------------------------- */
typedef struct hsr_tuning {
  int32_t tile;           /* raster tile edge in pixels: 8, 16 or 32 (16 and 32: 4 warps) */
  int32_t ctas_per_sm;    /* persistent raster CTAs per SM                          */
  int32_t warps_per_cta;  /* warps per raster CTA (one warp owns one tile)          */
  float bin_factor;       /* bin capacity = bin_factor * (faces + tiles) pairs      */
} hsr_tuning;
HSR_API int hsr_get_tuning(hsr_tuning* out);
HSR_API int hsr_set_tuning(const hsr_tuning* in);
/* Pick tile size (8, 16, 32), warps per CTA and CTAs per SM by timing the given batch (each
 * candidate renders it `reps` times into its targets), then search the bin capacity: the
 * smallest bin_factor of a ladder (0.5 .. 64) with which the batch runs without overflowing,
 * times 1.25 and at least 1.  Sets the choice and returns it in `out` (may be NULL). */
HSR_API int hsr_autotune(const hsr_draw_desc* descs, int32_t n, int32_t reps, hsr_tuning* out);

/* ---- failure injection for tests of the bounded device waits --------------------------
 * Host-side switches for hsr_draw / hsr_draw_batch (not plans or servers); no GPU fault is
 * involved.  poll_limit is the number of polls after which a bounded device wait gives up
 * (0 restores the default, about one second); once one dependency wait of a launch sequence
 * has given up, the others of that sequence stop waiting too.  faults is a mask of:
 *   HSR_FAULT_DEPENDENCY_STALL  raster tiles of a draw that reads another draw's target (its
 *                               shadow map) wait for one finished tile more than that draw
 *                               has, so the wait ends only by running out: the call returns
 *                               HSR_ERR_TIMEOUT and the device stays usable;
 *   HSR_FAULT_SCAN_STALL        the tile-count scan's first block withholds its prefix and
 *                               waits for a flag nothing sets, so every look-back runs out:
 *                               the call returns HSR_ERR_TIMEOUT and writes no target. */
#define HSR_FAULT_DEPENDENCY_STALL 1u
#define HSR_FAULT_SCAN_STALL 2u
HSR_API int hsr_set_fault_injection(uint32_t faults, int32_t poll_limit);

/* ---- statistics of the last completed draw sequence (for tests and benchmarks) ------- */
typedef struct hsr_stats {
  uint64_t records;       /* triangles that reached the raster                     */
  uint64_t clipped_faces; /* faces that went through the homogeneous clipper       */
  uint64_t bin_pairs;     /* (triangle, tile) pairs                                */
  uint64_t tiles;         /* tiles visited by the raster                           */
  uint64_t retries;       /* scratch re-sizes after an overflow                    */
  uint64_t kernel_launches; /* kernels this library launched since hsr_init         */
} hsr_stats;
HSR_API int hsr_get_stats(hsr_stats* out);

/* ---- plans: a batch recorded once into a CUDA graph and replayed ------------------------
 * hsr_plan_create validates the draws (same rules as hsr_draw_batch; a plan is one launch
 * sequence, so a draw that clears a target an earlier draw of the plan writes is refused with
 * HSR_ERR_INVALID_ARG), reserves the plan's own scratch, and records the whole launch sequence
 * (descriptor upload, counter reset, eight kernels) into a CUDA graph.  Between replays only uniforms may change
 * (hsr_plan_set_uniforms); meshes, textures, targets and shaders stay those of creation.
 * hsr_plan_launch replays the graph on the library stream and returns at once;
 * hsr_plan_wait blocks until it is done and re-runs it with larger scratch if the device
 * reported an overflow (the targets are left untouched by an overflowing run). */
typedef uint64_t hsr_plan;
HSR_API int hsr_plan_create(const hsr_draw_desc* descs, int32_t n, hsr_plan* out);
HSR_API int hsr_plan_set_uniforms(hsr_plan plan, int32_t draw, const hsr_shader_data* uniforms);
HSR_API int hsr_plan_launch(hsr_plan plan);
HSR_API int hsr_plan_wait(hsr_plan plan);
HSR_API int hsr_plan_release(hsr_plan plan);

/* ---- serving: continuous batching of render requests ------------------------------------
 * A server owns a scheduler thread.  Requests (one DrawModel::draw each: an optional shadow
 * pass into a shadow map of shadow_size^2, then the main pass) are queued by hsr_server_submit
 * and admitted in arrival order while the framebuffer pool has room for their targets
 * (pool_bytes, memory-based admission; a request larger than the whole pool fails with
 * HSR_ERR_OUT_OF_MEMORY).  Whenever one of the `slots` in-flight batches is free, everything
 * admitted so far (up to max_batch requests) becomes one launch sequence; launch sequences
 * run in turn on the server's compute stream while the next batch is formed and the previous
 * batch's results are copied out.  Colour / depth / prim ids of each request are
 * copied to the request's host pointers (page-locked memory recommended; NULL skips); the
 * targets return to the pool.  Results equal those of the same request drawn alone. */
typedef uint64_t hsr_server;
typedef struct hsr_server_config {
  uint64_t pool_bytes;     /* framebuffer pool budget for targets and shadow maps      */
  int32_t max_batch;       /* requests per launch sequence                              */
  int32_t slots;           /* batches in flight (each with its own copy stream)        */
} hsr_server_config;

typedef struct hsr_request {
  hsr_mesh mesh;
  int32_t shader;          /* hsr_shader_kind of the main pass                          */
  hsr_texture diffuse;
  hsr_texture normal;
  int32_t width, height;   /* main target                                               */
  int32_t shadow_size;     /* 0: no shadow pass; else an S x S shadow map (ShadowShader) */
  hsr_shader_data uniforms;
  uint8_t clear_rgba[4];
  float clear_depth;
  uint8_t shadow_clear_rgba[4];
  float shadow_clear_depth;
  uint8_t* out_rgba;       /* width*height*4 bytes, or NULL                            */
  float* out_depth;        /* width*height floats, or NULL                             */
  uint32_t* out_prim;      /* width*height, or NULL                                    */
} hsr_request;

typedef struct hsr_request_status {
  int32_t status;          /* HSR_OK, HSR_ERR_BUSY while pending, or the failure        */
  uint32_t batch;          /* sequence number of the batch that rendered it             */
  uint32_t batch_requests; /* requests in that batch                                    */
  uint32_t deferred;       /* times its targets could not be allocated at admission: the
                              request then stays queued at its place in arrival order and
                              is admitted again once memory frees up                    */
  double submit_ms;        /* times on the server's clock (ms since creation)           */
  double launch_ms;
  double done_ms;
} hsr_request_status;

HSR_API int hsr_server_create(const hsr_server_config* cfg, hsr_server* out);
HSR_API int hsr_server_submit(hsr_server s, const hsr_request* req, uint64_t* ticket);
HSR_API int hsr_server_poll(hsr_server s, uint64_t ticket, hsr_request_status* out);   /* HSR_ERR_BUSY if pending */
HSR_API int hsr_server_wait(hsr_server s, uint64_t ticket, int32_t timeout_ms, hsr_request_status* out);
HSR_API int hsr_server_now_ms(hsr_server s, double* out);
HSR_API int hsr_server_destroy(hsr_server s);   /* finishes in-flight work, fails queued requests */
/* Failure injection for tests of the admission path: the next n target allocations of the
 * server fail as if the device's memory pool were exhausted (no allocation is attempted).
 * Requests whose allocation fails are deferred, not failed: they stay queued in arrival
 * order and are admitted again when memory frees up; a request that still cannot get memory
 * with no batch in flight is failed with HSR_ERR_OUT_OF_MEMORY after 8 attempts. */
HSR_API int hsr_server_inject_alloc_failures(hsr_server s, int32_t n);

/* ---- timing of the last completed draw sequence (CUDA events on the library stream) --
 * batch_ms spans the upload of the view descriptors to the end of the raster kernel;
 * kernel_ms holds one entry per kernel of the launch sequence, in launch order, filled when
 * profiling is on:
 *   [0] vertex   screen vertices (k_vertex)
 *   [1] cull     fast accept, cull, viewport, bounding box, record (k_setup)
 *   [2] emit     shading payloads and tile counts of the surviving triangles (k_emit)
 *   [3] clip     homogeneous clipper for faces crossing a plane (k_post)
 *   [4] split    sub-records of triangles touching many tiles (k_big)
 *   [5] scan     prefix sums over the tile counts (k_scan)
 *   [6] scatter  tile lists, and the clear of tiles without triangles (k_scatter)
 *   [7] raster   coverage, depth test, shading, writes (k_raster) */
#define HSR_KERNEL_COUNT 8
typedef struct hsr_timing {
  float batch_ms;
  float kernel_ms[HSR_KERNEL_COUNT];
  uint32_t launches;       /* kernels launched by the sequence                         */
  uint32_t views;          /* draws in the sequence                                    */
  uint64_t h2d_bytes;      /* host -> device bytes of the sequence (view descriptors)  */
  uint64_t d2h_bytes;      /* device -> host bytes (control block)                     */
  uint64_t pixels;         /* target pixels covered by the draws' tile grids           */
  uint64_t shaded_pixels;  /* pixels whose visible fragment was shaded                 */
  uint64_t records;        /* triangles that reached the raster                        */
  uint64_t bin_pairs;      /* (triangle, tile) pairs                                   */
  uint64_t faces;          /* faces processed                                          */
  uint64_t vertices;       /* positions transformed                                    */
  uint64_t normals;        /* normals transformed once per normal (0: world normals are
                              transformed per corner of the triangles that survive setup) */
  uint64_t clipped_faces;  /* faces that went through the homogeneous clipper          */
  uint64_t fragments;      /* covered (pixel, triangle) pairs tested against the depth  */
  uint64_t raster_pixels;  /* pixels of the tiles the raster visited (tiles with triangles;
                              the fused clear of the others runs beside the binning)    */
  uint64_t tiles;          /* screen tiles of the sequence (all views)                  */
  uint64_t split_triangles;/* triangles split into sub-records (more than 32 tiles)     */
  uint64_t payload_bytes;  /* shading payload bytes written for the raster's records    */
} hsr_timing;
HSR_API int hsr_set_profiling(int on);
HSR_API int hsr_last_timing(hsr_timing* out);

/* Page-locked host memory for buffers passed to upload / download (fast DMA). */
HSR_API int hsr_host_alloc(size_t bytes, void** out);
HSR_API int hsr_host_free(void* p);

#ifdef __cplusplus
}
#endif
#endif /* HSR_H */
