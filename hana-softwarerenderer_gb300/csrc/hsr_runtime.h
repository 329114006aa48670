// hsr_runtime.h — host-side objects behind the C ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "hsr_internal.h"

namespace hsr {

struct MeshObj {  // Model (model.h:8-33) resident on the device
  float *px = nullptr, *py = nullptr, *pz = nullptr;
  float *nx = nullptr, *ny = nullptr, *nz = nullptr;
  float4 *p4 = nullptr, *n4 = nullptr;  // positions and normals as (x, y, z, 0)
  float4* pk = nullptr;  // meshes whose v, vt, vn indices agree: per vertex one 32-byte sector,
                         // (x, y, z, nx), (ny, nz, u, v)
  float2* uv = nullptr;
  int4 *fv = nullptr, *fvt = nullptr, *fvn = nullptr;
  int32_t npos = 0, nnrm = 0, nuv = 0, nfaces = 0;
  bool unified = false;  // v, vt and vn indices agree at every face corner
  ~MeshObj();
};

struct TexObj {  // TGAImage (tgaimage.h:66-98) as 32-bit BGRA words
  uint32_t* words = nullptr;
  int32_t w = 0, h = 0, bpp = 0;
  ~TexObj();
};

struct TargetObj {  // RenderBuffer (renderbuffer.h:5-22) + prim-id plane
  uint32_t* color = nullptr;  // RGBA8, byte order r, g, b, a
  float* depth = nullptr;
  uint32_t* prim = nullptr;
  int32_t w = 0, h = 0;
  char* block = nullptr;          // one stream-ordered allocation holding the three planes
  cudaStream_t stream = nullptr;  // the stream it was allocated on (and is freed on)
  bool pooled = false;  // memory owned by a server's pool (freed by the server, not here)
  ~TargetObj();
};

struct Arena {  // grow-only device scratch
  char* base = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes);
};

struct Pinned {  // grow-only pinned host staging
  char* base = nullptr;
  size_t cap = 0;
  int reserve(size_t bytes);
};

// One launch sequence: view descriptors, work chunks, scratch layout and capacities.
struct Plan {
  struct Off { size_t clip; };
  int n = 0, tile = 8, nscan = 0;
  std::vector<int> order;         // plan position -> index in the caller's array
  std::vector<DView> views;
  std::vector<Off> offs;
  int nvch = 0, nsch = 0, ncch = 0;  // vertex / setup / clear chunks of the batch (bases in each DView)
  uint32_t stash_warps = 0;          // raster warps with a stash (the device's SMs x kStashWarpsPerSm)
  size_t view_bytes = 0, total_faces = 0, total_tiles = 0, total_pos = 0, total_nrm = 0, total_pixels = 0;
  size_t rec_cap = 0, clip_cap = 0, bin_cap = 0, big_cap = 0;
  size_t o_views = 0, o_vout = 0, o_zero = 0, zero_bytes = 0, o_ctl = 0, o_done = 0,
         o_cnt = 0, o_fill = 0, o_stat = 0, o_toff = 0, o_neoff = 0, o_list = 0, o_recs = 0, o_pay = 0, o_clip = 0,
         o_big = 0, o_bins = 0, o_stash = 0;
  size_t dev_bytes = 0, host_bytes = 0, stage_bytes = 0;
  char* dev = nullptr;
  char* host = nullptr;
  Scratch sc = {};

  void layout();
  void bind(char* dev_base, char* host_base);
  int enqueue(cudaStream_t s, int num_sms, const hsr_tuning& tu, cudaEvent_t* ev);
  int kernel_count() const;
  bool grow(const Ctl& c);
};

// Index of the first draw that clears a target an earlier draw of the batch writes (n if none):
// a batch runs as one launch sequence up to there.
int first_reclear(const hsr_draw_desc* d, int n);

struct Runtime {
  int device = 0;
  int num_sms = 1;
  cudaStream_t stream = nullptr;
  uint64_t next_handle = 1;
  std::unordered_map<uint64_t, MeshObj*> meshes;
  std::unordered_map<uint64_t, TexObj*> textures;
  std::unordered_map<uint64_t, TargetObj*> targets;
  Arena arena;
  Pinned staging;
  hsr_tuning tuning = {8, 4, 8, 4.0f};
  hsr_stats stats = {};
  uint64_t launches = 0;
  size_t cap_rec_hint = 0, cap_clip_hint = 0, cap_bin_hint = 0, cap_big_hint = 0;
  bool profiling = false;
  uint32_t faults = 0;     // hsr_set_fault_injection: HSR_FAULT_* for hsr_draw / hsr_draw_batch
  int32_t poll_limit = 0;  // and the bounded waits' poll limit (0: default)
  static constexpr int kEvents = HSR_KERNEL_COUNT + 2;  // start, after the memset, after each kernel
  cudaEvent_t ev[kEvents] = {};
  hsr_timing timing = {};

  MeshObj* mesh(uint64_t h);
  TexObj* tex(uint64_t h);
  TargetObj* target(uint64_t h);
  int validate(const hsr_draw_desc& d);
  int plan_order(const hsr_draw_desc* d, int n, std::vector<int>& order, std::vector<int>& dep0,
                 std::vector<int>& dep1);
  int plan_build(const hsr_draw_desc* descs, int n, Plan& p);
  void record_result(const Plan& p, const Ctl& c);
  // A plan overflowed and grew: later plans start from at least its capacities (every path
  // that launches plans, so one overflow is not repeated by each later batch).
  void learn_caps(const Plan& p);
  int run_batch(const hsr_draw_desc* descs, int n);     // one or more launch sequences
  int run_sequence(const hsr_draw_desc* descs, int n);  // one launch sequence
  int clear_target(TargetObj* t, const uint8_t rgba[4], float depth);

 private:
  template <class T> T* get(std::unordered_map<uint64_t, T*>& m, uint64_t h);
};

extern Runtime* g_rt;
extern std::mutex g_mu;
extern thread_local std::string g_last_error;
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);
void mat_mul_ref(const float* a, const float* b, float* out);
void serve_shutdown();
int launch_clear(uint32_t* color, float* depth, uint32_t* prim, size_t n, uint32_t rgba, float d, cudaStream_t s);
int launch_pack_vertices(float4* pk, const float4* p4, const float4* n4, const float2* uv, int npos, int nnrm, int nuv,
                         cudaStream_t s);

}  // namespace hsr
