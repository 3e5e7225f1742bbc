// Internal device-side definitions shared by the kernels and the host layer.
//
// Arithmetic contract: every translation unit is compiled with -fmad=false,
// so `a * b + c` is a rounded multiply followed by a rounded add, exactly as
// the reference's expressions read and as the CPU oracle evaluates them;
// division and square root are the IEEE-rounded defaults.  Index, weight and
// int16 TSDF results are therefore bit-identical to the oracle.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "vs.h"

namespace vs {

constexpr int kMaxLevels = 3;
constexpr int kBrick = 8;             // 8^3 voxels per brick = reference sub-cube
constexpr int kBrickVox = 512;
constexpr float kQ = 32767.0f;
constexpr int kPartials = 32;         // partial slots per ICP block (29 used)
constexpr int kIcpMaxBlocks = 456;    // 3 blocks per SM on 152 SMs
constexpr int kMaxSlots = 64;         // sessions per batched launch

struct Level {
  int W, H;
  float K[4];  // fx, fy, cx, cy
};

// Pose and ICP state of one session, device resident.  The first 80 bytes
// (float pose and frame result) are what the host reads back per frame.
struct Pose {
  float Tgc[16];       // float copies read by the kernels
  int tracked;         // result of the last frame: 1 tracked (or first), 0 lost
  int iters_run;
  int valid_count;     // correspondences of the last iteration
  int frame;           // frames processed
  float Tcg[16];
  float center[3];     // camera centre in global coordinates
  float T21[16];       // float inverse of T12, read by the ICP term kernel
  double T_gc[16];     // FP64 master pose, global -> camera
  double T12[16];      // ICP increment of the current frame (camera t0 -> t1)
  int level_done[kMaxLevels];
  int failed;          // 6x6 system singular this frame
  int skip;            // no tracking this frame (first frame)
  float last_x[6];
  double last_sums[29];
};
constexpr size_t kPoseHeadBytes = 80;

// Everything a kernel needs to know about one session, copied to the device
// once at creation (pointers do not change afterwards).
struct SessionDev {
  Level lv[kMaxLevels];
  int levels;
  int dim[3];
  int nb[3];            // bricks per axis
  float origin[3];
  float vox, vox_inv, mu, max_w, r_cube;
  float cube_center[3];
  float th_icp, cos_normal;
  int iters[kMaxLevels];
  int reduce_mode, tsdf_type;
  float depth_scale;
  float gauss[5];       // bilateral spatial weights
  // frame buffers
  uint16_t* depth_mm;            // level-0 input (uint16)
  float* depth_raw;              // level-0 metres (integration input)
  float* depth[kMaxLevels];      // filtered pyramid
  float4* in_vtx[kMaxLevels];    // input vertex map (w = 1 valid, 0 invalid)
  float4* in_nrm[kMaxLevels];    // input normal map (w = 1 valid)
  uint8_t* in_code[kMaxLevels];  // normal-map pre-pass codes
  uint32_t* in_amask[kMaxLevels];// per-row bitmasks of normals failing the angle test
  uint32_t* in_rmask[kMaxLevels];// per-row rejection bitmasks
  float* m_depth[kMaxLevels];    // model (ray-cast) maps
  float4* m_vtx[kMaxLevels];     // xyz, w = 1 valid (invalid: -100)
  float4* m_nrm[kMaxLevels];
  uint8_t* m_img[kMaxLevels];
  // volume
  void* vol;                     // bricks, 512 words each
  uint32_t* brick_flag;          // per brick: stamp of the last integration that listed it (0: never / carved)
  uint32_t* brick_list;          // active bricks of this frame
  uint32_t* brick_count;         // [0] active bricks, [1] voxels updated (per frame), [2] activation stamp
  uint32_t* occ;                 // 1 bit per brick: some voxel has weight > 0 (NULL: not kept)
  uint8_t* band;                 // per brick: 1 if some voxel has weight > 0 and a TSDF value other
                                 // than 1 (a superset is allowed; NULL: not kept)
  uint8_t* bdist;                // per brick: Chebyshev distance in bricks to the nearest band brick,
                                 // saturating at kBandReach + 1 (rebuilt before every ray-cast)
  uint8_t* btmp;                 // the distance transform's intermediate (x and y passes)
  // ICP scratch
  double* partials;              // [kIcpMaxBlocks][2*kPartials]
  unsigned* icp_counter;
  Pose* pose;
  // tables built once per session with the reference's formulas
  float* lut_vox;                // voxel centre coordinate per axis: dim[0] + dim[1] + dim[2]
  float* lut_ray;                // level-0 K^-1 [x 1 1] (W) then [1 y 1] (H) components
  float4* ray_hit;               // surface points of a colour ray-cast (two launches), every level's
                                 // pixels in turn
  // colour (NULL pointers when the session keeps none)
  uint32_t* col;                 // colour bricks parallel to vol: per voxel 0x00BBGGRR
  uint8_t* rgb_in;               // level-0 colour frame, planar R, G, B
  uint32_t* rgb_packed;          // the same frame as one 0x00BBGGRR word per pixel
  uint32_t* m_rgb[kMaxLevels];   // ray-cast colour per pixel, 0x00BBGGRR
  float* lam_map;                // level-0 ray scale per pixel (NULL: computed per voxel)
  float2* dl_map;                // level-0 {depth (m), ray scale} per pixel, written by the ingest: one
                                 // gather per voxel in the integration (NULL: depth_raw and lam_map)
};

// Sessions advanced together by one launch of every per-frame kernel.  The
// kernels are persistent: a fixed grid walks the work items of all sessions
// (tiles, ICP block ranges, bricks), mapping an item to (slot, local index)
// through the prefix arrays, so one captured graph serves any set of
// sessions.  A session's items and their order do not depend on the other
// sessions of the table, so every result is the same alone and in a batch.
// One session alone is a table of one slot.
struct BatchTable {
  int n;
  int ray_lx;                          // ray tile of a warp: (1 << ray_lx) x (32 >> ray_lx) rays
  int bil_rows;                        // rows of a level-0 tile (bilateral, activation): 4, 8 or 16
  const SessionDev* s[kMaxSlots];
  int bil[kMaxSlots + 1];              // level-0 32 x bil_rows tiles (bilateral, activation)
  int pyr[kMaxLevels - 1][kMaxSlots + 1];  // 32x8 tiles of levels 1, 2
  int ipre[kMaxSlots + 1];             // input-map pre-pass 32x8 tiles, all levels
  int ipost[kMaxSlots + 1];            // input-map post-pass 16x16 tiles, all levels
  int scan[kMaxSlots + 1];             // input-map row scans: one per level
  int icp[kMaxLevels][kMaxSlots + 1];  // ICP block ranges per level
  int ray[kMaxSlots + 1];              // ray-cast tiles, all levels
  const uint16_t* frame[kMaxSlots];    // the uint16 frame each slot's ingest reads in place this step (device
                                       // memory, or pinned host memory the device can address; the ingest
                                       // also copies it into the session's frame buffer); NULL: that buffer
  int slab[kMaxSlots + 1];             // z slabs of bricks (band distance, x and y passes)
  int brow[kMaxSlots + 1];             // y rows of bricks (band distance, z pass)
  unsigned work[8];                    // work counters ([0..1] ray march, [2..3] ICP, [4..5] ray
                                       // shading); zero between launches
};

// slot of work item b (pre: prefix over n slots), or -1 past the last item
__device__ inline int find_slot(const int* pre, int n, int b, int& local) {
  if (b >= pre[n]) return -1;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (pre[mid] <= b)
      lo = mid;
    else
      hi = mid - 1;
  }
  local = b - pre[lo];
  return lo;
}

// ---------------------------------------------------------------------------
// small float3 helpers (the reference's ITMMath Vector3f operations)
// ---------------------------------------------------------------------------
struct F3 {
  float x, y, z;
};
__host__ __device__ inline F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__host__ __device__ inline F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline F3 scale(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline float length(F3 a) { return sqrtf(dot(a, a)); }
__host__ __device__ inline F3 normalised(F3 a) {
  float inv = 1.0f / sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
  return f3(a.x * inv, a.y * inv, a.z * inv);
}
// d_p_Project (_yooji_cuda_math.h:205-210)
__host__ __device__ inline void project(F3 p, const float* K, float& u, float& v) {
  u = K[0] * p.x / p.z + K[2];
  v = K[1] * p.y / p.z + K[3];
}
// d_bp_Back_Project (_yooji_cuda_math.h:212-226)
__host__ __device__ inline F3 back_project(float u, float v, const float* K, float d) {
  return f3(d * (u - K[2]) / K[0], d * (v - K[3]) / K[1], d);
}
// d_t_Transform / d_r_Rotate (_yooji_cuda_math.h:229-244)
__host__ __device__ inline F3 transform(F3 p, const float* M) {
  return f3(M[0] * p.x + M[1] * p.y + M[2] * p.z + M[3], M[4] * p.x + M[5] * p.y + M[6] * p.z + M[7],
            M[8] * p.x + M[9] * p.y + M[10] * p.z + M[11]);
}
__host__ __device__ inline F3 rotate(F3 p, const float* M) {
  return f3(M[0] * p.x + M[1] * p.y + M[2] * p.z, M[4] * p.x + M[5] * p.y + M[6] * p.z,
            M[8] * p.x + M[9] * p.y + M[10] * p.z);
}
// ROUNDF (_yooji_cuda_defines.h): half away from zero via truncation
__host__ __device__ inline int roundf_ref(float x) {
  return (x < 0.0f) ? (int)(x - 0.5f) : (int)(x + 0.5f);
}
// d_gpv_Get_Position_in_Voxel (_yooji_cuda_math.h:265-283)
__device__ inline bool pos_in_voxel(F3 p, const SessionDev& s, F3& v) {
  v.x = (p.x - s.origin[0]) * s.vox_inv - 0.5f;
  v.y = (p.y - s.origin[1]) * s.vox_inv - 0.5f;
  v.z = (p.z - s.origin[2]) * s.vox_inv - 0.5f;
  return !(v.x < -0.5f || v.x >= (float)s.dim[0] - 0.5f || v.y < -0.5f ||
           v.y >= (float)s.dim[1] - 0.5f || v.z < -0.5f || v.z >= (float)s.dim[2] - 0.5f);
}
// d_gpw_Get_Position_in_World (_yooji_cuda_math.h:285-302)
__device__ inline F3 pos_in_world(F3 v, const SessionDev& s) {
  return f3((v.x + 0.5f) / s.vox_inv + s.origin[0], (v.y + 0.5f) / s.vox_inv + s.origin[1],
            (v.z + 0.5f) / s.vox_inv + s.origin[2]);
}

// ---------------------------------------------------------------------------
// voxel storage
//   INT16: word = (uint16 weight << 16) | uint16(int16 q), tsdf = q / 32767
//   FP16 : word = (uint16 weight << 16) | half bits
//   FP32 : uint2 {float bits, uint32 weight}
// Bricks are 512 consecutive words, x fastest inside the brick; bricks are
// ordered x fastest, then y, then z.
// ---------------------------------------------------------------------------
__host__ __device__ inline uint32_t pack_rgb(uint32_t r, uint32_t g, uint32_t b) { return r | (g << 8) | (b << 16); }
__host__ __device__ inline uint32_t rgb_channel(uint32_t w, int k) { return (w >> (8 * k)) & 0xffu; }

// Band bricks and their distance field.  A ray-cast sample reads TSDF 1
// wherever the nearest voxel has weight 0 or value 1, and such samples leave
// the march's state and step unchanged; only a "band" brick (a voxel with
// weight > 0 and a value other than 1) can change them.  Before every ray-cast
// the Chebyshev distance (in bricks) from every brick to the nearest band
// brick is rebuilt, saturating at kBandReach + 1, so the march jumps through
// the box of bricks around its position that holds no band brick.  The field
// changes speed, never a sample.  Volumes have at most kMaxBricksAxis bricks
// per axis (1024 voxels).
constexpr int kBandReach = 7;
constexpr int kMaxBricksAxis = 128;

// sets bit i of a bitmap unless it is set already (the test keeps the atomics
// off words whose bits all settled in earlier frames)
__device__ inline void set_bit_once(uint32_t* bits, uint32_t i) {
  const uint32_t m = 1u << (i & 31);
  if (!(*((volatile uint32_t*)bits + (i >> 5)) & m)) atomicOr(bits + (i >> 5), m);
}

__host__ __device__ inline size_t brick_word_index(int x, int y, int z, const int* nb) {
  size_t b = ((size_t)(z >> 3) * nb[1] + (size_t)(y >> 3)) * nb[0] + (size_t)(x >> 3);
  return b * kBrickVox + (size_t)(((z & 7) << 6) | ((y & 7) << 3) | (x & 7));
}

__device__ inline float q_to_tsdf(int q) { return (float)q * (1.0f / kQ); }
__device__ inline int tsdf_to_q(float t) {
  float r = rintf(t * kQ);
  r = fminf(fmaxf(r, -kQ), kQ);
  return (int)r;
}

struct StoreI16 {
  typedef uint32_t word;
  __device__ static inline void decode(word v, float& t, uint32_t& w) {
    t = q_to_tsdf((int)(int16_t)(v & 0xffffu));
    w = v >> 16;
  }
  __device__ static inline word encode(float t, uint32_t w) {
    return (w << 16) | ((uint32_t)(uint16_t)(int16_t)tsdf_to_q(t));
  }
  __device__ static inline word initial() { return (uint32_t)(uint16_t)(int16_t)32767; }
  // weight > 0 and a value other than 1 (code 32767 is the only one that decodes to 1)
  __device__ static inline bool band(word v) { return v >= 0x10000u && (v & 0xffffu) != 0x7fffu; }
};
struct StoreF16 {
  typedef uint32_t word;
  __device__ static inline void decode(word v, float& t, uint32_t& w) {
    t = __half2float(__ushort_as_half((unsigned short)(v & 0xffffu)));
    w = v >> 16;
  }
  __device__ static inline word encode(float t, uint32_t w) {
    return (w << 16) | (uint32_t)__half_as_ushort(__float2half_rn(t));
  }
  __device__ static inline word initial() { return (uint32_t)__half_as_ushort(__float2half_rn(1.0f)); }
  __device__ static inline bool band(word v) { return v >= 0x10000u && (v & 0xffffu) != 0x3c00u; }
};
struct StoreF32 {
  typedef uint2 word;
  __device__ static inline void decode(word v, float& t, uint32_t& w) {
    t = __uint_as_float(v.x);
    w = v.y;
  }
  __device__ static inline word encode(float t, uint32_t w) { return make_uint2(__float_as_uint(t), w); }
  __device__ static inline word initial() { return make_uint2(__float_as_uint(1.0f), 0u); }
  __device__ static inline bool band(word v) { return v.y != 0u && v.x != 0x3f800000u; }
};

inline size_t voxel_bytes(int tsdf_type) { return tsdf_type == VS_TSDF_FP32 ? 8 : 4; }

// ---------------------------------------------------------------------------
// launch wrappers (one per kernel file).  `bt` is the device table and `hb`
// its host copy; grids are fixed (persistent), so a captured graph does not
// depend on the table's contents.
// ---------------------------------------------------------------------------
// Launch shape of the ray-cast kernels.  It changes grid sizes and how rays
// are grouped into warps, never a ray's computation, so every shape gives
// the same results (the autotuner picks among them by time).
struct LaunchShape {
  int ray_lx = 3;               // ray tile of a warp: (1 << ray_lx) x (32 >> ray_lx), ray_lx in 0..5
  int march_blocks_per_sm = 0;  // resident 128-thread blocks per SM of the march grid (0: as many as fit)
  int shade_blocks_per_sm = 0;
  int bil_rows = 8;             // level-0 tile rows of the bilateral filter and the activation: 4, 8, 16
  int integrate_blocks_per_sm = 0;  // 256-thread blocks per SM of the update grid (0: as many as fit)
};

int icp_blocks(int npix, int level);
int sm_count();
void fill_batch_table(BatchTable& hb, const SessionDev* const* host_recs, const SessionDev* const* dev_recs, int n,
                      int ray_lx = 3, int bil_rows = 8);
int ray_max_blocks_per_sm(int tsdf_type, bool shade);
void launch_filter(const BatchTable* bt, cudaStream_t st, int bil_rows = 8);
void launch_input_maps(const BatchTable* bt, cudaStream_t st);
void launch_bilateral_float(const SessionDev& h, const float* in, float* out, cudaStream_t st);
// ICP of every slot; the schedule runs levels max_levels-1 .. 0 with
// max_iters[l] launches each (slots with fewer levels or iterations skip)
void launch_icp(const BatchTable* bt, int max_levels, const int* max_iters, int reduce_mode, cudaStream_t st,
                bool frame_mode, const float* init_T12_dev);
// depth / Tgc / Tcg: explicit inputs of a one-slot table, or NULL for each
// session's own level-0 depth and pose; color: run the variant that also
// blends the colour of sessions that keep a colour volume
// blocks_per_sm: update grid (0: every block resident); dry: the update
// computes everything but stores no voxel (the autotuner's timing runs)
void launch_integrate(const BatchTable* bt, int tsdf_type, const float* depth, const float* Tgc,
                      const float* Tcg, bool gate_on_tracking, cudaStream_t st, bool color = false,
                      int blocks_per_sm = 0, bool dry = false);
// level < 0: every level of every slot into the sessions' model maps; else
// one level of a one-slot table into the external outputs with explicit poses;
// color: the shading variant that also interpolates colour
void launch_raycast(const BatchTable* bt, int tsdf_type, int level, const float* Tgc, const float* Tcg,
                    const float* center, float lx, float ly, float lz, bool gate_on_tracking, float* out_depth,
                    float* out_vtx3, float* out_nrm3, uint8_t* out_img, cudaStream_t st,
                    const LaunchShape& shape = LaunchShape(), uint8_t* out_rgb = nullptr, bool color = false,
                    int mode = 0);
// render variants (launch_raycast mode bits, external outputs only)
constexpr int kRayScene = 1;           // d_crtcs: camera centre to 2 r_cube, no cone test
constexpr int kRayGlobalNormals = 2;   // normals left in the global frame
constexpr int kRayNearestColor = 4;    // d_grvu nearest-voxel colour instead of d_grvi
constexpr int kRayWhiteBackground = 8; // colour 255 where nothing is hit
void launch_session_tables(const SessionDev& h, SessionDev* d, cudaStream_t st);
// planar colour frame -> one word per pixel (rgb: a device frame, or NULL for the session's own)
void launch_pack_color(const SessionDev& h, const uint8_t* rgb, cudaStream_t st);
// g_uvv_Update_Valid_Volume: valid = one byte per voxel, x fastest, 8-byte
// aligned; *carved (device) counts the sub-cubes reset
void launch_carve(const SessionDev& h, const SessionDev* d, const uint8_t* valid, unsigned* carved, cudaStream_t st);
// colour volume <-> reference layout (three planes of x-fastest bytes)
void launch_color_volume(const SessionDev& h, bool do_export, uint8_t* planes, cudaStream_t st);
void launch_color_map_export(const SessionDev& h, int level, uint8_t* planes, cudaStream_t st);
void launch_volume_init(const SessionDev& h, cudaStream_t st);
void launch_pose_set(const SessionDev* d, const double* T_gc, cudaStream_t st);
// pose heads of every slot, kPoseHeadBytes each, into out (kMaxSlots slots)
void launch_gather_heads(const BatchTable* bt, void* out, cudaStream_t st);
size_t occupancy_words(const SessionDev& h);  // 32-bit words of the per-brick occupancy bits
void launch_occupancy_clear(const SessionDev& h, cudaStream_t st);
void launch_occupancy_rebuild(const SessionDev& h, const SessionDev* d, cudaStream_t st);
void launch_maps_export(const SessionDev& h, int level, float* vtx3, float* nrm3, float* ivtx3, float* inrm3,
                        cudaStream_t st);

}  // namespace vs
