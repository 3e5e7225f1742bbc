/*
 * CPU oracle for the per-frame reconstruction path of vcl-volume-scanner.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py call it to
 * produce the expected results.  The product (the CUDA library) never links,
 * loads or calls it.
 *
 * It is a plain C++ restatement of the reference's algorithms, each function
 * citing the reference file:line it follows (paths relative to
 * VCL_Volume_Scanner/).  Parity status: the reference cannot be compiled on
 * Linux (MSVC/MFC project, CUDA 8 texture references, missing ITMMath and
 * KAISION headers), so the stage restatements are "parity unpinned" against
 * reference outputs; they are pinned by analytic known-answer tests, and the
 * host SE(3) exponential / 4x4 inverse are pinned against the reference's own
 * STAC/Util/_yooji_math_inlines.h compiled here (oracle/ref_pin.cpp).
 *
 * Arithmetic contract shared with the CUDA kernels: every expression is
 * evaluated in the same order with IEEE single precision, no fused
 * multiply-add (-ffp-contract=off here, -fmad=false there), correctly rounded
 * division and square root.  Integer / index / weight results are therefore
 * bit-exact; the only transcendental that differs is exp (glibc expf here,
 * __expf in the bilateral kernel, as in the reference).
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- configuration (mirrors the reference's scanner parameters) ---- */
typedef struct {
  int width, height;        /* level-0 image size                          */
  float fx, fy, cx, cy;     /* level-0 intrinsics                          */
  int levels;               /* pyramid levels (reference: 3)               */
  int dim[3];               /* volume voxels per axis (multiples of 8)     */
  float origin[3];          /* world position of voxel (-0.5,-0.5,-0.5)    */
  float voxel_size;         /* metres                                      */
  float mu;                 /* truncation distance (m)                     */
  float max_w;              /* weight cap (reference: 100)                 */
  float th_icp;             /* squared distance threshold (m^2)            */
  float cos_normal;         /* normal rejection: cos(angle); <= -2 = off   */
  int icp_iters[3];         /* iterations per level 0..2                   */
  int tsdf_store;           /* 0 = fp32, 1 = int16 (q*32767), 2 = fp16     */
  int reduce_mode;          /* 0 = reference tree, 1 = naive fp32,
                               2 = compensated fp32, 3 = fp64              */
  float depth_scale;        /* uint16 units -> metres (0.001)              */
} or_config;

/* single stages (float reference semantics) */
void or_depth_to_m(const uint16_t* in, int n, float scale, float* out);
void or_gaussian_table(float delta, int radius, float* out);
void or_bilateral(const float* in, int w, int h, float* out);
void or_pyramid_down(const float* in, int w, int h, float* out);
void or_point_normal_map(const float* depth, int w, int h, const float K[4],
                         float* vtx3, float* nrm3);
void or_level_intrinsics(const float K0[4], int levels, float* Kl);

/* ICP on explicit inputs.  depth[l]: input depth of level l; mvtx[l] / mnrm[l]:
 * model vertex / normal maps (AoS float3, camera frame of the previous pose);
 * nvtx[l]: input normal maps (may be NULL when cos_normal is off).
 * T_gc_prev: previous pose (global -> camera).  init_T12: optional initial
 * increment (NULL = identity, all levels; else level 0 only).
 * Returns 1 on success and writes T_gc_out; 0 on failure. info[0] = total
 * iterations run, info[1] = valid correspondences in the last iteration. */
int or_track(const or_config* cfg, const float* const* depth,
             const float* const* mvtx, const float* const* mnrm,
             const float* const* nnrm, const float* T_gc_prev,
             const float* init_T12, float* T_gc_out, int* info);
int or_track_f64(const or_config* cfg, const float* const* depth,
                 const float* const* mvtx, const float* const* mnrm,
                 const float* const* nnrm, const double* T_gc_prev,
                 const double* init_T12, double* T_gc_out, int* info);

/* ICP normal-equation sums for one iteration (27 unique + count + sum b^2),
 * reduced in the given mode.  T21: current increment, camera t1 -> t0. */
int or_icp_sums(const or_config* cfg, int level, const float* depth,
                const float* mvtx, const float* mnrm, const float* nnrm,
                const float* T21, double* out29);

/* pose helpers (reference float semantics) */
void or_pose_inverse(const float* T, float* Tinv);
void or_camera_center(const float* T_gc, float* c);
void or_se3_exp(const float* xi, float* T);
void or_se3_exp_f64(const double* xi, double* T);

/* volume: x-fastest linear arrays as in the reference (z*W*H + y*W + x) */
typedef struct or_volume or_volume;
or_volume* or_volume_create(const or_config* cfg);
void or_volume_destroy(or_volume* v);
void or_volume_reset(or_volume* v);
/* tsdf (dequantised float), weights; either may be NULL */
void or_volume_get(const or_volume* v, float* tsdf, uint16_t* w);
void or_volume_set(or_volume* v, const float* tsdf, const uint16_t* w);
/* flags of the last integrate call, one byte per 8^3 sub-cube */
void or_volume_flags(const or_volume* v, uint8_t* flags);
/* render variants: mode bits 1 scene ray-cast, 2 global normals, 4 nearest-voxel
 * colour, 8 colour 255 where nothing is hit; vtx3 / rgb may be NULL */
void or_render_variant(const or_volume* v, int level, int mode, const float* T_gc, const float* T_cg,
                       const float* cam_cen, const float* light, float* depth, float* vtx3, float* nrm3,
                       uint8_t* img, uint8_t* rgb);
/* valid-volume carving over the last integration's sub-cube flags */
uint32_t or_update_valid_volume(or_volume* v, const uint8_t* valid);
/* the expanded cube geometry: centre[3], r_cube, 1/voxel size */
void or_config_geometry(const or_config* cfg, float* out5);
/* single primitives of the restatement (float), pinned against the
 * reference's own _yooji_cuda_math.h: 6x6 Cholesky factor and solve, the
 * bilinear vertex / normal map lookups (normalise = 1: the normal form),
 * projection, back-projection, transform (rotate_only = 1: rotation part),
 * position in voxel / world coordinates */
void or_prim_cholesky6(const float* A, float* L);
int or_prim_chol_solve6(const float* L, const float* b, float* x);
int or_prim_bilinear3(float xf, float yf, int w, int h, const float* map3, int normalise, float* out3);
void or_prim_project(const float* p3, const float* K, float* uv);
void or_prim_back_project(float u, float v, const float* K, float d, float* p3);
void or_prim_transform(const float* p3, const float* T, int rotate_only, float* out3);
int or_prim_pos_in_voxel(const float* p3, const float* origin, const int* dim, float vox_inv, float* out3);
void or_prim_pos_in_world(const float* v, const float* origin, float vox_inv, float* out3);
/* one pixel's ICP term at a pyramid level (no input-normal test): A (6) and b;
 * returns 0 where the pixel gives no term */
int or_prim_icp_term(int x, int y, int w, int h, const float* K, const float* depth, const float* mvtx,
                     const float* mnrm, const float* T21, float th_icp, float* A6, float* b);
/* reference integration: sub-cube activation then TSDF update */
void or_integrate(or_volume* v, const float* depth, const float* T_gc,
                  const float* T_cg);
/* reference raycast of one level.  cam_cen / light: float3.
 * outputs: depth W*H, vertex/normal AoS float3, shaded image uint8. */
/* colour: g_ctvc with colour (registered colour image, planar R, G, B of the
 * depth image's size), the colour volume (three x-fastest planes), and the
 * ray-cast with the colour image (planar) */
void or_integrate_color(or_volume* v, const float* depth, const uint8_t* rgb, const float* T_gc,
                        const float* T_cg);
void or_volume_get_color(or_volume* v, uint8_t* rgb);
void or_volume_set_color(or_volume* v, const uint8_t* rgb);
void or_raycast_color(const or_volume* v, int level, const float* T_gc, const float* T_cg,
                      const float* cam_cen, const float* light, float* depth, float* vtx3, float* nrm3,
                      uint8_t* img, uint8_t* rgb);
/* depth map seen from a second camera (z-buffer, smaller depth wins) */
void or_warp_depth(const float* depth, int wd, int hd, const float* Kd, const float* T, const float* Kr, int wr,
                   int hr, float* out);
/* marching-tetrahedra mesh of the zero level set (9 floats / 9 colour bytes
 * per triangle, at most capacity written); returns the triangle count */
uint64_t or_extract_mesh(const or_volume* v, float* xyz, uint8_t* rgb, uint64_t capacity);
void or_raycast(const or_volume* v, int level, const float* T_gc,
                const float* T_cg, const float* cam_cen, const float* light,
                float* depth, float* vtx3, float* nrm3, uint8_t* img);

/* full per-frame pipeline (so_Scan_Object hot path) */
typedef struct or_session or_session;
or_session* or_session_create(const or_config* cfg);
void or_session_destroy(or_session* s);
/* returns 1 when the frame was tracked and fused, 0 on tracking failure */
int or_session_frame(or_session* s, const uint16_t* depth_mm);
void or_session_pose(const or_session* s, float* T_gc);
/* FP64 pipeline (precision-study ground truth) */
or_session* or_session_create_f64(const or_config* cfg);
void or_session_pose_f64(const or_session* s, double* T_gc);
or_volume* or_session_volume(or_session* s);
/* level l maps of the session (after the frame): model depth/vertex/normal,
 * input filtered depth */
void or_session_maps(const or_session* s, int level, float* mdepth, float* mvtx3,
                     float* mnrm3, float* in_depth);

#ifdef __cplusplus
}
#endif
