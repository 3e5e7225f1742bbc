/*
 * vs.h -- C ABI of the GB300-native reconstruction core for vcl-volume-scanner.
 *
 * The reference exposes its per-frame path as four C++ classes with global
 * __constant__ state (paths relative to VCL_Volume_Scanner/):
 *   LGKvImageProcessor   STAC/Engine/GPU/_yooji_cuda_img_proc.h:1-29
 *   LGKvPoseTracker      STAC/Engine/GPU/_yooji_cuda_pose_tracker.h:1-42
 *   LGKvVolumeIntegrator STAC/Engine/GPU/_yooji_cuda_volume_integrator.h:1-52
 *   LGKvRendererTSDF     STAC/Engine/GPU/_yooji_cuda_tsdf_renderer.h:1-95
 * plus the device containers GKvObjectCube / GKvTrackingState / GKvRgbdFrame
 * (STAC/Object/GPU/) and the per-frame caller so_Scan_Object
 * (STAC/Engine/CPU/z_yooji_object_scanner.cpp:472-629).
 *
 * Here the same surface is a plain C ABI over an opaque session: every
 * ip_Initialize_Parameters call becomes one vs_config given to
 * vs_session_create, the session owns what the reference kept in globals and
 * in its device containers, and any number of sessions can live in one
 * process.  Pointers are plain device (_dev) or host (_host) pointers; poses
 * are row-major 4x4 float, T_gc maps global to camera coordinates exactly as
 * in the reference.  Functions return VS_OK (0) or a negative VS_ERR_* code;
 * vs_last_error() describes the last failure of the calling thread.
 *
 * No function falls back to a CPU implementation: without a usable CUDA
 * device every compute entry point returns VS_ERR_CUDA.
 */
#ifndef VS_H
#define VS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VS_OK 0
#define VS_ERR_ARG (-1)     /* bad argument or size                          */
#define VS_ERR_CUDA (-2)    /* CUDA runtime failure / no device              */
#define VS_ERR_STATE (-3)   /* call out of order                             */
#define VS_ERR_MEMORY (-4)  /* device allocation failed                      */
#define VS_ERR_BUSY (-5)    /* queue full / budget exhausted; retry later     */

#define VS_MAX_BATCH 64     /* sessions advanced by one batched step          */

/* TSDF storage of the volume (the reference stores float + uchar weight) */
#define VS_TSDF_INT16 0     /* int16 q = rint(tsdf*32767), uint16 weight      */
#define VS_TSDF_FP16 1      /* IEEE half, uint16 weight                       */
#define VS_TSDF_FP32 2      /* float, uint32 weight (8 bytes per voxel)       */

/* combination of the ICP normal-equation sums across pixels */
#define VS_REDUCE_FP32 0    /* plain float sums                              */
#define VS_REDUCE_KAHAN 1   /* compensated (two-sum) float sums               */
#define VS_REDUCE_FP64 2    /* double sums of the float per-pixel terms       */

typedef struct {
  /* camera: level-0 depth size and intrinsics (ip_Initialize_Parameters of
   * the tracker, integrator and renderer) */
  int width, height;
  float fx, fy, cx, cy;
  int levels;               /* pyramid levels, 1..3 (reference: 3)           */
  /* volume (GKvObjectCube::create): voxels per axis, multiples of 8 */
  int dim[3];
  float origin[3];          /* world position of voxel corner (-0.5,-0.5,-0.5) */
  float voxel_size;         /* metres                                        */
  float mu;                 /* truncation distance (m)                        */
  float max_w;              /* weight cap (reference KV_MAX_W_TSDF = 100)    */
  /* tracking */
  float th_icp;             /* squared point distance threshold (m^2)        */
  float cos_normal;         /* input/model normal agreement, cos(angle);
                               <= -2 disables the test (the reference has none) */
  int icp_iters[3];         /* iterations at levels 0, 1, 2                   */
  int reduce_mode;          /* VS_REDUCE_*                                    */
  int tsdf_type;            /* VS_TSDF_*                                      */
  float depth_scale;        /* uint16 depth units -> metres (0.001)          */
  int color;                /* 1: keep an RGB volume, integrate and ray-cast
                               colour (the colour image is registered to the
                               depth image: same size and intrinsics)       */
} vs_config;

typedef struct vs_session vs_session;

/* fills reference defaults for a width x height camera */
void vs_config_default(vs_config* cfg, int width, int height);
const char* vs_last_error(void);
/* number of CUDA devices usable by this library (0 on a host without GPU) */
int vs_device_count(void);

/* session lifecycle: GKvObjectCube::create + GKvTrackingState::create +
 * GKvRgbdFrame::create + the four ip_Initialize_Parameters calls
 * (z_yooji_object_scanner.cpp:343-425).  Allocates every device buffer of the
 * session; the TSDF starts at 1 with zero weight, the pose at identity. */
int vs_session_create(const vs_config* cfg, vs_session** out);
int vs_session_destroy(vs_session* s);
int vs_session_reset(vs_session* s);
/* device bytes held by one session with this configuration */
size_t vs_session_bytes(const vs_config* cfg);

/* ---- reference-shaped stage entry points -------------------------------- */

/* LGKvImageProcessor::bfd_Bilateral_Filter_Depth
 * (_yooji_cuda_img_proc.h:12-15, z_yooji_cuda_img_proc.cu:394-417): host
 * float depth (m) in, filtered depth written to device memory. */
int vs_bilateral_filter_depth(vs_session* s, float* map_depth_filtered_dev,
                              const float* map_depth_host, int ww, int hh);
/* LGKvImageProcessor::bfd_Bilateral_Filter_Depth_Host (:17-20, .cu:420-442) */
int vs_bilateral_filter_depth_host(vs_session* s, float* map_depth_filtered_host,
                                   const float* map_depth_host, int ww, int hh);

/* LGKvPoseTracker::tp_Track_Pose (_yooji_cuda_pose_tracker.h:17-19,
 * z_yooji_cuda_pose_tracker.cu:790-1042): frame-to-model ICP of the
 * session's current input pyramid against its model maps.  init_T01_dev: an
 * optional device 4x4 initial increment (then only level 0 runs).  On success
 * the session pose becomes T_12 * T_gc; *tracked = 1 (0 when the 6x6 system
 * is singular, and the pose is left unchanged). */
int vs_track_pose(vs_session* s, const float* init_T01_dev, int* tracked);

/* LGKvVolumeIntegrator::cdtocc_Convert_Depth_to_TSDF_on_Cube_with_Color,
 * depth part (_yooji_cuda_volume_integrator.h:36-43,
 * z_yooji_cuda_volume_integrator.cu:976-1031): activate the 8^3 sub-cubes
 * near the depth rays, then update their voxels.  depth_dev: ww x hh float
 * metres; T_gc_dev / T_cg_dev: device 4x4. */
int vs_integrate_depth(vs_session* s, const float* map_depth_dev, int ww, int hh,
                       const float* T_gc_dev, const float* T_cg_dev);

/* LGKvRendererTSDF::rmi_Render_Maps_for_ICP (_yooji_cuda_tsdf_renderer.h:16-30,
 * z_yooji_cuda_tsdf_renderer.cu:1642-1700): ray-cast the session volume at
 * pyramid level `level` (size ww x hh).  Outputs in the reference layout:
 * depth float, vertex / normal float3 AoS in the camera frame (-100 where
 * invalid), shaded normal image uint8.  cam_cen / light: host float[3]. */
int vs_render_maps(vs_session* s, int ww, int hh, const float* T_gc_dev,
                   const float* T_cg_dev, const float* cam_cen, const float* light,
                   int level, float* map_depth_dev, float* map_vertex_dev,
                   float* map_normals_dev, uint8_t* img_normals_dev);

/* ---- colour (sessions created with cfg.color = 1) ------------------------
 * The colour image is planar uint8 R, G, B, each plane width x height, as the
 * reference's img_color (plane stride ww*hh), registered to the depth image
 * (the reference's flag_on_rgb path).  The colour volume holds 8-bit R, G, B
 * per voxel, initialised to 0. */

/* LGKvVolumeIntegrator::cdtocc_Convert_Depth_to_TSDF_on_Cube_with_Color
 * (z_yooji_cuda_volume_integrator.cu:265-455): the depth update of
 * vs_integrate_depth plus, for every updated voxel, the colour sampled
 * bilinearly at the voxel's projection (d_gii_Get_Interpolated_Intensity,
 * _yooji_cuda_math.h:305-332) and blended as (w * old + sample) / (w + 1),
 * truncated to 8 bits.  A sample the reference cannot interpolate (outside
 * the image, or a texel <= 0) leaves the voxel's colour unchanged (the
 * reference would blend an uninitialised value). */
int vs_integrate_depth_color(vs_session* s, const float* map_depth_dev, const uint8_t* img_color_dev, int ww,
                             int hh, const float* T_gc_dev, const float* T_cg_dev);
/* rmi_Render_Maps_for_ICP with its img_color output
 * (z_yooji_cuda_tsdf_renderer.cu:1165-1174): as vs_render_maps plus the
 * trilinear colour at every hit (d_grvi_Get_RGB_Value_Interpolated,
 * :232-284), planar uint8, 0 where there is no hit or a neighbour has weight
 * 0.  img_color_dev: 3 * ww * hh bytes. */
int vs_render_maps_color(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                         const float* cam_cen, const float* light, int level, float* map_depth_dev,
                         float* map_vertex_dev, float* map_normals_dev, uint8_t* img_normals_dev,
                         uint8_t* img_color_dev);
/* the colour frame the next vs_scan_frame / batch step integrates (planar,
 * host or device pointer) */
int vs_set_color_frame(vs_session* s, const uint8_t* img_color, int is_host);
/* the colour volume in the reference layout: three planes (R, G, B) of
 * dim[0]*dim[1]*dim[2] bytes, x fastest (cube_color) */
int vs_get_color_volume(vs_session* s, uint8_t* rgb_host);
int vs_set_color_volume(vs_session* s, const uint8_t* rgb_host);
/* the colour image of the last frame's ray-cast at a level, planar */
int vs_get_color_map(vs_session* s, int level, uint8_t* rgb_host);

/* ---- scene rendering and valid-volume carving --------------------------------
 * Render variants of LGKvRendererTSDF (z_yooji_cuda_tsdf_renderer.cu).  All
 * write external device outputs only (the session's model maps are not
 * touched) in the layout of vs_render_maps; normals stay in the global frame
 * and the shaded image uses them with `light` as given.  Where nothing is
 * hit: depth 0, vertex and normal -100, image 0. */

/* rmis_Render_Maps_for_Scene with a vertex map (:1761-1814, kernel
 * :1338-1446), the scanner's per-frame ray-cast for scene input
 * (z_yooji_object_scanner.cpp:1318): level-0 size and intrinsics; every ray
 * starts at the camera centre and ends 2 r_cube away, with no test against
 * the cube's view cone (d_crtcs_Cast_Ray_on_TSDF_Cube_for_Scene, :908-1066);
 * vertex in the camera frame; colour (optional, colour sessions) of the
 * nearest voxel with weight > 0 (d_grvu, :155-229), 0 otherwise.  The
 * reference writes the green channel into the red plane there, marked as
 * temporary; the true red is written here. */
int vs_render_maps_scene(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                         const float* cam_cen, const float* light, float* map_depth_dev, float* map_vertex_dev,
                         float* map_normals_dev, uint8_t* img_normals_dev, uint8_t* img_color_dev);
/* rmis_Render_Maps_for_Scene without a vertex map (:1817-1862, kernel
 * :1448-1548), the viewer's render (VCL_Volume_Scanner_View.cpp:1921): the
 * scene ray-cast with the trilinear colour of vs_render_maps_color. */
int vs_render_view_scene(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                         const float* cam_cen, const float* light, float* map_depth_dev, float* map_normals_dev,
                         uint8_t* img_normals_dev, uint8_t* img_color_dev);
/* rmi_Render_Maps_for_ICP without a vertex map (:1703-1757, kernel
 * :1211-1336): the object ray-cast of vs_render_maps at `level`, normals in
 * the global frame, trilinear colour, and colour 255 in every channel where
 * nothing is hit. */
int vs_render_view(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                   const float* cam_cen, const float* light, int level, float* map_depth_dev,
                   float* map_normals_dev, uint8_t* img_normals_dev, uint8_t* img_color_dev);

/* LGKvVolumeIntegrator::uvv_Update_Valid_Volume
 * (z_yooji_cuda_volume_integrator.cu:1035-1060, kernel :718-799): carve the
 * volume with a valid-voxel mask (e.g. a visual hull), one byte per voxel
 * (0 = outside), dim[0]*dim[1]*dim[2] bytes x fastest; a device pointer must
 * be 8-byte aligned.  Each 8^3 sub-cube that the last integration activated
 * (the reference's cube_valid flags) and that holds no valid voxel is reset
 * to the empty state (TSDF 1, weight 0, colour 0) and loses its flag, so a
 * second carving before the next integration leaves it alone.  Sub-cubes
 * with at least one valid voxel are kept whole.  *carved (optional): the
 * number of sub-cubes reset. */
int vs_update_valid_volume(vs_session* s, const uint8_t* vol_valid, int is_host, uint32_t* carved);

/* ---- depth -> colour camera registration ------------------------------------
 * z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates
 * (z_yooji_object_scanner.cpp:2429-2476): the depth map as seen from a second
 * (colour) camera, for rigs whose colour camera is not the depth camera.  Each
 * depth pixel with depth d > 0 is back-projected with K_d, moved by the 4x4
 * depth-to-colour transform T_rgb_wrt_d (row-major, metres), projected with
 * K_rgb and rounded (half away from zero); a colour pixel keeps the smallest
 * depth landing on it, 0 where none does.  K_*: host {fx, fy, cx, cy};
 * T_rgb_wrt_d: host float[16]; buffers on the device; asynchronous on stream.
 * The result (colour-camera depth, registered to the colour image) can feed
 * a session configured with the colour camera's intrinsics. */
int vs_warp_depth_to_color(const float* depth_dev, int w_d, int h_d, const float* K_d, const float* T_rgb_wrt_d,
                           const float* K_rgb, int w_rgb, int h_rgb, float* depth_rgb_dev, void* stream);
/* the same on uint16 depth units (depth_scale: units -> metres), giving a
 * uint16 frame for vs_scan_frame */
int vs_warp_depth_mm_to_color(const uint16_t* depth_mm_dev, int w_d, int h_d, float depth_scale, const float* K_d,
                              const float* T_rgb_wrt_d, const float* K_rgb, int w_rgb, int h_rgb,
                              uint16_t* depth_mm_rgb_dev, void* stream);

/* ---- per-frame hot path (so_Scan_Object) -------------------------------- */

/* One frame on device input, asynchronous on `stream` (cudaStream_t, NULL =
 * the session's stream): uint16 ingest + bilateral + pyramid + input
 * vertex/normal maps, ICP (skipped on the first frame), TSDF integration of
 * the raw depth, ray-cast of every level.  Runs as one CUDA graph; a
 * tracking failure skips integration and ray-casting on the device. */
int vs_scan_frame(vs_session* s, const uint16_t* depth_mm_dev, void* stream);
/* Same with host input and output: copies the frame in, runs it, copies the
 * pose and the tracking flag out and waits.  T_gc_out may be NULL. */
int vs_scan_frame_host(vs_session* s, const uint16_t* depth_mm_host, float* T_gc_out,
                       int* tracked);
/* waits for the session's work */
int vs_session_sync(vs_session* s);

/* stages of vs_scan_frame, one call each (device input, session stream) */
int vs_stage_filter(vs_session* s, const uint16_t* depth_mm_dev);
int vs_stage_track(vs_session* s);
int vs_stage_integrate(vs_session* s);
int vs_stage_raycast(vs_session* s);

/* ---- state access ------------------------------------------------------- */

/* pose: T_gc (float, as used by the kernels) and its FP64 master copy; any
 * output may be NULL.  info (may be NULL): [0] tracked flag of the last frame,
 * [1] ICP iterations run, [2] valid correspondences of the last iteration,
 * [3] frames processed. */
int vs_get_pose(vs_session* s, float* T_gc, double* T_gc_f64, int* info);
int vs_set_pose(vs_session* s, const double* T_gc_f64);
/* the normal equations of the last ICP iteration run (tp_Track_Pose's ATA /
 * ATb, z_yooji_cuda_pose_tracker.cu:937-943): sums29 = the 21 entries of
 * the upper triangle of ATA row by row, the 6 of ATb, the correspondence
 * count and the sum of b^2, as summed (FP64); x6 = the increment solved from
 * them (twist [w; v], rounded to float).  Either pointer may be NULL. */
int vs_get_icp_system(vs_session* s, double* sums29, float* x6);
/* Diagnostic of the ray-cast's free-space skipping (no reference
 * counterpart): per sub-cube, x fastest (z * nb_x * nb_y + y * nb_x + x, nb =
 * dim / 8), band = 1 where some voxel has weight > 0 and a TSDF value other
 * than 1 (the only sub-cubes whose samples can change the march), and dist =
 * the Chebyshev distance in sub-cubes to the nearest band sub-cube as the
 * last ray-cast computed it, saturating at 8.  Either pointer may be NULL. */
int vs_get_band(vs_session* s, uint8_t* band, uint8_t* dist);
/* GKvObjectCube::to_host / from_host (_yooji_cuda_object_cube.hpp:6-85): the
 * volume in the reference's x-fastest layout (z*W*H + y*W + x), TSDF as float
 * and weight as uint16; either pointer may be NULL. */
int vs_get_volume(vs_session* s, float* tsdf_host, uint16_t* weight_host);
int vs_set_volume(vs_session* s, const float* tsdf_host, const uint16_t* weight_host);
/* sub-cubes activated by the last integration: count, and optionally their
 * indices (z*nby*nbx + y*nbx + x), unsorted */
int vs_get_active_bricks(vs_session* s, uint32_t* count, uint32_t* bricks_host,
                         uint32_t capacity);
/* level maps in the reference layout (host outputs, any may be NULL): model
 * depth / vertex float3 / normal float3 / shaded image from the last
 * ray-cast, filtered input depth, input vertex / normal float3 */
int vs_get_maps(vs_session* s, int level, float* model_depth, float* model_vertex3,
                float* model_normal3, uint8_t* model_img, float* input_depth,
                float* input_vertex3, float* input_normal3);
/* ---- snapshot / resume ---------------------------------------------------
 * The reference saves scans through a closed KAISION writer (.vcl,
 * z_yooji_object_scanner.cpp:2732-2745) and moves the cube with
 * to_host / from_host (_yooji_cuda_object_cube.hpp:6-85).  The snapshot here
 * is this library's own file: "VSSNAP01", the vs_config, the FP64 pose and
 * frame count, then only the sub-cubes holding data (index list, their TSDF
 * words, and their colour words when the session keeps colour).  Loading
 * creates a session, restores volume, occupancy and pose, and ray-casts the
 * model maps, so the next frame continues exactly as the saved session
 * would. */
int vs_session_save(vs_session* s, const char* path);
/* the configuration a session was created with (e.g. after vs_session_load) */
int vs_session_config(vs_session* s, vs_config* out);
int vs_session_load(const char* path, vs_session** out);

/* ---- surface extraction ---------------------------------------------------
 * The zero level set of the TSDF as a triangle soup, by marching tetrahedra:
 * every cell of 2x2x2 voxels whose eight corners have weight > 0 is split
 * into six tetrahedra around its (0,0,0)-(1,1,1) diagonal; a vertex is the
 * linear zero crossing on a tetrahedron edge, in world coordinates, and each
 * triangle faces positive TSDF (free space).  xyz: 9 floats per triangle;
 * rgb (may be NULL; sessions with colour): 9 bytes per triangle, the edge's
 * two voxel colours mixed with the same weights and rounded.  Writes at most
 * capacity triangles and returns the total in *n_triangles (call again with a
 * larger buffer when it exceeds capacity).  Host buffers; the order of the
 * triangles is not fixed. */
int vs_extract_mesh(vs_session* s, float* xyz_host, uint8_t* rgb_host, uint64_t capacity, uint64_t* n_triangles);
/* the same mesh written as a binary little-endian PLY (vertex x y z [r g b],
 * face vertex_indices) */
int vs_save_mesh_ply(vs_session* s, const char* path);

/* ---- instrumentation (the reference prints per-stage stopwatch times,
 * z_yooji_object_scanner.cpp:489-604) ------------------------------------- */

/* records CUDA events between the stages of the per-frame graph (the graph is
 * re-captured on the next frame) */
int vs_set_stage_timing(vs_session* s, int enable);
/* device milliseconds of the last frame: filter (ingest, bilateral, pyramid,
 * input maps), track, integrate, ray-cast; waits for the frame */
int vs_get_stage_times(vs_session* s, float* ms4);
/* counters of the last frame: [0] active sub-cubes, [1] voxels updated,
 * [2] ICP iterations run, [3] correspondences of the last iteration */
int vs_get_frame_stats(vs_session* s, uint32_t* stats4);
/* kernel launches one vs_scan_frame performs for this configuration (-1 if
 * the configuration is invalid) */
int vs_kernels_per_frame(const vs_config* cfg);

/* level-0 depth in metres as converted from the last uint16 input frame (the
 * integration input, musf_Matrix_Ushort_to_Float with the depth scale,
 * z_yooji_frame_capture.cpp:597) */
int vs_get_input_raw(vs_session* s, float* depth_m_host);
/* raw device pointers of the session buffers (for zero-copy callers):
 * which = 0 raw depth (float m, level 0), 1..3 filtered depth levels 0..2 */
int vs_get_device_buffer(vs_session* s, int which, void** ptr);

/* ---- allocation-free integration ----------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (code running inside a host framework's own device-memory pool or arena,
 * real-time loops that cannot afford an allocation's driver lock, processes
 * that size all device memory up front): the same TSDF update as
 * vs_integrate_depth, into a volume buffer the caller owns, with no device
 * allocation by this library.  Scratch is a fixed ~2 MiB __device__ array
 * inside the library (held by every GPU that loads it until exit), which caps
 * the volume at 262,144 sub-cubes (512^3 voxels); larger volumes return
 * VS_ERR_ARG.  The first call on a device looks up the scratch address
 * (cudaGetSymbolAddress) and should come before any stream capture.  Calls
 * share the scratch: calls on one stream run in order, calls that overlap on
 * the GPU race.  Asynchronous on `stream` (cudaStream_t, NULL = default).
 *   volume_dev: (dim/8)^3 sub-cubes of 512 uint32 words each, sub-cubes x
 *     fastest then y then z, voxels x fastest inside a sub-cube; a word is
 *     (uint16 weight << 16) | uint16(int16 q) with TSDF = q / 32767.  A new
 *     volume is every word 0x00007FFF (TSDF 1, weight 0).  It must be
 *     16-byte aligned (sub-cubes move as 16-byte vectors); another address
 *     returns VS_ERR_ARG before anything runs.
 *   dim, origin: 3 ints / 3 floats; K: host fx, fy, cx, cy; depth ww x hh
 *   float metres and the 4x4 poses on the device, as vs_integrate_depth. */
int vs_integrate_depth_noalloc(uint32_t* volume_dev, const int* dim, const float* origin,
                               float voxel_size, float mu, float max_w, const float* map_depth_dev,
                               int ww, int hh, const float* K, const float* T_gc_dev,
                               const float* T_cg_dev, void* stream);

/* ---- batched frames ------------------------------------------------------
 * A batch runner advances several sessions by one frame each with ONE launch
 * per stage: every per-frame kernel is persistent over the work items of all
 * sessions of a device-resident table, so the runner captures one CUDA graph
 * and replays it for any set of sessions (sizes, volumes and levels may
 * differ; reduce_mode and tsdf_type must agree).  Each session's items and
 * their summation order are those it has alone, so a session's poses,
 * volume and maps are identical whether it runs alone (vs_scan_frame) or in
 * any batch.  The reference has one session per process and no batching;
 * the step replaces n calls of so_Scan_Object's per-frame body
 * (z_yooji_object_scanner.cpp:501-597).
 *
 * A session must not be used by two runners, or by its own entry points, while
 * a step that includes it is in flight; vs_batch_sync() ends all of them. */
typedef struct vs_batch vs_batch;

int vs_batch_create(vs_batch** out);
int vs_batch_destroy(vs_batch* b);
/* one frame for each of n (1..VS_MAX_BATCH) distinct sessions.
 * depth_mm_dev[i]: device uint16 frame of session i, or NULL (or a NULL
 * array) when the frame is already in the session's input buffer.  Enqueued
 * on `stream` (NULL: the runner's own stream); returns without waiting.  The
 * step's first kernel reads each frame in place (no copy), so a frame must
 * not change until the step is done (work enqueued after it on the same
 * stream is ordered after it). */
int vs_batch_step(vs_batch* b, vs_session* const* sessions, int n, const uint16_t* const* depth_mm_dev,
                  void* stream);
/* host frames in, poses out (T_gc_out: n x 16 floats, tracked_out: n ints,
 * either may be NULL); returns when the step has finished.  A frame in pinned
 * host memory (cudaHostAlloc / cudaHostRegister) is read in place by the
 * step's first kernel over the host link; a pageable one is copied first. */
int vs_batch_step_host(vs_batch* b, vs_session* const* sessions, int n, const uint16_t* const* depth_mm_host,
                       float* T_gc_out, int* tracked_out);
int vs_batch_sync(vs_batch* b);
/* stage events inside the batch graph; ms[4] as vs_get_stage_times, for the
 * last finished step */
int vs_batch_set_stage_timing(vs_batch* b, int enable);
int vs_batch_get_stage_times(vs_batch* b, float* ms);
/* kernels one step launches (the same for every batch size) */
int vs_batch_kernels_per_step(vs_batch* b);

/* Launch shape of a runner's steps: a warp's 32 rays form a
 * (1 << ray_tile_log2) x (32 >> ray_tile_log2) pixel tile, and the ray-cast
 * grid (march and shading in one launch; colour sessions: the march grid,
 * then the shading grid) holds that many 128-thread blocks per SM (0: as
 * many as fit);
 * the bilateral filter and the sub-cube activation work on 32 x
 * bilateral_rows pixel tiles (4, 8 or 16; 0: 8); the integration's update
 * grid holds integrate_blocks_per_sm 256-thread blocks per SM (0: as many as
 * fit).  The shape changes no result, only time. */
typedef struct {
  int ray_tile_log2;        /* 0..5, default 3 (8 x 4 rays)                  */
  int march_blocks_per_sm;
  int shade_blocks_per_sm;
  int bilateral_rows;
  int integrate_blocks_per_sm;
} vs_launch_shape;

int vs_batch_get_launch_shape(vs_batch* b, vs_launch_shape* out);
int vs_batch_set_launch_shape(vs_batch* b, const vs_launch_shape* in);
/* Autotuner: times three stages of these sessions (their current frames,
 * volumes and poses; no state changes) under their candidate shapes, reps
 * launches each, and keeps the fastest of each for the runner's later steps:
 * the ray-cast (ray tile and march grid), the filter (tile rows) and the
 * integration (update grid, timed as dry runs that store no voxel); for the
 * last two a shape other than the default must be more than 3 % faster.
 * best and best_ms (ms per ray-cast stage) may be NULL. */
int vs_batch_autotune(vs_batch* b, vs_session* const* sessions, int n, int reps, vs_launch_shape* best,
                      float* best_ms);

/* ---- serving ---------------------------------------------------------------
 * A server takes frames from many sessions as they arrive and runs them with
 * continuous batching: a worker thread forms each step from the sessions that
 * have a frame waiting (one frame per session per step, oldest first, round
 * robin) and launches it through one of `lanes` batch runners, each on its
 * own stream, so several steps run on the GPU at once (by default three, one
 * step per lane); a completion thread per lane timestamps each frame's
 * result.  Every session's volume, pose and maps stay on the device
 * between frames.  Sessions are admitted while the resident set fits the HBM
 * budget (vs_session_bytes of each) and a resident slot is free; a session
 * that does not fit yet waits, queues its frames, and is admitted when closed
 * sessions free memory.  Results equal those of the session run alone. */
typedef struct vs_server vs_server;

typedef struct {
  size_t hbm_budget;        /* device bytes resident sessions may hold (0: 150 GB) */
  int max_resident;         /* resident sessions, 1..VS_MAX_BATCH (0: VS_MAX_BATCH) */
  int max_batch;            /* sessions per step, 1..VS_MAX_BATCH (0: VS_MAX_BATCH) */
  int queue_depth;          /* frames buffered per session, 1..256 (0: 8)    */
  int pipeline;             /* steps in flight per lane, 1..2 (0: 1)         */
  int lanes;                /* steps run at the same time, each on its own
                               stream and batch runner, 1..4 (0: 3); with
                               more than one, a session joins a step only
                               when none of its frames is in flight        */
} vs_server_config;

typedef struct {
  int session;              /* id from vs_server_open                         */
  int frame;                /* 0-based index of the frame in its session      */
  int tracked;
  int batch;                /* sessions in the step that ran the frame        */
  float T_gc[16];
  double t_submit;          /* seconds, vs_server_clock() time base           */
  double t_done;            /* result on the host                             */
  double latency_ms;
} vs_result;

typedef struct {
  uint64_t steps, frames;
  double mean_batch;
  int max_batch_seen;
  int resident, waiting, closed;
  size_t bytes_resident, bytes_budget;
} vs_server_stats;

#define VS_SESSION_WAITING 0
#define VS_SESSION_RESIDENT 1
#define VS_SESSION_CLOSED 2

void vs_server_config_default(vs_server_config* c);
int vs_server_create(const vs_server_config* c, vs_server** out);
/* finishes every queued frame, then frees all sessions */
int vs_server_destroy(vs_server* s);
/* VS_ERR_MEMORY when the session alone exceeds the budget */
int vs_server_open(vs_server* s, const vs_config* cfg, int* id);
int vs_server_state(vs_server* s, int id, int* state);
/* copies the frame (width x height uint16) into the session's queue;
 * VS_ERR_BUSY when queue_depth frames are already waiting */
int vs_server_submit(vs_server* s, int id, const uint16_t* depth_mm_host);
/* the session leaves after its queued frames; its memory admits waiters */
int vs_server_close(vs_server* s, int id);
/* up to max results, waiting at most timeout_ms for the first; returns the
 * count (>= 0) or a VS_ERR_* code */
int vs_server_poll(vs_server* s, vs_result* out, int max, int timeout_ms);
/* waits until every submitted frame has finished */
int vs_server_drain(vs_server* s);
/* the resident session behind an id (state access; call after a drain) */
int vs_server_get_session(vs_server* s, int id, vs_session** out);
int vs_server_get_stats(vs_server* s, vs_server_stats* st);
/* seconds on the monotonic clock of t_submit / t_done */
double vs_server_clock(void);

#ifdef __cplusplus
}
#endif
#endif /* VS_H */
