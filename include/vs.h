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
 *     volume is every word 0x00007FFF (TSDF 1, weight 0).
 *   dim, origin: 3 ints / 3 floats; K: host fx, fy, cx, cy; depth ww x hh
 *   float metres and the 4x4 poses on the device, as vs_integrate_depth. */
int vs_integrate_depth_noalloc(uint32_t* volume_dev, const int* dim, const float* origin,
                               float voxel_size, float mu, float max_w, const float* map_depth_dev,
                               int ww, int hh, const float* K, const float* T_gc_dev,
                               const float* T_cg_dev, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* VS_H */
