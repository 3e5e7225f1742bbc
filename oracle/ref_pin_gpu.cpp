// Harness around the reference's own GPU sources, compiled as host C++ (TEST
// INFRASTRUCTURE ONLY; nothing here runs on a GPU).
//
// oracle/build_oracle.py rewrites the kernel-launch syntax of
// STAC/Engine/GPU/z_yooji_cuda_tsdf_renderer.cu and
// z_yooji_cuda_volume_integrator.cu (and of STAC/Util/z_yooji_cuda_math.cu,
// which fills device buffers) into calls of the host launch loop of
// ref_shim/gpu/ref_gpu_shim.h, writes the result under oracle/_ref/gen/ and
// compiles it with this file once per source (the two files define the same
// __constant__ names, so each gets its own library):
//   oracle/_ref/libref_pin_render.so  (REF_PIN_RENDER)
//   oracle/_ref/libref_pin_integ.so   (REF_PIN_INTEG)
//   oracle/_ref/libref_pin_track.so   (REF_PIN_TRACK: the per-pixel ICP term
//     d_cssfp_Compute_Single_Summand_with_Forward_Params of
//     z_yooji_cuda_pose_tracker.cu, and the whole of tp_Track_Pose, whose
//     block reductions use shared memory and barriers and so run as
//     cooperative block threads, vs_block_threads of the shim)
//   oracle/_ref/libref_pin_imgproc.so (REF_PIN_IMGPROC: the bilateral filter
//     of z_yooji_cuda_img_proc.cu through LGKvImageProcessor, its texture
//     reference given by the texture stand-in of ref_gpu_shim.h)
// The reference's own host code then runs unchanged on host memory: the cube
// class, ip_Initialize_Parameters, rmi_Render_Maps_for_ICP and
// cdtocc_Convert_Depth_to_TSDF_on_Cube_with_Color with their kernels
// (g_rmi_Render_Maps_for_ICP with d_crtc_Cast_Ray_on_TSDF_Cube_NEW, d_gtvu,
// d_gtvi, d_csnt; g_fvsc_Find_Visible_Sub_Cubes, g_ctvc_...).  The volume is
// the reference's: float TSDF, uchar weights, x fastest.
#include "ref_gpu_shim.h"

#if defined(REF_PIN_RENDER)
#include "renderer.cu.cpp"

extern "C" int ref_render_icp(int W, int H, const float* K0, int level, const int* dim, const float* origin,
                              const float* center, float vox, float mu, float max_w, const float* tsdf,
                              const uint8_t* w, const float* T_gc, const float* T_cg, const float* cam,
                              const float* light, float* depth, float* vtx3, float* nrm3, uint8_t* img) {
  GKvObjectCubeFloat cube;
  if (!cube.create(Vector3i(dim[0], dim[1], dim[2]), Vector3f(origin[0], origin[1], origin[2]),
                   Vector3f(center[0], center[1], center[2]), vox, false))
    return 0;
  const size_t n = (size_t)dim[0] * dim[1] * dim[2];
  std::memcpy(cube.vp_tsdf(), tsdf, n * sizeof(float));
  std::memcpy(cube.vp_w(), w, n);
  LGKvRendererTSDF r;
  r.ip_Initialize_Parameters(&cube, W, H, K0[0], K0[1], K0[2], K0[3], mu, max_w);
  int lw = W, lh = H;
  for (int l = 0; l < level; l++) lw /= 2, lh /= 2;
  r.rmi_Render_Maps_for_ICP(&cube, lw, lh, T_gc, T_cg, Vector3f(cam[0], cam[1], cam[2]),
                            Vector3f(light[0], light[1], light[2]), level, depth, vtx3, nrm3, img, nullptr);
  return 1;
}

// the other renders of a colour cube: variant 0 rmis_Render_Maps_for_Scene
// with a vertex map, 1 the same without one, 2 rmi_Render_Maps_for_ICP
// without a vertex map at the given level; rgb_img: three planes of the image
extern "C" int ref_render_variant(int variant, int W, int H, const float* K0, int level, const int* dim,
                                  const float* origin, const float* center, float vox, float mu, float max_w,
                                  const float* tsdf, const uint8_t* w, const uint8_t* rgb, const float* T_gc,
                                  const float* T_cg, const float* cam, const float* light, float* depth, float* vtx3,
                                  float* nrm3, uint8_t* img, uint8_t* rgb_img) {
  GKvObjectCubeFloat cube;
  if (!cube.create(Vector3i(dim[0], dim[1], dim[2]), Vector3f(origin[0], origin[1], origin[2]),
                   Vector3f(center[0], center[1], center[2]), vox, true))
    return 0;
  const size_t n = (size_t)dim[0] * dim[1] * dim[2];
  std::memcpy(cube.vp_tsdf(), tsdf, n * sizeof(float));
  std::memcpy(cube.vp_w(), w, n);
  std::memcpy(cube.vp_rgb(), rgb, 3 * n);
  LGKvRendererTSDF r;
  r.ip_Initialize_Parameters(&cube, W, H, K0[0], K0[1], K0[2], K0[3], mu, max_w);
  const Vector3f c(cam[0], cam[1], cam[2]), li(light[0], light[1], light[2]);
  if (variant == 0) {
    r.rmis_Render_Maps_for_Scene(&cube, W, H, T_gc, T_cg, c, li, depth, vtx3, nrm3, img, rgb_img);
  } else if (variant == 1) {
    r.rmis_Render_Maps_for_Scene(&cube, W, H, T_gc, T_cg, c, li, depth, nrm3, img, rgb_img);
  } else {
    int lw = W, lh = H;
    for (int l = 0; l < level; l++) lw /= 2, lh /= 2;
    r.rmi_Render_Maps_for_ICP(&cube, lw, lh, T_gc, T_cg, c, li, level, depth, nrm3, img, rgb_img);
  }
  return 1;
}
#endif

#if defined(REF_PIN_INTEG)
#include "integrator.cu.cpp"

// one cdtocc call on a cube given and returned in the reference layout (rgb:
// three planes of the cube; img_rgb: three planes of the image, registered to
// the depth image), then, where vol_valid (one byte per voxel) is given, one
// uvv_Update_Valid_Volume carving over the sub-cubes this integration flagged
extern "C" int ref_integrate_color(int W, int H, const float* K0, const int* dim, const float* origin,
                                   const float* center, float vox, float mu, float max_w, float* tsdf, uint8_t* w,
                                   uint8_t* rgb, const float* depth, const uint8_t* img_rgb, const float* T_gc,
                                   const float* T_cg, const uint8_t* vol_valid) {
  GKvObjectCubeFloat cube;
  if (!cube.create(Vector3i(dim[0], dim[1], dim[2]), Vector3f(origin[0], origin[1], origin[2]),
                   Vector3f(center[0], center[1], center[2]), vox, true))
    return 0;
  const size_t n = (size_t)dim[0] * dim[1] * dim[2];
  std::memcpy(cube.vp_tsdf(), tsdf, n * sizeof(float));
  std::memcpy(cube.vp_w(), w, n);
  std::memcpy(cube.vp_rgb(), rgb, 3 * n);
  LGKvVolumeIntegrator integ;
  integ.ip_Initialize_Parameters(&cube, W, H, K0[0], K0[1], K0[2], K0[3], mu, max_w);
  integ.cdtocc_Convert_Depth_to_TSDF_on_Cube_with_Color(&cube, depth, img_rgb, W, H, T_gc, T_cg, true);
  if (vol_valid) {
    // carving over this integration's sub-cube flags (uvv_Update_Valid_Volume)
    GKvVolumeBool vv;
    vv.create(dim[0], dim[1], dim[2], 1, true);
    for (size_t i = 0; i < n; i++) vv.vp()[i] = vol_valid[i] != 0;
    integ.uvv_Update_Valid_Volume(&cube, &vv);
  }
  std::memcpy(tsdf, cube.vp_tsdf(), n * sizeof(float));
  std::memcpy(w, cube.vp_w(), n);
  std::memcpy(rgb, cube.vp_rgb(), 3 * n);
  return 1;
}
#endif

#if defined(REF_PIN_TRACK)
#include "tracker.cu.cpp"

// the reference's per-pixel ICP term at level 0 for every pixel of a frame:
// ATA (36 per pixel) and ATb (6 per pixel) where the pixel gives a term,
// ok[pixel] = 1 there; vertex / normal maps in the reference's float3 layout
extern "C" void ref_icp_terms(int W, int H, const float* K, const float* depth_t1, const float* depth_t0,
                              const float* vtx3_t0, const float* nrm3_t0, const float* T21, float th_icp, float* ATA,
                              float* ATb, uint8_t* ok) {
  for (int k = 0; k < 4; k++) K_dev[k] = K[k];
  for (int y = 0; y < H; y++)
    for (int x = 0; x < W; x++) {
      const size_t i = (size_t)y * W + x;
      ok[i] = d_cssfp_Compute_Single_Summand_with_Forward_Params(x, y, depth_t1, depth_t0, vtx3_t0, nrm3_t0, T21, 0,
                                                                 W, H, th_icp, ATA + 36 * i, ATb + 6 * i)
                  ? 1
                  : 0;
    }
}

// the reference's tp_Track_Pose: t0 maps (model depth / vertex / normal of
// each level, the reference's float3 layout), t1 depth levels, the previous
// pose T_gc (row-major 4x4) and an optional initial increment T_12; writes
// the tracked T_gc and returns 1, or returns 0 where the solve failed
extern "C" int ref_track_pose(int W, int H, const float* K0, float th_icp, const float* const* depth_t1,
                              const float* const* depth_t0, const float* const* vtx3_t0,
                              const float* const* nrm3_t0, const float* T_gc_prev, const float* init_T12,
                              float* T_gc_out) {
  GKvTrackingState ts;
  GKvRgbdFrame fr;
  if (!ts.create(Vector2i(W, H)) || !fr.create(Vector2i(W, H))) return -1;
  for (int l = 0; l < GK_LEVEL_OF_IMAGE_PYRAMID; l++) {
    const size_t n = (size_t)(W >> l) * (H >> l);
    std::memcpy(ts.vp_map_depth(l), depth_t0[l], n * sizeof(float));
    std::memcpy(ts.vp_map_vertex(l), vtx3_t0[l], 3 * n * sizeof(float));
    std::memcpy(ts.vp_map_normal(l), nrm3_t0[l], 3 * n * sizeof(float));
    std::memcpy(fr.vp_map_depth(l), depth_t1[l], n * sizeof(float));
  }
  GKvMatrixFloat prev, init;
  prev.create(4, 4, 1);
  std::memcpy(prev.vp(), T_gc_prev, 16 * sizeof(float));
  ts.set_transform(&prev, false);
  if (init_T12) {
    init.create(4, 4, 1);
    std::memcpy(init.vp(), init_T12, 16 * sizeof(float));
  }
  LGKvPoseTracker tr;
  tr.ip_Initialize_Parameters(W, H, K0[0], K0[1], K0[2], K0[3], th_icp);
  vs_block_threads = true;
  const bool ok = tr.tp_Track_Pose(&ts, &fr, init_T12 ? &init : nullptr);
  vs_block_threads = false;
  std::fflush(stdout);  // the tracker prints ATA every iteration
  std::memcpy(T_gc_out, ts.vp_T_gc(), 16 * sizeof(float));
  return ok ? 1 : 0;
}
#endif

#if defined(REF_PIN_IMGPROC)
#include "imgproc.cu.cpp"

// the reference's bilateral filter of one depth frame (metres in, metres out)
extern "C" void ref_bilateral(int W, int H, const float* depth, float* out) {
  LGKvImageProcessor ip;
  ip.bfd_Bilateral_Filter_Depth_Host(out, depth, W, H);
  ip.r_Release();
}
#endif
