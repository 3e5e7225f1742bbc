// Harness around member functions of the reference's CPU image processor
// (STAC/Engine/CPU/z_yooji_image_processor.cpp), its intrinsics class
// (STAC/Object/CPU/z_yooji_camera_parameters.cpp) and its pyramid class
// (STAC/Object/CPU/z_yooji_image_pyramid.cpp), compiled as host C++ (TEST
// INFRASTRUCTURE ONLY).  oracle/build_oracle.py copies those functions'
// definitions, unchanged, from the reference tree into
// oracle/_ref/gen/cpu_functions.cpp (a build product, never committed); the
// KAISION SDK types they are written on are the stand-ins of
// ref_shim/cpu/ref_kaision_shim.h.
//   cpdd_Construct_Pyramids_Down_Depth = sdg5 (5x5 Gaussian) + ddh (half)
//   cpm_Compute_Point_Map + enm_Estimate_Normal_Map (half window 1)
//   dih_Downsample_Intrinsics_Half
//   z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates with convert_pixel_coord
#include <cstdint>

#include "ref_kaision_shim.h"
#include "cpu_functions.cpp"

// the depth pyramid of `levels` levels: level l (w >> l by h >> l) at
// out + the sum of the sizes of the levels before it
extern "C" void ref_depth_pyramid(const float* depth, int w, int h, int levels, float* out) {
  LCKvYooji_Image_Processor ip;
  CKvMatrixFloat d;
  std::memcpy(d.c_Create(h, w)[0], depth, sizeof(float) * w * h);
  CKvYooji_Pyramid_Mat_Float pyr;
  ip.cpdd_Construct_Pyramids_Down_Depth(&d, &pyr, levels);
  size_t off = 0;
  for (int l = 0; l < levels; l++) {
    const size_t n = (size_t)pyr.imgs[l].mw() * pyr.imgs[l].mh();
    std::memcpy(out + off, pyr.imgs[l].vp(), n * sizeof(float));
    off += n;
  }
}

// the point and normal maps of one depth map (x, y, z per pixel, -100 where
// invalid), with intrinsics fx, fy, cx, cy
extern "C" void ref_point_normal_map(const float* depth, int w, int h, const float* K, float* vtx3, float* nrm3) {
  LCKvYooji_Image_Processor ip;
  CKvMatrixFloat d;
  std::memcpy(d.c_Create(h, w)[0], depth, sizeof(float) * w * h);
  CKvYooji_Intrinsics in;
  in.set_from_params(K[0], K[1], K[2], K[3]);
  CKvSet2d_of_Point3Df p3d, nrm;
  ip.cpm_Compute_Point_Map(&d, &in, &p3d);
  ip.enm_Estimate_Normal_Map(&p3d, &nrm);
  std::memcpy(vtx3, p3d.vp(), sizeof(float) * 3 * w * h);
  std::memcpy(nrm3, nrm.vp(), sizeof(float) * 3 * w * h);
}

// the intrinsics of `levels` pyramid levels (fx, fy, cx, cy each)
extern "C" void ref_level_intrinsics(const float* K0, int levels, float* Kl) {
  LCKvYooji_Image_Processor ip;
  std::vector<CKvYooji_Intrinsics> in(levels);
  in[0].set_from_params(K0[0], K0[1], K0[2], K0[3]);
  for (int l = 1; l < levels; l++) ip.dih_Downsample_Intrinsics_Half(&in[l - 1], &in[l]);
  for (int l = 0; l < levels; l++) {
    float dmin, dmax;
    in[l].get_params(Kl[4 * l], Kl[4 * l + 1], Kl[4 * l + 2], Kl[4 * l + 3], dmin, dmax);
  }
}

// the depth map seen from the colour camera: depth (wd x hd, metres) through
// the depth intrinsics Kd, the depth-to-colour transform T (4x4 row-major)
// and the colour intrinsics Kr into out (wr x hr), nearest depth kept
extern "C" void ref_warp_depth(const float* depth, int wd, int hd, const float* Kd, const float* T, const float* Kr,
                               int wr, int hr, float* out) {
  CKvYooji_MatrixRgbD rig;
  rig.zz_intrin_d.set_from_params(Kd[0], Kd[1], Kd[2], Kd[3]);
  rig.zz_intrin_rgb.set_from_params(Kr[0], Kr[1], Kr[2], Kr[3]);
  rig.zz_extrin_rgb_wrt_d.set_matrix(T);
  rig.zz_image_rgb.c_Create(hr, wr);
  CKvMatrixFloat d, o;
  std::memcpy(d.c_Create(hd, wd)[0], depth, sizeof(float) * wd * hd);
  o.c_Create(hr, wr);
  CKvYooji_3D_Object_Scanner sc;
  sc.z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates(&rig, &d, &o);
  std::memcpy(out, o.vp(), sizeof(float) * wr * hr);
}
