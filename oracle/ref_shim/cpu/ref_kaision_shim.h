// Stand-ins for the closed KAISION SDK types that the reference's CPU image
// processor is written on, and declarations of the reference classes whose
// member functions oracle/build_oracle.py takes from the reference tree
// (TEST INFRASTRUCTURE ONLY).  Only what those functions use is here, with the
// semantics their call sites imply (ROUNDF comes from the reference's own
// STAC/Util/_yooji_SITM_defines.h):
//   CKvMatrixFloat / CKvSet2d_of_Point3Df: a row-major matrix; ms(w, h) and
//     mps(w, h) report width and height (mps also returns the row pointers),
//     c_Create(rows, cols[, value]) sizes it (zero-filled without a value),
//     vp() is the first element, mw() / mh() width / height.
//   CKvPoint3Df::n_Normalize(): each component divided by the Euclidean norm.
//   PI: the double closest to pi.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

using std::abs;
using std::cos;
using std::max;
using std::sqrt;
using std::vector;

#define PI 3.14159265358979323846
#include "_yooji_SITM_defines.h"

struct CKvClass {};
struct CKvPixel {
  int x = 0, y = 0;
};
struct CKvPointf {
  float x = 0, y = 0;
};
struct CKvPoint3Df {
  float x = 0, y = 0, z = 0;
  void n_Normalize() {
    const float n = std::sqrt(x * x + y * y + z * z);
    x /= n, y /= n, z /= n;
  }
};

template <class T>
class KvMatrix {
 public:
  KvMatrix() {}
  KvMatrix(const KvMatrix& a) : d_(a.d_), w_(a.w_), h_(a.h_) { relink(); }
  KvMatrix& operator=(const KvMatrix& a) {
    d_ = a.d_, w_ = a.w_, h_ = a.h_;
    relink();
    return *this;
  }
  T** c_Create(int rows, int cols, T v = T()) {
    w_ = cols, h_ = rows;
    d_.assign((size_t)w_ * h_, v);
    relink();
    return rows_.data();
  }
  void ms(int& ww, int& hh) const { ww = w_, hh = h_; }
  T** mps(int& ww, int& hh) {
    ww = w_, hh = h_;
    return rows_.data();
  }
  T* vp() { return d_.data(); }
  int mw() const { return w_; }
  int mh() const { return h_; }
  void cp_Copy(KvMatrix* a) { *this = *a; }

 private:
  void relink() {
    rows_.resize(h_);
    for (int r = 0; r < h_; r++) rows_[r] = d_.data() + (size_t)r * w_;
  }
  std::vector<T> d_;
  std::vector<T*> rows_;
  int w_ = 0, h_ = 0;
};
typedef KvMatrix<float> CKvMatrixFloat;
typedef KvMatrix<CKvPoint3Df> CKvSet2d_of_Point3Df;
typedef KvMatrix<unsigned char> CKvMatrixUcharRgb;  // only its size is used

// the reference's own classes (STAC/Object/CPU/_yooji_camera_parameters.h,
// _yooji_image_pyramid.h, STAC/Engine/CPU/_yooji_image_processor.h), declared
// with the members the taken functions use
class CKvYooji_Intrinsics : CKvClass {
 public:
  CKvYooji_Intrinsics() { zz_mat.c_Create(3, 3, 0.0f); }
  bool set_from_params(float in_fx, float in_fy, float in_px, float in_py, float in_dmin = 0.0f,
                       float in_dmax = 100.0f);
  void get_params(float& in_fx, float& in_fy, float& in_px, float& in_py, float& in_dmin, float& in_dmax);
  void back_project(CKvPixel& in_xy, float in_Z, CKvPoint3Df& out_p3d);
  void back_project(CKvPointf& in_xy, float in_Z, CKvPoint3Df& out_p3d);
  bool project(CKvPoint3Df& in_p3d, CKvPointf& out_p);

 protected:
  CKvMatrixFloat zz_mat;
  float zz_fx = 0, zz_fy = 0, zz_px = 0, zz_py = 0;
  float zz_d_min = 0, zz_d_max = 0;
};

class CKvYooji_Extrinsics : CKvClass {
 public:
  CKvYooji_Extrinsics() { zz_mat.c_Create(4, 4, 0.0f); }
  // the harness sets the 4x4 row-major transform directly
  void set_matrix(const float* T) { std::memcpy(zz_mat.vp(), T, 16 * sizeof(float)); }
  void transform(CKvPoint3Df& in_p3d, CKvPoint3Df& out_p);

 protected:
  CKvMatrixFloat zz_mat;
};

class CKvYooji_MatrixRgbD : public CKvClass {
 public:
  bool convert_pixel_coord(CKvPointf& in_point_depth, float in_depth, CKvPointf& out_point_rgb);
  CKvYooji_Intrinsics zz_intrin_d, zz_intrin_rgb;
  CKvYooji_Extrinsics zz_extrin_rgb_wrt_d;
  CKvMatrixUcharRgb zz_image_rgb;
};

class CKvYooji_3D_Object_Scanner {
 public:
  void z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates(CKvYooji_MatrixRgbD* in_rgbd_img, CKvMatrixFloat* in_img_d,
                                                         CKvMatrixFloat* out_img_d_transformed);
};

class CKvYooji_Pyramid_Mat_Float : public CKvClass {
 public:
  void c_Create(int in_ww_bottom, int in_hh_bottom, int in_level_of_scale = 3);
  int levOfScale = 0;
  vector<CKvMatrixFloat> imgs;
};

class LCKvYooji_Image_Processor {
 public:
  void cpm_Compute_Point_Map(CKvMatrixFloat* in_map_depth, CKvYooji_Intrinsics* in_intrinsics,
                             CKvSet2d_of_Point3Df* out_map_p3d);
  void enm_Estimate_Normal_Map(CKvSet2d_of_Point3Df* in_map_p3d, CKvSet2d_of_Point3Df* out_map_normal,
                               int in_sz_mask_half = 1);
  void cpdd_Construct_Pyramids_Down_Depth(CKvMatrixFloat* in_map_depth, CKvYooji_Pyramid_Mat_Float* out_pyrams_map,
                                          int in_level_of_pyrams);
  void sdg5_Smooth_Depthmap_Gaussian_5x5(CKvMatrixFloat* in_map_depth, CKvMatrixFloat* out_map_smooth,
                                         bool in_flag_boundary_padding, CKvMatrixFloat* in_map_for_padding);
  void ddh_Downsample_Depthmap_Half(CKvMatrixFloat* in_map_depth, CKvMatrixFloat* out_map_downsampled);
  void dih_Downsample_Intrinsics_Half(CKvYooji_Intrinsics* in_intrinsics,
                                      CKvYooji_Intrinsics* out_intrinsics_downsampled);

 private:
  CKvMatrixFloat zz_map_tmp[3];
  CKvMatrixFloat zz_map_padding[3];
};
