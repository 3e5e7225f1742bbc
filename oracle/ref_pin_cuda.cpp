// Harness around the reference's own device math header, compiled as host
// C++ from the reference source tree where it lies (TEST INFRASTRUCTURE ONLY).
//
// STAC/Util/_yooji_cuda_math.h holds the per-pixel and per-voxel helpers of the
// hot path as inline functions; with the stand-ins of ref_shim/ref_cuda_shim.h
// for the CUDA qualifiers and ITMMath's vector types it builds with g++, and
// oracle/build_oracle.py compiles this file into oracle/_ref/libref_pin_cuda.so.
// The exported functions pin the oracle's restatements of:
//   d_lld_LL_Decomposition, d_sls_Solve_Linear_System_using_LLD  :489-592
//   d_giv_Get_Interpolated_Vertex, d_gin_Get_Interpolated_Normal  :365-481
//   d_gid_Get_Interpolated_Depth                                  :335-362
//   d_p_Project, d_bp_Back_Project, d_t_Transform, d_r_Rotate     :200-250
//   d_gcc_Get_Camera_Center                                       :247-257
//   d_gpv_Get_Position_in_Voxel, d_gpw_Get_Position_in_World      :265-300
#include "ref_cuda_shim.h"
#include "_yooji_math_inlines.h"
#include "_yooji_cuda_math.h"

extern "C" {
int ref_lld6(const float* A, float* L) { return d_lld_LL_Decomposition<float>(A, 6, L) ? 1 : 0; }
int ref_sls6(const float* L, const float* b, float* x) {
  float y[6];
  return d_sls_Solve_Linear_System_using_LLD<float>(L, b, y, 6, x) ? 1 : 0;
}
int ref_giv(float xf, float yf, int w, int h, const float* map3, float* out3) {
  Vector2f p;
  p.x = xf;
  p.y = yf;
  Vector3f o;
  const bool ok = d_giv_Get_Interpolated_Vertex(p, w, h, map3, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
  return ok ? 1 : 0;
}
int ref_gin(float xf, float yf, int w, int h, const float* map3, float* out3) {
  Vector2f p;
  p.x = xf;
  p.y = yf;
  Vector3f o;
  const bool ok = d_gin_Get_Interpolated_Normal(p, w, h, map3, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
  return ok ? 1 : 0;
}
int ref_gid(float xf, float yf, int w, int h, const float* map, float* out) {
  Vector2f p;
  p.x = xf;
  p.y = yf;
  return d_gid_Get_Interpolated_Depth(p, w, h, map, *out) ? 1 : 0;
}
void ref_project(const float* p3, const float* K, float* uv) {
  Vector3f p;
  p.x = p3[0], p.y = p3[1], p.z = p3[2];
  Vector2f o;
  d_p_Project(p, K, o);
  uv[0] = o.x, uv[1] = o.y;
}
void ref_back_project(float u, float v, const float* K, float d, float* p3) {
  Vector2f p;
  p.x = u, p.y = v;
  Vector3f o;
  d_bp_Back_Project(p, K, d, o);
  p3[0] = o.x, p3[1] = o.y, p3[2] = o.z;
}
void ref_transform(const float* p3, const float* T, float* out3) {
  Vector3f p, o;
  p.x = p3[0], p.y = p3[1], p.z = p3[2];
  d_t_Transform(p, T, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
}
void ref_rotate(const float* p3, const float* T, float* out3) {
  Vector3f p, o;
  p.x = p3[0], p.y = p3[1], p.z = p3[2];
  d_r_Rotate(p, T, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
}
void ref_camera_center(const float* T, float* c) {
  Vector3f o;
  d_gcc_Get_Camera_Center(T, o);
  c[0] = o.x, c[1] = o.y, c[2] = o.z;
}
int ref_pos_in_voxel(const float* p3, const float* origin, const int* dim, float vox_inv, float* out3) {
  Vector3f p, o;
  p.x = p3[0], p.y = p3[1], p.z = p3[2];
  const bool ok = d_gpv_Get_Position_in_Voxel(p, origin, dim, vox_inv, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
  return ok ? 1 : 0;
}
void ref_pos_in_world(const float* v3, const float* origin, const int* dim, float vox_inv, float* out3) {
  Vector3f p, o;
  p.x = v3[0], p.y = v3[1], p.z = v3[2];
  d_gpw_Get_Position_in_World(p, origin, dim, vox_inv, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
}
}
