// Depth -> colour camera registration (vs_warp_depth_to_color,
// vs_warp_depth_mm_to_color in include/vs.h).
//
// Reference: z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates
// (STAC/Engine/CPU/z_yooji_object_scanner.cpp:2429-2476) with
// CKvYooji_MatrixRgbD::convert_pixel_coord (STAC/Object/CPU/
// z_yooji_matrix_rgbd.cpp:101-118) and the KAISION-style camera helpers of
// STAC/Object/CPU/z_yooji_camera_parameters.cpp:89-108,678-685: every depth
// pixel with depth d > 0 is back-projected with the depth intrinsics,
// transformed by the depth-to-colour extrinsics, projected with the colour
// intrinsics and rounded with ROUNDF; a colour pixel keeps the smallest depth
// that lands on it (the depth value of the depth camera, as the reference
// stores it), 0 where none lands.  The reference runs this per frame on the
// host ("always start from the depth seen by the RGB camera",
// z_yooji_object_scanner.cpp:806-820).  Here one thread per depth pixel
// lands its depth with an atomic minimum on the value's bits, which orders
// positive floats (and uint16) as their values, so the result does not
// depend on the order the threads arrive in.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

struct WarpArgs {
  int wd, hd, wr, hr;
  float Kd[4], Kr[4], T[12];
  float scale;  // depth units -> metres (1 for metres)
};

// T: depth type (float metres or uint16 units); out holds the minimum as
// unsigned bits, "empty" = all ones
template <class T>
__global__ void k_warp_depth(const T* __restrict__ in, WarpArgs a, unsigned* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.wd || j >= a.hd) return;
  const T raw = in[(size_t)j * a.wd + i];
  const float td = (float)raw * a.scale;
  if (!(td > 0.0f)) return;
  const F3 p = transform(back_project((float)i, (float)j, a.Kd, td), a.T);
  float u, v;
  project(p, a.Kr, u, v);
  if (isnan(u) || isnan(v)) return;
  const int tx = roundf_ref(u), ty = roundf_ref(v);
  if (tx < 0 || tx > a.wr - 1 || ty < 0 || ty > a.hr - 1) return;
  unsigned bits;
  if (sizeof(T) == 4)
    bits = __float_as_uint(td);
  else
    bits = (unsigned)raw;
  atomicMin(out + (size_t)ty * a.wr + tx, bits);
}

template <class T>
__global__ void k_warp_finish(const unsigned* __restrict__ bits, T* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned b = bits[i];
  if (sizeof(T) == 4)
    reinterpret_cast<unsigned*>(out)[i] = (b == 0xffffffffu) ? 0u : b;
  else
    out[i] = (T)((b == 0xffffffffu) ? 0u : b);
}

}  // namespace

template <class T>
void launch_warp_depth(const T* in, int wd, int hd, const float* Kd, const float* T_rgb_d, const float* Kr, int wr,
                       int hr, float scale, unsigned* scratch, T* out, cudaStream_t st) {
  WarpArgs a;
  a.wd = wd;
  a.hd = hd;
  a.wr = wr;
  a.hr = hr;
  for (int k = 0; k < 4; k++) a.Kd[k] = Kd[k], a.Kr[k] = Kr[k];
  for (int k = 0; k < 12; k++) a.T[k] = T_rgb_d[k];
  a.scale = scale;
  const int n = wr * hr;
  cudaMemsetAsync(scratch, 0xff, (size_t)n * 4, st);
  k_warp_depth<T><<<dim3((wd + 31) / 32, (hd + 7) / 8), dim3(32, 8), 0, st>>>(in, a, scratch);
  k_warp_finish<T><<<(n + 255) / 256, 256, 0, st>>>(scratch, out, n);
}

template void launch_warp_depth<float>(const float*, int, int, const float*, const float*, const float*, int, int,
                                       float, unsigned*, float*, cudaStream_t);
template void launch_warp_depth<uint16_t>(const uint16_t*, int, int, const float*, const float*, const float*, int,
                                          int, float, unsigned*, uint16_t*, cudaStream_t);

}  // namespace vs
