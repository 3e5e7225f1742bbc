// Stand-ins that let the reference's STAC/Util/_yooji_cuda_math.h compile as
// plain host C++ (TEST INFRASTRUCTURE ONLY: the reference-pin harness in
// oracle/ref_pin_cuda.cpp includes this file first).
//
// The header normally comes after _yooji_cuda_defines.h, which pulls in the
// CUDA runtime and InfiniTAM's ITMMath (InfiniTAM v2, 2014; not vendored in the
// reference tree).  Only what the pinned functions touch is given here:
//   * the CUDA qualifiers as nothing, int2 / int3, uchar, and declarations of
//     the three runtime calls that uninstantiated templates name;
//   * ITMMath's Vector2f / Vector2i / Vector3f / Vector3u as plain structs with
//     the component-wise operators ITMMath defines (scalar * vector multiplies
//     each component, vector + vector adds component by component).  A
//     default-constructed Vector3f here is zero; ITMMath leaves it
//     uninitialised, and the reference multiplies such a vector by a zero
//     interpolation weight, so 0 is the value the oracle assumes.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>

#define __device__
#define __host__
#define __forceinline__ inline
#define _CPU_AND_GPU_CODE_

using std::abs;
using std::sqrt;

typedef unsigned char uchar;
struct int2 {
  int x, y;
};
struct int3 {
  int x, y, z;
};
int cudaFree(void*);
int cudaMalloc(void**, size_t);
int cudaMemcpy(void*, const void*, size_t, int);
enum { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
// _yooji_cuda_math.hpp:98 (GKvMatrix<T>::to_host) names an undeclared
// `out_vol`; MSVC never checks the uninstantiated template, GCC needs the name
// to exist.  Nothing here instantiates it.
static void* out_vol;

struct Vector2f {
  float x = 0.0f, y = 0.0f;
};
struct Vector2i {
  int x = 0, y = 0;
};
struct Vector3u {
  unsigned char x = 0, y = 0, z = 0;
};
struct Vector3f {
  float x = 0.0f, y = 0.0f, z = 0.0f;
  // ITMMath's Vector3::normalised: v * (1 / |v|)
  Vector3f normalised() const {
    const float norm = 1.0f / std::sqrt(x * x + y * y + z * z);
    Vector3f r;
    r.x = x * norm;
    r.y = y * norm;
    r.z = z * norm;
    return r;
  }
};
// named by helpers of the header that are not pinned (declared only; inline
// functions that are never called are never emitted)
float dot(const Vector3f&, const Vector3f&);
Vector3f cross(const Vector3f&, const Vector3f&);
Vector3f normalize(const Vector3f&);
inline Vector3f operator*(float s, const Vector3f& v) {
  Vector3f r = v;
  r.x *= s;
  r.y *= s;
  r.z *= s;
  return r;
}
inline Vector3f operator+(const Vector3f& a, const Vector3f& b) {
  Vector3f r = a;
  r.x += b.x;
  r.y += b.y;
  r.z += b.z;
  return r;
}
