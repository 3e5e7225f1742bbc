// Harness around the reference's own host math header, compiled from the
// reference source tree where it lies (TEST INFRASTRUCTURE ONLY).
//
// STAC/Util/_yooji_math_inlines.h needs nothing but the C++ standard library,
// so unlike the rest of the reference it builds on Linux: g++ -fpermissive
// (MSVC resolves the template's non-dependent calls late; GCC needs the flag).
// oracle/build.py compiles this file into oracle/_ref/libref_pin.so with the
// reference include directory on the include path.  The exported functions pin
// the oracle's SE(3) exponential and 4x4 inverse:
//   d_cme_Compute_Matrix_Exponential  _yooji_math_inlines.h:114-194
//   d_im_Inverse_Matrix_4x4           _yooji_math_inlines.h:403-465
//   d_mmm_Multiply_Matrix_Matrix      _yooji_math_inlines.h:228-246
#include <cmath>
#include <cstdlib>
// MSVC's <cmath> puts the float overloads of abs/sqrt/sin/cos in the global
// namespace, which the header relies on.
using std::abs;
using std::cos;
using std::sin;
using std::sqrt;
#include "_yooji_math_inlines.h"

extern "C" {
void ref_se3_exp(const float* xi, float* T) {
  float x[6];
  for (int i = 0; i < 6; i++) x[i] = xi[i];
  d_cme_Compute_Matrix_Exponential(x, T);
}
int ref_inverse4(const float* M, float* Minv) {
  float m[16];
  for (int i = 0; i < 16; i++) m[i] = M[i];
  return d_im_Inverse_Matrix_4x4(m, Minv) ? 1 : 0;
}
void ref_matmul4(const float* A, const float* B, float* C) {
  float a[16], b[16];
  for (int i = 0; i < 16; i++) a[i] = A[i], b[i] = B[i];
  d_mmm_Multiply_Matrix_Matrix(a, b, 4, 4, 4, C);
}
}
