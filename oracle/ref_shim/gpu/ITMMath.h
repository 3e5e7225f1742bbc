// stand-in for InfiniTAM's ITMMath (InfiniTAM v2, 2014; not in the reference
// tree): the vector types and free functions the reference's GPU sources use,
// restated as plain structs whose operators work component by component.
#pragma once
#include "ref_gpu_shim.h"

template <class T>
struct Vector2_ {
  T x = 0, y = 0;
  Vector2_() {}
  Vector2_(T a, T b) : x(a), y(b) {}
  Vector2_& operator=(T a) {
    x = y = a;
    return *this;
  }
  Vector2_& operator/=(T s) {
    x /= s, y /= s;
    return *this;
  }
  Vector2_& operator*=(T s) {
    x *= s, y *= s;
    return *this;
  }
  // a friend, not a template, so a scalar of another type converts to T
  friend Vector2_ operator/(Vector2_ a, T s) { return a /= s; }
};
template <class T>
struct Vector3_ {
  T x = 0, y = 0, z = 0;
  Vector3_() {}
  Vector3_(T a, T b, T c) : x(a), y(b), z(c) {}
  explicit Vector3_(T a) : x(a), y(a), z(a) {}
  Vector3_& operator=(T a) {
    x = y = z = a;
    return *this;
  }
  Vector3_& operator+=(const Vector3_& o) {
    x += o.x, y += o.y, z += o.z;
    return *this;
  }
  Vector3_& operator-=(const Vector3_& o) {
    x -= o.x, y -= o.y, z -= o.z;
    return *this;
  }
  Vector3_& operator*=(T s) {
    x *= s, y *= s, z *= s;
    return *this;
  }
  Vector3_& operator/=(T s) {
    x /= s, y /= s, z /= s;
    return *this;
  }
  // the floor and the remainder v - floor(v), the InfiniTAM convention the
  // oracle restates (the reference's CPU twin of the trilinear read,
  // z_yooji_cube_tsdf_float.cpp:376-378, truncates instead; the two differ
  // only for a coordinate in (-1, 0), where the floor's tap at -1 makes the
  // read invalid)
  Vector3_<int> toInt(Vector3_<float>& residual) const {
    const Vector3_<int> i((int)std::floor(x), (int)std::floor(y), (int)std::floor(z));
    residual = Vector3_<float>((float)(x - (T)i.x), (float)(y - (T)i.y), (float)(z - (T)i.z));
    return i;
  }
  // round half away from zero, clamp to 0..255
  Vector3_<unsigned char> toUChar() const {
    auto r = [](T v) {
      int i = (int)((v < (T)0) ? (v - (T)0.5f) : (v + (T)0.5f));
      return (unsigned char)(i < 0 ? 0 : (i > 255 ? 255 : i));
    };
    return Vector3_<unsigned char>(r(x), r(y), r(z));
  }
  // ITMMath's Vector3::normalised: v * (1 / |v|)
  Vector3_ normalised() const {
    const T norm = (T)1.0f / (T)std::sqrt((float)(x * x + y * y + z * z));
    return Vector3_(x * norm, y * norm, z * norm);
  }
};
template <class T>
inline Vector3_<T> operator+(Vector3_<T> a, const Vector3_<T>& b) { return a += b; }
template <class T>
inline Vector3_<T> operator-(Vector3_<T> a, const Vector3_<T>& b) { return a -= b; }
template <class T>
inline Vector3_<T> operator-(const Vector3_<T>& a) { return Vector3_<T>(-a.x, -a.y, -a.z); }
template <class T>
inline Vector3_<T> operator*(Vector3_<T> a, T s) { return a *= s; }
template <class T>
inline Vector3_<T> operator*(T s, Vector3_<T> a) { return a *= s; }
template <class T>
inline Vector3_<T> operator/(Vector3_<T> a, T s) { return a /= s; }
template <class T>
inline T dot(const Vector3_<T>& a, const Vector3_<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T>
inline Vector3_<T> cross(const Vector3_<T>& a, const Vector3_<T>& b) {
  return Vector3_<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T>
inline T length(const Vector3_<T>& a) { return (T)std::sqrt((float)dot(a, a)); }
template <class T>
inline Vector3_<T> normalize(const Vector3_<T>& a) { return a.normalised(); }

typedef Vector2_<float> Vector2f;
typedef Vector2_<int> Vector2i;
typedef Vector3_<float> Vector3f;
typedef Vector3_<int> Vector3i;
typedef Vector3_<unsigned char> Vector3u;
typedef Vector3_<short> Vector3s;
