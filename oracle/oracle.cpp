// CPU oracle for the per-frame reconstruction path (TEST INFRASTRUCTURE ONLY;
// see oracle.h).  Paths cited as file:line are relative to VCL_Volume_Scanner/
// of the reference repository.
//
// Build: g++ -O2 -std=c++17 -ffp-contract=off -fPIC -shared (oracle/build.py).
// Every stage is templated on the arithmetic type T: T = float restates the
// reference semantics; T = double is the FP64 oracle used as ground truth by
// the precision study.
#include "oracle.h"

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

// ---------------------------------------------------------------------------
// small vector type (the reference uses InfiniTAM's ITMMath Vector2f/3f;
// ITMMath is not part of the reference repository, its published semantics
// are restated: componentwise + - *, dot = x*x'+y*y'+z*z', length = sqrt(dot),
// normalised = v * (1/length))
// ---------------------------------------------------------------------------
template <class T>
struct V3 {
  T x, y, z;
};
template <class T>
inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T>
inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T>
inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T>
inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T>
inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T>
inline T tsqrt(T x) { return std::sqrt(x); }
template <class T>
inline T length(V3<T> a) { return tsqrt(dot(a, a)); }
template <class T>
inline V3<T> normalised(V3<T> a) {
  T inv = T(1) / tsqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return {a.x * inv, a.y * inv, a.z * inv};
}

// _yooji_cuda_math.h:205-210 d_p_Project
template <class T>
inline void project(V3<T> p, const T* K, T& u, T& v) {
  u = K[0] * p.x / p.z + K[2];
  v = K[1] * p.y / p.z + K[3];
}
// _yooji_cuda_math.h:212-226 d_bp_Back_Project
template <class T>
inline V3<T> back_project(T u, T v, const T* K, T d) {
  return {d * (u - K[2]) / K[0], d * (v - K[3]) / K[1], d};
}
// _yooji_cuda_math.h:229-235 d_t_Transform
template <class T>
inline V3<T> transform(V3<T> p, const T* M) {
  return {M[0] * p.x + M[1] * p.y + M[2] * p.z + M[3],
          M[4] * p.x + M[5] * p.y + M[6] * p.z + M[7],
          M[8] * p.x + M[9] * p.y + M[10] * p.z + M[11]};
}
// _yooji_cuda_math.h:238-244 d_r_Rotate
template <class T>
inline V3<T> rotate(V3<T> p, const T* M) {
  return {M[0] * p.x + M[1] * p.y + M[2] * p.z, M[4] * p.x + M[5] * p.y + M[6] * p.z,
          M[8] * p.x + M[9] * p.y + M[10] * p.z};
}
// _yooji_cuda_math.h:247-262 d_gcc_Get_Camera_Center
template <class T>
inline V3<T> camera_center(const T* M) {
  T tx = M[3], ty = M[7], tz = M[11];
  return {-M[0] * tx - M[4] * ty - M[8] * tz, -M[1] * tx - M[5] * ty - M[9] * tz,
          -M[2] * tx - M[6] * ty - M[10] * tz};
}

// ROUNDF macro (_yooji_cuda_defines.h ROUNDF): (x<0) ? (int)(x-0.5) : (int)(x+0.5)
template <class T>
inline int roundf_ref(T x) {
  return (x < T(0)) ? (int)(x - T(0.5)) : (int)(x + T(0.5));
}
// The reference writes ROUNDF(v)/sz_sc; the unparenthesised macro makes that
// (v<0) ? (int)(v-0.5) : (int)(v+0.5)/sz_sc  (z_yooji_cuda_volume_integrator.cu:133-135)
template <class T>
inline int roundf_div_ref(T x, int d) {
  return (x < T(0)) ? (int)(x - T(0.5)) : (int)(x + T(0.5)) / d;
}
// __float2int_rn (z_yooji_cuda_volume_integrator.cu:347): round half to even,
// NaN -> 0, saturating (the PTX cvt.rni.s32 rule, restated)
template <class T>
inline int float2int_rn(T x) {
  if (std::isnan(x)) return 0;
  T r = std::nearbyint(x);
  if (r >= T(2147483647.0)) return 2147483647;
  if (r <= T(-2147483648.0)) return (-2147483647 - 1);
  return (int)r;
}

// d_gpv_Get_Position_in_Voxel (_yooji_cuda_math.h:265-283)
template <class T>
inline bool pos_in_voxel(V3<T> p, const T* origin, const int* dim, T inv, V3<T>& v) {
  v.x = (p.x - origin[0]) * inv - T(0.5);
  v.y = (p.y - origin[1]) * inv - T(0.5);
  v.z = (p.z - origin[2]) * inv - T(0.5);
  bool valid = true;
  if (v.x < T(-0.5) || v.x >= (T)dim[0] - T(0.5) || v.y < T(-0.5) ||
      v.y >= (T)dim[1] - T(0.5) || v.z < T(-0.5) || v.z >= (T)dim[2] - T(0.5))
    valid = false;
  return valid;
}
// d_gpw_Get_Position_in_World (_yooji_cuda_math.h:285-302)
template <class T>
inline V3<T> pos_in_world(V3<T> v, const T* origin, T inv) {
  return {(v.x + T(0.5)) / inv + origin[0], (v.y + T(0.5)) / inv + origin[1],
          (v.z + T(0.5)) / inv + origin[2]};
}

// ---------------------------------------------------------------------------
// half precision conversion (IEEE binary16, round to nearest even), used for
// the FP16 TSDF storage variant of the precision study
// ---------------------------------------------------------------------------
inline uint16_t f2h(float f) {
  uint32_t x;
  std::memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t ax = x & 0x7fffffffu;
  if (ax >= 0x7f800000u) return (uint16_t)(sign | (ax > 0x7f800000u ? 0x7e00u : 0x7c00u));
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to inf
  if (ax < 0x38800000u) {                                      // half subnormal
    if (ax < 0x33000000u) return (uint16_t)sign;               // below half of 2^-24
    int e = (int)(ax >> 23);                                   // 102 .. 112
    uint32_t mant = (ax & 0x7fffffu) | 0x800000u;              // value = mant * 2^(e-150)
    int sh = 126 - e;                                          // q = mant * 2^(e-126) units of 2^-24
    uint32_t q = mant >> sh;
    uint32_t rem = mant & ((1u << sh) - 1u);
    uint32_t halfway = 1u << (sh - 1);
    if (rem > halfway || (rem == halfway && (q & 1u))) q++;
    return (uint16_t)(sign | q);
  }
  uint32_t e = (ax >> 23) - 112;  // rebias 127 -> 15
  uint32_t m = ax & 0x7fffffu;
  uint32_t h = (e << 10) | (m >> 13);
  uint32_t rem = m & 0x1fffu;
  if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
  return (uint16_t)(sign | h);
}
inline float h2f(uint16_t h) {
  uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
  uint32_t e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
  uint32_t x;
  if (e == 0) {
    if (m == 0) {
      x = sign;
    } else {
      float f = std::ldexp((float)m, -24);
      std::memcpy(&x, &f, 4);
      x |= sign;
    }
  } else if (e == 31) {
    x = sign | 0x7f800000u | (m << 13);
  } else {
    x = sign | ((e + 112) << 23) | (m << 13);
  }
  float f;
  std::memcpy(&f, &x, 4);
  return f;
}

const float kQ = 32767.0f;
const float kInvQ = 1.0f / 32767.0f;

// storage rounding of a freshly averaged TSDF value
template <class T>
inline T store_tsdf(T v, int /*mode*/) {
  return v;
}
template <>
inline float store_tsdf<float>(float v, int mode) {
  if (mode == 1) {
    float q = std::nearbyint(v * kQ);
    if (q > 32767.0f) q = 32767.0f;
    if (q < -32767.0f) q = -32767.0f;
    return q * kInvQ;
  }
  if (mode == 2) return h2f(f2h(v));
  return v;
}

// ---------------------------------------------------------------------------
// configuration expanded per level
// ---------------------------------------------------------------------------
template <class T>
struct Cfg {
  int W[3], H[3];
  T K[3][4];
  int levels;
  int dim[3];
  T origin[3];
  T vox, vox_inv, mu, max_w, th_icp, r_cube;
  T center[3];
  float cos_normal;
  int iters[3];
  int tsdf_store, reduce_mode;
  float depth_scale;
};

// intrinsics pyramid: z_yooji_cuda_pose_tracker.cu:764-776 and
// z_yooji_cuda_tsdf_renderer.cu:1611-1623 (same rule as the CPU
// dih_Downsample_Intrinsics_Half, z_yooji_image_processor.cpp:599-612)
template <class T>
Cfg<T> expand(const or_config* c) {
  Cfg<T> g;
  std::memset(&g, 0, sizeof(g));
  g.levels = c->levels;
  T fx = (T)c->fx, fy = (T)c->fy, px = (T)c->cx, py = (T)c->cy;
  int w = c->width, h = c->height;
  for (int k = 0; k < 3; k++) {
    g.W[k] = w;
    g.H[k] = h;
    g.K[k][0] = fx;
    g.K[k][1] = fy;
    g.K[k][2] = px;
    g.K[k][3] = py;
    fx = T(0.5) * fx;
    fy = T(0.5) * fy;
    px = T(0.5) * (px - T(0.5));
    py = T(0.5) * (py - T(0.5));
    w /= 2;
    h /= 2;
  }
  for (int k = 0; k < 3; k++) {
    g.dim[k] = c->dim[k];
    g.origin[k] = (T)c->origin[k];
  }
  g.vox = (T)c->voxel_size;
  g.vox_inv = T(1) / g.vox;  // z_yooji_cuda_volume_integrator.cu:847
  g.mu = (T)c->mu;
  g.max_w = (T)c->max_w;
  g.th_icp = (T)c->th_icp;
  // cube centre = origin + dim*sz_vox/2 (z_yooji_object_scanner.cpp:306)
  for (int k = 0; k < 3; k++) g.center[k] = g.origin[k] + (T)g.dim[k] * g.vox / T(2);
  V3<T> d = v3(g.origin[0] - g.center[0], g.origin[1] - g.center[1], g.origin[2] - g.center[2]);
  g.r_cube = length(d);  // z_yooji_cuda_tsdf_renderer.cu:1601
  g.cos_normal = c->cos_normal;
  for (int k = 0; k < 3; k++) g.iters[k] = c->icp_iters[k];
  g.tsdf_store = c->tsdf_store;
  g.reduce_mode = c->reduce_mode;
  g.depth_scale = c->depth_scale;
  return g;
}

// ---------------------------------------------------------------------------
// a2: bilateral filter, z_yooji_cuda_img_proc.cu:86-141 (kernel), :275-286
// (Gaussian table), constants :42-45 (sigma_s = 4 px, sigma_r = 0.1 m, r = 2).
// The reference samples a linear-filtered float texture at integer
// coordinates (:119,126,214-217): each tap is the mean of the 2x2 texels
// (X-1..X, Y-1..Y).  The texture asks for mirror addressing, which CUDA only
// honours for normalised coordinates; with the unnormalised coordinates used
// here the texture unit clamps to the edge, so taps clamp.
// ---------------------------------------------------------------------------
template <class T>
void gaussian_table(T delta, int radius, T* g) {
  for (int i = 0; i < 2 * radius + 1; ++i) {
    T x = (T)(i - radius);
    g[i] = std::exp(-(x * x) / (2 * delta * delta));
  }
}

template <class T>
inline T tex_tap(const T* img, int w, int h, int X, int Y) {
  auto at = [&](int x, int y) {
    x = x < 0 ? 0 : (x >= w ? w - 1 : x);
    y = y < 0 ? 0 : (y >= h ? h - 1 : y);
    return img[(size_t)y * w + x];
  };
  return T(0.25) * ((at(X - 1, Y - 1) + at(X, Y - 1)) + (at(X - 1, Y) + at(X, Y)));
}

template <class T>
void bilateral(const T* in, int w, int h, T* out) {
  const int r = 2;
  const T e_d = (T)0.1f;
  T g[5];
  gaussian_table<T>((T)4.0f, r, g);
  const T denom = T(2) * e_d * e_d;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < h; y++) {
    for (int x = 0; x < w; x++) {
      T sum = 0, t = 0;
      T center = tex_tap(in, w, h, x, y);
      bool zero = false;
      for (int i = -r; i <= r && !zero; i++) {
        for (int j = -r; j <= r; j++) {
          T cur = tex_tap(in, w, h, x + j, y + i);
          if (cur <= T(0)) {
            zero = true;
            break;
          }
          T mod = (center - cur) * (center - cur);
          T factor = g[i + r] * g[j + r] * std::exp(-mod / denom);
          t += factor * cur;
          sum += factor;
        }
      }
      out[(size_t)y * w + x] = zero ? T(0) : t / sum;
    }
  }
}

// ---------------------------------------------------------------------------
// a4: depth pyramid.  cpdd_Construct_Pyramids_Down_Depth
// (z_yooji_image_processor.cpp:368-407) = sdg5_Smooth_Depthmap_Gaussian_5x5
// (:857-937, [1 4 6 4 1] separable, no validity mask, borders 0) followed by
// ddh_Downsample_Depthmap_Half (:567-596, keep pixel (2i+1, 2j+1)).
// ---------------------------------------------------------------------------
template <class T>
void pyramid_down(const T* in, int w, int h, T* out) {
  std::vector<T> pad((size_t)w * h, T(0)), sm((size_t)w * h, T(0));
  const T f0 = 1, f1 = 4, f2 = 6;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < h; j++)
    for (int i = 2; i < w - 2; i++) {
      const T* p = in + (size_t)j * w;
      pad[(size_t)j * w + i] = f0 * p[i - 2] + f0 * p[i + 2] + f1 * p[i - 1] + f1 * p[i + 1] + f2 * p[i];
    }
#pragma omp parallel for schedule(static)
  for (int i = 2; i < w - 2; i++)
    for (int j = 2; j < h - 2; j++) {
      const T* p = pad.data() + i;
      sm[(size_t)j * w + i] =
          (f0 * p[(size_t)(j - 2) * w] + f0 * p[(size_t)(j + 2) * w] + f1 * p[(size_t)(j - 1) * w] +
           f1 * p[(size_t)(j + 1) * w] + f2 * p[(size_t)j * w]) /
          (T(16) * T(16));
    }
  int w2 = w / 2, h2 = h / 2;
  for (int j2 = 0; j2 < h2; j2++)
    for (int i2 = 0; i2 < w2; i2++) out[(size_t)j2 * w2 + i2] = sm[(size_t)(2 * j2 + 1) * w + (2 * i2 + 1)];
}

// ---------------------------------------------------------------------------
// a5: input vertex / normal maps.  cpm_Compute_Point_Map
// (z_yooji_image_processor.cpp:119-152) and enm_Estimate_Normal_Map
// (:155-227, half window 1).  Invalid = -100.  The normal loop rewrites the
// point map in place when it rejects a normal (-n_z < cos 60 deg), so a
// rejected pixel also invalidates the right and lower neighbours' normals:
// this raster-order side effect is reproduced exactly.
// ---------------------------------------------------------------------------
template <class T>
void point_normal_map(const T* depth, int w, int h, const T* K, T* vtx, T* nrm) {
  size_t n = (size_t)w * h;
  for (size_t k = 0; k < 3 * n; k++) vtx[k] = nrm[k] = T(-100);
#pragma omp parallel for schedule(static)
  for (int i = 0; i < h; i++)
    for (int j = 0; j < w; j++) {
      size_t t = (size_t)i * w + j;
      T d = depth[t];
      if (d <= T(0)) continue;
      V3<T> p = back_project((T)j, (T)i, K, d);
      vtx[3 * t] = p.x;
      vtx[3 * t + 1] = p.y;
      vtx[3 * t + 2] = p.z;
    }
  const double cos60 = std::cos(M_PI * 60.0 / 180.0);
  for (int i = 1; i < h - 1; i++)
    for (int j = 1; j < w - 1; j++) {
      size_t t = (size_t)i * w + j;
      const T* c = vtx + 3 * t;
      const T* x1 = vtx + 3 * (t - 1);
      const T* x2 = vtx + 3 * (t + 1);
      const T* y1 = vtx + 3 * (t - w);
      const T* y2 = vtx + 3 * (t + w);
      if (c[0] == T(-100) || x1[0] == T(-100) || x2[0] == T(-100) || y1[0] == T(-100) ||
          y2[0] == T(-100))
        continue;
      T dx = x2[0] - x1[0];
      if (std::fabs(dx) < T(1.0e-7f)) continue;
      T dy = y2[1] - y1[1];
      if (std::fabs(dy) < T(1.0e-7f)) continue;
      T dzdx = (x2[2] - x1[2]) / dx;
      T dzdy = (y2[2] - y1[2]) / dy;
      T len = tsqrt(dzdx * dzdx + dzdy * dzdy + T(1));
      T nx = dzdx / len, ny = dzdy / len, nz = T(-1) / len;
      if (-(double)nz < cos60) {
        vtx[3 * t] = vtx[3 * t + 1] = vtx[3 * t + 2] = T(-100);
        continue;  // normal stays -100
      }
      nrm[3 * t] = nx;
      nrm[3 * t + 1] = ny;
      nrm[3 * t + 2] = nz;
    }
}

// ---------------------------------------------------------------------------
// a6: per-pixel ICP term, d_cssfp_Compute_Single_Summand_with_Forward_Params
// (z_yooji_cuda_pose_tracker.cu:279-395) with the bilinear model lookups
// d_giv / d_gin (_yooji_cuda_math.h:365-481).  Taps that get zero weight are
// not read; their value is taken as 0 (the reference leaves them
// uninitialised).
// ---------------------------------------------------------------------------
template <class T>
inline bool bilinear3(T xf, T yf, int w, int h, const float* map, V3<T>& out) {
  // NaN coordinates (a point at z = 0) are rejected; the reference leaves
  // them to an undefined float-to-int conversion
  if (!(xf >= T(0) && xf <= T(w - 1) && yf >= T(0) && yf <= T(h - 1))) return false;
  int x = (int)xf, y = (int)yf;
  T rx = xf - (T)x, ry = yf - (T)y;
  V3<T> a{0, 0, 0}, b{0, 0, 0}, c{0, 0, 0}, d{0, 0, 0};
  const float* p = map + 3 * ((size_t)y * w + x);
  if (p[0] == -100.0f) return false;
  a = v3<T>(p[0], p[1], p[2]);
  if (rx > T(0)) {
    p = map + 3 * ((size_t)y * w + x + 1);
    if (p[0] == -100.0f) return false;
    b = v3<T>(p[0], p[1], p[2]);
  }
  if (ry > T(0)) {
    p = map + 3 * ((size_t)(y + 1) * w + x);
    if (p[0] == -100.0f) return false;
    c = v3<T>(p[0], p[1], p[2]);
  }
  if (rx > T(0) && ry > T(0)) {
    p = map + 3 * ((size_t)(y + 1) * w + x + 1);
    if (p[0] == -100.0f) return false;
    d = v3<T>(p[0], p[1], p[2]);
  }
  T ix = T(1) - rx, iy = T(1) - ry;
  out.x = iy * (ix * a.x + rx * b.x) + ry * (ix * c.x + rx * d.x);
  out.y = iy * (ix * a.y + rx * b.y) + ry * (ix * c.y + rx * d.y);
  out.z = iy * (ix * a.z + rx * b.z) + ry * (ix * c.z + rx * d.z);
  return true;
}

template <class T>
inline bool icp_term(int x, int y, int w, int h, const T* K, const float* depth,
                     const float* mvtx, const float* mnrm, const float* nnrm, const T* T21,
                     T th_icp, float cos_normal, T A[6], T& b) {
  T d1 = (T)depth[(size_t)y * w + x];
  if (d1 < T(1.0e-6f)) return false;
  V3<T> tp = back_project((T)x, (T)y, K, d1);
  V3<T> p1 = transform(tp, T21);
  T u, v;
  project(p1, K, u, v);
  V3<T> p0;
  if (!bilinear3(u, v, w, h, mvtx, p0)) return false;
  T dd = (p0.x - p1.x) * (p0.x - p1.x) + (p0.y - p1.y) * (p0.y - p1.y) + (p0.z - p1.z) * (p0.z - p1.z);
  if (dd > th_icp) return false;
  V3<T> n;
  if (!bilinear3(u, v, w, h, mnrm, n)) return false;
  n = normalised(n);
  if (cos_normal > -2.0f && nnrm) {
    // build extension (not in the reference): reject when the input normal,
    // rotated into the model frame, is more than acos(cos_normal) away from
    // the model normal.
    const float* q = nnrm + 3 * ((size_t)y * w + x);
    if (q[0] == -100.0f) return false;
    V3<T> nin = rotate(v3<T>(q[0], q[1], q[2]), T21);
    if (dot(nin, n) < (T)cos_normal) return false;
  }
  A[0] = p1.z * n.y + (-p1.y) * n.z;
  A[1] = (-p1.z) * n.x + p1.x * n.z;
  A[2] = p1.y * n.x + (-p1.x) * n.y;
  A[3] = -n.x;
  A[4] = -n.y;
  A[5] = -n.z;
  b = dot(n, p0 - p1);
  return true;
}

// 27 unique sums in the order (i<=j row-major upper triangle of ATA: 21), ATb (6)
inline int tri_index(int i, int j) {  // i <= j
  return i * 6 - i * (i - 1) / 2 + (j - i);
}

// a7: reduction.  Mode 0 restates the reference: a 16x16 thread block per
// tile, a shared-memory tree (256 -> 1, :623-669) per quantity, then a serial
// float sum of block partials on the host (:937-943).
template <class T>
void icp_sums(const Cfg<T>& g, int lev, const float* depth, const float* mvtx, const float* mnrm,
              const float* nnrm, const T* T21, double* out29) {
  const int w = g.W[lev], h = g.H[lev];
  const T* K = g.K[lev];
  for (int k = 0; k < 29; k++) out29[k] = 0;
  const int mode = g.reduce_mode;
  auto term = [&](int x, int y, T v[29]) -> bool {
    T A[6], b;
    for (int k = 0; k < 29; k++) v[k] = 0;
    if (!icp_term(x, y, w, h, K, depth, mvtx, mnrm, nnrm, T21, g.th_icp, g.cos_normal, A, b))
      return false;
    for (int i = 0; i < 6; i++)
      for (int j = i; j < 6; j++) v[tri_index(i, j)] = A[i] * A[j];
    for (int i = 0; i < 6; i++) v[21 + i] = A[i] * b;
    v[27] = 1;
    v[28] = b * b;
    return true;
  };
  if (mode == 0) {
    int gx = (w + 15) / 16, gy = (h + 15) / 16;
    std::vector<T> part((size_t)gx * gy * 29);
#pragma omp parallel
    {
      std::vector<T> cache((size_t)256 * 29);
#pragma omp for schedule(static)
      for (int bidx = 0; bidx < gx * gy; bidx++) {
        int bx = bidx % gx, by = bidx / gx;
        for (int ty = 0; ty < 16; ty++)
          for (int tx = 0; tx < 16; tx++) {
            int x = bx * 16 + tx, y = by * 16 + ty, cidx = tx + ty * 16;
            T v[29];
            for (int k = 0; k < 29; k++) v[k] = 0;
            if (x < w && y < h) term(x, y, v);
            for (int k = 0; k < 29; k++) cache[(size_t)cidx * 29 + k] = v[k];
          }
        for (int i = 128; i != 0; i /= 2)
          for (int c = 0; c < i; c++)
            for (int k = 0; k < 29; k++) cache[(size_t)c * 29 + k] += cache[(size_t)(c + i) * 29 + k];
        for (int k = 0; k < 29; k++) part[(size_t)bidx * 29 + k] = cache[k];
      }
    }
    T host[29];
    for (int k = 0; k < 29; k++) host[k] = 0;
    for (int bidx = 0; bidx < gx * gy; bidx++)
      for (int k = 0; k < 29; k++) host[k] += part[(size_t)bidx * 29 + k];
    for (int k = 0; k < 29; k++) out29[k] = (double)host[k];
    return;
  }
  T acc[29], comp[29];
  double dacc[29];
  for (int k = 0; k < 29; k++) acc[k] = comp[k] = 0, dacc[k] = 0;
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      T v[29];
      if (!term(x, y, v)) continue;
      for (int k = 0; k < 29; k++) {
        if (mode == 1) {
          acc[k] += v[k];
        } else if (mode == 2) {  // Kahan compensated
          T yk = v[k] - comp[k];
          T tk = acc[k] + yk;
          comp[k] = (tk - acc[k]) - yk;
          acc[k] = tk;
        } else {
          dacc[k] += (double)v[k];
        }
      }
    }
  for (int k = 0; k < 29; k++) out29[k] = (mode == 3) ? dacc[k] : (double)acc[k];
}

// ---------------------------------------------------------------------------
// a8: 6x6 solve and pose update.
// d_lld_LL_Decomposition / d_sls_Solve_Linear_System_using_LLD
// (_yooji_cuda_math.h:489-592), convergence |x|_inf < 5e-7
// (z_yooji_cuda_pose_tracker.cu:971-972), z_uitme (:50-149) = exp(xi)*T,
// d_im_Inverse_Matrix_4x4 (_yooji_math_inlines.h:404-465).
// ---------------------------------------------------------------------------
template <class T>
void cholesky(const T* A, T* L) {
  for (int i = 0; i < 36; i++) L[i] = T(0);
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      if (i < j) continue;
      if (i == j) {
        T s = 0;
        for (int k = 0; k < j; k++) s += L[j * 6 + k] * L[j * 6 + k];
        L[j * 6 + j] = tsqrt(A[j * 6 + j] - s);
      } else if (std::fabs(L[j * 6 + j]) >= T(1e-8f)) {
        T s = 0;
        for (int k = 0; k < j; k++) s += L[i * 6 + k] * L[j * 6 + k];
        L[i * 6 + j] = (A[i * 6 + j] - s) / L[j * 6 + j];
      } else {
        L[i * 6 + j] = T(0);
      }
    }
}
template <class T>
bool chol_solve(const T* L, const T* b, T* x) {
  for (int i = 0; i < 6; i++)
    if (std::fabs(L[i * 6 + i]) < T(1.0e-8f)) return false;
  T y[6];
  for (int i = 0; i < 6; i++) {
    T s = 0;
    for (int k = 0; k < i; k++) s += L[i * 6 + k] * y[k];
    y[i] = (b[i] - s) / L[i * 6 + i];
  }
  for (int i = 5; i >= 0; i--) {
    T s = 0;
    for (int k = i + 1; k < 6; k++) s += L[k * 6 + i] * x[k];
    x[i] = (y[i] - s) / L[i * 6 + i];
  }
  return true;
}
// d_niv_Norm_Infinity_Vector (_yooji_math_inlines.h:57-62): a NaN entry never
// raises the running maximum (its comparison is false)
template <class T>
T norm_inf(const T* x) {
  T n = T(-100000.0f);
  for (int i = 0; i < 6; i++) {
    T a = std::fabs(x[i]);
    if (n < a) n = a;
  }
  return n;
}

template <class T>
void matmul4(const T* a, const T* b, T* c) {
  for (int j = 0; j < 4; j++)
    for (int i = 0; i < 4; i++) {
      T s = 0;
      for (int k = 0; k < 4; k++) s += a[j * 4 + k] * b[k * 4 + i];
      c[j * 4 + i] = s;
    }
}

// exp(xi) of the twist xi = [w; v] (Ma et al., eq. 2.30), as
// z_uitme_Update_Incremental_Tracking_with_Matrix_Exponential builds it: w is
// normalised by theta = |w|, v is divided by theta, R = I + sin(theta)[w]x +
// (1-cos(theta))[w]x^2, t = (I-R)[w]x v + w w^T v theta.  The reference
// divides by theta unguarded (0/0 for a zero rotation); here theta == 0 takes
// the limit R = I, t = v.
template <class T>
void se3_exp(const T* xi, T* E) {
  T w[3] = {xi[0], xi[1], xi[2]};
  T theta = 0;
  for (int i = 0; i < 3; i++) theta += w[i] * w[i];
  theta = tsqrt(theta);
  for (int i = 0; i < 16; i++) E[i] = T(0);
  E[15] = T(1);
  if (theta == T(0)) {
    E[0] = E[5] = E[10] = T(1);
    E[3] = xi[3];
    E[7] = xi[4];
    E[11] = xi[5];
    return;
  }
  T v[3];
  for (int i = 0; i < 3; i++) w[i] /= theta;
  for (int i = 0; i < 3; i++) v[i] = xi[3 + i] / theta;
  T wx[9] = {T(0), -w[2], w[1], w[2], T(0), -w[0], -w[1], w[0], T(0)};
  T wx2[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      T s = 0;
      for (int k = 0; k < 3; k++) s += wx[j * 3 + k] * wx[k * 3 + i];
      wx2[j * 3 + i] = s;
    }
  T sn = std::sin(theta), cs = T(1) - std::cos(theta);
  T tm[9], R[9];
  for (int i = 0; i < 9; i++) tm[i] = sn * wx[i] + cs * wx2[i];
  for (int i = 0; i < 9; i++) R[i] = tm[i];
  R[0] += T(1);
  R[4] += T(1);
  R[8] += T(1);
  for (int i = 0; i < 9; i++) tm[i] *= T(-1);
  T tm2[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      T s = 0;
      for (int k = 0; k < 3; k++) s += tm[j * 3 + k] * wx[k * 3 + i];
      tm2[j * 3 + i] = s;
    }
  T tv[3];
  for (int j = 0; j < 3; j++) {
    T s = 0;
    for (int i = 0; i < 3; i++) s += tm2[j * 3 + i] * v[i];
    tv[j] = s;
  }
  T ts = 0;
  for (int i = 0; i < 3; i++) ts += w[i] * v[i];
  ts *= theta;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) E[j * 4 + i] = R[j * 3 + i];
  for (int j = 0; j < 3; j++) E[j * 4 + 3] = tv[j] + w[j] * ts;
}

template <class T>
bool inverse4(const T* m, T* o) {
  T m11 = m[0], m12 = m[1], m13 = m[2], m14 = m[3];
  T m21 = m[4], m22 = m[5], m23 = m[6], m24 = m[7];
  T m31 = m[8], m32 = m[9], m33 = m[10], m34 = m[11];
  T m41 = m[12], m42 = m[13], m43 = m[14], m44 = m[15];
  T t[12];
  t[0] = m33 * m44;
  t[1] = m34 * m42;
  t[2] = m32 * m43;
  t[3] = m34 * m43;
  t[4] = m32 * m44;
  t[5] = m33 * m42;
  t[6] = m31 * m44;
  t[7] = m33 * m41;
  t[8] = m34 * m41;
  t[9] = m31 * m43;
  t[10] = m31 * m42;
  t[11] = m32 * m41;
  o[0] = m22 * t[0] + m23 * t[1] + m24 * t[2] - m22 * t[3] - m23 * t[4] - m24 * t[5];
  o[1] = m12 * t[3] + m13 * t[4] + m14 * t[5] - m12 * t[0] - m13 * t[1] - m14 * t[2];
  o[2] = m12 * m23 * m44 + m13 * m24 * m42 + m14 * m22 * m43 - m12 * m24 * m43 - m13 * m22 * m44 - m14 * m23 * m42;
  o[3] = m12 * m24 * m33 + m13 * m22 * m34 + m14 * m23 * m32 - m12 * m23 * m34 - m13 * m24 * m32 - m14 * m22 * m33;
  T det = m11 * o[0] + m21 * o[1] + m31 * o[2] + m41 * o[3];
  if (det == T(0)) return false;
  o[4] = m21 * t[3] + m23 * t[6] + m24 * t[7] - m21 * t[0] - m23 * t[8] - m24 * t[9];
  o[5] = m11 * t[0] + m13 * t[8] + m14 * t[9] - m11 * t[3] - m13 * t[6] - m14 * t[7];
  o[6] = m11 * m24 * m43 + m13 * m21 * m44 + m14 * m23 * m41 - m11 * m23 * m44 - m13 * m24 * m41 - m14 * m21 * m43;
  o[7] = m11 * m23 * m34 + m13 * m24 * m31 + m14 * m21 * m33 - m11 * m24 * m33 - m13 * m21 * m34 - m14 * m23 * m31;
  o[8] = m21 * t[4] + m22 * t[8] + m24 * t[10] - m21 * t[1] - m22 * t[6] - m24 * t[11];
  o[9] = m11 * t[1] + m12 * t[6] + m14 * t[11] - m11 * t[4] - m12 * t[8] - m14 * t[10];
  o[10] = m11 * m22 * m44 + m12 * m24 * m41 + m14 * m21 * m42 - m11 * m24 * m42 - m12 * m21 * m44 - m14 * m22 * m41;
  o[11] = m11 * m24 * m32 + m12 * m21 * m34 + m14 * m22 * m31 - m11 * m22 * m34 - m12 * m24 * m31 - m14 * m21 * m32;
  o[12] = m21 * t[5] + m22 * t[9] + m23 * t[11] - m21 * t[2] - m22 * t[7] - m23 * t[10];
  o[13] = m11 * t[2] + m12 * t[11] + m13 * t[10] - m11 * t[5] - m12 * t[9] - m13 * t[11];
  o[14] = m11 * m23 * m42 + m12 * m21 * m43 + m13 * m22 * m41 - m11 * m22 * m43 - m12 * m23 * m41 - m13 * m21 * m42;
  o[15] = m11 * m22 * m33 + m12 * m23 * m31 + m13 * m21 * m32 - m11 * m23 * m32 - m12 * m21 * m33 - m13 * m22 * m31;
  det = T(1) / det;
  for (int i = 0; i < 16; i++) o[i] *= det;
  return true;
}

// tp_Track_Pose (z_yooji_cuda_pose_tracker.cu:790-1042): coarse to fine over
// levels n = L-1 .. 0 (only level 0 with an initial increment), iterations
// per level from the configuration, T_12 <- exp(x) T_12, T_21 = inv(T_12),
// final T_gc <- T_12 T_gc.
template <class T>
int track(const Cfg<T>& g, const float* const* depth, const float* const* mvtx,
          const float* const* mnrm, const float* const* nnrm, const T* T_gc_prev,
          const T* init_T12, T* T_gc_out, int* info) {
  T T12[16], T21[16];
  for (int i = 0; i < 16; i++) T12[i] = T21[i] = (i % 4 == i / 4) ? T(1) : T(0);
  int lev = g.levels;
  if (init_T12) {
    for (int i = 0; i < 16; i++) T12[i] = init_T12[i];
    inverse4(T12, T21);
    lev = 1;
  }
  bool valid = true;
  int total = 0, last_count = 0;
  for (int n = lev - 1; n >= 0; n--) {
    for (int it = 0; it < g.iters[n]; it++) {
      if (!valid) break;
      double s[29];
      icp_sums(g, n, depth[n], mvtx[n], mnrm[n], nnrm ? nnrm[n] : nullptr, T21, s);
      total++;
      last_count = (int)s[27];
      T A[36], bv[6], L[36], x[6];
      for (int i = 0; i < 6; i++)
        for (int j = i; j < 6; j++) A[i * 6 + j] = A[j * 6 + i] = (T)s[tri_index(i, j)];
      for (int i = 0; i < 6; i++) bv[i] = (T)s[21 + i];
      cholesky(A, L);
      valid = chol_solve(L, bv, x);
      if (!valid) break;
      if (norm_inf(x) < T(5.0e-7f)) break;
      T E[16], tmp[16];
      se3_exp(x, E);
      matmul4(E, T12, tmp);
      for (int i = 0; i < 16; i++) T12[i] = tmp[i];
      inverse4(T12, T21);
    }
  }
  if (info) {
    info[0] = total;
    info[1] = last_count;
  }
  if (!valid) return 0;
  matmul4(T12, T_gc_prev, T_gc_out);
  return 1;
}

// ---------------------------------------------------------------------------
// volume
// ---------------------------------------------------------------------------
template <class T>
struct Volume {
  Cfg<T> g;
  std::vector<T> tsdf;
  std::vector<uint16_t> w;
  std::vector<uint8_t> flags;  // 8^3 sub-cube activity of the last frame
  std::vector<uint8_t> col;    // cube_color: R, G, B planes, x fastest (empty until colour is used)
  int nsc[3];
  void init(const Cfg<T>& c) {
    g = c;
    size_t n = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
    // setDeviceMem3D(tsdf, 1.0f), z_yooji_object_scanner.cpp:347 (in the
    // storage format: int16 keeps 32767, read back as 32767/32767)
    tsdf.assign(n, store_tsdf<T>(T(1), g.tsdf_store));
    w.assign(n, 0);
    for (int k = 0; k < 3; k++) nsc[k] = (g.dim[k] + 7) / 8;
    flags.assign((size_t)nsc[0] * nsc[1] * nsc[2], 0);
    col.clear();
  }
  void enable_color() {
    if (col.empty()) col.assign((size_t)3 * g.dim[0] * g.dim[1] * g.dim[2], 0);
  }
};

// a9: g_fvsc_Find_Visible_Sub_Cubes (z_yooji_cuda_volume_integrator.cu:84-152)
// after the per-frame flag reset (:1006-1010)
template <class T>
void find_visible_subcubes(Volume<T>& V, const float* depth, const T* T_cg) {
  const Cfg<T>& g = V.g;
  const int w = g.W[0], h = g.H[0];
  const T* K = g.K[0];
  std::fill(V.flags.begin(), V.flags.end(), 0);
#pragma omp parallel for schedule(static)
  for (int ty = 0; ty < h; ty++)
    for (int tx = 0; tx < w; tx++) {
      T td = (T)depth[(size_t)ty * w + tx];
      if (!(td > T(0))) continue;
      V3<T> p = transform(back_project((T)tx, (T)ty, K, td), T_cg);
      V3<T> pe = transform(back_project((T)tx, (T)ty, K, T(100.0f)), T_cg);
      V3<T> dv = normalised(pe - p);
      for (int n = -4; n <= 1; n++) {
        V3<T> tp = p + (((T)n) * g.mu) * dv;
        V3<T> vox;
        if (!pos_in_voxel(tp, g.origin, g.dim, g.vox_inv, vox)) continue;
        int xs = roundf_div_ref(vox.x, 8), ys = roundf_div_ref(vox.y, 8), zs = roundf_div_ref(vox.z, 8);
        if (xs < 0 || xs >= V.nsc[0] || ys < 0 || ys >= V.nsc[1] || zs < 0 || zs >= V.nsc[2]) break;
        uint8_t& f = V.flags[((size_t)zs * V.nsc[1] + ys) * V.nsc[0] + xs];
#pragma omp atomic write
        f = 1;
      }
    }
}

// a10: g_ctvc_Compute_TSDF_of_Voxels_with_Color, depth part
// (z_yooji_cuda_volume_integrator.cu:265-402), for every voxel of an
// activated sub-cube.
template <class T>
void update_tsdf(Volume<T>& V, const float* depth, const T* T_gc, const T* T_cg) {
  const Cfg<T>& g = V.g;
  const int w = g.W[0], h = g.H[0];
  const T* K = g.K[0];
  const int X = g.dim[0], Y = g.dim[1];
  const int nsc = V.nsc[0] * V.nsc[1] * V.nsc[2];
#pragma omp parallel for schedule(dynamic, 16)
  for (int sc = 0; sc < nsc; sc++) {
    const int xs = sc % V.nsc[0], ys = (sc / V.nsc[0]) % V.nsc[1], zs = sc / (V.nsc[0] * V.nsc[1]);
        if (!V.flags[sc]) continue;
        for (int lz = 0; lz < 8; lz++)
          for (int ly = 0; ly < 8; ly++)
            for (int lx = 0; lx < 8; lx++) {
              int xc = xs * 8 + lx, yc = ys * 8 + ly, zc = zs * 8 + lz;
              V3<T> pg = pos_in_world(v3<T>((T)xc, (T)yc, (T)zc), g.origin, g.vox_inv);
              V3<T> pc = transform(pg, T_gc);
              T u, v;
              project(pc, K, u, v);
              int x = float2int_rn(u), y = float2int_rn(v);
              if (x < 0 || x > w - 1 || y < 0 || y > h - 1) continue;
              T dm = (T)depth[(size_t)y * w + x];
              if (!(dm > T(0))) continue;
              V3<T> r = back_project((T)x, (T)y, K, T(1));
              T lam = T(1) / tsqrt(r.x * r.x + r.y * r.y + T(1));
              V3<T> dc = v3(pg.x - T_cg[3], pg.y - T_cg[7], pg.z - T_cg[11]);
              T nrm = tsqrt(dc.x * dc.x + dc.y * dc.y + dc.z * dc.z);
              T sdf = dm - lam * nrm;
              if (sdf < -g.mu) continue;
              T ts = std::fmin(T(1), sdf / g.mu);
              size_t idx = ((size_t)zc * Y + yc) * X + xc;
              T oldW = (T)V.w[idx];
              T newW = oldW + T(1);
              T inewW = T(1) / newW;
              if (oldW >= g.max_w) continue;
              V.tsdf[idx] = store_tsdf<T>((oldW * V.tsdf[idx] + ts) * inewW, g.tsdf_store);
              V.w[idx] = (uint16_t)newW;
            }
      }
}

// d_gii_Get_Interpolated_Intensity (_yooji_cuda_math.h:305-332) on one 8-bit
// plane: bilinear, a used texel <= 0 fails; NaN coordinates fail (the
// reference's comparisons let them through to an undefined conversion).
template <class T>
bool interp_intensity(T xf, T yf, int w, int h, const uint8_t* map, T& out) {
  if (!(xf >= T(0) && xf <= (T)(w - 1) && yf >= T(0) && yf <= (T)(h - 1))) return false;
  int x = (int)xf, y = (int)yf;
  T rx = xf - (T)x, ry = yf - (T)y;
  T d2 = 0, d3 = 0, d4 = 0;
  T d1 = (T)map[(size_t)y * w + x];
  if (d1 <= T(0)) return false;
  if (rx > T(0)) {
    d2 = (T)map[(size_t)y * w + x + 1];
    if (d2 <= T(0)) return false;
  }
  if (ry > T(0)) {
    d3 = (T)map[(size_t)(y + 1) * w + x];
    if (d3 <= T(0)) return false;
  }
  if (rx > T(0) && ry > T(0)) {
    d4 = (T)map[(size_t)(y + 1) * w + x + 1];
    if (d4 <= T(0)) return false;
  }
  out = (T(1) - ry) * ((T(1) - rx) * d1 + rx * d2) + ry * ((T(1) - rx) * d3 + rx * d4);
  return true;
}

// g_ctvc_Compute_TSDF_of_Voxels_with_Color, depth and colour
// (z_yooji_cuda_volume_integrator.cu:265-455), registered colour
// (flag_on_rgb: the colour is sampled at the voxel's projection into the
// depth camera).  The colour planes have the depth image's size, as the
// reference indexes them (&img_color[k*ww*hh]).  A channel that cannot be
// interpolated leaves the voxel's colour unchanged (the reference would blend
// an uninitialised value).
template <class T>
void update_tsdf_color(Volume<T>& V, const float* depth, const uint8_t* rgb, const T* T_gc, const T* T_cg) {
  const Cfg<T>& g = V.g;
  const int w = g.W[0], h = g.H[0];
  const T* K = g.K[0];
  const int X = g.dim[0], Y = g.dim[1];
  const size_t n3 = (size_t)X * Y * g.dim[2], n2 = (size_t)w * h;
  V.enable_color();
  const int nsc = V.nsc[0] * V.nsc[1] * V.nsc[2];
#pragma omp parallel for schedule(dynamic, 16)
  for (int sc = 0; sc < nsc; sc++) {
    const int xs = sc % V.nsc[0], ys = (sc / V.nsc[0]) % V.nsc[1], zs = sc / (V.nsc[0] * V.nsc[1]);
    if (!V.flags[sc]) continue;
    for (int lz = 0; lz < 8; lz++)
      for (int ly = 0; ly < 8; ly++)
        for (int lx = 0; lx < 8; lx++) {
          int xc = xs * 8 + lx, yc = ys * 8 + ly, zc = zs * 8 + lz;
          V3<T> pg = pos_in_world(v3<T>((T)xc, (T)yc, (T)zc), g.origin, g.vox_inv);
          V3<T> pc = transform(pg, T_gc);
          T u, v;
          project(pc, K, u, v);
          int x = float2int_rn(u), y = float2int_rn(v);
          if (x < 0 || x > w - 1 || y < 0 || y > h - 1) continue;
          T dm = (T)depth[(size_t)y * w + x];
          if (!(dm > T(0))) continue;
          V3<T> r = back_project((T)x, (T)y, K, T(1));
          T lam = T(1) / tsqrt(r.x * r.x + r.y * r.y + T(1));
          V3<T> dc = v3(pg.x - T_cg[3], pg.y - T_cg[7], pg.z - T_cg[11]);
          T nrm = tsqrt(dc.x * dc.x + dc.y * dc.y + dc.z * dc.z);
          T sdf = dm - lam * nrm;
          if (sdf < -g.mu) continue;
          T ts = std::fmin(T(1), sdf / g.mu);
          size_t idx = ((size_t)zc * Y + yc) * X + xc;
          T oldW = (T)V.w[idx];
          T newW = oldW + T(1);
          T inewW = T(1) / newW;
          if (oldW >= g.max_w) continue;
          V.tsdf[idx] = store_tsdf<T>((oldW * V.tsdf[idx] + ts) * inewW, g.tsdf_store);
          V.w[idx] = (uint16_t)newW;
          T smp[3];
          bool ok = true;
          for (int k = 0; k < 3; k++) ok = ok && interp_intensity(u, v, w, h, rgb + k * n2, smp[k]);
          if (!ok) continue;
          for (int k = 0; k < 3; k++) {
            uint8_t& c = V.col[idx + k * n3];
            c = (uint8_t)(std::fmax(T(0), std::fmin(T(255.0f), (oldW * (T)c + smp[k]) * inewW)));
          }
        }
  }
}

// ---------------------------------------------------------------------------
// a11/a12: raycast.  g_rmi_Render_Maps_for_ICP (z_yooji_cuda_tsdf_renderer.cu:
// 1069-1209), d_crtc_Cast_Ray_on_TSDF_Cube_NEW (:466-635), d_gtvu (:68-97),
// d_gtvi (:100-153), d_csnt (:288-464), host set-up (:1642-1700).
// ---------------------------------------------------------------------------
template <class T>
inline bool gtvu(const Volume<T>& V, V3<T> p, T& out) {
  out = T(1);
  if (std::isnan(p.x) || std::isnan(p.y) || std::isnan(p.z)) return false;
  int x = roundf_ref(p.x), y = roundf_ref(p.y), z = roundf_ref(p.z);
  const int* d = V.g.dim;
  if (x < 0 || x >= d[0] || y < 0 || y >= d[1] || z < 0 || z >= d[2]) return false;
  size_t idx = ((size_t)z * d[1] + y) * d[0] + x;
  if (V.w[idx] == 0) return false;
  out = V.tsdf[idx];
  return true;
}
// ITMMath Vector3f::toInt(residual): the reference's CPU twin of this lookup
// truncates (z_yooji_cube_tsdf_float.cpp:376-378); floor is used, which is the
// same for the non-negative coordinates inside the cube.
template <class T>
inline void to_int_floor(V3<T> p, int o[3], V3<T>& r) {
  T fx = std::floor(p.x), fy = std::floor(p.y), fz = std::floor(p.z);
  o[0] = (int)fx;
  o[1] = (int)fy;
  o[2] = (int)fz;
  r = v3(p.x - fx, p.y - fy, p.z - fz);
}
template <class T>
inline bool gtvi(const Volume<T>& V, V3<T> p, T& out) {
  out = T(1);
  if (std::isnan(p.x) || std::isnan(p.y) || std::isnan(p.z)) return false;
  int o[3];
  V3<T> r;
  to_int_floor(p, o, r);
  static const int dx1[4] = {0, 1, 0, 1}, dy1[4] = {0, 0, 1, 1};
  T f[4], b[4];
  for (int i = 0; i < 4; i++)
    if (!gtvu(V, v3<T>((T)(o[0] + dx1[i]), (T)(o[1] + dy1[i]), (T)o[2]), f[i])) return false;
  for (int i = 0; i < 4; i++)
    if (!gtvu(V, v3<T>((T)(o[0] + dx1[i]), (T)(o[1] + dy1[i]), (T)(o[2] + 1)), b[i])) return false;
  T inf = (T(1) - r.y) * ((T(1) - r.x) * f[0] + r.x * f[1]) + r.y * ((T(1) - r.x) * f[2] + r.x * f[3]);
  T inb = (T(1) - r.y) * ((T(1) - r.x) * b[0] + r.x * b[1]) + r.y * ((T(1) - r.x) * b[2] + r.x * b[3]);
  out = (T(1) - r.z) * inf + r.z * inb;
  return true;
}

template <class T>
bool surface_normal(const Volume<T>& V, V3<T> p3d, V3<T>& nout) {
  const Cfg<T>& g = V.g;
  V3<T> vox;
  if (!pos_in_voxel(p3d, g.origin, g.dim, g.vox_inv, vox)) return false;
  if (std::isnan(vox.x) || std::isnan(vox.y) || std::isnan(vox.z)) return false;
  int o[3];
  V3<T> r;
  to_int_floor(vox, o, r);
  static const int dx1[4] = {0, 1, 0, 1}, dy1[4] = {0, 0, 1, 1};
  static const int dx2[12] = {0, 1, -1, 0, 1, 2, -1, 0, 1, 2, 0, 1};
  static const int dy2[12] = {-1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2};
  T fm[4], fr[12], bk[12], bm[4];
  for (int i = 0; i < 4; i++)
    if (!gtvu(V, v3<T>((T)(o[0] + dx1[i]), (T)(o[1] + dy1[i]), (T)(o[2] - 1)), fm[i])) return false;
  for (int i = 0; i < 12; i++)
    if (!gtvu(V, v3<T>((T)(o[0] + dx2[i]), (T)(o[1] + dy2[i]), (T)o[2]), fr[i])) return false;
  for (int i = 0; i < 12; i++)
    if (!gtvu(V, v3<T>((T)(o[0] + dx2[i]), (T)(o[1] + dy2[i]), (T)(o[2] + 1)), bk[i])) return false;
  for (int i = 0; i < 4; i++)
    if (!gtvu(V, v3<T>((T)(o[0] + dx1[i]), (T)(o[1] + dy1[i]), (T)(o[2] + 2)), bm[i])) return false;
  const T rx = r.x, ry = r.y, rz = r.z;
  T a4[4], b4[4], a2[2], b2[2], gx, gy, gz;
  a4[0] = (T(1) - rz) * fr[2] + rz * bk[2];
  a4[1] = (T(1) - rz) * fr[3] + rz * bk[3];
  a4[2] = (T(1) - rz) * fr[4] + rz * bk[4];
  a4[3] = (T(1) - rz) * fr[5] + rz * bk[5];
  b4[0] = (T(1) - rz) * fr[6] + rz * bk[6];
  b4[1] = (T(1) - rz) * fr[7] + rz * bk[7];
  b4[2] = (T(1) - rz) * fr[8] + rz * bk[8];
  b4[3] = (T(1) - rz) * fr[9] + rz * bk[9];
  a2[0] = (T(1) - rx) * a4[0] + rx * a4[1];
  a2[1] = (T(1) - rx) * b4[0] + rx * b4[1];
  b2[0] = (T(1) - rx) * a4[2] + rx * a4[3];
  b2[1] = (T(1) - rx) * b4[2] + rx * b4[3];
  gx = (T(1) - ry) * b2[0] + ry * b2[1];
  gx -= (T(1) - ry) * a2[0] + ry * a2[1];
  a4[0] = (T(1) - rz) * fr[0] + rz * bk[0];
  a4[1] = (T(1) - rz) * fr[3] + rz * bk[3];
  a4[2] = (T(1) - rz) * fr[7] + rz * bk[7];
  a4[3] = (T(1) - rz) * fr[10] + rz * bk[10];
  b4[0] = (T(1) - rz) * fr[1] + rz * bk[1];
  b4[1] = (T(1) - rz) * fr[4] + rz * bk[4];
  b4[2] = (T(1) - rz) * fr[8] + rz * bk[8];
  b4[3] = (T(1) - rz) * fr[11] + rz * bk[11];
  a2[0] = (T(1) - ry) * a4[0] + ry * a4[1];
  a2[1] = (T(1) - ry) * b4[0] + ry * b4[1];
  b2[0] = (T(1) - ry) * a4[2] + ry * a4[3];
  b2[1] = (T(1) - ry) * b4[2] + ry * b4[3];
  gy = (T(1) - rx) * b2[0] + rx * b2[1];
  gy -= (T(1) - rx) * a2[0] + rx * a2[1];
  a4[0] = (T(1) - ry) * fm[0] + ry * fm[2];
  a4[1] = (T(1) - ry) * fr[3] + ry * fr[7];
  a4[2] = (T(1) - ry) * bk[3] + ry * bk[7];
  a4[3] = (T(1) - ry) * bm[0] + ry * bm[2];
  b4[0] = (T(1) - ry) * fm[1] + ry * fm[3];
  b4[1] = (T(1) - ry) * fr[4] + ry * fr[8];
  b4[2] = (T(1) - ry) * bk[4] + ry * bk[8];
  b4[3] = (T(1) - ry) * bm[1] + ry * bm[3];
  a2[0] = (T(1) - rz) * a4[0] + rz * a4[1];
  a2[1] = (T(1) - rz) * b4[0] + rz * b4[1];
  b2[0] = (T(1) - rz) * a4[2] + rz * a4[3];
  b2[1] = (T(1) - rz) * b4[2] + rz * b4[3];
  gz = (T(1) - rx) * b2[0] + rx * b2[1];
  gz -= (T(1) - rx) * a2[0] + rx * a2[1];
  if (gx == T(0) && gy == T(0) && gz == T(0)) return false;
  nout = normalised(v3(gx, gy, gz));
  return true;
}

// The reference loop has no iteration bound; a ray whose fine steps keep
// alternating direction never ends there.  Both this restatement and the
// CUDA kernel stop after max_ray_iterations() steps and report no hit.
inline int max_ray_iterations(float total_step_max) { return 4 * (int)total_step_max + 64; }

// object mode: d_crtc_Cast_Ray_on_TSDF_Cube_NEW (z_yooji_cuda_tsdf_renderer.cu
// :466-635), the ray segment through the cube's bounding sphere, rays outside
// the cube's view cone rejected; scene mode: d_crtcs_Cast_Ray_on_TSDF_Cube_for
// _Scene (:908-1066), from the camera centre to 2 r_cube, no cone test.  The
// march itself is the same in both.
template <class T>
bool cast_ray(const Volume<T>& V, int lev, T px, T py, const T* T_cg, V3<T> cam, V3<T> ncc,
              T dist_cc, T theta_max, V3<T>& p3d, bool scene = false) {
  const Cfg<T>& g = V.g;
  enum { COARSE, FINE, BEHIND };
  T dmin = scene ? T(0) : dist_cc - g.r_cube, dmax = scene ? T(2) * g.r_cube : dist_cc + g.r_cube;
  V3<T> pe = transform(back_project(px, py, g.K[lev], dmax), T_cg);
  V3<T> rd = normalised(pe - cam);
  if (!scene) {
    T theta = std::acos(dot(rd, ncc));
    if (theta > theta_max) return false;
  }
  V3<T> ps = cam + dmin * rd;
  T step_scale = T(0.9f) * g.mu * g.vox_inv;
  T step = step_scale, coarse = step_scale;
  T total_max = T(2) * g.r_cube * g.vox_inv;
  T total = 0, tsdf;
  V3<T> vs;
  pos_in_voxel(ps, g.origin, g.dim, g.vox_inv, vs);
  int state;
  bool ok = gtvu(V, vs, tsdf);
  if (!ok)
    state = COARSE;
  else if (tsdf >= T(0))
    state = FINE;
  else
    return false;
  const int cap = max_ray_iterations((float)total_max);
  int it = 0;
  while (state != BEHIND) {
    if (++it > cap) return false;
    if (state == COARSE)
      step = coarse;
    else
      step = (tsdf > T(0)) ? std::fmax(step_scale * tsdf, T(1)) : std::fmin(step_scale * tsdf, T(-1));
    vs = vs + step * rd;
    total += step;
    if (total > total_max) break;
    gtvu(V, vs, tsdf);
    if (tsdf > T(-1) && tsdf < T(1)) {
      gtvi(V, vs, tsdf);
      if (tsdf < T(0)) {
        if (state == COARSE) break;
        state = BEHIND;
      } else if (tsdf == T(0)) {
        p3d = pos_in_world(vs, g.origin, g.vox_inv);
        return true;
      } else if (state == COARSE) {
        state = FINE;
      }
    }
    // else: the reference's `state == SEARCH_COARSE;` (:591) is a no-op
  }
  if (state == BEHIND) {
    step = step_scale * tsdf;
    vs = vs + step * rd;
    gtvi(V, vs, tsdf);
    step = step_scale * tsdf;
    vs = vs + step * rd;
    p3d = pos_in_world(vs, g.origin, g.vox_inv);
    return true;
  }
  return false;
}

// d_grvi_Get_RGB_Value_Interpolated (z_yooji_cuda_tsdf_renderer.cu:232-284)
// with d_grvu (:194-229) for the eight neighbours (in range, weight > 0), and
// InfiniTAM's Vector3f::toUChar: round half away from zero, clamp 0..255.
template <class T>
void trilinear_color(const Volume<T>& V, V3<T> pg, uint8_t out[3]) {
  out[0] = out[1] = out[2] = 0;
  if (V.col.empty()) return;
  const Cfg<T>& g = V.g;
  V3<T> pv;
  pos_in_voxel(pg, g.origin, g.dim, g.vox_inv, pv);
  if (std::isnan(pv.x) || std::isnan(pv.y) || std::isnan(pv.z)) return;
  int o[3];
  V3<T> r;
  to_int_floor(pv, o, r);
  const size_t n3 = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
  size_t idx[8];
  for (int i = 0; i < 8; i++) {
    int x = o[0] + (i & 1), y = o[1] + ((i >> 1) & 1), z = o[2] + (i >> 2);
    if (x < 0 || x >= g.dim[0] || y < 0 || y >= g.dim[1] || z < 0 || z >= g.dim[2]) return;
    idx[i] = ((size_t)z * g.dim[1] + y) * g.dim[0] + x;
    if (V.w[idx[i]] == 0) return;
  }
  for (int k = 0; k < 3; k++) {
    T f[4], b[4];
    for (int i = 0; i < 4; i++) {
      f[i] = (T)V.col[idx[i] + k * n3];
      b[i] = (T)V.col[idx[4 + i] + k * n3];
    }
    T inf = (T(1) - r.y) * ((T(1) - r.x) * f[0] + r.x * f[1]) + r.y * ((T(1) - r.x) * f[2] + r.x * f[3]);
    T inb = (T(1) - r.y) * ((T(1) - r.x) * b[0] + r.x * b[1]) + r.y * ((T(1) - r.x) * b[2] + r.x * b[3]);
    T val = (T(1) - r.z) * inf + r.z * inb;
    T rounded = (val < T(0)) ? (val - T(0.5f)) : (val + T(0.5f));
    out[k] = (uint8_t)std::fmax(T(0), std::fmin(T(255.0f), rounded));
  }
}

// d_grvu_Get_RGB_Value_Uninterpolated (z_yooji_cuda_tsdf_renderer.cu:155-229):
// the colour of the nearest voxel (ROUNDF) when it is in range with weight > 0,
// else 0.  The reference's Vector3u overload reads the green plane for red
// (:178), and the scene kernel writes green into the red plane (:1432-1434,
// marked there as temporary); the true red is returned here.
template <class T>
void nearest_color(const Volume<T>& V, V3<T> pg, uint8_t out[3]) {
  out[0] = out[1] = out[2] = 0;
  if (V.col.empty()) return;
  const Cfg<T>& g = V.g;
  V3<T> pv;
  pos_in_voxel(pg, g.origin, g.dim, g.vox_inv, pv);
  if (std::isnan(pv.x) || std::isnan(pv.y) || std::isnan(pv.z)) return;
  const int x = roundf_ref(pv.x), y = roundf_ref(pv.y), z = roundf_ref(pv.z);
  if (x < 0 || x >= g.dim[0] || y < 0 || y >= g.dim[1] || z < 0 || z >= g.dim[2]) return;
  const size_t n3 = (size_t)g.dim[0] * g.dim[1] * g.dim[2];
  const size_t i = ((size_t)z * g.dim[1] + y) * g.dim[0] + x;
  if (V.w[i] == 0) return;
  for (int k = 0; k < 3; k++) out[k] = V.col[i + k * n3];
}

// render variants (bits of `mode`), as the CUDA library's
enum { kRayScene = 1, kRayGlobalNormals = 2, kRayNearestColor = 4, kRayWhiteBackground = 8 };

// mode 0: g_rmi_Render_Maps_for_ICP (z_yooji_cuda_tsdf_renderer.cu:1070-1209);
// kRayScene | kRayGlobalNormals | kRayNearestColor: g_rmis with a vertex map
// (:1338-1446); kRayScene | kRayGlobalNormals: g_rmis without one
// (:1448-1548); kRayGlobalNormals | kRayWhiteBackground: g_rmi without one
// (:1211-1336).  vtx may be NULL.
template <class T>
void raycast(const Volume<T>& V, int lev, const T* T_gc, const T* T_cg, V3<T> cam, V3<T> light,
             T* depth, T* vtx, T* nrm, uint8_t* img, uint8_t* rgb = nullptr, int mode = 0) {
  const Cfg<T>& g = V.g;
  const int w = g.W[lev], h = g.H[lev];
  V3<T> cc = v3(g.center[0], g.center[1], g.center[2]);
  V3<T> vcc = cc - cam;
  V3<T> ncc = normalised(vcc);
  T dist_cc = length(vcc);
  T theta_max = std::asin(g.r_cube / dist_cc);
#pragma omp parallel for schedule(dynamic, 4)
  for (int ty = 0; ty < h; ty++)
    for (int tx = 0; tx < w; tx++) {
      size_t t = (size_t)ty * w + tx;
      V3<T> pg, sn;
      bool valid = cast_ray(V, lev, (T)tx, (T)ty, T_cg, cam, ncc, dist_cc, theta_max, pg, (mode & kRayScene) != 0);
      if (valid && surface_normal(V, pg, sn)) {
        V3<T> pc = transform(pg, T_gc);
        depth[t] = pc.z;
        if (vtx) {
          vtx[3 * t] = pc.x;
          vtx[3 * t + 1] = pc.y;
          vtx[3 * t + 2] = pc.z;
        }
        V3<T> sc = (mode & kRayGlobalNormals) ? sn : rotate(sn, T_gc);
        nrm[3 * t] = sc.x;
        nrm[3 * t + 1] = sc.y;
        nrm[3 * t + 2] = sc.z;
        T ang = sc.x * light.x + sc.y * light.y + sc.z * light.z;
        T s = (T(0.8f) * ang + T(0.2f)) * T(255.0f);
        s = std::fmax(T(0), std::fmin(T(255.0f), s));
        img[t] = (uint8_t)s;
        if (rgb) {
          uint8_t c[3];
          if (mode & kRayNearestColor)
            nearest_color(V, pg, c);
          else
            trilinear_color(V, pg, c);
          for (int k = 0; k < 3; k++) rgb[t + k * (size_t)w * h] = c[k];
        }
      } else {
        depth[t] = 0;
        if (vtx) vtx[3 * t] = vtx[3 * t + 1] = vtx[3 * t + 2] = T(-100);
        nrm[3 * t] = nrm[3 * t + 1] = nrm[3 * t + 2] = T(-100);
        img[t] = 0;
        if (rgb)
          for (int k = 0; k < 3; k++) rgb[t + k * (size_t)w * h] = (mode & kRayWhiteBackground) ? 255 : 0;
      }
    }
}

// ---------------------------------------------------------------------------
// surface extraction: marching tetrahedra over the cells whose eight corners
// have weight > 0; six tetrahedra around the (0,0,0)-(1,1,1) diagonal; a vertex
// is the linear zero crossing on an edge, in world coordinates; triangles face
// the positive side; colour mixed along the edge with the same weight and
// rounded (half up).  Same operations and corner order as the CUDA kernel.
// ---------------------------------------------------------------------------
template <class T>
uint64_t extract_mesh(const Volume<T>& V, float* xyz, uint8_t* rgb, uint64_t capacity) {
  static const int tet[6][4] = {{0, 7, 1, 3}, {0, 7, 3, 2}, {0, 7, 2, 6}, {0, 7, 6, 4}, {0, 7, 4, 5}, {0, 7, 5, 1}};
  const Cfg<T>& g = V.g;
  const int X = g.dim[0], Y = g.dim[1], Z = g.dim[2];
  const size_t n3 = (size_t)X * Y * Z;
  uint64_t count = 0;
  struct EV {
    V3<T> p;
    T c[3];
  };
  auto emit = [&](const EV& a, const EV& b, const EV& c, V3<T> ci, V3<T> co) {
    V3<T> u = b.p - a.p, v = c.p - a.p;
    V3<T> n = v3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
    V3<T> d = co - ci;
    bool flip = (n.x * d.x + n.y * d.y + n.z * d.z) < T(0);
    const EV* t[3] = {&a, flip ? &c : &b, flip ? &b : &c};
    if (count < capacity) {
      for (int k = 0; k < 3; k++) {
        xyz[9 * count + 3 * k] = (float)t[k]->p.x;
        xyz[9 * count + 3 * k + 1] = (float)t[k]->p.y;
        xyz[9 * count + 3 * k + 2] = (float)t[k]->p.z;
        if (rgb)
          for (int ch = 0; ch < 3; ch++)
            rgb[9 * count + 3 * k + ch] = (uint8_t)std::fmin(T(255.0f), std::fmax(T(0), t[k]->c[ch] + T(0.5f)));
      }
    }
    count++;
  };
  for (int z = 0; z + 1 < Z; z++)
    for (int y = 0; y + 1 < Y; y++)
      for (int x = 0; x + 1 < X; x++) {
        T v[8], col[8][3];
        bool ok = true;
        for (int c = 0; c < 8 && ok; c++) {
          size_t idx = ((size_t)(z + (c >> 2)) * Y + (y + ((c >> 1) & 1))) * X + (x + (c & 1));
          ok = V.w[idx] != 0;
          v[c] = V.tsdf[idx];
          for (int k = 0; k < 3; k++) col[c][k] = V.col.empty() ? T(0) : (T)V.col[idx + k * n3];
        }
        if (!ok) continue;
        unsigned neg = 0;
        for (int c = 0; c < 8; c++) neg |= (v[c] < T(0) ? 1u : 0u) << c;
        if (neg == 0u || neg == 0xffu) continue;
        auto P = [&](int c) { return v3<T>((T)(x + (c & 1)), (T)(y + ((c >> 1) & 1)), (T)(z + (c >> 2))); };
        auto E = [&](int a, int c) {
          T t = (T(0) - v[a]) / (v[c] - v[a]);
          V3<T> pa = P(a), pb = P(c);
          V3<T> pv = v3(pa.x + t * (pb.x - pa.x), pa.y + t * (pb.y - pa.y), pa.z + t * (pb.z - pa.z));
          EV e;
          e.p = pos_in_world(pv, g.origin, g.vox_inv);
          for (int k = 0; k < 3; k++) e.c[k] = col[a][k] + t * (col[c][k] - col[a][k]);
          return e;
        };
        for (int t = 0; t < 6; t++) {
          int in[4], out[4], ni = 0, no = 0;
          for (int k = 0; k < 4; k++) {
            int c = tet[t][k];
            if ((neg >> c) & 1u)
              in[ni++] = c;
            else
              out[no++] = c;
          }
          if (ni == 0 || no == 0) continue;
          V3<T> ci = v3<T>(0, 0, 0), co = v3<T>(0, 0, 0);
          for (int k = 0; k < ni; k++) ci = ci + P(in[k]);
          for (int k = 0; k < no; k++) co = co + P(out[k]);
          ci = (T(1) / (T)ni) * ci;
          co = (T(1) / (T)no) * co;
          if (ni == 1 || no == 1) {
            int lone = (ni == 1) ? in[0] : out[0];
            const int* rest = (ni == 1) ? out : in;
            emit(E(lone, rest[0]), E(lone, rest[1]), E(lone, rest[2]), ci, co);
          } else {
            EV e00 = E(in[0], out[0]), e01 = E(in[0], out[1]), e11 = E(in[1], out[1]), e10 = E(in[1], out[0]);
            emit(e00, e01, e11, ci, co);
            emit(e00, e11, e10, ci, co);
          }
        }
      }
  return count;
}

// ---------------------------------------------------------------------------
// session: so_Scan_Object hot path (z_yooji_object_scanner.cpp:472-629)
// ---------------------------------------------------------------------------
template <class T>
struct Session {
  Cfg<T> g;
  Volume<T> V;
  T T_gc[16], T_cg[16];
  V3<T> center;
  int frame = 0;
  std::vector<float> raw, lvl[3], in_nrm[3], in_vtx[3];
  std::vector<float> mdepth[3], mvtx[3], mnrm[3];
  std::vector<uint8_t> mimg[3];
  void init(const or_config* c) {
    g = expand<T>(c);
    V.init(g);
    for (int i = 0; i < 16; i++) T_gc[i] = T_cg[i] = (i % 4 == i / 4) ? T(1) : T(0);
    center = v3<T>(0, 0, 0);
    raw.assign((size_t)g.W[0] * g.H[0], 0.f);
    for (int l = 0; l < 3; l++) {
      size_t n = (size_t)g.W[l] * g.H[l];
      lvl[l].assign(n, 0.f);
      in_vtx[l].assign(3 * n, -100.f);
      in_nrm[l].assign(3 * n, -100.f);
      mdepth[l].assign(n, 0.f);
      mvtx[l].assign(3 * n, -100.f);
      mnrm[l].assign(3 * n, -100.f);
      mimg[l].assign(n, 0);
    }
  }
  // set_transform (_yooji_cuda_tracking_state.h:59-94)
  void set_pose(const T* Tgc) {
    for (int i = 0; i < 16; i++) T_gc[i] = Tgc[i];
    inverse4(T_gc, T_cg);
    center = camera_center(T_gc);
  }
  int step(const uint16_t* mm) {
    const int w0 = g.W[0], h0 = g.H[0];
    size_t n0 = (size_t)w0 * h0;
    for (size_t i = 0; i < n0; i++) raw[i] = (float)mm[i] * g.depth_scale;
    // z_uid: bilateral of the raw depth -> level 0 of the pyramid
    if (std::is_same<T, float>::value) {
      bilateral<float>(raw.data(), w0, h0, lvl[0].data());
    } else {
      std::vector<double> a(raw.begin(), raw.end()), b(n0);
      bilateral<double>(a.data(), w0, h0, b.data());
      for (size_t i = 0; i < n0; i++) lvl[0][i] = (float)b[i];
    }
    // z_cip: pyramid
    for (int l = 1; l < g.levels; l++) {
      if (std::is_same<T, float>::value) {
        pyramid_down<float>(lvl[l - 1].data(), g.W[l - 1], g.H[l - 1], lvl[l].data());
      } else {
        std::vector<double> a(lvl[l - 1].begin(), lvl[l - 1].end()), b((size_t)g.W[l] * g.H[l]);
        pyramid_down<double>(a.data(), g.W[l - 1], g.H[l - 1], b.data());
        for (size_t i = 0; i < b.size(); i++) lvl[l][i] = (float)b[i];
      }
    }
    // input vertex / normal maps (needed by the normal rejection test)
    if (g.cos_normal > -2.0f) {
      for (int l = 0; l < g.levels; l++) {
        size_t n = (size_t)g.W[l] * g.H[l];
        std::vector<T> d(lvl[l].begin(), lvl[l].end()), vv(3 * n), nn(3 * n);
        point_normal_map<T>(d.data(), g.W[l], g.H[l], g.K[l], vv.data(), nn.data());
        for (size_t i = 0; i < 3 * n; i++) in_vtx[l][i] = (float)vv[i], in_nrm[l][i] = (float)nn[i];
      }
    }
    // z_ecp: track (skipped on the first frame, zz_flag_track false)
    int ok = 1;
    if (frame > 0) {
      const float* dp[3] = {lvl[0].data(), lvl[1].data(), lvl[2].data()};
      const float* vp[3] = {mvtx[0].data(), mvtx[1].data(), mvtx[2].data()};
      const float* np[3] = {mnrm[0].data(), mnrm[1].data(), mnrm[2].data()};
      const float* ip[3] = {in_nrm[0].data(), in_nrm[1].data(), in_nrm[2].data()};
      T out[16];
      ok = track(g, dp, vp, np, g.cos_normal > -2.0f ? ip : nullptr, T_gc, (const T*)nullptr, out,
                 nullptr);
      if (ok) set_pose(out);
    }
    frame++;
    if (!ok) return 0;
    // z_uom: integrate the raw depth (z_yooji_object_scanner.cpp:1274-1281)
    find_visible_subcubes(V, raw.data(), T_cg);
    update_tsdf(V, raw.data(), T_gc, T_cg);
    // z_uts: raycast every level, light (0,0,-1) (:1313, :1333-1356)
    for (int l = 0; l < g.levels; l++) {
      size_t n = (size_t)g.W[l] * g.H[l];
      std::vector<T> d(n), vv(3 * n), nn(3 * n);
      raycast(V, l, T_gc, T_cg, center, v3<T>(0, 0, -1), d.data(), vv.data(), nn.data(),
              mimg[l].data());
      for (size_t i = 0; i < n; i++) mdepth[l][i] = (float)d[i];
      for (size_t i = 0; i < 3 * n; i++) mvtx[l][i] = (float)vv[i], mnrm[l][i] = (float)nn[i];
    }
    return 1;
  }
};

}  // namespace

// ===========================================================================
// C API
// ===========================================================================
struct or_volume {
  Volume<float> v;
};
struct or_session {
  or_config cfg;
  Session<float>* f = nullptr;
  Session<double>* d = nullptr;
  or_volume view;  // float view of the volume (refreshed on request)
};

extern "C" {

void or_depth_to_m(const uint16_t* in, int n, float scale, float* out) {
  for (int i = 0; i < n; i++) out[i] = (float)in[i] * scale;
}
void or_gaussian_table(float delta, int radius, float* out) { gaussian_table<float>(delta, radius, out); }
void or_bilateral(const float* in, int w, int h, float* out) { bilateral<float>(in, w, h, out); }
void or_pyramid_down(const float* in, int w, int h, float* out) { pyramid_down<float>(in, w, h, out); }
void or_point_normal_map(const float* depth, int w, int h, const float K[4], float* vtx3, float* nrm3) {
  point_normal_map<float>(depth, w, h, K, vtx3, nrm3);
}
void or_level_intrinsics(const float K0[4], int levels, float* Kl) {
  or_config c;
  std::memset(&c, 0, sizeof(c));
  c.fx = K0[0];
  c.fy = K0[1];
  c.cx = K0[2];
  c.cy = K0[3];
  c.width = 1 << 12;
  c.height = 1 << 12;
  c.levels = levels;
  c.voxel_size = 1;
  Cfg<float> g = expand<float>(&c);
  for (int l = 0; l < levels && l < 3; l++)
    for (int k = 0; k < 4; k++) Kl[4 * l + k] = g.K[l][k];
}

int or_track(const or_config* cfg, const float* const* depth, const float* const* mvtx,
             const float* const* mnrm, const float* const* nnrm, const float* T_gc_prev,
             const float* init_T12, float* T_gc_out, int* info) {
  Cfg<float> g = expand<float>(cfg);
  return track<float>(g, depth, mvtx, mnrm, nnrm, T_gc_prev, init_T12, T_gc_out, info);
}
int or_track_f64(const or_config* cfg, const float* const* depth, const float* const* mvtx,
                 const float* const* mnrm, const float* const* nnrm, const double* T_gc_prev,
                 const double* init_T12, double* T_gc_out, int* info) {
  Cfg<double> g = expand<double>(cfg);
  return track<double>(g, depth, mvtx, mnrm, nnrm, T_gc_prev, init_T12, T_gc_out, info);
}
int or_icp_sums(const or_config* cfg, int level, const float* depth, const float* mvtx,
                const float* mnrm, const float* nnrm, const float* T21, double* out29) {
  Cfg<float> g = expand<float>(cfg);
  icp_sums<float>(g, level, depth, mvtx, mnrm, nnrm, T21, out29);
  return (int)out29[27];
}

void or_pose_inverse(const float* T, float* Tinv) { inverse4<float>(T, Tinv); }
void or_camera_center(const float* T_gc, float* c) {
  V3<float> v = camera_center(T_gc);
  c[0] = v.x;
  c[1] = v.y;
  c[2] = v.z;
}
void or_se3_exp(const float* xi, float* T) { se3_exp<float>(xi, T); }
void or_se3_exp_f64(const double* xi, double* T) { se3_exp<double>(xi, T); }

or_volume* or_volume_create(const or_config* cfg) {
  or_volume* v = new or_volume;
  v->v.init(expand<float>(cfg));
  return v;
}
void or_volume_destroy(or_volume* v) { delete v; }
void or_volume_reset(or_volume* v) { v->v.init(v->v.g); }
void or_volume_get(const or_volume* v, float* tsdf, uint16_t* w) {
  if (tsdf) std::memcpy(tsdf, v->v.tsdf.data(), v->v.tsdf.size() * sizeof(float));
  if (w) std::memcpy(w, v->v.w.data(), v->v.w.size() * sizeof(uint16_t));
}
void or_volume_set(or_volume* v, const float* tsdf, const uint16_t* w) {
  if (tsdf) std::memcpy(v->v.tsdf.data(), tsdf, v->v.tsdf.size() * sizeof(float));
  if (w) std::memcpy(v->v.w.data(), w, v->v.w.size() * sizeof(uint16_t));
}
void or_volume_flags(const or_volume* v, uint8_t* flags) {
  std::memcpy(flags, v->v.flags.data(), v->v.flags.size());
}
void or_integrate(or_volume* v, const float* depth, const float* T_gc, const float* T_cg) {
  find_visible_subcubes(v->v, depth, T_cg);
  update_tsdf(v->v, depth, T_gc, T_cg);
}
void or_integrate_color(or_volume* v, const float* depth, const uint8_t* rgb, const float* T_gc,
                        const float* T_cg) {
  find_visible_subcubes(v->v, depth, T_cg);
  update_tsdf_color(v->v, depth, rgb, T_gc, T_cg);
}
void or_volume_get_color(or_volume* v, uint8_t* rgb) {
  v->v.enable_color();
  std::memcpy(rgb, v->v.col.data(), v->v.col.size());
}
void or_volume_set_color(or_volume* v, const uint8_t* rgb) {
  v->v.enable_color();
  std::memcpy(v->v.col.data(), rgb, v->v.col.size());
}
void or_raycast_color(const or_volume* v, int level, const float* T_gc, const float* T_cg, const float* cam_cen,
                      const float* light, float* depth, float* vtx3, float* nrm3, uint8_t* img, uint8_t* rgb) {
  raycast<float>(v->v, level, T_gc, T_cg, v3(cam_cen[0], cam_cen[1], cam_cen[2]),
                 v3(light[0], light[1], light[2]), depth, vtx3, nrm3, img, rgb);
}
// z_tdrcc_Transform_Depth_to_Rgb_Camera_Coordinates
// (z_yooji_object_scanner.cpp:2429-2476), raster order, z-buffer keeping the
// smaller depth; NaN projections are dropped (the reference's ROUNDF of NaN is
// undefined)
void or_warp_depth(const float* depth, int wd, int hd, const float* Kd, const float* T, const float* Kr, int wr,
                   int hr, float* out) {
  for (int i = 0; i < wr * hr; i++) out[i] = 0.0f;
  for (int j = 0; j < hd; j++)
    for (int i = 0; i < wd; i++) {
      float td = depth[(size_t)j * wd + i];
      if (!(td > 0.0f)) continue;
      V3<float> p = transform(back_project((float)i, (float)j, Kd, td), T);
      float u, v;
      project(p, Kr, u, v);
      if (std::isnan(u) || std::isnan(v)) continue;
      int tx = roundf_ref(u), ty = roundf_ref(v);
      if (tx < 0 || tx > wr - 1 || ty < 0 || ty > hr - 1) continue;
      float& cur = out[(size_t)ty * wr + tx];
      if (cur > td || cur <= 0.0f) cur = td;
    }
}
void or_render_variant(const or_volume* v, int level, int mode, const float* T_gc, const float* T_cg,
                       const float* cam_cen, const float* light, float* depth, float* vtx3, float* nrm3,
                       uint8_t* img, uint8_t* rgb) {
  raycast<float>(v->v, level, T_gc, T_cg, v3(cam_cen[0], cam_cen[1], cam_cen[2]),
                 v3(light[0], light[1], light[2]), depth, vtx3, nrm3, img, rgb, mode);
}
// g_uvv_Update_Valid_Volume (z_yooji_cuda_volume_integrator.cu:718-799): each
// sub-cube flagged by the last integration (cube_valid) with no valid voxel is
// reset (TSDF 1, weight 0, colour 0) and unflagged; returns the number reset
uint32_t or_update_valid_volume(or_volume* ov, const uint8_t* valid) {
  Volume<float>& V = ov->v;
  const Cfg<float>& g = V.g;
  const int X = g.dim[0], Y = g.dim[1], Z = g.dim[2];
  const size_t n3 = (size_t)X * Y * Z;
  uint32_t carved = 0;
  for (int zs = 0; zs < V.nsc[2]; zs++)
    for (int ys = 0; ys < V.nsc[1]; ys++)
      for (int xs = 0; xs < V.nsc[0]; xs++) {
        uint8_t& f = V.flags[((size_t)zs * V.nsc[1] + ys) * V.nsc[0] + xs];
        if (!f) continue;
        int cnt = 0;
        for (int z = zs * 8; z < zs * 8 + 8 && z < Z; z++)
          for (int y = ys * 8; y < ys * 8 + 8 && y < Y; y++)
            for (int x = xs * 8; x < xs * 8 + 8 && x < X; x++)
              if (valid[((size_t)z * Y + y) * X + x]) cnt++;
        if (cnt > 0) continue;
        f = 0;
        carved++;
        for (int z = zs * 8; z < zs * 8 + 8 && z < Z; z++)
          for (int y = ys * 8; y < ys * 8 + 8 && y < Y; y++)
            for (int x = xs * 8; x < xs * 8 + 8 && x < X; x++) {
              const size_t i = ((size_t)z * Y + y) * X + x;
              V.tsdf[i] = store_tsdf<float>(1.0f, g.tsdf_store);
              V.w[i] = 0;
              if (!V.col.empty())
                for (int k = 0; k < 3; k++) V.col[i + k * n3] = 0;
            }
      }
  return carved;
}
// the expanded cube geometry of a configuration: centre[3], r_cube, 1/voxel
void or_config_geometry(const or_config* cfg, float* out5) {
  const Cfg<float> g = expand<float>(cfg);
  for (int k = 0; k < 3; k++) out5[k] = g.center[k];
  out5[3] = g.r_cube;
  out5[4] = g.vox_inv;
}
// single primitives of the restatement (float), for the reference pin
void or_prim_cholesky6(const float* A, float* L) { cholesky<float>(A, L); }
int or_prim_chol_solve6(const float* L, const float* b, float* x) { return chol_solve<float>(L, b, x) ? 1 : 0; }
int or_prim_bilinear3(float xf, float yf, int w, int h, const float* map3, int normalise, float* out3) {
  V3<float> o{0, 0, 0};
  if (!bilinear3<float>(xf, yf, w, h, map3, o)) return 0;
  if (normalise) o = normalised(o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
  return 1;
}
void or_prim_project(const float* p3, const float* K, float* uv) {
  project<float>(v3<float>(p3[0], p3[1], p3[2]), K, uv[0], uv[1]);
}
void or_prim_back_project(float u, float v, const float* K, float d, float* p3) {
  const V3<float> o = back_project<float>(u, v, K, d);
  p3[0] = o.x, p3[1] = o.y, p3[2] = o.z;
}
void or_prim_transform(const float* p3, const float* T, int rotate_only, float* out3) {
  const V3<float> p = v3<float>(p3[0], p3[1], p3[2]);
  const V3<float> o = rotate_only ? rotate<float>(p, T) : transform<float>(p, T);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
}
int or_prim_pos_in_voxel(const float* p3, const float* origin, const int* dim, float vox_inv, float* out3) {
  V3<float> o;
  const bool ok = pos_in_voxel<float>(v3<float>(p3[0], p3[1], p3[2]), origin, dim, vox_inv, o);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
  return ok ? 1 : 0;
}
int or_prim_icp_term(int x, int y, int w, int h, const float* K, const float* depth, const float* mvtx,
                     const float* mnrm, const float* T21, float th_icp, float* A6, float* b) {
  float A[6], bb = 0;
  if (!icp_term<float>(x, y, w, h, K, depth, mvtx, mnrm, nullptr, T21, th_icp, -3.0f, A, bb)) return 0;
  for (int i = 0; i < 6; i++) A6[i] = A[i];
  *b = bb;
  return 1;
}
void or_prim_pos_in_world(const float* v, const float* origin, float vox_inv, float* out3) {
  const V3<float> o = pos_in_world<float>(v3<float>(v[0], v[1], v[2]), origin, vox_inv);
  out3[0] = o.x, out3[1] = o.y, out3[2] = o.z;
}
uint64_t or_extract_mesh(const or_volume* v, float* xyz, uint8_t* rgb, uint64_t capacity) {
  return extract_mesh<float>(v->v, xyz, rgb, capacity);
}
void or_raycast(const or_volume* v, int level, const float* T_gc, const float* T_cg,
                const float* cam_cen, const float* light, float* depth, float* vtx3, float* nrm3,
                uint8_t* img) {
  raycast<float>(v->v, level, T_gc, T_cg, v3(cam_cen[0], cam_cen[1], cam_cen[2]),
                 v3(light[0], light[1], light[2]), depth, vtx3, nrm3, img);
}

or_session* or_session_create(const or_config* cfg) {
  or_session* s = new or_session;
  s->cfg = *cfg;
  s->f = new Session<float>;
  s->f->init(cfg);
  return s;
}
// FP64 pipeline (precision-study ground truth): same algorithm in double
or_session* or_session_create_f64(const or_config* cfg) {
  or_session* s = new or_session;
  s->cfg = *cfg;
  s->d = new Session<double>;
  s->d->init(cfg);
  return s;
}
void or_session_destroy(or_session* s) {
  delete s->f;
  delete s->d;
  delete s;
}
int or_session_frame(or_session* s, const uint16_t* depth_mm) {
  return s->f ? s->f->step(depth_mm) : s->d->step(depth_mm);
}
void or_session_pose(const or_session* s, float* T_gc) {
  for (int i = 0; i < 16; i++) T_gc[i] = s->f ? s->f->T_gc[i] : (float)s->d->T_gc[i];
}
void or_session_pose_f64(const or_session* s, double* T_gc) {
  for (int i = 0; i < 16; i++) T_gc[i] = s->f ? (double)s->f->T_gc[i] : s->d->T_gc[i];
}
or_volume* or_session_volume(or_session* s) {
  if (s->f) {
    s->view.v.g = s->f->V.g;
    s->view.v.tsdf = s->f->V.tsdf;
    s->view.v.w = s->f->V.w;
    s->view.v.flags = s->f->V.flags;
    for (int k = 0; k < 3; k++) s->view.v.nsc[k] = s->f->V.nsc[k];
  } else {
    const Volume<double>& d = s->d->V;
    s->view.v.g = expand<float>(&s->cfg);
    s->view.v.tsdf.assign(d.tsdf.begin(), d.tsdf.end());
    s->view.v.w = d.w;
    s->view.v.flags = d.flags;
    for (int k = 0; k < 3; k++) s->view.v.nsc[k] = d.nsc[k];
  }
  return &s->view;
}
void or_session_maps(const or_session* s, int level, float* mdepth, float* mvtx3, float* mnrm3,
                     float* in_depth) {
  auto copy = [&](auto* S) {
    size_t n = S->mdepth[level].size();
    if (mdepth) std::memcpy(mdepth, S->mdepth[level].data(), n * 4);
    if (mvtx3) std::memcpy(mvtx3, S->mvtx[level].data(), 3 * n * 4);
    if (mnrm3) std::memcpy(mnrm3, S->mnrm[level].data(), 3 * n * 4);
    if (in_depth) std::memcpy(in_depth, S->lvl[level].data(), n * 4);
  };
  if (s->f)
    copy(s->f);
  else
    copy(s->d);
}

}  // extern "C"
