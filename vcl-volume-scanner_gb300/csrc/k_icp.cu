// Projective point-to-plane ICP, entirely on the device.
//
// The reference (STAC/Engine/GPU/z_yooji_cuda_pose_tracker.cu:548-697 and
// :790-1042) launches one kernel per iteration, copies 1200 x 42 block
// partial sums to the host, adds them serially in FP32, solves the 6x6 system
// with an FP32 Cholesky on the host and copies the new increment back: three
// blocking transfers per iteration.  Here one launch per iteration does it
// all:
//   per pixel   FP32 Jacobian row A (6) and residual b (d_cssfp, :279-395)
//   per thread  accumulation of the 27 unique sums (21 of ATA, 6 of ATb)
//               plus count and sum b^2, in the configured precision
//   per block   warp-shuffle butterfly, then shared memory across warps
//   per grid    single pass: the last block to finish (atomic ticket) sums
//               the block partials in a fixed order, solves the 6x6 system in
//               FP64 (Cholesky LL^T with the reference's failure rules,
//               _yooji_cuda_math.h:489-592), tests convergence
//               (|x|_inf < 5e-7, :971-972) and applies the SE(3) update in
//               FP64 (T_12 <- exp(x) T_12, :976-978)
// Convergence and failure are flags in device memory that the following
// launches read first, so a whole frame of iterations is one CUDA graph with
// no host round trip.  Nothing in these kernels waits on another block.
//
// Batches: one launch per iteration serves every session of a batch table.
// A session at level l owns icp_blocks(W_l H_l) block ranges ("virtual
// blocks"), laid out as they would be in a grid of that size; the persistent
// grid walks the ranges of all sessions, each session has its own partial
// buffer and arrival counter, and the range that arrives last for a session
// reduces and solves that session's system.  Sums therefore run in the same
// order whatever else shares the launch.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int kThreads = 256;

// Bilinear taps of a float4 map at (xf, yf) (d_gii-style interpolation of the
// reference, _yooji_cuda_math.h:365-481): taps with zero weight are neither
// tested nor used (they count as 0), a used tap holding the -100 sentinel
// rejects the sample, and NaN coordinates are rejected (see the oracle).
// The four reads are issued together; a zero-weight tap reads its row/column
// neighbour inside the map and is replaced by 0 before use, which gives the
// read-and-test-in-turn form's result exactly.
struct Taps {
  int i00, i01, i10, i11;
  float rx, ry;
};

__device__ inline bool tap_setup(float xf, float yf, int w, int h, Taps& t) {
  if (!(xf >= 0.0f && xf <= (float)(w - 1) && yf >= 0.0f && yf <= (float)(h - 1))) return false;
  const int x = (int)xf, y = (int)yf;
  t.rx = xf - (float)x;
  t.ry = yf - (float)y;
  const int xb = t.rx > 0.0f ? x + 1 : x, yb = t.ry > 0.0f ? y + 1 : y;
  t.i00 = y * w + x;
  t.i01 = y * w + xb;
  t.i10 = yb * w + x;
  t.i11 = yb * w + xb;
  return true;
}

__device__ inline bool interp(const Taps& t, float4 a, float4 b, float4 c, float4 d, F3& out) {
  const bool ub = t.rx > 0.0f, uc = t.ry > 0.0f, ud = ub && uc;
  if (a.x == -100.0f || (ub && b.x == -100.0f) || (uc && c.x == -100.0f) || (ud && d.x == -100.0f)) return false;
  const F3 A = f3(a.x, a.y, a.z);
  const F3 B = ub ? f3(b.x, b.y, b.z) : f3(0, 0, 0);
  const F3 C = uc ? f3(c.x, c.y, c.z) : f3(0, 0, 0);
  const F3 D = ud ? f3(d.x, d.y, d.z) : f3(0, 0, 0);
  const float rx = t.rx, ry = t.ry, ix = 1.0f - rx, iy = 1.0f - ry;
  out.x = iy * (ix * A.x + rx * B.x) + ry * (ix * C.x + rx * D.x);
  out.y = iy * (ix * A.y + rx * B.y) + ry * (ix * C.y + rx * D.y);
  out.z = iy * (ix * A.z + rx * B.z) + ry * (ix * C.z + rx * D.z);
  return true;
}

// d_cssfp_Compute_Single_Summand_with_Forward_Params.  Two rounds of reads:
// the pixel's depth (and input normal), then the eight model-map taps.
// The per-pixel arithmetic is the reference's, operation for operation
// (IEEE divisions and square root): every pixel's term, and therefore every
// correspondence decision at the distance threshold, equals the float
// oracle's.  (Products with inverse focal lengths, one reciprocal of z and a
// reciprocal square root were 4 % faster, but moved the correspondence set
// of frames whose pixels sit on the threshold, up to 3.5e-4 rad per frame.)
__device__ inline bool icp_term(int x, int y, int w, int h, const float* K, float d1, float4 q,
                                const float4* __restrict__ mvtx, const float4* __restrict__ mnrm, const float* T21,
                                float th_icp, float cos_normal, float A[6], float& b) {
  const bool ntest = cos_normal > -2.0f;
  if (d1 < 1.0e-6f) return false;
  F3 tp = back_project((float)x, (float)y, K, d1);
  F3 p1 = transform(tp, T21);
  float u, v;
  project(p1, K, u, v);
  Taps t;
  if (!tap_setup(u, v, w, h, t)) return false;
  const float4 va = __ldg(mvtx + t.i00), vb = __ldg(mvtx + t.i01), vc = __ldg(mvtx + t.i10), vd = __ldg(mvtx + t.i11);
  F3 p0;
  if (!interp(t, va, vb, vc, vd, p0)) return false;
  float dd = (p0.x - p1.x) * (p0.x - p1.x) + (p0.y - p1.y) * (p0.y - p1.y) + (p0.z - p1.z) * (p0.z - p1.z);
  if (dd > th_icp) return false;
  const float4 na = __ldg(mnrm + t.i00), nb = __ldg(mnrm + t.i01), nc = __ldg(mnrm + t.i10), nd = __ldg(mnrm + t.i11);
  F3 n;
  if (!interp(t, na, nb, nc, nd, n)) return false;
  n = normalised(n);
  if (ntest) {
    if (q.w == 0.0f) return false;
    F3 nin = rotate(f3(q.x, q.y, q.z), T21);
    if (dot(nin, n) < cos_normal) return false;
  }
  A[0] = p1.z * n.y + (-p1.y) * n.z;
  A[1] = (-p1.z) * n.x + p1.x * n.z;
  A[2] = p1.y * n.x + (-p1.x) * n.y;
  A[3] = -n.x;
  A[4] = -n.y;
  A[5] = -n.z;
  b = dot(n, sub(p0, p1));
  return true;
}

// error-free addition (Knuth two-sum): s + e == a + b exactly
__device__ inline void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

// Per-thread sums of the (few) pixels a thread owns are plain float (FP32
// and compensated modes) or double (FP64 mode); the compensated mode carries
// (sum, error) pairs only from the warp reduction on, where thousands of
// values meet, so the pixel loop keeps 29 accumulators in registers.
//
// Warp reduction: a butterfly reduce-scatter over the 29 sums (padded to
// 32).  At the level of lane bit m every lane keeps one half of its current
// values, sends the other half to lane ^ m and adds what it receives, so the
// five levels cost 16 + 8 + 4 + 2 + 1 exchanges instead of 29 per level, and
// lane q ends with the warp's sum of quantity q, in a fixed order.
template <int HALF, int M, class T>
__device__ __forceinline__ void rs_level(T* a, int lane) {
  const bool hi = (lane & M) != 0;
#pragma unroll
  for (int i = 0; i < HALF; i++) {
    const T keep = hi ? a[HALF + i] : a[i];
    const T send = hi ? a[i] : a[HALF + i];
    a[i] = keep + __shfl_xor_sync(0xffffffffu, send, M);
  }
}
template <int HALF, int M>
__device__ __forceinline__ void rs_level_pair(float* s, float* c, int lane) {
  const bool hi = (lane & M) != 0;
#pragma unroll
  for (int i = 0; i < HALF; i++) {
    const float ks = hi ? s[HALF + i] : s[i], kc = hi ? c[HALF + i] : c[i];
    const float ss = hi ? s[i] : s[HALF + i], sc = hi ? c[i] : c[HALF + i];
    const float rs = __shfl_xor_sync(0xffffffffu, ss, M), rc = __shfl_xor_sync(0xffffffffu, sc, M);
    float t, e;
    two_sum(ks, rs, t, e);
    s[i] = t;
    c[i] = kc + rc + e;
  }
}

template <int MODE>
struct Acc;
template <>
struct Acc<VS_REDUCE_FP32> {
  float s[32];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < 32; k++) s[k] = 0.0f;
  }
  __device__ void add(int k, float v) { s[k] += v; }
  // lane q < 29 returns the warp's sum of quantity q
  __device__ float2 reduce_scatter(int lane) {
    rs_level<16, 16>(s, lane);
    rs_level<8, 8>(s, lane);
    rs_level<4, 4>(s, lane);
    rs_level<2, 2>(s, lane);
    rs_level<1, 1>(s, lane);
    return make_float2(s[0], 0.0f);
  }
};
template <>
struct Acc<VS_REDUCE_KAHAN> {
  float s[32];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < 32; k++) s[k] = 0.0f;
  }
  __device__ void add(int k, float v) { s[k] += v; }
  __device__ float2 reduce_scatter(int lane) {
    float c[16];
    // first level: plain values in, (sum, error) pairs out
    {
      const bool hi = (lane & 16) != 0;
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const float keep = hi ? s[16 + i] : s[i];
        const float send = hi ? s[i] : s[16 + i];
        float t, e;
        two_sum(keep, __shfl_xor_sync(0xffffffffu, send, 16), t, e);
        s[i] = t;
        c[i] = e;
      }
    }
    rs_level_pair<8, 8>(s, c, lane);
    rs_level_pair<4, 4>(s, c, lane);
    rs_level_pair<2, 2>(s, c, lane);
    rs_level_pair<1, 1>(s, c, lane);
    return make_float2(s[0], c[0]);
  }
};
template <>
struct Acc<VS_REDUCE_FP64> {
  double s[32];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < 32; k++) s[k] = 0.0;
  }
  __device__ void add(int k, float v) { s[k] += (double)v; }
  __device__ double2 reduce_scatter(int lane) {
    rs_level<16, 16>(s, lane);
    rs_level<8, 8>(s, lane);
    rs_level<4, 4>(s, lane);
    rs_level<2, 2>(s, lane);
    rs_level<1, 1>(s, lane);
    return make_double2(s[0], 0.0);
  }
};

// Partial sums travel as (sum, error) pairs in the mode's own type: float2
// for the FP32 and compensated modes (no conversions to double, which run on
// the narrow FP64 pipe), double2 for the FP64 mode.
template <int MODE>
struct PartT {
  typedef float2 type;
};
template <>
struct PartT<VS_REDUCE_FP64> {
  typedef double2 type;
};
__device__ inline float2 combine(float2 a, float2 b, int mode) {
  if (mode == VS_REDUCE_FP32) return make_float2(a.x + b.x, 0.0f);
  float t, e;
  two_sum(a.x, b.x, t, e);
  return make_float2(t, a.y + b.y + e);
}
__device__ inline double2 combine(double2 a, double2 b, int) { return make_double2(a.x + b.x, 0.0); }
__device__ inline float2 shfl_xor2(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}
__device__ inline double2 shfl_xor2(double2 v, int m) {
  return make_double2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

__device__ inline int tri_index(int i, int j) { return i * 6 - i * (i - 1) / 2 + (j - i); }

// ---- FP64 pose algebra, spread over the lanes of one warp ------------------
// FP64 runs on a narrow pipe on this part: a dependent double operation costs
// tens of cycles whatever the number of active lanes, so the 6x6 solve, the
// SE(3) exponential and the 4x4 products keep every lane busy on its own
// matrix element instead of running as one long single-thread chain.

// lane -> (row, col) of the lower triangle, row-major: lane = row*(row+1)/2 + col
__device__ __forceinline__ int low_lane(int r, int c) { return r * (r + 1) / 2 + c; }
__device__ __forceinline__ void low_rc(int lane, int& r, int& c) {
  r = 0;
  while (low_lane(r + 1, 0) <= lane) r++;
  c = lane - low_lane(r, 0);
}

// The 6x6 solve: d_lld_LL_Decomposition + d_sls_Solve_Linear_System_using_LLD
// (_yooji_cuda_math.h:489-592), restated as an L D L^T factorisation
// (D_j = L_jj^2).  The factorisation is done twice.  In float - the
// reference's own precision - it decides failure by the reference's pivot
// rules unchanged: a pivot with sqrt(D_j) < 1e-8 fails the solve (returns 1);
// a negative or NaN pivot makes the reference's square root NaN, its column
// zero and the solution NaN, which the convergence test reads as converged
// (returns 2).  In FP64, from the FP64 sums, it gives the solution: forward
// and back substitution with the double factors.  Lane i < 6 returns x_i.
template <class T>
__device__ void warp_ldl_solve(T l, T D, int lane, T& v) {
  const unsigned M = 0xffffffffu;
  // v: right-hand side in lanes 0..5 on entry, solution on exit
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const T vj = __shfl_sync(M, v, j);
    const bool upd = lane < 6 && lane > j;
    const T lij = __shfl_sync(M, l, upd ? low_lane(lane, j) : lane);
    if (upd) v -= lij * vj;
  }
  const T dd = __shfl_sync(M, D, lane < 6 ? low_lane(lane, lane) : lane);
  if (lane < 6) v = v / dd;
#pragma unroll
  for (int j = 5; j >= 0; j--) {
    const T xj = __shfl_sync(M, v, j);
    const bool upd = lane < j;
    const T lji = __shfl_sync(M, l, upd ? low_lane(j, lane) : lane);
    if (upd) v -= lji * xj;
  }
}

// 1 / d in FP64 for a positive pivot d: the float reciprocal refined by two
// Newton-Raphson steps r <- r + r (1 - d r) (the error squares each step:
// 2^-23, 2^-46, then below the double rounding), four dependent FP64
// operations instead of a double division on the narrow FP64 pipe
__device__ __forceinline__ double recip_f64(double d) {
  double r = (double)(1.0f / (float)d);
  if (!(r > 0.0 && r < 1e300)) return 1.0 / d;  // outside the float range
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

// The two factorisations share one loop over the columns: the float chain
// (the reference's decisions) and the FP64 chain (the solution) are
// independent, so the scheduler overlaps their latencies.
__device__ int warp_solve6(const double* fin, int lane, double& x) {
  const unsigned M = 0xffffffffu;
  int r = 0, c = 0;
  if (lane < 21) low_rc(lane, r, c);
  float a = (lane < 21) ? (float)fin[tri_index(c, r)] : 0.0f;
  double ad = (lane < 21) ? fin[tri_index(c, r)] : 0.0;
  double inv = 0.0;  // lane j < 6: 1 / D_j of the FP64 factors
  bool nanp = false, fail = false, dfail = false;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const float d = __shfl_sync(M, a, low_lane(j, j));
    const double dd = __shfl_sync(M, ad, low_lane(j, j));
    const bool neg = !(d >= 0.0f);
    const bool tiny = !neg && !(sqrtf(d) >= 1e-8f);
    nanp |= neg;
    fail |= tiny;
    const bool ok = !neg && !tiny;
    const bool dok = dd > 0.0;
    dfail |= !dok;
    const double di = dok ? recip_f64(dd) : 0.0;
    if (lane == j) inv = di;
    if (lane < 21 && c == j && r > j) {
      a = ok ? a / d : 0.0f;
      ad = ad * di;
    }
    const bool upd = lane < 21 && c > j;
    const int sr = upd ? low_lane(r, j) : lane, sc = upd ? low_lane(c, j) : lane;
    const float lr = __shfl_sync(M, a, sr), lc = __shfl_sync(M, a, sc);
    const double lrd = __shfl_sync(M, ad, sr), lcd = __shfl_sync(M, ad, sc);
    if (upd && ok) a -= lr * d * lc;
    if (upd && dok) ad -= lrd * dd * lcd;
  }
  if (fail) return 1;
  if (nanp || dfail) {
    // nanp: the reference's solution is NaN here and reads as converged; the
    // pose is not updated, so the float factors' (finite) solution is only
    // recorded.  dfail: a pivot that float rounding left positive and FP64
    // does not (a system singular to FP64 precision): the float solution.
    float vf = (lane < 6) ? (float)fin[21 + lane] : 0.0f;
    warp_ldl_solve<float>(a, a, lane, vf);
    x = (lane < 6) ? (double)vf : 0.0;
    return nanp ? 2 : 0;
  }
  // L D L^T x = b with the FP64 factors and the inverse pivots
  double v = (lane < 6) ? fin[21 + lane] : 0.0;
#pragma unroll
  for (int j = 0; j < 6; j++) {
    const double vj = __shfl_sync(M, v, j);
    const bool upd = lane < 6 && lane > j;
    const double lij = __shfl_sync(M, ad, upd ? low_lane(lane, j) : lane);
    if (upd) v -= lij * vj;
  }
  if (lane < 6) v *= inv;
#pragma unroll
  for (int j = 5; j >= 0; j--) {
    const double xj = __shfl_sync(M, v, j);
    const bool upd = lane < j;
    const double lji = __shfl_sync(M, ad, upd ? low_lane(j, lane) : lane);
    if (upd) v -= lji * xj;
  }
  x = (lane < 6) ? v : 0.0;
  return 0;
}

// SE(3) exponential of the twist [w; v] in the reference's parameterisation
// (z_uitme_Update_Incremental_Tracking_with_Matrix_Exponential,
// z_yooji_cuda_pose_tracker.cu:50-149: R = I + sin(th)[u]x +
// (1 - cos(th))[u]x^2 with u = w / th, t = (I - R)[u]x v / th + u u^T v),
// written with W = [w]x as R = I + A W + B W^2, t = v + B (w x v) +
// C (w (w.v) - th^2 v), A = sin(th)/th, B = (1 - cos(th))/th^2,
// C = (th - sin(th))/th^3 - the same function, with no division by th.  For
// th < 0.1 the three coefficients come from their Taylor series in th^2
// (truncation below 1e-17 relative), one per lane; otherwise from sin/cos.
// Lane l < 16 returns element l of the 4x4 result; x is lane i's component.
__device__ double warp_se3_exp(double x, int lane) {
  const unsigned M = 0xffffffffu;
  double q[6];
#pragma unroll
  for (int k = 0; k < 6; k++) q[k] = __shfl_sync(M, x, k);
  const double th2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
  double coef = 0.0;
  if (th2 < 0.01) {
    const double t = th2;
    if (lane == 0)  // sin(th)/th
      coef = 1.0 - t * (1.0 / 6.0) * (1.0 - t * (1.0 / 20.0) * (1.0 - t * (1.0 / 42.0) * (1.0 - t * (1.0 / 72.0) * (1.0 - t * (1.0 / 110.0)))));
    else if (lane == 1)  // (1 - cos(th))/th^2
      coef = 0.5 * (1.0 - t * (1.0 / 12.0) * (1.0 - t * (1.0 / 30.0) * (1.0 - t * (1.0 / 56.0) * (1.0 - t * (1.0 / 90.0) * (1.0 - t * (1.0 / 132.0))))));
    else if (lane == 2)  // (th - sin(th))/th^3
      coef = (1.0 / 6.0) * (1.0 - t * (1.0 / 20.0) * (1.0 - t * (1.0 / 42.0) * (1.0 - t * (1.0 / 72.0) * (1.0 - t * (1.0 / 110.0) * (1.0 - t * (1.0 / 156.0))))));
  } else if (lane < 3) {
    const double th = sqrt(th2);
    const double sn = sin(th), cs = cos(th);
    coef = (lane == 0) ? sn / th : (lane == 1) ? (1.0 - cs) / th2 : (th - sn) / (th2 * th);
  }
  const double A = __shfl_sync(M, coef, 0), B = __shfl_sync(M, coef, 1), C = __shfl_sync(M, coef, 2);
  const int r = (lane >> 2) & 3, cc = lane & 3;
  if (lane >= 16 || r == 3) return (lane == 15) ? 1.0 : 0.0;
  const double W[9] = {0.0, -q[2], q[1], q[2], 0.0, -q[0], -q[1], q[0], 0.0};
  if (cc < 3) {
    const double dl = (r == cc) ? 1.0 : 0.0;
    return dl + A * W[r * 3 + cc] + B * (q[r] * q[cc] - th2 * dl);
  }
  const double wxv[3] = {q[1] * q[5] - q[2] * q[4], q[2] * q[3] - q[0] * q[5], q[0] * q[4] - q[1] * q[3]};
  const double wv = q[0] * q[3] + q[1] * q[4] + q[2] * q[5];
  return q[3 + r] + B * wxv[r] + C * (q[r] * wv - th2 * q[3 + r]);
}

// out = A * B (4x4, lane l < 16 computes element l); A in shared memory
__device__ void warp_compose(const double* A, const double* B, double* out, int lane) {
  if (lane < 16) {
    const int r = lane >> 2, c = lane & 3;
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 4; k++) s += A[r * 4 + k] * B[k * 4 + c];
    out[lane] = s;
  }
  __syncwarp();
}
// inverse of a rigid transform [R t; 0 1] held in shared memory; lane l < 16
// receives element l
__device__ void warp_rigid_inverse(const double* T, int lane, double& out) {
  out = 0.0;
  if (lane < 16) {
    const int r = lane >> 2, c = lane & 3;
    if (r == 3)
      out = (c == 3) ? 1.0 : 0.0;
    else if (c < 3)
      out = T[c * 4 + r];
    else
      out = -(T[0 * 4 + r] * T[3] + T[1 * 4 + r] * T[7] + T[2 * 4 + r] * T[11]);
  }
}
// T12 <- E * T12 and T21 = float(inv(T12)); E and scratch Tn in shared memory
__device__ void warp_compose_and_invert(const double* E, double* T12, double* Tn, int lane, double* T12_out,
                                        float* T21_out) {
  warp_compose(E, T12, Tn, lane);
  double ti;
  warp_rigid_inverse(Tn, lane, ti);
  if (lane < 16) {
    T12_out[lane] = Tn[lane];
    T21_out[lane] = (float)ti;
  }
}
// single-thread inverse used once per frame by k_icp_begin
__device__ void rigid_inverse(const double* T, double* I) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) I[i * 4 + j] = T[j * 4 + i];
  for (int i = 0; i < 3; i++) I[i * 4 + 3] = -(T[0 * 4 + i] * T[3] + T[1 * 4 + i] * T[7] + T[2 * 4 + i] * T[11]);
  I[12] = I[13] = I[14] = 0.0;
  I[15] = 1.0;
}

__global__ void k_icp_begin(const BatchTable* __restrict__ bt, int allow_skip, int with_init,
                            const float* init) {
  const int i = threadIdx.x;
  if (i >= bt->n) return;
  Pose* P = bt->s[i]->pose;
  P->skip = (allow_skip && P->frame == 0) ? 1 : 0;
  P->failed = 0;
  P->iters_run = 0;
  P->valid_count = 0;
  for (int l = 0; l < kMaxLevels; l++) P->level_done[l] = (with_init && l > 0) ? 1 : 0;
  double T[16];
  for (int k = 0; k < 16; k++) T[k] = (k % 5 == 0) ? 1.0 : 0.0;
  if (with_init && init)
    for (int k = 0; k < 16; k++) T[k] = (double)init[k];
  double I[16];
  rigid_inverse(T, I);
  for (int k = 0; k < 16; k++) {
    P->T12[k] = T[k];
    P->T21[k] = (float)I[k];
  }
}

// warp 0 of the block that closed a session's iteration: FP64 solve and SE(3)
// update, lane-parallel (kept out of line so the pixel loop's register
// allocation does not carry it)
__device__ __noinline__ void icp_solve_update(Pose* P, const double* fin, int level) {
  const int ln = threadIdx.x;
  if (ln < 29) P->last_sums[ln] = fin[ln];
  if (ln == 0) {
    P->iters_run += 1;
    P->valid_count = (int)fin[27];
  }
  double x;
  const int st = warp_solve6(fin, ln, x);
  if (st == 1) {
    if (ln == 0) P->failed = 1;
    return;
  }
  if (ln < 6) P->last_x[ln] = (float)x;
  // |x|_inf < 5e-7 ends the level (d_niv_Norm_Infinity_Vector: NaN entries never
  // raise the maximum, so an all-NaN solution also ends it)
  const bool big = (ln < 6) && (fabs(x) >= 5.0e-7);
  if (st == 2 || !__any_sync(0xffffffffu, big)) {
    if (ln == 0) P->level_done[level] = 1;
    return;
  }
  __shared__ double E[16], Tn[16];
  const double e = warp_se3_exp(x, ln);
  if (ln < 16) E[ln] = e;
  __syncwarp();
  warp_compose_and_invert(E, P->T12, Tn, ln, P->T12, P->T21);
  __syncwarp();
}

// Blocks take ranges from an atomic counter: a block that closes a session
// (reduction + solve, ~10 us) simply takes no new range meanwhile, so the
// closing work of different sessions overlaps instead of queueing behind a
// static assignment.  The last block to leave clears the counters.
#ifndef VS_ICP_MIN_BLOCKS
#define VS_ICP_MIN_BLOCKS 3  // resident 256-thread blocks per SM the register allocation must allow
#endif

template <int MODE>
__global__ void __launch_bounds__(kThreads, VS_ICP_MIN_BLOCKS)
    k_icp_iter(const BatchTable* __restrict__ bt, unsigned* __restrict__ work, int level, int iter) {
  typedef typename PartT<MODE>::type PT;
  __shared__ PT wsum[kThreads / 32][29];
  __shared__ int s_last, s_item;
  __shared__ double fin[29];
  __shared__ float sT21[12], sK[4];
  const int n = bt->n;
  const int* pre = bt->icp[level];
  const int total = pre[n];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(work, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= total) break;
    int vb;
    const int slot = find_slot(pre, n, item, vb);
    const SessionDev* __restrict__ s = bt->s[slot];
    Pose* P = s->pose;
    // uniform across the session's ranges: no range of this session has
    // closed the iteration yet when any of them reads the flags
    if (iter >= s->iters[level] || (P->skip | P->failed | P->level_done[level])) {
      // the session sits this launch out (its flags do not change during the
      // launch): move the counter past its remaining ranges at once
      if (threadIdx.x == 0) atomicMax(work, (unsigned)pre[slot + 1]);
      __syncthreads();  // every thread has read s_item before the next fetch
      continue;
    }
    const int nvb = pre[slot + 1] - pre[slot];
    const int w = s->lv[level].W, h = s->lv[level].H;
    // the pose and intrinsics are read from shared memory in the pixel loop,
    // which leaves the registers to the 29 running sums
    if (threadIdx.x < 12) sT21[threadIdx.x] = P->T21[threadIdx.x];
    if (threadIdx.x < 4) sK[threadIdx.x] = s->lv[level].K[threadIdx.x];
    __syncthreads();
    const float* K = sK;
    const float* T21 = sT21;
    const float th = s->th_icp, cosn = s->cos_normal;
    const float* depth = s->depth[level];
    const float4* mvtx = s->m_vtx[level];
    const float4* mnrm = s->m_nrm[level];
    const float4* innrm = s->in_nrm[level];

    Acc<MODE> acc;
    acc.zero();
    const int npix = w * h;
    const int stride = nvb * kThreads;
    const bool ntest = cosn > -2.0f;
    // the first-round reads (depth, input normal) of a thread's next pixel are
    // in flight while its current pixel's taps are read
    int p = vb * kThreads + threadIdx.x;
    float d_next = 0.0f;
    float4 q_next = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (p < npix) {
      d_next = __ldg(depth + p);
      if (ntest) q_next = __ldg(innrm + p);
    }
    while (p < npix) {
      const float d1 = d_next;
      const float4 qn = q_next;
      const int y = p / w, x = p - y * w;
      p += stride;
      if (p < npix) {
        d_next = __ldg(depth + p);
        if (ntest) q_next = __ldg(innrm + p);
      }
      float A[6], b;
      if (!icp_term(x, y, w, h, K, d1, qn, mvtx, mnrm, T21, th, cosn, A, b)) continue;
#pragma unroll
      for (int i = 0; i < 6; i++)
#pragma unroll
        for (int j = i; j < 6; j++) acc.add(tri_index(i, j), A[i] * A[j]);
#pragma unroll
      for (int i = 0; i < 6; i++) acc.add(21 + i, A[i] * b);
      acc.add(27, 1.0f);
      acc.add(28, b * b);
    }
    const PT mine = acc.reduce_scatter(lane);
    if (lane < 29) wsum[warp][lane] = mine;
    __syncthreads();
    PT* part = reinterpret_cast<PT*>(s->partials) + (size_t)vb * kPartials;
    if (threadIdx.x < 29) {
      PT v = wsum[0][threadIdx.x];
      for (int q = 1; q < kThreads / 32; q++) v = combine(v, wsum[q][threadIdx.x], MODE);
      part[threadIdx.x] = v;
      __threadfence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned t = atomicAdd(s->icp_counter, 1u);
      s_last = (t == (unsigned)nvb - 1u);
    }
    __syncthreads();
    if (s_last) {
      // ---- last range of this session: deterministic sum, then the solve ----
      __threadfence();
      {
        // 8 threads per quantity, each a fixed stride over the ranges, then a
        // fixed shuffle tree
        const int k = threadIdx.x >> 3, j = threadIdx.x & 7;
        PT v;
        v.x = 0;
        v.y = 0;
        if (k < 29) {
          // four partials in flight per thread, combined in the same order
          // as one at a time (a missing one combines as an exact zero)
          const PT* base = reinterpret_cast<const PT*>(s->partials);
          for (int bb = j; bb < nvb; bb += 32) {
            PT t4[4];
#pragma unroll
            for (int u = 0; u < 4; u++) {
              const int q = bb + 8 * u;
              t4[u].x = 0;
              t4[u].y = 0;
              if (q < nvb) t4[u] = __ldcg(base + (size_t)q * kPartials + k);
            }
#pragma unroll
            for (int u = 0; u < 4; u++) v = combine(v, t4[u], MODE);
          }
        }
#pragma unroll
        for (int m = 4; m >= 1; m >>= 1) v = combine(v, shfl_xor2(v, m), MODE);
        if (k < 29 && j == 0) fin[k] = (double)v.x + (double)v.y;
      }
      __syncthreads();
      if (threadIdx.x < 32) {
        if (threadIdx.x == 0) *s->icp_counter = 0u;
        icp_solve_update(P, fin, level);
      }
    }
    __syncthreads();  // shared sums and s_item are reused by the next range
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(work + 1, 1u) == gridDim.x - 1) {
      work[0] = 0u;
      work[1] = 0u;
      __threadfence();
    }
  }
}

// one warp per slot
__global__ void k_icp_finish(const BatchTable* __restrict__ bt, int frame_mode) {
  if ((int)blockIdx.x >= bt->n) return;
  Pose* P = bt->s[blockIdx.x]->pose;
  const int ln = threadIdx.x;
  __shared__ double Tn[16], A[16];
  if (!P->skip && !P->failed) {
    if (ln < 16) A[ln] = P->T12[ln];
    __syncwarp();
    double Ti;
    warp_compose(A, P->T_gc, Tn, ln);
    if (ln < 16) P->T_gc[ln] = Tn[ln];
    warp_rigid_inverse(Tn, ln, Ti);
    if (ln < 16) {
      P->Tgc[ln] = (float)Tn[ln];
      P->Tcg[ln] = (float)Ti;
    }
    if (ln == 3 || ln == 7 || ln == 11) P->center[ln >> 2] = (float)Ti;
  }
  if (ln == 0) {
    P->tracked = P->skip ? 1 : (P->failed ? 0 : 1);
    if (frame_mode) P->frame += 1;
  }
}

__global__ void k_pose_set(SessionDev* s, const double* T) {
  Pose* P = s->pose;
  const int ln = threadIdx.x;
  __shared__ double Tn[16];
  if (ln < 16) Tn[ln] = T[ln];
  __syncwarp();
  double Ti;
  warp_rigid_inverse(Tn, ln, Ti);
  if (ln < 16) {
    P->T_gc[ln] = Tn[ln];
    P->Tgc[ln] = (float)Tn[ln];
    P->Tcg[ln] = (float)Ti;
  }
  if (ln == 3 || ln == 7 || ln == 11) P->center[ln >> 2] = (float)Ti;
}

// the 80-byte pose heads (float pose, tracked, iterations, count, frame) of
// every slot, packed slot after slot for one device-to-host copy
__global__ void k_gather_heads(const BatchTable* __restrict__ bt, uint32_t* __restrict__ out) {
  const int slot = blockIdx.x;
  if (slot >= bt->n) return;
  constexpr int kWords = (int)(kPoseHeadBytes / 4);
  const uint32_t* src = reinterpret_cast<const uint32_t*>(bt->s[slot]->pose);
  if (threadIdx.x < kWords) out[slot * kWords + threadIdx.x] = src[threadIdx.x];
}

}  // namespace

void launch_gather_heads(const BatchTable* bt, void* out, cudaStream_t st) {
  k_gather_heads<<<kMaxSlots, 32, 0, st>>>(bt, reinterpret_cast<uint32_t*>(out));
}

// pixels per ICP range at level 0 and at the coarser levels.  A range is
// the unit between two block barriers and one partial write: long ranges
// spend less of the launch in barriers and reductions, short ranges keep
// more blocks busy on the small coarse levels (and on a lone session).
#ifndef VS_ICP_PIXELS_PER_RANGE
#define VS_ICP_PIXELS_PER_RANGE 2048
#endif
#ifndef VS_ICP_PIXELS_PER_RANGE_COARSE
#define VS_ICP_PIXELS_PER_RANGE_COARSE 512
#endif

int icp_blocks(int npix, int level) {
  const int ppr = level == 0 ? VS_ICP_PIXELS_PER_RANGE : VS_ICP_PIXELS_PER_RANGE_COARSE;
  int b = (npix + ppr - 1) / ppr;
  if (b < 1) b = 1;
  if (b > kIcpMaxBlocks) b = kIcpMaxBlocks;
  return b;
}

void launch_icp(const BatchTable* bt, int max_levels, const int* max_iters, int reduce_mode, cudaStream_t st,
                bool frame_mode, const float* init_T12) {
  // frame-level calls skip tracking on the first frame as so_Scan_Object does
  // (zz_flag_track, z_yooji_object_scanner.cpp:534,572-576); explicit
  // tp_Track_Pose calls always track
  const bool with_init = init_T12 != nullptr;
  k_icp_begin<<<1, kMaxSlots, 0, st>>>(bt, frame_mode ? 1 : 0, with_init ? 1 : 0, init_T12);
  const int grid = sm_count() * VS_ICP_MIN_BLOCKS;  // every block resident
  unsigned* work = const_cast<unsigned*>(bt->work) + 2;
  for (int l = max_levels - 1; l >= 0; l--) {
    for (int i = 0; i < max_iters[l]; i++) {
      switch (reduce_mode) {
        case VS_REDUCE_FP32:
          k_icp_iter<VS_REDUCE_FP32><<<grid, kThreads, 0, st>>>(bt, work, l, i);
          break;
        case VS_REDUCE_FP64:
          k_icp_iter<VS_REDUCE_FP64><<<grid, kThreads, 0, st>>>(bt, work, l, i);
          break;
        default:
          k_icp_iter<VS_REDUCE_KAHAN><<<grid, kThreads, 0, st>>>(bt, work, l, i);
          break;
      }
    }
  }
  k_icp_finish<<<kMaxSlots, 32, 0, st>>>(bt, frame_mode ? 1 : 0);
}

void launch_pose_set(const SessionDev* d, const double* T_gc, cudaStream_t st) {
  k_pose_set<<<1, 32, 0, st>>>(const_cast<SessionDev*>(d), T_gc);
}

}  // namespace vs
