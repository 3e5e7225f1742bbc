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
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int kThreads = 256;

__device__ inline bool bilinear4(float xf, float yf, int w, int h, const float4* __restrict__ map, F3& out) {
  // NaN coordinates are rejected (see the oracle)
  if (!(xf >= 0.0f && xf <= (float)(w - 1) && yf >= 0.0f && yf <= (float)(h - 1))) return false;
  int x = (int)xf, y = (int)yf;
  float rx = xf - (float)x, ry = yf - (float)y;
  F3 a = f3(0, 0, 0), b = f3(0, 0, 0), c = f3(0, 0, 0), d = f3(0, 0, 0);
  float4 p = __ldg(map + (size_t)y * w + x);
  if (p.x == -100.0f) return false;
  a = f3(p.x, p.y, p.z);
  if (rx > 0.0f) {
    p = __ldg(map + (size_t)y * w + x + 1);
    if (p.x == -100.0f) return false;
    b = f3(p.x, p.y, p.z);
  }
  if (ry > 0.0f) {
    p = __ldg(map + (size_t)(y + 1) * w + x);
    if (p.x == -100.0f) return false;
    c = f3(p.x, p.y, p.z);
  }
  if (rx > 0.0f && ry > 0.0f) {
    p = __ldg(map + (size_t)(y + 1) * w + x + 1);
    if (p.x == -100.0f) return false;
    d = f3(p.x, p.y, p.z);
  }
  float ix = 1.0f - rx, iy = 1.0f - ry;
  out.x = iy * (ix * a.x + rx * b.x) + ry * (ix * c.x + rx * d.x);
  out.y = iy * (ix * a.y + rx * b.y) + ry * (ix * c.y + rx * d.y);
  out.z = iy * (ix * a.z + rx * b.z) + ry * (ix * c.z + rx * d.z);
  return true;
}

// d_cssfp_Compute_Single_Summand_with_Forward_Params
__device__ inline bool icp_term(int x, int y, int w, int h, const float* K, const float* __restrict__ depth,
                                const float4* __restrict__ mvtx, const float4* __restrict__ mnrm,
                                const float4* __restrict__ innrm, const float* T21, float th_icp,
                                float cos_normal, float A[6], float& b) {
  float d1 = __ldg(depth + (size_t)y * w + x);
  if (d1 < 1.0e-6f) return false;
  F3 tp = back_project((float)x, (float)y, K, d1);
  F3 p1 = transform(tp, T21);
  float u, v;
  project(p1, K, u, v);
  F3 p0;
  if (!bilinear4(u, v, w, h, mvtx, p0)) return false;
  float dd = (p0.x - p1.x) * (p0.x - p1.x) + (p0.y - p1.y) * (p0.y - p1.y) + (p0.z - p1.z) * (p0.z - p1.z);
  if (dd > th_icp) return false;
  F3 n;
  if (!bilinear4(u, v, w, h, mnrm, n)) return false;
  n = normalised(n);
  if (cos_normal > -2.0f) {
    float4 q = __ldg(innrm + (size_t)y * w + x);
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

template <int MODE>
struct Acc;
template <>
struct Acc<VS_REDUCE_FP32> {
  float s[29];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < 29; k++) s[k] = 0.0f;
  }
  __device__ void add(int k, float v) { s[k] += v; }
  __device__ void shfl_add(unsigned m) {
#pragma unroll
    for (int k = 0; k < 29; k++) s[k] += __shfl_xor_sync(0xffffffffu, s[k], m);
  }
  __device__ double2 get(int k) const { return make_double2((double)s[k], 0.0); }
};
template <>
struct Acc<VS_REDUCE_KAHAN> {
  float s[29], c[29];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < 29; k++) s[k] = c[k] = 0.0f;
  }
  __device__ void add(int k, float v) {
    float t, e;
    two_sum(s[k], v, t, e);
    s[k] = t;
    c[k] += e;
  }
  __device__ void shfl_add(unsigned m) {
#pragma unroll
    for (int k = 0; k < 29; k++) {
      float os = __shfl_xor_sync(0xffffffffu, s[k], m);
      float oc = __shfl_xor_sync(0xffffffffu, c[k], m);
      float t, e;
      two_sum(s[k], os, t, e);
      s[k] = t;
      c[k] = c[k] + oc + e;
    }
  }
  __device__ double2 get(int k) const { return make_double2((double)s[k], (double)c[k]); }
};
template <>
struct Acc<VS_REDUCE_FP64> {
  double s[29];
  __device__ void zero() {
#pragma unroll
    for (int k = 0; k < 29; k++) s[k] = 0.0;
  }
  __device__ void add(int k, float v) { s[k] += (double)v; }
  __device__ void shfl_add(unsigned m) {
#pragma unroll
    for (int k = 0; k < 29; k++) s[k] += __shfl_xor_sync(0xffffffffu, s[k], m);
  }
  __device__ double2 get(int k) const { return make_double2(s[k], 0.0); }
};

// combine two partials (hi, lo) in the mode's arithmetic
template <int MODE>
__device__ inline double2 combine(double2 a, double2 b) {
  if (MODE == VS_REDUCE_FP32) return make_double2((double)((float)a.x + (float)b.x), 0.0);
  if (MODE == VS_REDUCE_KAHAN) {
    float t, e;
    two_sum((float)a.x, (float)b.x, t, e);
    return make_double2((double)t, (double)((float)a.y + (float)b.y + e));
  }
  return make_double2(a.x + b.x, 0.0);
}

__device__ inline int tri_index(int i, int j) { return i * 6 - i * (i - 1) / 2 + (j - i); }

// ---- FP64 pose algebra (single thread) ------------------------------------
__device__ void mat4_mul(const double* a, const double* b, double* c) {
  for (int j = 0; j < 4; j++)
    for (int i = 0; i < 4; i++) {
      double s = 0.0;
      for (int k = 0; k < 4; k++) s += a[j * 4 + k] * b[k * 4 + i];
      c[j * 4 + i] = s;
    }
}
// inverse of a rigid transform [R t; 0 1]
__device__ void rigid_inverse(const double* T, double* I) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) I[i * 4 + j] = T[j * 4 + i];
  for (int i = 0; i < 3; i++) I[i * 4 + 3] = -(T[0 * 4 + i] * T[3] + T[1 * 4 + i] * T[7] + T[2 * 4 + i] * T[11]);
  I[12] = I[13] = I[14] = 0.0;
  I[15] = 1.0;
}
// SE(3) exponential in the reference's parameterisation
// (z_uitme_Update_Incremental_Tracking_with_Matrix_Exponential, :50-149):
// R = I + sin(th)[w]x + (1-cos(th))[w]x^2 with w normalised,
// t = (I-R)[w]x v/th + w w^T v; below th = 1e-10 the first-order limit is used
// (the reference divides by th unguarded).
__device__ void se3_exp(const double* xi, double* E) {
  double th = sqrt(xi[0] * xi[0] + xi[1] * xi[1] + xi[2] * xi[2]);
  for (int i = 0; i < 16; i++) E[i] = 0.0;
  E[15] = 1.0;
  if (th < 1e-10) {
    E[0] = E[5] = E[10] = 1.0;
    E[1] = -xi[2];
    E[2] = xi[1];
    E[4] = xi[2];
    E[6] = -xi[0];
    E[8] = -xi[1];
    E[9] = xi[0];
    E[3] = xi[3];
    E[7] = xi[4];
    E[11] = xi[5];
    return;
  }
  double w[3] = {xi[0] / th, xi[1] / th, xi[2] / th};
  double v[3] = {xi[3] / th, xi[4] / th, xi[5] / th};
  double wx[9] = {0.0, -w[2], w[1], w[2], 0.0, -w[0], -w[1], w[0], 0.0};
  double wx2[9];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      double s = 0.0;
      for (int k = 0; k < 3; k++) s += wx[j * 3 + k] * wx[k * 3 + i];
      wx2[j * 3 + i] = s;
    }
  double sn = sin(th), cs = 1.0 - cos(th);
  double R[9], M[9];
  for (int i = 0; i < 9; i++) R[i] = sn * wx[i] + cs * wx2[i];
  for (int i = 0; i < 9; i++) M[i] = -R[i];  // I - R without the identity
  R[0] += 1.0;
  R[4] += 1.0;
  R[8] += 1.0;
  double wv = w[0] * v[0] + w[1] * v[1] + w[2] * v[2];
  for (int j = 0; j < 3; j++) {
    double s = 0.0;
    for (int i = 0; i < 3; i++) {
      double mw = 0.0;
      for (int k = 0; k < 3; k++) mw += M[j * 3 + k] * wx[k * 3 + i];
      s += mw * v[i];
    }
    E[j * 4 + 3] = s + w[j] * wv * th;
  }
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) E[j * 4 + i] = R[j * 3 + i];
}

// d_lld_LL_Decomposition + d_sls_Solve_Linear_System_using_LLD in FP64 with
// the reference's rules: a pivot whose magnitude is below 1e-8 fails the
// solve; a negative pivot (square root of a negative number) propagates NaN,
// which the infinity-norm test then treats as converged.
__device__ bool solve6(const double* A, const double* b, double* x) {
  double L[36];
  for (int i = 0; i < 36; i++) L[i] = 0.0;
  for (int i = 0; i < 6; i++)
    for (int j = 0; j <= i; j++) {
      if (i == j) {
        double s = 0.0;
        for (int k = 0; k < j; k++) s += L[j * 6 + k] * L[j * 6 + k];
        L[j * 6 + j] = sqrt(A[j * 6 + j] - s);
      } else if (fabs(L[j * 6 + j]) >= 1e-8) {
        double s = 0.0;
        for (int k = 0; k < j; k++) s += L[i * 6 + k] * L[j * 6 + k];
        L[i * 6 + j] = (A[i * 6 + j] - s) / L[j * 6 + j];
      }
    }
  for (int i = 0; i < 6; i++)
    if (fabs(L[i * 6 + i]) < 1e-8) return false;
  double y[6];
  for (int i = 0; i < 6; i++) {
    double s = 0.0;
    for (int k = 0; k < i; k++) s += L[i * 6 + k] * y[k];
    y[i] = (b[i] - s) / L[i * 6 + i];
  }
  for (int i = 5; i >= 0; i--) {
    double s = 0.0;
    for (int k = i + 1; k < 6; k++) s += L[k * 6 + i] * x[k];
    x[i] = (y[i] - s) / L[i * 6 + i];
  }
  return true;
}

__device__ void refresh_float_pose(Pose* P) {
  double I[16];
  rigid_inverse(P->T_gc, I);
  for (int i = 0; i < 16; i++) {
    P->Tgc[i] = (float)P->T_gc[i];
    P->Tcg[i] = (float)I[i];
  }
  P->center[0] = (float)I[3];
  P->center[1] = (float)I[7];
  P->center[2] = (float)I[11];
}

__global__ void k_icp_begin(SessionDev* s, int allow_skip, int with_init, const float* init) {
  Pose* P = s->pose;
  P->skip = (allow_skip && P->frame == 0) ? 1 : 0;
  P->failed = 0;
  P->iters_run = 0;
  P->valid_count = 0;
  for (int l = 0; l < kMaxLevels; l++) P->level_done[l] = (with_init && l > 0) ? 1 : 0;
  double T[16];
  for (int i = 0; i < 16; i++) T[i] = (i % 5 == 0) ? 1.0 : 0.0;
  if (with_init && init)
    for (int i = 0; i < 16; i++) T[i] = (double)init[i];
  double I[16];
  rigid_inverse(T, I);
  for (int i = 0; i < 16; i++) {
    P->T12[i] = T[i];
    P->T21[i] = (float)I[i];
  }
}

template <int MODE>
__global__ void __launch_bounds__(kThreads) k_icp_iter(const SessionDev* __restrict__ s, int level) {
  Pose* P = s->pose;
  if (P->skip | P->failed | P->level_done[level]) return;  // uniform across the grid
  const int w = s->lv[level].W, h = s->lv[level].H;
  float K[4], T21[12];
#pragma unroll
  for (int k = 0; k < 4; k++) K[k] = s->lv[level].K[k];
#pragma unroll
  for (int k = 0; k < 12; k++) T21[k] = P->T21[k];
  const float th = s->th_icp, cosn = s->cos_normal;
  const float* depth = s->depth[level];
  const float4* mvtx = s->m_vtx[level];
  const float4* mnrm = s->m_nrm[level];
  const float4* innrm = s->in_nrm[level];

  Acc<MODE> acc;
  acc.zero();
  const int npix = w * h;
  for (int p = blockIdx.x * kThreads + threadIdx.x; p < npix; p += gridDim.x * kThreads) {
    int y = p / w, x = p - y * w;
    float A[6], b;
    if (!icp_term(x, y, w, h, K, depth, mvtx, mnrm, innrm, T21, th, cosn, A, b)) continue;
#pragma unroll
    for (int i = 0; i < 6; i++)
#pragma unroll
      for (int j = i; j < 6; j++) acc.add(tri_index(i, j), A[i] * A[j]);
#pragma unroll
    for (int i = 0; i < 6; i++) acc.add(21 + i, A[i] * b);
    acc.add(27, 1.0f);
    acc.add(28, b * b);
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc.shfl_add(m);

  __shared__ double2 wsum[kThreads / 32][29];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 29; k++) wsum[warp][k] = acc.get(k);
  __syncthreads();
  double2* part = reinterpret_cast<double2*>(s->partials) + (size_t)blockIdx.x * kPartials;
  if (threadIdx.x < 29) {
    double2 v = wsum[0][threadIdx.x];
    for (int q = 1; q < kThreads / 32; q++) v = combine<MODE>(v, wsum[q][threadIdx.x]);
    part[threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = atomicAdd(s->icp_counter, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return;

  // ---- last block: deterministic grid sum, then the solve ----
  __threadfence();
  __shared__ double fin[29];
  {
    // 8 threads per quantity, each a fixed stride over blocks, then a fixed
    // shuffle tree
    const int k = threadIdx.x >> 3, j = threadIdx.x & 7;
    double2 v = make_double2(0.0, 0.0);
    if (k < 29) {
      const double2* base = reinterpret_cast<const double2*>(s->partials);
      for (int bb = j; bb < (int)gridDim.x; bb += 8) v = combine<MODE>(v, __ldcg(base + (size_t)bb * kPartials + k));
    }
#pragma unroll
    for (int m = 4; m >= 1; m >>= 1) {
      double2 o;
      o.x = __shfl_xor_sync(0xffffffffu, v.x, m);
      o.y = __shfl_xor_sync(0xffffffffu, v.y, m);
      v = combine<MODE>(v, o);
    }
    if (k < 29 && j == 0) fin[k] = v.x + v.y;
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  *s->icp_counter = 0u;
  double A6[36], b6[6], x[6];
  for (int i = 0; i < 6; i++)
    for (int j = i; j < 6; j++) A6[i * 6 + j] = A6[j * 6 + i] = fin[tri_index(i, j)];
  for (int i = 0; i < 6; i++) b6[i] = fin[21 + i];
  for (int k = 0; k < 29; k++) P->last_sums[k] = fin[k];
  P->iters_run += 1;
  P->valid_count = (int)fin[27];
  if (!solve6(A6, b6, x)) {
    P->failed = 1;
    return;
  }
  for (int i = 0; i < 6; i++) P->last_x[i] = (float)x[i];
  // d_niv_Norm_Infinity_Vector: NaN entries never raise the maximum
  double ninf = -100000.0;
  for (int i = 0; i < 6; i++) {
    double a = fabs(x[i]);
    if (ninf < a) ninf = a;
  }
  if (ninf < 5.0e-7) {
    P->level_done[level] = 1;
    return;
  }
  double E[16], T[16], I[16];
  se3_exp(x, E);
  mat4_mul(E, P->T12, T);
  rigid_inverse(T, I);
  for (int i = 0; i < 16; i++) {
    P->T12[i] = T[i];
    P->T21[i] = (float)I[i];
  }
}

__global__ void k_icp_finish(SessionDev* s, int frame_mode) {
  Pose* P = s->pose;
  if (!P->skip) {
    if (!P->failed) {
      double T[16];
      mat4_mul(P->T12, P->T_gc, T);
      for (int i = 0; i < 16; i++) P->T_gc[i] = T[i];
      refresh_float_pose(P);
      P->tracked = 1;
    } else {
      P->tracked = 0;
    }
  } else {
    P->tracked = 1;
  }
  if (frame_mode) P->frame += 1;
}

__global__ void k_pose_set(SessionDev* s, const double* T) {
  Pose* P = s->pose;
  for (int i = 0; i < 16; i++) P->T_gc[i] = T[i];
  refresh_float_pose(P);
}

int icp_blocks(int npix) {
  int b = (npix + 511) / 512;
  if (b < 1) b = 1;
  if (b > kIcpMaxBlocks) b = kIcpMaxBlocks;
  return b;
}

}  // namespace

void launch_icp(const SessionDev* d, const SessionDev& h, cudaStream_t st, bool frame_mode,
                const float* init_T12) {
  SessionDev* dm = const_cast<SessionDev*>(d);
  // frame-level calls skip tracking on the first frame as so_Scan_Object does
  // (zz_flag_track, z_yooji_object_scanner.cpp:534,572-576); explicit
  // tp_Track_Pose calls always track
  const bool with_init = init_T12 != nullptr;
  k_icp_begin<<<1, 1, 0, st>>>(dm, frame_mode ? 1 : 0, with_init ? 1 : 0, init_T12);
  for (int l = h.levels - 1; l >= 0; l--) {
    int nb = icp_blocks(h.lv[l].W * h.lv[l].H);
    for (int i = 0; i < h.iters[l]; i++) {
      switch (h.reduce_mode) {
        case VS_REDUCE_FP32:
          k_icp_iter<VS_REDUCE_FP32><<<nb, kThreads, 0, st>>>(d, l);
          break;
        case VS_REDUCE_FP64:
          k_icp_iter<VS_REDUCE_FP64><<<nb, kThreads, 0, st>>>(d, l);
          break;
        default:
          k_icp_iter<VS_REDUCE_KAHAN><<<nb, kThreads, 0, st>>>(d, l);
          break;
      }
    }
  }
  k_icp_finish<<<1, 1, 0, st>>>(dm, frame_mode ? 1 : 0);
}

void launch_pose_set(const SessionDev* d, const double* T_gc, cudaStream_t st) {
  k_pose_set<<<1, 1, 0, st>>>(const_cast<SessionDev*>(d), T_gc);
}

}  // namespace vs
