// TSDF integration: sub-cube activation + gated update of the active bricks.
//
// Reference: g_fvsc_Find_Visible_Sub_Cubes and g_ctvc_Compute_TSDF_of_Voxels
// _with_Color (STAC/Engine/GPU/z_yooji_cuda_volume_integrator.cu:84-152,
// 265-402, host :976-1031).  The reference resets a byte flag per 8^3
// sub-cube, marks the sub-cubes that lie on every depth ray between 4 mu in
// front of and 1 mu behind the measured point, then runs one thread per
// sub-cube over its 512 voxels in the x-fastest global layout: uncoalesced,
// and most threads of its 512x512x1-voxel launch grid idle.
//
// GB300 layout: the volume is stored as bricks (one brick = one sub-cube =
// 512 consecutive 32-bit words, 2 KB), so an active sub-cube is one
// contiguous, perfectly coalesced 2 KB read and write.  Activation appends a
// brick to a compact list the first time its flag flips (atomicExch), and the
// update kernel is persistent: one warp per listed brick, 16-byte vector
// loads, 16 voxels per lane.  Flags are cleared by the warp that consumes the
// brick, so no full-volume pass touches HBM.  Voxel centres and the per-pixel
// ray scale K^-1 [x y 1] come from per-session tables built once with the
// same IEEE operations as the per-voxel reference formula, so the result
// stays bit-identical while the divisions leave the inner loop.
//
// Batches: activation is persistent over the level-0 tiles of every session
// of a batch table, each session filling its own brick list; the update
// kernel walks the concatenation of the lists (a brick touches only its own
// session's voxels, so the order across sessions changes no result).
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int kIntThreads = 256;
constexpr int kMaxDimLut = 1024;   // voxels per axis (bricks fit 21 index bits)
constexpr int kMaxImgLut = 2048;   // pixels per image axis

// ROUNDF(v)/8 as the unparenthesised reference macro evaluates it
// (z_yooji_cuda_volume_integrator.cu:133-135)
__device__ inline int roundf_div8_ref(float x) { return (x < 0.0f) ? (int)(x - 0.5f) : (int)(x + 0.5f) / 8; }

// 1 / w for every weight an update can produce (w = 1..65535), IEEE-rounded
// exactly as the division it replaces
__device__ float g_inv_weight[65536];

// per-session tables: voxel centre coordinate per axis
// (d_gpw_Get_Position_in_World), the level-0 ray components K^-1 [x y 1] and,
// when kept, the per-pixel ray scale lambda^-1 = 1 / |K^-1 [x y 1]| of
// g_ctvc (z_yooji_cuda_volume_integrator.cu:357-372), each with the
// reference's own operations
__global__ void k_session_tables(SessionDev* s) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int d0 = s->dim[0], d1 = s->dim[1], d2 = s->dim[2];
  if (i < d0) s->lut_vox[i] = ((float)i + 0.5f) / s->vox_inv + s->origin[0];
  if (i < d1) s->lut_vox[d0 + i] = ((float)i + 0.5f) / s->vox_inv + s->origin[1];
  if (i < d2) s->lut_vox[d0 + d1 + i] = ((float)i + 0.5f) / s->vox_inv + s->origin[2];
  const float* K = s->lv[0].K;
  const int W = s->lv[0].W, H = s->lv[0].H;
  if (i < W) s->lut_ray[i] = 1.0f * ((float)i - K[2]) / K[0];
  if (i < H) s->lut_ray[W + i] = 1.0f * ((float)i - K[3]) / K[1];
  if (i < 65536) g_inv_weight[i] = 1.0f / (float)i;
  if (s->lam_map && i < W * H) {
    const int x = i % W, y = i / W;
    const float rx = 1.0f * ((float)x - K[2]) / K[0], ry = 1.0f * ((float)y - K[3]) / K[1];
    s->lam_map[i] = 1.0f / sqrtf(rx * rx + ry * ry + 1.0f);
  }
}

// frame counters of every slot, and the activation stamp.  A brick's flag
// holds the stamp of the last integration that activated it, so no pass
// clears flags: the flagged set of the last integration is {b : flag[b] ==
// stamp != 0}, the reference's per-sub-cube bytes (cube_valid) after its
// reset and marking (z_yooji_cuda_volume_integrator.cu:1006-1016), which
// g_uvv_Update_Valid_Volume visits later.  A session whose tracking failed
// (gate) does not integrate and keeps its stamp and flags.
__global__ void k_integrate_prepare(const BatchTable* __restrict__ bt, int gate) {
  const int i = threadIdx.x;
  if (i < bt->n) {
    const SessionDev* s = bt->s[i];
    s->brick_count[0] = 0u;
    s->brick_count[1] = 0u;
    if (!(gate && s->pose->failed)) {
      const uint32_t stamp = s->brick_count[2] + 1u;
      s->brick_count[2] = stamp ? stamp : 1u;
    }
  }
}

__global__ void __launch_bounds__(256) k_activate(const BatchTable* __restrict__ bt, const float* __restrict__ depth_ext,
                                                  const float* __restrict__ Tcg_ext, int gate) {
  const int n = bt->n;
  const int total = bt->bil[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int t;
    const int slot = find_slot(bt->bil, n, item, t);
    const SessionDev* __restrict__ s = bt->s[slot];
    if (gate && s->pose->failed) continue;
    const int W = s->lv[0].W, H = s->lv[0].H;
    const int tw = (W + 31) / 32;
    const int rows = bt->bil_rows;
    for (int ty = threadIdx.y; ty < rows; ty += blockDim.y) {
      const int x = (t % tw) * 32 + threadIdx.x, y = (t / tw) * rows + ty;
      if (x >= W || y >= H) continue;
      const float* depth = depth_ext ? depth_ext : s->depth_raw;
      const float td = depth[(size_t)y * W + x];
      if (!(td > 0.0f)) continue;
      const float* Tcg_in = Tcg_ext ? Tcg_ext : s->pose->Tcg;
      float T[12];
  #pragma unroll
      for (int k = 0; k < 12; k++) T[k] = Tcg_in[k];
      const float* K = s->lv[0].K;
      F3 p = transform(back_project((float)x, (float)y, K, td), T);
      F3 pe = transform(back_project((float)x, (float)y, K, 100.0f), T);
      F3 dv = normalised(sub(pe, p));
      const int nb0 = s->nb[0], nb1 = s->nb[1], nb2 = s->nb[2];
      const uint32_t stamp = s->brick_count[2];
      int prev = -1;
      for (int m = -4; m <= 1; m++) {
        F3 tp = add(p, scale(((float)m) * s->mu, dv));
        F3 v;
        if (!pos_in_voxel(tp, *s, v)) continue;
        int xs = roundf_div8_ref(v.x), ys = roundf_div8_ref(v.y), zs = roundf_div8_ref(v.z);
        if (xs < 0 || xs >= nb0 || ys < 0 || ys >= nb1 || zs < 0 || zs >= nb2) break;
        int b = (zs * nb1 + ys) * nb0 + xs;
        if (b == prev) continue;
        prev = b;
        // an L1-cached read of the flag may be stale, but only ever with an
        // older stamp, and the exchange then decides: it returns the current
        // stamp to every thread but the first
        uint32_t* f = s->brick_flag + b;
        if (*f != stamp && atomicExch(f, stamp) != stamp) {
          uint32_t pos = atomicAdd(s->brick_count, 1u);
          s->brick_list[pos] = (uint32_t)b;
        }
      }
    }
  }
}

// per-warp copy of the session parameters the update needs
struct IntParams {
  const float* depth;
  const float* lut_vox;
  const float* lut_ray;
  const float* lam_map;
  const uint32_t* list;
  uint32_t* counters;
  void* vol;
  uint32_t* col;            // colour bricks (NULL: no colour)
  const uint32_t* rgb;      // packed colour frame
  float T[12];
  float C[3];
  float K[4];
  float mu, max_w;
  int W, H, nb0, nb1, d0, d1;
};

__device__ inline void load_params(IntParams& q, const SessionDev* __restrict__ s, const float* depth_ext,
                                   const float* Tgc_ext, const float* Tcg_ext) {
  q.depth = depth_ext ? depth_ext : s->depth_raw;
  q.lut_vox = s->lut_vox;
  q.lut_ray = s->lut_ray;
  q.lam_map = s->lam_map;
  q.list = s->brick_list;
  q.counters = s->brick_count;
  q.vol = s->vol;
  q.col = s->col;
  q.rgb = s->rgb_packed;
  const float* Tgc = Tgc_ext ? Tgc_ext : s->pose->Tgc;
  const float* Tcg = Tcg_ext ? Tcg_ext : s->pose->Tcg;
#pragma unroll
  for (int k = 0; k < 12; k++) q.T[k] = Tgc[k];
  q.C[0] = Tcg[3];
  q.C[1] = Tcg[7];
  q.C[2] = Tcg[11];
#pragma unroll
  for (int k = 0; k < 4; k++) q.K[k] = s->lv[0].K[k];
  q.mu = s->mu;
  q.max_w = s->max_w;
  q.W = s->lv[0].W;
  q.H = s->lv[0].H;
  q.nb0 = s->nb[0];
  q.nb1 = s->nb[1];
  q.d0 = s->dim[0];
  q.d1 = s->dim[1];
}

// the values of the per-voxel loop of the update kernel
struct VoxParams {
  // depth source: the session's packed {depth, lambda^-1} map (packed), or
  // a depth map with the lambda^-1 map beside it (lam) or without (NULL:
  // computed per voxel from the ray table)
  const void* src;
  const float* lam;
  float K[4];
  float mu, inv_mu, max_w;
  int W, H;
  bool packed;
  bool fast;  // principal point within the bound of nearest_pixel's fast path
};

__device__ inline void load_vox_params(VoxParams& p, const SessionDev* __restrict__ s, const float* depth_ext) {
  p.packed = !depth_ext && s->dl_map;
  p.src = p.packed ? static_cast<const void*>(s->dl_map) : static_cast<const void*>(depth_ext ? depth_ext : s->depth_raw);
  p.lam = p.packed ? nullptr : s->lam_map;
#pragma unroll
  for (int k = 0; k < 4; k++) p.K[k] = s->lv[0].K[k];
  p.mu = s->mu;
  p.inv_mu = 1.0f / s->mu;
  p.max_w = s->max_w;
  p.W = s->lv[0].W;
  p.H = s->lv[0].H;
  p.fast = fabsf(p.K[2]) < 4096.0f && fabsf(p.K[3]) < 4096.0f;
}

// A load the compiler may neither hoist out of the brick loop nor keep in a
// register across it: the session's brick-level values are read again at each
// brick (L1 hits), so they take no registers while the voxels are processed.
template <class T>
__device__ __forceinline__ T reload(const T* p) {
  return *reinterpret_cast<const volatile T*>(p);
}
template <class T>
__device__ __forceinline__ T* reload(T* const* p) {
  return *reinterpret_cast<T* const volatile*>(p);
}

// The colour part of g_ctvc (z_yooji_cuda_volume_integrator.cu:404-455, the
// registered-colour path): for every voxel of the round whose depth was just
// updated, the colour at its projection, interpolated as
// d_gii_Get_Interpolated_Intensity (_yooji_cuda_math.h:305-332) per channel,
// is blended as (w * old + sample) / (w + 1) and truncated to 8 bits.  When a
// channel cannot be interpolated (outside the image, or a used texel <= 0) the
// voxel keeps its colour (the reference would blend an uninitialised value).
// The four taps and the old colour of four voxels are read in one round.
__device__ inline bool interp_channel(uint32_t a, uint32_t b, uint32_t c, uint32_t d, int k, float rx, float ry,
                                      float& out) {
  const float d1 = (float)rgb_channel(a, k);
  if (d1 <= 0.0f) return false;
  float d2 = 0.0f, d3 = 0.0f, d4 = 0.0f;
  if (rx > 0.0f) {
    d2 = (float)rgb_channel(b, k);
    if (d2 <= 0.0f) return false;
  }
  if (ry > 0.0f) {
    d3 = (float)rgb_channel(c, k);
    if (d3 <= 0.0f) return false;
  }
  if (rx > 0.0f && ry > 0.0f) {
    d4 = (float)rgb_channel(d, k);
    if (d4 <= 0.0f) return false;
  }
  out = (1.0f - ry) * ((1.0f - rx) * d1 + rx * d2) + ry * ((1.0f - rx) * d3 + rx * d4);
  return true;
}

// wv: the round's words, [vector][voxel in vector]; v0: the lane's index of
// the round's first voxel
template <class S, int kPerVec, int kRound, class IP, class WV>
__device__ void color_round(const IP& q, unsigned upd, int v0, int lane, int bx, int by, int bz, uint32_t b,
                            const WV& wv, const float* __restrict__ lx, const float* __restrict__ ly,
                            const float* __restrict__ lz) {
  constexpr int kG = 4;
#pragma unroll
  for (int g = 0; g < kRound; g += kG) {
    uint32_t t00[kG], t01[kG], t10[kG], t11[kG], oc[kG];
    float rxs[kG], rys[kG];
    bool ok[kG];
#pragma unroll
    for (int j = 0; j < kG; j++) {
      ok[j] = false;
      if (!((upd >> (g + j)) & 1u)) continue;
      const int v = v0 + g + j, k = v / kPerVec, e = v % kPerVec;
      const int li = (k * 32 + lane) * kPerVec + e;
      const int xc = bx * 8 + (li & 7), yc = by * 8 + ((li >> 3) & 7), zc = bz * 8 + (li >> 6);
      const F3 pg = f3(__ldg(lx + xc), __ldg(ly + yc), __ldg(lz + zc));
      float u, vv;
      project(transform(pg, q.T), q.K, u, vv);
      if (!(u >= 0.0f && u <= (float)(q.W - 1) && vv >= 0.0f && vv <= (float)(q.H - 1))) continue;
      const int x = (int)u, y = (int)vv;
      rxs[j] = u - (float)x;
      rys[j] = vv - (float)y;
      const int xb = rxs[j] > 0.0f ? x + 1 : x, yb = rys[j] > 0.0f ? y + 1 : y;
      t00[j] = __ldg(q.rgb + y * q.W + x);
      t01[j] = __ldg(q.rgb + y * q.W + xb);
      t10[j] = __ldg(q.rgb + yb * q.W + x);
      t11[j] = __ldg(q.rgb + yb * q.W + xb);
      oc[j] = q.col[(size_t)b * kBrickVox + li];
      ok[j] = true;
    }
#pragma unroll
    for (int j = 0; j < kG; j++) {
      if (!ok[j]) continue;
      const int v = v0 + g + j, k = v / kPerVec, e = v % kPerVec;
      const int li = (k * 32 + lane) * kPerVec + e;
      float tn;
      uint32_t wn;
      S::decode(wv[(g + j) / kPerVec][e], tn, wn);  // the updated word: weight w + 1
      const float oldW = (float)(wn - 1u), inewW = __ldg(g_inv_weight + wn);
      float smp[3];
      bool good = true;
#pragma unroll
      for (int c = 0; c < 3; c++) good &= interp_channel(t00[j], t01[j], t10[j], t11[j], c, rxs[j], rys[j], smp[c]);
      if (!good) continue;
      uint32_t ch[3];
#pragma unroll
      for (int c = 0; c < 3; c++)
        ch[c] = (uint32_t)(uint8_t)(fmaxf(0.0f, fminf(255.0f, (oldW * (float)rgb_channel(oc[j], c) + smp[c]) * inewW)));
      q.col[(size_t)b * kBrickVox + li] = pack_rgb(ch[0], ch[1], ch[2]);
    }
  }
}

#ifndef VS_INT_MIN_BLOCKS
#define VS_INT_MIN_BLOCKS 4  // resident 256-thread blocks per SM the register allocation must allow
#endif

// rcp.approx.ftz.f32: the reciprocal with at most 1 ulp of error (PTX ISA,
// "rcp.approx"), one special-function instruction
__device__ __forceinline__ float rcp_approx(float z) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(z));
  return r;
}

// Nearest pixel of a camera-frame point: (__float2int_rn(u), __float2int_rn(v))
// of d_p_Project's u = K0 x / z + K2, v = K1 y / z + K3 with IEEE division
// (_yooji_cuda_math.h:205-210, z_yooji_cuda_volume_integrator.cu:344-347),
// bit for bit, at the price of a reciprocal instead of two divisions for all
// but a few voxels.
//
// u' = RN(RN(K0 x * rcp(z)) + K2) differs from u = RN(RN(K0 x / z) + K2) by
// at most 2^-22 |K0 x / z| + ulp(u): rcp has at most 1 ulp of error and each
// product / sum one rounding.  A pixel inside an image of at most 2048
// columns needs |u| < 2048, so |K0 x / z| < 2048 + |K2| < 6144 when
// |K2| < 4096, and |u' - u| < 1.5e-3 + 2.5e-4 < 2^-8 =: m.  If u' is farther
// than m from every half-integer, no rounding boundary lies between u and
// u', so rint(u') = rint(u).  Otherwise, and for z <= 1e-4 (or NaN), the
// IEEE divisions run.  (Outside the image both forms give columns out of
// range, where the exact value does not matter.)  `fast` is false when the
// principal point is out of the bound.
__device__ __forceinline__ void nearest_pixel(float x, float y, float z, const float* K, bool fast, int& px,
                                              int& py) {
  constexpr float kEdge = 0.5f - 1.0f / 256.0f;
  const float a = K[0] * x, b = K[1] * y;
  float u = 0.0f, v = 0.0f;
  bool exact = !(fast && z > 1e-4f);
  if (!exact) {
    const float r = rcp_approx(z);
    u = a * r + K[2];
    v = b * r + K[3];
    exact = fabsf(u - rintf(u)) > kEdge || fabsf(v - rintf(v)) > kEdge;
  }
  if (exact) {
    u = a / z + K[2];
    v = b / z + K[3];
  }
  px = __float2int_rn(u);
  py = __float2int_rn(v);
}

// g_ctvc's depth update, per voxel in the reference's operation order
// (z_yooji_cuda_volume_integrator.cu:340-402): world centre p_g, camera point
// T_gc p_g, nearest pixel, depth d; lambda^-1 |p_g - C|; sdf = d - that;
// skip if sdf < -mu; tsdf = min(1, sdf / mu); weighted mean with the old
// value; weight + 1.  The weights and the skip decisions are bit-identical
// to that order.  Two rewrites that keep every rounding:
//  * a lane's voxels share their y coordinate, take kPerVec x and kLaneVec
//    z values, so the partial sums M0 x + M1 y (and M4, M8 rows) and
//    (x - Cx)^2 + (y - Cy)^2 are formed once per x value, and the rest of
//    each sum is added in the same order as the full expression;
//  * the pixel rounding uses nearest_pixel above.
// The one change of a rounding: sdf / mu is the product with 1 / mu and one
// Markstein correction step (q = s r; e = fma(-q, mu, s); q + e r, P.
// Markstein, IBM J. Res. Dev. 34(1), 1990), which returns the IEEE quotient in
// all but rare cases and otherwise differs by one ulp (6e-8 of a TSDF value,
// below 0.002 of an int16 step), inside the one-step tolerance.
template <class S, bool COLOR>
__global__ void __launch_bounds__(kIntThreads, COLOR ? 2 : VS_INT_MIN_BLOCKS)
    k_integrate(const BatchTable* __restrict__ bt, const float* __restrict__ depth_ext,
                const float* __restrict__ Tgc_ext, const float* __restrict__ Tcg_ext, int color, int dry) {
  __shared__ uint32_t pre[kMaxSlots + 1];  // prefix of the slots' active-brick counts
  // per thread, per x value of its voxels: the transform rows' partial sums
  // M0 x + M1 y, M4 x + M5 y, M8 x + M9 y and (x - Cx)^2 + (y - Cy)^2
  // ([x value][thread]: a warp's 16-byte reads are consecutive, no bank conflicts)
  __shared__ float4 xpart[16 / sizeof(typename S::word)][kIntThreads];
  const int n = bt->n;
  if (threadIdx.x < 32) {
    const int ln = threadIdx.x;
    const uint32_t c0 = (2 * ln < n) ? *((volatile uint32_t*)bt->s[2 * ln]->brick_count) : 0u;
    const uint32_t c1 = (2 * ln + 1 < n) ? *((volatile uint32_t*)bt->s[2 * ln + 1]->brick_count) : 0u;
    uint32_t v = c0 + c1;
#pragma unroll
    for (int m = 1; m < 32; m <<= 1) {
      const uint32_t o = __shfl_up_sync(0xffffffffu, v, m);
      if (ln >= m) v += o;
    }
    pre[2 * ln + 2] = v;
    pre[2 * ln + 1] = v - c1;
    if (ln == 0) pre[0] = 0u;
  }
  __syncthreads();
  const uint32_t total = pre[n];

  typedef typename S::word word;
  constexpr int kPerVec = 16 / sizeof(word);    // voxels per 16-byte vector, consecutive in x
  constexpr int kVecs = kBrickVox / kPerVec;    // 16-byte vectors per brick
  constexpr int kLaneVec = kVecs / 32;          // vectors per lane, one z value each
  constexpr int kRV = 4 / kPerVec > 0 ? 4 / kPerVec : 1;  // 16-byte vectors per round
  constexpr int kRound = kRV * kPerVec;                    // 4 voxels per round, gathers in flight together
  constexpr int kRounds = kLaneVec / kRV;
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  // the lane's voxel coordinates inside a brick: word (k * 32 + lane) * kPerVec + e
  // is x = x0 + e, y = y0, z = z0 + k * kPerVec / 2
  const int x0 = (lane * kPerVec) & 7, y0 = ((lane * kPerVec) >> 3) & 7, z0 = (lane * kPerVec) >> 6;
  constexpr int kZStep = kPerVec / 2;
  // Per-session values: the voxel loop's in registers (VoxParams); the
  // brick-level ones (pointers, rotation, centre, brick grid) are read from
  // the session record at each brick, so they hold no registers across the
  // loop.  The colour variant keeps the whole IntParams for color_round.
  IntParams q;
  VoxParams vp;
  const SessionDev* __restrict__ sp = nullptr;
  int cur = -1;

  for (uint32_t i = gwarp; i < total; i += nwarps) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (pre[mid] <= i)
        lo = mid;
      else
        hi = mid - 1;
    }
    if (lo != cur) {
      cur = lo;
      sp = bt->s[lo];
      load_vox_params(vp, sp, depth_ext);
      if (COLOR) {
        load_params(q, sp, depth_ext, Tgc_ext, Tcg_ext);
        if (!color) q.col = nullptr;
      }
    }
    const uint32_t b = reload(sp->brick_list + (i - pre[lo]));
    int nupd = 0;
    bool band = false;  // some voxel of the brick, after the update, is a band voxel
    const uint32_t nb0 = (uint32_t)reload(&sp->nb[0]), nb1 = (uint32_t)reload(&sp->nb[1]);
    const int bx = (int)(b % nb0), by = (int)((b / nb0) % nb1), bz = (int)(b / (nb0 * nb1));
    uint4* bv = reinterpret_cast<uint4*>(reinterpret_cast<word*>(reload(&sp->vol)) + (size_t)b * kBrickVox);
    const int d0 = reload(&sp->dim[0]), d1 = reload(&sp->dim[1]);
    const float* __restrict__ lx = reload(&sp->lut_vox);
    const float* __restrict__ ly = lx + d0;
    const float* __restrict__ lz = lx + d0 + d1;
    // per-x partial sums of the transform rows and of |p_g - C|^2
    const float* Tg = Tgc_ext ? Tgc_ext : reload(&sp->pose)->Tgc;
    const float* Tc = Tcg_ext ? Tcg_ext : reload(&sp->pose)->Tcg;
    float Tr[12];
#pragma unroll
    for (int k = 0; k < 12; k++) Tr[k] = reload(Tg + k);
    const float C0 = reload(Tc + 3), C1 = reload(Tc + 7), C2 = reload(Tc + 11);
    const float py = __ldg(ly + by * 8 + y0);
    const float dy = py - C1;
    // kept in shared memory (one 16-byte read per voxel) rather than in 16
    // registers per thread
#pragma unroll
    for (int e = 0; e < kPerVec; e++) {
      const float px = __ldg(lx + bx * 8 + x0 + e);
      const float dx = px - C0;
      xpart[e][threadIdx.x] = make_float4(Tr[0] * px + Tr[1] * py, Tr[4] * px + Tr[5] * py, Tr[8] * px + Tr[9] * py,
                          dx * dx + dy * dy);
    }
    // Rounds of kRV vectors (4 voxels): the next round's vectors are read
    // while this round's voxels run, and a round's vectors are written back
    // as soon as it ends, so at most two rounds of voxel words are live.
    uint4 cur[kRV], nxt[kRV];
#pragma unroll
    for (int v = 0; v < kRV; v++) cur[v] = bv[v * 32 + lane];
#pragma unroll
    for (int r = 0; r < kRounds; r++) {
      if (r + 1 < kRounds) {
#pragma unroll
        for (int v = 0; v < kRV; v++) nxt[v] = bv[((r + 1) * kRV + v) * 32 + lane];
      }
      word wv[kRV][kPerVec];
#pragma unroll
      for (int v = 0; v < kRV; v++) memcpy(wv[v], &cur[v], 16);
      // this round's z values, one per vector
      float tz0[kRV], tz1[kRV], tz2[kRV], dz2[kRV];
#pragma unroll
      for (int v = 0; v < kRV; v++) {
        const float pz = __ldg(lz + bz * 8 + z0 + (r * kRV + v) * kZStep);
        tz0[v] = Tr[2] * pz;
        tz1[v] = Tr[6] * pz;
        tz2[v] = Tr[10] * pz;
        const float dz = pz - C2;
        dz2[v] = dz * dz;
      }
      // nearest pixel of every voxel, then its gathers, all in flight together
      float2 g[kRound];
      int pix[kRound];
#pragma unroll
      for (int j = 0; j < kRound; j++) {
        const int v = j / kPerVec, e = j % kPerVec;
        float told;
        uint32_t wold;
        S::decode(wv[v][e], told, wold);
        pix[j] = -1;
        if ((float)wold >= vp.max_w) continue;
        // T_gc p_g, each row summed as M0 x + M1 y + M2 z + M3
        const float4 xp = xpart[e][threadIdx.x];
        const float cx = (xp.x + tz0[v]) + Tr[3];
        const float cy = (xp.y + tz1[v]) + Tr[7];
        const float cz = (xp.z + tz2[v]) + Tr[11];
        int x, y;
        nearest_pixel(cx, cy, cz, vp.K, vp.fast, x, y);
        if ((unsigned)x > (unsigned)(vp.W - 1) || (unsigned)y > (unsigned)(vp.H - 1)) continue;
        pix[j] = y * vp.W + x;
      }
#pragma unroll
      for (int j = 0; j < kRound; j++) {
        g[j] = make_float2(0.0f, 0.0f);
        if (pix[j] >= 0) {
          if (vp.packed) {
            g[j] = __ldg(reinterpret_cast<const float2*>(vp.src) + pix[j]);
          } else {
            g[j].x = __ldg(reinterpret_cast<const float*>(vp.src) + pix[j]);
            if (vp.lam) g[j].y = __ldg(vp.lam + pix[j]);
          }
        }
      }
      bool changed[kRV];
#pragma unroll
      for (int v = 0; v < kRV; v++) changed[v] = false;
      unsigned upd = 0u;  // voxels of this round whose depth was updated
#pragma unroll
      for (int j = 0; j < kRound; j++) {
        const int v = j / kPerVec, e = j % kPerVec;
        if (pix[j] < 0 || !(g[j].x > 0.0f)) continue;
        float told;
        uint32_t wold;
        S::decode(wv[v][e], told, wold);
        const float oldW = (float)wold;
        float lm = g[j].y;
        if (!vp.packed && !vp.lam) {
          const float* rx_t = reload(&sp->lut_ray);
          const int x = pix[j] % vp.W, y = pix[j] / vp.W;
          const float rx = __ldg(rx_t + x), ry = __ldg(rx_t + vp.W + y);
          lm = 1.0f / sqrtf(rx * rx + ry * ry + 1.0f);
        }
        const float nrm = sqrtf(xpart[e][threadIdx.x].w + dz2[v]);
        const float sdf = g[j].x - lm * nrm;
        if (sdf < -vp.mu) continue;
        const float q0 = sdf * vp.inv_mu;
        const float ts = fminf(1.0f, fmaf(fmaf(-q0, vp.mu, sdf), vp.inv_mu, q0));
        const float newW = oldW + 1.0f;
        const float inewW = __ldg(g_inv_weight + (int)newW);
        const float tnew = (oldW * told + ts) * inewW;
        wv[v][e] = S::encode(tnew, (uint32_t)newW);
        changed[v] = true;
        upd |= 1u << j;
        nupd++;
      }
      if (COLOR && q.col && upd && !dry)
        color_round<S, kPerVec, kRound>(q, upd, r * kRound, lane, bx, by, bz, b, wv, lx, ly, lz);
#pragma unroll
      for (int v = 0; v < kRV; v++)
#pragma unroll
        for (int e = 0; e < kPerVec; e++) band |= S::band(wv[v][e]);
#pragma unroll
      for (int v = 0; v < kRV; v++)
        if (changed[v] && !dry) {
          memcpy(&cur[v], wv[v], 16);
          bv[(r * kRV + v) * 32 + lane] = cur[v];
        }
      if (r + 1 < kRounds) {
#pragma unroll
        for (int v = 0; v < kRV; v++) cur[v] = nxt[v];
      }
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) nupd += __shfl_xor_sync(0xffffffffu, nupd, m);
    band = __any_sync(0xffffffffu, band);
    if (lane == 0 && !dry) {
      // the brick's band state from its words after this update (the
      // brick's own warp is its only writer)
      uint8_t* bb = reload(&sp->band);
      if (bb) bb[b] = band ? 1 : 0;
      if (nupd) {
        atomicAdd(reload(&sp->brick_count) + 1, (uint32_t)nupd);
        // weights never decrease, so a brick that got an update stays occupied
        uint32_t* occ = reload(&sp->occ);
        if (occ) set_bit_once(occ, b);
      }
    }
  }
}

template <class S>
__global__ void k_volume_fill(typename S::word* vol, size_t n) {
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const typename S::word v = S::initial();
  for (; i < n; i += (size_t)gridDim.x * blockDim.x) vol[i] = v;
}

// bricked <-> x-fastest linear layout, for a slab of z in [z0, z0 + nz)
template <class S>
__global__ void k_volume_export(const typename S::word* vol, int X, int Y, int z0, int nz, const int* nb3,
                                int nb0, int nb1, float* tsdf, uint16_t* w) {
  size_t n = (size_t)X * Y * nz;
  int nb[3] = {nb0, nb1, 0};
  (void)nb3;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % X), y = (int)((i / X) % Y), z = z0 + (int)(i / ((size_t)X * Y));
    float t;
    uint32_t ww;
    S::decode(vol[brick_word_index(x, y, z, nb)], t, ww);
    if (tsdf) tsdf[i] = t;
    if (w) w[i] = (uint16_t)(ww > 65535u ? 65535u : ww);
  }
}
template <class S>
__global__ void k_volume_import(typename S::word* vol, int X, int Y, int z0, int nz, int nb0, int nb1,
                                const float* tsdf, const uint16_t* w) {
  size_t n = (size_t)X * Y * nz;
  int nb[3] = {nb0, nb1, 0};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    int x = (int)(i % X), y = (int)((i / X) % Y), z = z0 + (int)(i / ((size_t)X * Y));
    size_t idx = brick_word_index(x, y, z, nb);
    float t;
    uint32_t ww;
    S::decode(vol[idx], t, ww);
    if (tsdf) t = tsdf[i];
    if (w) ww = w[i];
    vol[idx] = S::encode(t, ww);
  }
}

// recomputes the occupancy bits and band flags from the volume (after an import);
// one warp per brick
template <class S>
__global__ void k_occupancy(const SessionDev* __restrict__ s) {
  const typename S::word* vol = reinterpret_cast<const typename S::word*>(s->vol);
  const int nb0 = s->nb[0], nb1 = s->nb[1];
  const size_t nbr = (size_t)nb0 * nb1 * s->nb[2];
  const int lane = threadIdx.x & 31;
  const size_t gw = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarp = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t b = gw; b < nbr; b += nwarp) {
    bool any = false, band = false;
    for (int k = lane; k < kBrickVox; k += 32) {
      const typename S::word v = vol[b * kBrickVox + k];
      float t;
      uint32_t w;
      S::decode(v, t, w);
      any |= w != 0u;
      band |= S::band(v);
    }
    const unsigned m = __ballot_sync(0xffffffffu, any);
    band = __any_sync(0xffffffffu, band);
    if (lane == 0) {
      if (m) set_bit_once(s->occ, (uint32_t)b);
      if (s->band) s->band[b] = band ? 1 : 0;
    }
  }
}

__global__ void k_pack_color(const uint8_t* __restrict__ rgb, uint32_t* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = pack_rgb(rgb[i], rgb[n + i], rgb[2 * n + i]);
}

// bricked colour words <-> three planes of x-fastest bytes (cube_color)
__global__ void k_color_volume(uint32_t* col, int X, int Y, int Z, int nb0, int nb1, uint8_t* planes, int do_export) {
  const size_t n = (size_t)X * Y * Z;
  int nb[3] = {nb0, nb1, 0};
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % X), y = (int)((i / X) % Y), z = (int)(i / ((size_t)X * Y));
    const size_t w = brick_word_index(x, y, z, nb);
    if (do_export) {
      const uint32_t c = col[w];
      planes[i] = (uint8_t)rgb_channel(c, 0);
      planes[n + i] = (uint8_t)rgb_channel(c, 1);
      planes[2 * n + i] = (uint8_t)rgb_channel(c, 2);
    } else {
      col[w] = pack_rgb(planes[i], planes[n + i], planes[2 * n + i]);
    }
  }
}

__global__ void k_color_map_export(const uint32_t* __restrict__ m, int n, uint8_t* __restrict__ planes) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const uint32_t c = m[i];
    planes[i] = (uint8_t)rgb_channel(c, 0);
    planes[n + i] = (uint8_t)rgb_channel(c, 1);
    planes[2 * n + i] = (uint8_t)rgb_channel(c, 2);
  }
}

}  // namespace

void launch_pack_color(const SessionDev& h, const uint8_t* rgb, cudaStream_t st) {
  const int n = h.lv[0].W * h.lv[0].H;
  k_pack_color<<<(n + 255) / 256, 256, 0, st>>>(rgb ? rgb : h.rgb_in, h.rgb_packed, n);
}

void launch_color_volume(const SessionDev& h, bool do_export, uint8_t* planes, cudaStream_t st) {
  k_color_volume<<<sm_count() * 8, 256, 0, st>>>(h.col, h.dim[0], h.dim[1], h.dim[2], h.nb[0], h.nb[1], planes,
                                                 do_export ? 1 : 0);
}

void launch_color_map_export(const SessionDev& h, int level, uint8_t* planes, cudaStream_t st) {
  const int n = h.lv[level].W * h.lv[level].H;
  k_color_map_export<<<(n + 255) / 256, 256, 0, st>>>(h.m_rgb[level], n, planes);
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
  }
  return n;
}

template <class S, bool COLOR>
int resident_blocks() {
  // one query per kernel variant (the answer depends only on the compiled kernel)
  static int per_sm = -1;
  if (per_sm < 0) {
    int v = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_integrate<S, COLOR>, kIntThreads, 0) != cudaSuccess ||
        v < 1)
      v = 1;
    per_sm = v;
  }
  return sm_count() * per_sm;
}

template <class S>
void launch_update(const BatchTable* bt, const float* depth, const float* Tgc, const float* Tcg, bool color,
                   cudaStream_t st, int blocks_per_sm, bool dry) {
  const int most = color ? resident_blocks<S, true>() : resident_blocks<S, false>();
  const int grid = (blocks_per_sm > 0 && blocks_per_sm * sm_count() < most) ? blocks_per_sm * sm_count() : most;
  if (color)
    k_integrate<S, true><<<grid, kIntThreads, 0, st>>>(bt, depth, Tgc, Tcg, 1, dry ? 1 : 0);
  else
    k_integrate<S, false><<<grid, kIntThreads, 0, st>>>(bt, depth, Tgc, Tcg, 0, dry ? 1 : 0);
}

void launch_session_tables(const SessionDev& h, SessionDev* d, cudaStream_t st) {
  int m = 65536;
  for (int v : {h.dim[0], h.dim[1], h.dim[2], h.lv[0].W * h.lv[0].H}) m = v > m ? v : m;
  k_session_tables<<<(m + 255) / 256, 256, 0, st>>>(d);
}

void launch_integrate(const BatchTable* bt, int tsdf_type, const float* depth, const float* Tgc, const float* Tcg,
                      bool gate, cudaStream_t st, bool color, int blocks_per_sm, bool dry) {
  const int c = color ? 1 : 0;
  k_integrate_prepare<<<1, kMaxSlots, 0, st>>>(bt, gate ? 1 : 0);
  k_activate<<<sm_count() * 8, dim3(32, 8), 0, st>>>(bt, depth, Tcg, gate ? 1 : 0);
  // persistent grid: every block resident at once
  switch (tsdf_type) {
    case VS_TSDF_FP16:
      launch_update<StoreF16>(bt, depth, Tgc, Tcg, c != 0, st, blocks_per_sm, dry);
      break;
    case VS_TSDF_FP32:
      launch_update<StoreF32>(bt, depth, Tgc, Tcg, c != 0, st, blocks_per_sm, dry);
      break;
    default:
      launch_update<StoreI16>(bt, depth, Tgc, Tcg, c != 0, st, blocks_per_sm, dry);
      break;
  }
}

void launch_volume_init(const SessionDev& h, cudaStream_t st) {
  size_t n = (size_t)h.nb[0] * h.nb[1] * h.nb[2] * kBrickVox;
  int blocks = sm_count() * 8;
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      k_volume_fill<StoreF16><<<blocks, 256, 0, st>>>((uint32_t*)h.vol, n);
      break;
    case VS_TSDF_FP32:
      k_volume_fill<StoreF32><<<blocks, 256, 0, st>>>((uint2*)h.vol, n);
      break;
    default:
      k_volume_fill<StoreI16><<<blocks, 256, 0, st>>>((uint32_t*)h.vol, n);
      break;
  }
}

// exports / imports one z-slab [z0, z0+nz) through device staging buffers
void launch_volume_slab(const SessionDev& h, bool do_export, int z0, int nz, float* tsdf, uint16_t* w,
                        cudaStream_t st) {
  int blocks = sm_count() * 8;
  const int X = h.dim[0], Y = h.dim[1];
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      if (do_export)
        k_volume_export<StoreF16><<<blocks, 256, 0, st>>>((const uint32_t*)h.vol, X, Y, z0, nz, nullptr, h.nb[0],
                                                          h.nb[1], tsdf, w);
      else
        k_volume_import<StoreF16><<<blocks, 256, 0, st>>>((uint32_t*)h.vol, X, Y, z0, nz, h.nb[0], h.nb[1], tsdf, w);
      break;
    case VS_TSDF_FP32:
      if (do_export)
        k_volume_export<StoreF32><<<blocks, 256, 0, st>>>((const uint2*)h.vol, X, Y, z0, nz, nullptr, h.nb[0],
                                                          h.nb[1], tsdf, w);
      else
        k_volume_import<StoreF32><<<blocks, 256, 0, st>>>((uint2*)h.vol, X, Y, z0, nz, h.nb[0], h.nb[1], tsdf, w);
      break;
    default:
      if (do_export)
        k_volume_export<StoreI16><<<blocks, 256, 0, st>>>((const uint32_t*)h.vol, X, Y, z0, nz, nullptr, h.nb[0],
                                                          h.nb[1], tsdf, w);
      else
        k_volume_import<StoreI16><<<blocks, 256, 0, st>>>((uint32_t*)h.vol, X, Y, z0, nz, h.nb[0], h.nb[1], tsdf, w);
      break;
  }
}
// g_uvv_Update_Valid_Volume (z_yooji_cuda_volume_integrator.cu:718-799, host
// :1035-1060): every sub-cube flagged by the last integration whose voxels
// are all invalid in `valid` (one byte per voxel, x fastest, 0 = invalid) is
// reset to the empty state (TSDF 1, weight 0, colour 0) and unflagged;
// sub-cubes with a valid voxel, and unflagged ones, are left as they are.
// One warp per brick: a lane tests rows 2 lane and 2 lane + 1 (8 bytes
// each, aligned: dim[0] is a multiple of 8 and `valid` 8-byte aligned).  The
// brick's occupancy bit is cleared (it holds no weight any more); the coarse
// cells around it stay set, which only costs the ray-caster a skip.
template <class S>
__global__ void k_carve(const SessionDev* __restrict__ s, const uint8_t* __restrict__ valid, unsigned* carved) {
  typename S::word* vol = reinterpret_cast<typename S::word*>(s->vol);
  const int nb0 = s->nb[0], nb1 = s->nb[1];
  const size_t nbr = (size_t)nb0 * nb1 * s->nb[2];
  const size_t X = (size_t)s->dim[0], XY = X * (size_t)s->dim[1];
  const uint32_t stamp = s->brick_count[2];
  const int lane = threadIdx.x & 31;
  const size_t gw = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarp = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t b = gw; b < nbr; b += nwarp) {
    const uint32_t f = s->brick_flag[b];
    if (f == 0u || f != stamp) continue;  // the same for the whole warp
    const int bx = (int)(b % nb0), by = (int)((b / nb0) % nb1), bz = (int)(b / ((size_t)nb0 * nb1));
    bool any = false;
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const int r = 2 * lane + k;
      const size_t o = (size_t)(bz * 8 + (r >> 3)) * XY + (size_t)(by * 8 + (r & 7)) * X + (size_t)bx * 8;
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(valid + o));
      any |= (v.x | v.y) != 0u;
    }
    if (__any_sync(0xffffffffu, any)) continue;
    const typename S::word e = S::initial();
    for (int k = lane; k < kBrickVox; k += 32) vol[b * kBrickVox + k] = e;
    if (s->col)
      for (int k = lane; k < kBrickVox; k += 32) s->col[b * kBrickVox + k] = 0u;
    if (lane == 0) {
      s->brick_flag[b] = 0u;
      if (s->band) s->band[b] = 0;
      atomicAnd(s->occ + (b >> 5), ~(1u << (b & 31)));
      atomicAdd(carved, 1u);
    }
  }
}

size_t occupancy_words(const SessionDev& h) { return (((size_t)h.nb[0] * h.nb[1] * h.nb[2]) + 31) / 32; }

void launch_occupancy_clear(const SessionDev& h, cudaStream_t st) {
  cudaMemsetAsync(h.occ, 0, occupancy_words(h) * 4, st);
  if (h.band) cudaMemsetAsync(h.band, 0, (size_t)h.nb[0] * h.nb[1] * h.nb[2], st);
}

void launch_occupancy_rebuild(const SessionDev& h, const SessionDev* d, cudaStream_t st) {
  launch_occupancy_clear(h, st);
  const int blocks = sm_count() * 8;
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      k_occupancy<StoreF16><<<blocks, 256, 0, st>>>(d);
      break;
    case VS_TSDF_FP32:
      k_occupancy<StoreF32><<<blocks, 256, 0, st>>>(d);
      break;
    default:
      k_occupancy<StoreI16><<<blocks, 256, 0, st>>>(d);
      break;
  }
}

void launch_carve(const SessionDev& h, const SessionDev* d, const uint8_t* valid, unsigned* carved, cudaStream_t st) {
  const int blocks = sm_count() * 8;
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      k_carve<StoreF16><<<blocks, 256, 0, st>>>(d, valid, carved);
      break;
    case VS_TSDF_FP32:
      k_carve<StoreF32><<<blocks, 256, 0, st>>>(d, valid, carved);
      break;
    default:
      k_carve<StoreI16><<<blocks, 256, 0, st>>>(d, valid, carved);
      break;
  }
}

int integrate_max_dim() { return kMaxDimLut; }
int integrate_max_image() { return kMaxImgLut; }

}  // namespace vs
