// Depth ingest, bilateral filter, depth pyramid and input vertex/normal maps.
//
// HBM-bound streaming stages: one pass over the uint16 frame, shared-memory
// tiles with halos, coalesced 2D blocks.  Each kernel restates one reference
// routine (paths relative to VCL_Volume_Scanner/):
//   k_bilateral      d_bilateral_filter  STAC/Engine/GPU/z_yooji_cuda_img_proc.cu:103-141
//   k_pyramid_down   sdg5 + ddh          STAC/Engine/CPU/z_yooji_image_processor.cpp:567-596,857-937
//   k_inmap_*        cpm + enm           STAC/Engine/CPU/z_yooji_image_processor.cpp:119-227
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int BX = 32, BY = 8;  // output tile of the bilateral filter

// The reference reads a linear-filtered texture at integer coordinates, so
// every tap is the mean of the 2x2 texels (X-1..X, Y-1..Y); out-of-range texel
// coordinates clamp to the edge.  A tile of BX x BY outputs needs taps
// X in [x0-2, x0+BX+1] and texels in [x0-3, x0+BX+1].
template <bool FROM_MM>
__global__ void __launch_bounds__(BX* BY)
    k_bilateral(const uint16_t* __restrict__ mm, const float* __restrict__ fin, float scale,
                float* __restrict__ raw_out, float* __restrict__ out, int W, int H, float g0,
                float g1, float g2) {
  __shared__ float tex[BY + 5][BX + 6];
  __shared__ float tap[BY + 4][BX + 5];
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int tid = threadIdx.y * BX + threadIdx.x;
  for (int i = tid; i < (BY + 5) * (BX + 5); i += BX * BY) {
    int ty = i / (BX + 5), tx = i - ty * (BX + 5);
    int gx = min(max(x0 - 3 + tx, 0), W - 1);
    int gy = min(max(y0 - 3 + ty, 0), H - 1);
    float v;
    if (FROM_MM)
      v = (float)mm[(size_t)gy * W + gx] * scale;
    else
      v = fin[(size_t)gy * W + gx];
    tex[ty][tx] = v;
  }
  __syncthreads();
  for (int i = tid; i < (BY + 4) * (BX + 4); i += BX * BY) {
    int ty = i / (BX + 4), tx = i - ty * (BX + 4);
    tap[ty][tx] = 0.25f * ((tex[ty][tx] + tex[ty][tx + 1]) + (tex[ty + 1][tx] + tex[ty + 1][tx + 1]));
  }
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  if (x >= W || y >= H) return;
  if (FROM_MM) raw_out[(size_t)y * W + x] = tex[ty + 3][tx + 3];
  const float g[5] = {g0, g1, g2, g1, g0};
  const float denom = 2.0f * 0.1f * 0.1f;  // 2 sigma_r^2, sigma_r = 0.1 m (z_yooji_cuda_img_proc.cu:44,91)
  const float center = tap[ty + 2][tx + 2];
  float t = 0.0f, sum = 0.0f;
#pragma unroll
  for (int i = -2; i <= 2; i++) {
#pragma unroll
    for (int j = -2; j <= 2; j++) {
      float cur = tap[ty + 2 + i][tx + 2 + j];
      if (cur <= 0.0f) {
        out[(size_t)y * W + x] = 0.0f;
        return;
      }
      float mod = (center - cur) * (center - cur);
      float factor = g[i + 2] * g[j + 2] * __expf(-mod / denom);
      t += factor * cur;
      sum += factor;
    }
  }
  out[(size_t)y * W + x] = t / sum;
}

// level l -> l+1: separable [1 4 6 4 1] smoothing (borders 0, no validity
// mask) evaluated only at the kept pixel (2 i2 + 1, 2 j2 + 1)
__global__ void k_pyramid_down(const float* __restrict__ in, int w, int h, float* __restrict__ out,
                               int w2, int h2) {
  int i2 = blockIdx.x * blockDim.x + threadIdx.x;
  int j2 = blockIdx.y * blockDim.y + threadIdx.y;
  if (i2 >= w2 || j2 >= h2) return;
  int i = 2 * i2 + 1, j = 2 * j2 + 1;
  float v = 0.0f;
  if (i >= 2 && i < w - 2 && j >= 2 && j < h - 2) {
    float pad[5];
#pragma unroll
    for (int r = 0; r < 5; r++) {
      const float* p = in + (size_t)(j - 2 + r) * w;
      pad[r] = p[i - 2] + p[i + 2] + 4.0f * p[i - 1] + 4.0f * p[i + 1] + 6.0f * p[i];
    }
    v = (pad[0] + pad[4] + 4.0f * pad[1] + 4.0f * pad[3] + 6.0f * pad[2]) / (16.0f * 16.0f);
  }
  out[(size_t)j2 * w2 + i2] = v;
}

// ---------------------------------------------------------------------------
// input vertex / normal maps (enm_Estimate_Normal_Map semantics)
//
// pass 1 (parallel): per interior pixel, code 0 = no normal (an invalid
//   point among the 5, or |dx|,|dy| < 1e-7), 1 = normal accepted,
//   2 = normal rejected by the 60 degree test; candidate normals are stored.
// pass 2 (one warp per level, rows in order): the reference rewrites the
//   point map in place on a rejection, which blocks the right and lower
//   neighbours.  With C = code2 & ~R(row above), a row solves
//   R_j = C_j & ~R_{j-1}: inside each run of C the rejected pixels alternate
//   starting at the run's first pixel.  Runs are smeared with one addition
//   per 32-bit word; the words of a row and the rows themselves are swept as
//   a wavefront across the lanes of the warp.
// pass 3 (parallel): vertex valid = depth > 0 and not rejected; normal valid =
//   code 1 and neither the left nor the upper neighbour rejected.
// ---------------------------------------------------------------------------
struct LevelPtrs {
  const float* depth;
  float4* vtx;
  float4* nrm;
  uint8_t* code;
  uint32_t* amask;
  uint32_t* rmask;
  int w, h;
  float K[4];
};
struct InmapArgs {
  LevelPtrs lv[kMaxLevels];
  int levels;
  int tiles[kMaxLevels + 1];  // prefix of tiles per level (32x8 for pre, 16x16 for post)
  int tiles_pre[kMaxLevels + 1];
};

__device__ inline bool bp_valid(const float* depth, int w, int x, int y, const float* K, F3& p) {
  float d = depth[(size_t)y * w + x];
  if (d <= 0.0f) return false;
  p = back_project((float)x, (float)y, K, d);
  return true;
}

__global__ void __launch_bounds__(256) k_inmap_pre(InmapArgs a) {
  int b = blockIdx.x, l = 0;
  while (l + 1 < a.levels && b >= a.tiles_pre[l + 1]) l++;
  const LevelPtrs& L = a.lv[l];
  const int t = b - a.tiles_pre[l];
  const int tw = (L.w + 31) / 32;
  const int x = (t % tw) * 32 + threadIdx.x, y = (t / tw) * 8 + threadIdx.y;
  if (y >= L.h) return;  // whole warp (a warp is one 32-pixel row segment)
  uint8_t code = 0;
  float4 n = make_float4(-100.0f, -100.0f, -100.0f, 0.0f);
  if (x >= 1 && x < L.w - 1 && y >= 1 && y < L.h - 1) {
    F3 c, x1, x2, y1, y2;
    bool ok = bp_valid(L.depth, L.w, x, y, L.K, c) && bp_valid(L.depth, L.w, x - 1, y, L.K, x1) &&
              bp_valid(L.depth, L.w, x + 1, y, L.K, x2) && bp_valid(L.depth, L.w, x, y - 1, L.K, y1) &&
              bp_valid(L.depth, L.w, x, y + 1, L.K, y2);
    if (ok) {
      float dx = x2.x - x1.x;
      float dy = y2.y - y1.y;
      if (!(fabsf(dx) < 1.0e-7f) && !(fabsf(dy) < 1.0e-7f)) {
        float dzdx = (x2.z - x1.z) / dx;
        float dzdy = (y2.z - y1.z) / dy;
        float len = sqrtf(dzdx * dzdx + dzdy * dzdy + 1.0f);
        float nx = dzdx / len, ny = dzdy / len, nz = -1.0f / len;
        // -n_z < cos(60 deg), the threshold taken in double as the reference's cos()
        if (-(double)nz < 0.50000000000000011) {
          code = 2;
        } else {
          code = 1;
          n = make_float4(nx, ny, nz, 0.0f);
        }
      }
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, code == 2);
  if (threadIdx.x == 0) L.amask[(size_t)y * tw + (t % tw)] = m;
  if (x >= L.w) return;
  L.code[(size_t)y * L.w + x] = code;
  L.nrm[(size_t)y * L.w + x] = n;
}

// one block per level: the block stages the level's code-2 bitmasks in
// shared memory, then warp 0 sweeps the rows as a wavefront: at step t lane l
// solves row t - l for its words, taking the carry of the row's earlier words
// from lane l - 1 (computed at step t - 1) and the rejections of the row above
// from its own registers, so one step costs one shuffle.
__global__ void __launch_bounds__(1024) k_inmap_scan(InmapArgs a) {
  extern __shared__ uint32_t amask[];  // [h][nw]
  const LevelPtrs& L = a.lv[blockIdx.x];
  const int nw = (L.w + 31) >> 5;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwords = L.h * nw;
  for (int i = threadIdx.x; i < nwords; i += blockDim.x) amask[i] = L.amask[i];
  __syncthreads();
  if (warp != 0) return;
  const uint32_t M0 = 0x55555555u, M1 = 0xaaaaaaaau;
  const int wpl = (nw + 31) >> 5;  // words per lane (1 up to 1024 pixels, 2 up to 2048)
  const int steps = L.h + 31;
  if (wpl == 1) {
    // both outcomes of a word are formed before its carry arrives, so a step's
    // critical path is one shuffle and one select
    const bool act = lane < nw;
    uint32_t rup = 0u, cout = 0u;
    for (int t = 0; t < steps; t++) {
      const int row = t - lane;
      const bool valid = act && row >= 0 && row < L.h;
      uint32_t R0 = 0u, R1 = 0u;
      if (valid && row > 0) {  // row 0 is never processed (interior rows only)
        const uint32_t C = amask[row * nw + lane] & ~rup;
        const uint32_t st = C & ~(C << 1);  // run starts (bit 0 counted as a start)
        const uint32_t ev = (C & ((C + ((st & ~1u) & M0)) ^ C)) & M0;
        const uint32_t od = (C & ((C + ((st & ~1u) & M1)) ^ C)) & M1;
        // a run at bit 0 continues the previous word's alternation: even
        // parity after a clear carry, odd after a set one
        const uint32_t b0 = st & 1u;
        R0 = ev | ((C & ((C + b0) ^ C)) & M0) | od;
        R1 = ev | od | ((C & ((C + b0) ^ C)) & M1);
      }
      uint32_t cin = __shfl_up_sync(0xffffffffu, cout, 1);
      if (lane == 0) cin = 0u;
      const uint32_t R = cin ? R1 : R0;
      if (valid) {
        L.rmask[(size_t)row * nw + lane] = R;
        rup = R;
      }
      cout = valid ? (R >> 31) : 0u;
    }
    return;
  }
  uint32_t rup[2] = {0u, 0u};  // this lane's words of the row above
  uint32_t cout_prev = 0u;
  for (int t = 0; t < steps; t++) {
    uint32_t cin = __shfl_up_sync(0xffffffffu, cout_prev, 1);
    if (lane == 0) cin = 0u;
    const int row = t - lane;
    uint32_t cout = 0u;
    if (row >= 0 && row < L.h) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int wi = lane * wpl + q;
        if (q < wpl && wi < nw) {
          uint32_t R = 0u;
          if (row > 0) {
            const uint32_t C = amask[row * nw + wi] & ~rup[q];
            const uint32_t st = C & ~(C << 1);
            const uint32_t rest = st & ~1u;
            const uint32_t se = (rest & M0) | (cin ? 0u : (st & 1u));
            const uint32_t so = (rest & M1) | (cin ? (st & 1u) : 0u);
            R = ((C & ((C + se) ^ C)) & M0) | ((C & ((C + so) ^ C)) & M1);
          }
          L.rmask[(size_t)row * nw + wi] = R;
          rup[q] = R;
          cin = R >> 31;
        }
      }
      cout = cin;
    }
    cout_prev = cout;
  }
}

__global__ void k_inmap_post(InmapArgs a) {
  int b = blockIdx.x, l = 0;
  while (l + 1 < a.levels && b >= a.tiles[l + 1]) l++;
  const LevelPtrs& L = a.lv[l];
  int t = b - a.tiles[l];
  int tw = (L.w + 15) / 16;
  int x = (t % tw) * 16 + threadIdx.x, y = (t / tw) * 16 + threadIdx.y;
  if (x >= L.w || y >= L.h) return;
  const int nw = (L.w + 31) >> 5;
  auto rej = [&](int xx, int yy) -> bool {
    if (xx < 0 || yy < 0) return false;
    return (L.rmask[(size_t)yy * nw + (xx >> 5)] >> (xx & 31)) & 1u;
  };
  size_t idx = (size_t)y * L.w + x;
  float d = L.depth[idx];
  float4 v = make_float4(-100.0f, -100.0f, -100.0f, 0.0f);
  if (d > 0.0f && !rej(x, y)) {
    F3 p = back_project((float)x, (float)y, L.K, d);
    v = make_float4(p.x, p.y, p.z, 1.0f);
  }
  L.vtx[idx] = v;
  uint8_t code = L.code[idx];
  float4 n = L.nrm[idx];
  if (code == 1 && !rej(x - 1, y) && !rej(x, y - 1)) {
    n.w = 1.0f;
  } else {
    n = make_float4(-100.0f, -100.0f, -100.0f, 0.0f);
  }
  L.nrm[idx] = n;
}

InmapArgs make_inmap_args(const SessionDev& h) {
  InmapArgs a;
  a.levels = h.levels;
  a.tiles[0] = 0;
  a.tiles_pre[0] = 0;
  for (int l = 0; l < kMaxLevels; l++) {
    LevelPtrs& L = a.lv[l];
    L.depth = h.depth[l];
    L.vtx = h.in_vtx[l];
    L.nrm = h.in_nrm[l];
    L.code = h.in_code[l];
    L.amask = h.in_amask[l];
    L.rmask = h.in_rmask[l];
    L.w = h.lv[l].W;
    L.h = h.lv[l].H;
    for (int k = 0; k < 4; k++) L.K[k] = h.lv[l].K[k];
    int nt = (l < h.levels) ? ((L.w + 15) / 16) * ((L.h + 15) / 16) : 0;
    a.tiles[l + 1] = a.tiles[l] + nt;
    int np = (l < h.levels) ? ((L.w + 31) / 32) * ((L.h + 7) / 8) : 0;
    a.tiles_pre[l + 1] = a.tiles_pre[l] + np;
  }
  return a;
}

}  // namespace

void launch_filter(const SessionDev* /*d*/, const SessionDev& h, cudaStream_t st) {
  const int W = h.lv[0].W, H = h.lv[0].H;
  dim3 blk(BX, BY), grd((W + BX - 1) / BX, (H + BY - 1) / BY);
  k_bilateral<true><<<grd, blk, 0, st>>>(h.depth_mm, nullptr, h.depth_scale, h.depth_raw, h.depth[0],
                                         W, H, h.gauss[0], h.gauss[1], h.gauss[2]);
  for (int l = 1; l < h.levels; l++) {
    dim3 b2(32, 8), g2((h.lv[l].W + 31) / 32, (h.lv[l].H + 7) / 8);
    k_pyramid_down<<<g2, b2, 0, st>>>(h.depth[l - 1], h.lv[l - 1].W, h.lv[l - 1].H, h.depth[l],
                                      h.lv[l].W, h.lv[l].H);
  }
}

void launch_bilateral_float(const SessionDev* /*d*/, const SessionDev& h, const float* in, float* out,
                            cudaStream_t st) {
  const int W = h.lv[0].W, H = h.lv[0].H;
  dim3 blk(BX, BY), grd((W + BX - 1) / BX, (H + BY - 1) / BY);
  k_bilateral<false><<<grd, blk, 0, st>>>(nullptr, in, 1.0f, nullptr, out, W, H, h.gauss[0], h.gauss[1],
                                          h.gauss[2]);
}

size_t inmap_scan_smem(const SessionDev& h) {
  size_t m = 0;
  for (int l = 0; l < h.levels; l++) {
    size_t b = (size_t)h.lv[l].H * ((h.lv[l].W + 31) / 32) * 4;
    if (b > m) m = b;
  }
  return m;
}

void launch_input_maps(const SessionDev* /*d*/, const SessionDev& h, cudaStream_t st) {
  InmapArgs a = make_inmap_args(h);
  dim3 b16(16, 16);
  k_inmap_pre<<<a.tiles_pre[h.levels], dim3(32, 8), 0, st>>>(a);
  size_t smem = inmap_scan_smem(h);
  k_inmap_scan<<<h.levels, 1024, smem, st>>>(a);
  k_inmap_post<<<a.tiles[h.levels], b16, 0, st>>>(a);
}

void configure_filter_kernels() {
  cudaFuncSetAttribute(k_inmap_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
}

}  // namespace vs
