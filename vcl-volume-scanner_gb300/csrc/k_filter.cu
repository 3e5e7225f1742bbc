// Depth ingest, bilateral filter, depth pyramid and input vertex/normal maps.
//
// HBM-bound streaming stages: one pass over the uint16 frame, shared-memory
// tiles with halos, coalesced 2D blocks.  Every kernel is persistent over the
// tiles of all sessions of a batch table (one session = a table of one).
// Each kernel restates one reference routine (paths relative to
// VCL_Volume_Scanner/):
//   k_bilateral_*    d_bilateral_filter  STAC/Engine/GPU/z_yooji_cuda_img_proc.cu:103-141
//   k_pyramid_batch  sdg5 + ddh          STAC/Engine/CPU/z_yooji_image_processor.cpp:567-596,857-937
//   k_inmap_*        cpm + enm           STAC/Engine/CPU/z_yooji_image_processor.cpp:119-227
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstring>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int BX = 32, BY = 8;  // output tile of the bilateral filter (BY: default rows; 4 and 16 also built)
constexpr int kScanSmem = 64 * 1024;  // staged normal-rejection bitmasks of one level

// The reference reads a linear-filtered texture at integer coordinates, so
// every tap is the mean of the 2x2 texels (X-1..X, Y-1..Y); out-of-range texel
// coordinates clamp to the edge.  A tile of BX x BY outputs needs taps
// X in [x0-2, x0+BX+1] and texels in [x0-3, x0+BX+1].
template <int R>
struct BilateralSmem {
  float tex[R + 5][BX + 6];
  float tap[R + 4][BX + 5];
};

template <int R>
__device__ inline float bilateral_px(const BilateralSmem<R>& m, int tx, int ty, const float g[5]) {
  // The reference's exponent is -mod / (2 sigma_r^2), 2 sigma_r^2 = 2.0f *
  // 0.1f * 0.1f with sigma_r = 0.1 m (z_yooji_cuda_img_proc.cu:44,91).  Here
  // it is the product with the folded constant -1 / (2 sigma_r^2): one
  // rounding more than the quotient (a relative 1.2e-7 of an exponent that
  // matters only below ~20), far inside the 1e-5 m tolerance of the filtered
  // depth, and no division per tap.
  constexpr float kNegInvDenom = -1.0f / (2.0f * 0.1f * 0.1f);
  const float center = m.tap[ty + 2][tx + 2];
  float t = 0.0f, sum = 0.0f;
#pragma unroll
  for (int i = -2; i <= 2; i++) {
#pragma unroll
    for (int j = -2; j <= 2; j++) {
      float cur = m.tap[ty + 2 + i][tx + 2 + j];
      if (cur <= 0.0f) return 0.0f;
      float mod = (center - cur) * (center - cur);
      float factor = g[i + 2] * g[j + 2] * __expf(mod * kNegInvDenom);
      t += factor * cur;
      sum += factor;
    }
  }
  return t / sum;
}

// one BX x R output tile; the block's BX x R threads all take part (two barriers)
template <bool FROM_MM, int R>
__device__ inline void bilateral_tile(BilateralSmem<R>& m, const uint16_t* __restrict__ mm,
                                      const float* __restrict__ fin, float scale, float* __restrict__ raw_out,
                                      float* __restrict__ out, int W, int H, int x0, int y0, const float g[5],
                                      float2* __restrict__ dl_out = nullptr, const float* __restrict__ lam = nullptr) {
  const int tid = threadIdx.y * BX + threadIdx.x;
  for (int i = tid; i < (R + 5) * (BX + 5); i += BX * R) {
    int ty = i / (BX + 5), tx = i - ty * (BX + 5);
    int gx = min(max(x0 - 3 + tx, 0), W - 1);
    int gy = min(max(y0 - 3 + ty, 0), H - 1);
    float v;
    if (FROM_MM)
      v = (float)mm[(size_t)gy * W + gx] * scale;
    else
      v = fin[(size_t)gy * W + gx];
    m.tex[ty][tx] = v;
  }
  __syncthreads();
  for (int i = tid; i < (R + 4) * (BX + 4); i += BX * R) {
    int ty = i / (BX + 4), tx = i - ty * (BX + 4);
    m.tap[ty][tx] = 0.25f * ((m.tex[ty][tx] + m.tex[ty][tx + 1]) + (m.tex[ty + 1][tx] + m.tex[ty + 1][tx + 1]));
  }
  __syncthreads();
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x = x0 + tx, y = y0 + ty;
  if (x < W && y < H) {
    if (FROM_MM) {
      const float raw = m.tex[ty + 3][tx + 3];
      raw_out[(size_t)y * W + x] = raw;
      if (dl_out) dl_out[(size_t)y * W + x] = make_float2(raw, __ldg(lam + (size_t)y * W + x));
    }
    out[(size_t)y * W + x] = bilateral_px(m, tx, ty, g);
  }
}

template <int R>
__global__ void __launch_bounds__(BX* R) k_bilateral_batch(const BatchTable* __restrict__ bt) {
  __shared__ BilateralSmem<R> m;
  const int n = bt->n;
  const int total = bt->bil[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int t;
    const int slot = find_slot(bt->bil, n, item, t);
    const SessionDev* __restrict__ s = bt->s[slot];
    const int W = s->lv[0].W, H = s->lv[0].H;
    const int tw = (W + BX - 1) / BX;
    const float g[5] = {s->gauss[0], s->gauss[1], s->gauss[2], s->gauss[1], s->gauss[0]};
    const uint16_t* __restrict__ mm = bt->frame[slot] ? bt->frame[slot] : s->depth_mm;
    bilateral_tile<true, R>(m, mm, nullptr, s->depth_scale, s->depth_raw, s->depth[0], W, H, (t % tw) * BX,
                            (t / tw) * R, g, s->lam_map ? s->dl_map : nullptr, s->lam_map);
    if (mm != s->depth_mm) {
      // a frame read in place: the session's own frame buffer is kept current
      const int x = (t % tw) * BX + threadIdx.x, y = (t / tw) * R + threadIdx.y;
      if (x < W && y < H) s->depth_mm[(size_t)y * W + x] = mm[(size_t)y * W + x];
    }
    if (s->rgb_packed) {
      // the colour frame as one word per pixel, for the integration's gathers
      const int x = (t % tw) * BX + threadIdx.x, y = (t / tw) * R + threadIdx.y;
      if (x < W && y < H) {
        const size_t i = (size_t)y * W + x, plane = (size_t)W * H;
        s->rgb_packed[i] = pack_rgb(s->rgb_in[i], s->rgb_in[plane + i], s->rgb_in[2 * plane + i]);
      }
    }
    __syncthreads();  // the next tile overwrites the shared tiles
  }
}

__global__ void __launch_bounds__(BX* BY)
    k_bilateral_float(const float* __restrict__ in, float* __restrict__ out, int W, int H, float g0, float g1,
                      float g2) {
  __shared__ BilateralSmem<BY> m;
  const float g[5] = {g0, g1, g2, g1, g0};
  bilateral_tile<false, BY>(m, nullptr, in, 1.0f, nullptr, out, W, H, blockIdx.x * BX, blockIdx.y * BY, g);
}

// level l -> l+1: separable [1 4 6 4 1] smoothing (borders 0, no validity
// mask) evaluated only at the kept pixel (2 i2 + 1, 2 j2 + 1)
__global__ void __launch_bounds__(256) k_pyramid_batch(const BatchTable* __restrict__ bt, int l2) {
  const int n = bt->n;
  const int* pre = bt->pyr[l2 - 1];
  const int total = pre[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int t;
    const int slot = find_slot(pre, n, item, t);
    const SessionDev* __restrict__ s = bt->s[slot];
    const int w = s->lv[l2 - 1].W, h = s->lv[l2 - 1].H, w2 = s->lv[l2].W, h2 = s->lv[l2].H;
    const int tw = (w2 + 31) / 32;
    const int i2 = (t % tw) * 32 + threadIdx.x, j2 = (t / tw) * 8 + threadIdx.y;
    if (i2 >= w2 || j2 >= h2) continue;
    const float* __restrict__ in = s->depth[l2 - 1];
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
    s->depth[l2][(size_t)j2 * w2 + i2] = v;
  }
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
// A session's items cover its levels in order; the per-level tile counts
// follow from the level sizes.
// ---------------------------------------------------------------------------
__device__ inline int level_of_tile(const SessionDev& s, int tile_w, int tile_h, int& t) {
  int l = 0;
  for (; l < s.levels - 1; l++) {
    const int nt = ((s.lv[l].W + tile_w - 1) / tile_w) * ((s.lv[l].H + tile_h - 1) / tile_h);
    if (t < nt) break;
    t -= nt;
  }
  return l;
}

__device__ inline bool bp_valid(const float* depth, int w, int x, int y, const float* K, F3& p) {
  float d = depth[(size_t)y * w + x];
  if (d <= 0.0f) return false;
  p = back_project((float)x, (float)y, K, d);
  return true;
}

__global__ void __launch_bounds__(256) k_inmap_pre(const BatchTable* __restrict__ bt) {
  const int n = bt->n;
  const int total = bt->ipre[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int t;
    const int slot = find_slot(bt->ipre, n, item, t);
    const SessionDev& s = *bt->s[slot];
    const int l = level_of_tile(s, 32, 8, t);
    const int w = s.lv[l].W, h = s.lv[l].H;
    const float K[4] = {s.lv[l].K[0], s.lv[l].K[1], s.lv[l].K[2], s.lv[l].K[3]};
    const float* __restrict__ depth = s.depth[l];
    const int tw = (w + 31) / 32;
    const int x = (t % tw) * 32 + threadIdx.x, y = (t / tw) * 8 + threadIdx.y;
    if (y >= h) continue;  // whole warp (a warp is one 32-pixel row segment)
    uint8_t code = 0;
    float4 nv = make_float4(-100.0f, -100.0f, -100.0f, 0.0f);
    if (x >= 1 && x < w - 1 && y >= 1 && y < h - 1) {
      F3 c, x1, x2, y1, y2;
      bool ok = bp_valid(depth, w, x, y, K, c) && bp_valid(depth, w, x - 1, y, K, x1) &&
                bp_valid(depth, w, x + 1, y, K, x2) && bp_valid(depth, w, x, y - 1, K, y1) &&
                bp_valid(depth, w, x, y + 1, K, y2);
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
            nv = make_float4(nx, ny, nz, 0.0f);
          }
        }
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, code == 2);
    if (threadIdx.x == 0) s.in_amask[l][(size_t)y * tw + (t % tw)] = m;
    if (x >= w) continue;
    s.in_code[l][(size_t)y * w + x] = code;
    s.in_nrm[l][(size_t)y * w + x] = nv;
  }
}

// Row sweep of one level: warp 0 sweeps the rows as a wavefront: at step t
// lane l solves row t - l for its words, taking the carry of the row's earlier
// words from lane l - 1 (computed at step t - 1) and the rejections of the row
// above from its own registers, so one step costs one shuffle.  am: the
// level's code-2 bitmasks (shared memory when they fit, else global).
__device__ void scan_level(const uint32_t* am, uint32_t* __restrict__ rmask, int w, int h) {
  const int nw = (w + 31) >> 5;
  const int lane = threadIdx.x & 31;
  const uint32_t M0 = 0x55555555u, M1 = 0xaaaaaaaau;
  const int wpl = (nw + 31) >> 5;  // words per lane (1 up to 1024 pixels, 2 up to 2048)
  const int steps = h + 31;
  if (wpl == 1) {
    // both outcomes of a word are formed before its carry arrives, so a step's
    // critical path is one shuffle and one select
    const bool act = lane < nw;
    uint32_t rup = 0u, cout = 0u;
    for (int t = 0; t < steps; t++) {
      const int row = t - lane;
      const bool valid = act && row >= 0 && row < h;
      uint32_t R0 = 0u, R1 = 0u;
      if (valid && row > 0) {  // row 0 is never processed (interior rows only)
        const uint32_t C = am[row * nw + lane] & ~rup;
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
        rmask[(size_t)row * nw + lane] = R;
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
    if (row >= 0 && row < h) {
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int wi = lane * wpl + q;
        if (q < wpl && wi < nw) {
          uint32_t R = 0u;
          if (row > 0) {
            const uint32_t C = am[row * nw + wi] & ~rup[q];
            const uint32_t st = C & ~(C << 1);
            const uint32_t rest = st & ~1u;
            const uint32_t se = (rest & M0) | (cin ? 0u : (st & 1u));
            const uint32_t so = (rest & M1) | (cin ? (st & 1u) : 0u);
            R = ((C & ((C + se) ^ C)) & M0) | ((C & ((C + so) ^ C)) & M1);
          }
          rmask[(size_t)row * nw + wi] = R;
          rup[q] = R;
          cin = R >> 31;
        }
      }
      cout = cin;
    }
    cout_prev = cout;
  }
}

// one block per (session, level) item
__global__ void __launch_bounds__(1024) k_inmap_scan(const BatchTable* __restrict__ bt) {
  extern __shared__ uint32_t amask[];  // [h][nw] of the current item
  const int n = bt->n;
  const int total = bt->scan[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int l;
    const int slot = find_slot(bt->scan, n, item, l);
    const SessionDev& s = *bt->s[slot];
    const int w = s.lv[l].W, h = s.lv[l].H;
    const int nwords = h * ((w + 31) >> 5);
    const uint32_t* src = s.in_amask[l];
    const bool staged = nwords * 4 <= kScanSmem;
    if (staged)
      for (int i = threadIdx.x; i < nwords; i += blockDim.x) amask[i] = src[i];
    __syncthreads();
    if (threadIdx.x < 32) scan_level(staged ? amask : src, s.in_rmask[l], w, h);
    __syncthreads();  // the next item restages the shared masks
  }
}

__global__ void __launch_bounds__(256) k_inmap_post(const BatchTable* __restrict__ bt) {
  const int n = bt->n;
  const int total = bt->ipost[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int t;
    const int slot = find_slot(bt->ipost, n, item, t);
    const SessionDev& s = *bt->s[slot];
    const int l = level_of_tile(s, 16, 16, t);
    const int w = s.lv[l].W, h = s.lv[l].H;
    const int tw = (w + 15) / 16;
    const int x = (t % tw) * 16 + threadIdx.x, y = (t / tw) * 16 + threadIdx.y;
    if (x >= w || y >= h) continue;
    const int nw = (w + 31) >> 5;
    const uint32_t* __restrict__ rm = s.in_rmask[l];
    auto rej = [&](int xx, int yy) -> bool {
      if (xx < 0 || yy < 0) return false;
      return (rm[(size_t)yy * nw + (xx >> 5)] >> (xx & 31)) & 1u;
    };
    const size_t idx = (size_t)y * w + x;
    const float d = s.depth[l][idx];
    float4 v = make_float4(-100.0f, -100.0f, -100.0f, 0.0f);
    if (d > 0.0f && !rej(x, y)) {
      F3 p = back_project((float)x, (float)y, s.lv[l].K, d);
      v = make_float4(p.x, p.y, p.z, 1.0f);
    }
    s.in_vtx[l][idx] = v;
    const uint8_t code = s.in_code[l][idx];
    float4 nv = s.in_nrm[l][idx];
    if (code == 1 && !rej(x - 1, y) && !rej(x, y - 1)) {
      nv.w = 1.0f;
    } else {
      nv = make_float4(-100.0f, -100.0f, -100.0f, 0.0f);
    }
    s.in_nrm[l][idx] = nv;
  }
}

}  // namespace

void launch_filter(const BatchTable* bt, cudaStream_t st, int rows) {
  const int grid = sm_count() * 8;
  switch (rows) {
    case 4:
      k_bilateral_batch<4><<<grid * 2, dim3(BX, 4), 0, st>>>(bt);
      break;
    case 16:
      k_bilateral_batch<16><<<grid / 2, dim3(BX, 16), 0, st>>>(bt);
      break;
    default:
      k_bilateral_batch<BY><<<grid, dim3(BX, BY), 0, st>>>(bt);
      break;
  }
  for (int l = 1; l < kMaxLevels; l++) k_pyramid_batch<<<grid, dim3(32, 8), 0, st>>>(bt, l);
}

void launch_input_maps(const BatchTable* bt, cudaStream_t st) {
  const int grid = sm_count() * 8;
  k_inmap_pre<<<grid, dim3(32, 8), 0, st>>>(bt);
  k_inmap_scan<<<kMaxSlots * kMaxLevels, 1024, kScanSmem, st>>>(bt);
  k_inmap_post<<<grid, dim3(16, 16), 0, st>>>(bt);
}

void launch_bilateral_float(const SessionDev& h, const float* in, float* out, cudaStream_t st) {
  const int W = h.lv[0].W, H = h.lv[0].H;
  dim3 blk(BX, BY), grd((W + BX - 1) / BX, (H + BY - 1) / BY);
  k_bilateral_float<<<grd, blk, 0, st>>>(in, out, W, H, h.gauss[0], h.gauss[1], h.gauss[2]);
}

void configure_filter_kernels() {
  cudaFuncSetAttribute(k_inmap_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, kScanSmem);
}

// work-item prefixes of a batch; host_recs are the host copies of the
// session records, dev_recs their device addresses
void fill_batch_table(BatchTable& hb, const SessionDev* const* host_recs, const SessionDev* const* dev_recs, int n,
                      int ray_lx, int bil_rows) {
  std::memset(&hb, 0, sizeof(hb));
  hb.n = n;
  hb.ray_lx = ray_lx;
  hb.bil_rows = (bil_rows == 4 || bil_rows == 16) ? bil_rows : BY;
  const int rx = 1 << ray_lx, ry = 32 >> ray_lx;
  for (int i = 0; i < n; i++) {
    const SessionDev& h = *host_recs[i];
    hb.s[i] = dev_recs[i];
    const bool nm = h.cos_normal > -2.0f;
    int ipre = 0, ipost = 0, ray = 0;
    for (int l = 0; l < h.levels; l++) {
      const int w = h.lv[l].W, hh = h.lv[l].H;
      ipre += ((w + 31) / 32) * ((hh + 7) / 8);
      ipost += ((w + 15) / 16) * ((hh + 15) / 16);
      ray += ((w + rx - 1) / rx) * ((hh + ry - 1) / ry);
    }
    hb.bil[i + 1] = hb.bil[i] + ((h.lv[0].W + BX - 1) / BX) * ((h.lv[0].H + hb.bil_rows - 1) / hb.bil_rows);
    for (int l = 1; l < kMaxLevels; l++)
      hb.pyr[l - 1][i + 1] =
          hb.pyr[l - 1][i] + (l < h.levels ? ((h.lv[l].W + 31) / 32) * ((h.lv[l].H + 7) / 8) : 0);
    hb.ipre[i + 1] = hb.ipre[i] + (nm ? ipre : 0);
    hb.ipost[i + 1] = hb.ipost[i] + (nm ? ipost : 0);
    hb.scan[i + 1] = hb.scan[i] + (nm ? h.levels : 0);
    for (int l = 0; l < kMaxLevels; l++)
      hb.icp[l][i + 1] = hb.icp[l][i] + (l < h.levels ? icp_blocks(h.lv[l].W * h.lv[l].H, l) : 0);
    hb.ray[i + 1] = hb.ray[i] + ray;
    hb.slab[i + 1] = hb.slab[i] + (h.bdist ? h.nb[2] : 0);
    hb.brow[i + 1] = hb.brow[i] + (h.bdist ? h.nb[1] : 0);
  }
}

}  // namespace vs
