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
// ray scale K^-1 [x y 1] come from shared-memory tables built with the same
// IEEE operations as the per-voxel reference formula, so the result stays
// bit-identical while the divisions leave the inner loop.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int kIntThreads = 256;
constexpr int kMaxDimLut = 1024;   // voxels per axis
constexpr int kMaxImgLut = 2048;   // pixels per image axis

// ROUNDF(v)/8 as the unparenthesised reference macro evaluates it
// (z_yooji_cuda_volume_integrator.cu:133-135)
__device__ inline int roundf_div8_ref(float x) { return (x < 0.0f) ? (int)(x - 0.5f) : (int)(x + 0.5f) / 8; }

__global__ void k_activate(const SessionDev* __restrict__ s, const float* __restrict__ depth,
                           const float* __restrict__ Tcg_in, int gate) {
  if (gate && s->pose->failed) return;
  const int W = s->lv[0].W, H = s->lv[0].H;
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= W || y >= H) return;
  float td = depth[(size_t)y * W + x];
  if (!(td > 0.0f)) return;
  float T[12];
#pragma unroll
  for (int k = 0; k < 12; k++) T[k] = Tcg_in[k];
  const float* K = s->lv[0].K;
  F3 p = transform(back_project((float)x, (float)y, K, td), T);
  F3 pe = transform(back_project((float)x, (float)y, K, 100.0f), T);
  F3 dv = normalised(sub(pe, p));
  const int nb0 = s->nb[0], nb1 = s->nb[1], nb2 = s->nb[2];
  int prev = -1;
  for (int n = -4; n <= 1; n++) {
    F3 tp = add(p, scale(((float)n) * s->mu, dv));
    F3 v;
    if (!pos_in_voxel(tp, *s, v)) continue;
    int xs = roundf_div8_ref(v.x), ys = roundf_div8_ref(v.y), zs = roundf_div8_ref(v.z);
    if (xs < 0 || xs >= nb0 || ys < 0 || ys >= nb1 || zs < 0 || zs >= nb2) break;
    int b = (zs * nb1 + ys) * nb0 + xs;
    if (b == prev) continue;
    prev = b;
    uint32_t* f = s->brick_flag + b;
    if (*((volatile uint32_t*)f) == 0u && atomicExch(f, 1u) == 0u) {
      uint32_t pos = atomicAdd(s->brick_count, 1u);
      s->brick_list[pos] = (uint32_t)b;
    }
  }
}

template <class S>
__global__ void __launch_bounds__(kIntThreads)
    k_integrate(const SessionDev* __restrict__ s, const float* __restrict__ depth,
                const float* __restrict__ Tgc_in, const float* __restrict__ Tcg_in, int gate) {
  if (gate && s->pose->failed) return;
  __shared__ float lut_p[3][kMaxDimLut];  // voxel centre coordinate per axis
  __shared__ float lut_rx[kMaxImgLut], lut_ry[kMaxImgLut];
  const int W = s->lv[0].W, H = s->lv[0].H;
  const float K0 = s->lv[0].K[0], K1 = s->lv[0].K[1], K2 = s->lv[0].K[2], K3 = s->lv[0].K[3];
  for (int a = 0; a < 3; a++)
    for (int i = threadIdx.x; i < s->dim[a]; i += blockDim.x)
      lut_p[a][i] = ((float)i + 0.5f) / s->vox_inv + s->origin[a];  // d_gpw_Get_Position_in_World
  for (int i = threadIdx.x; i < W; i += blockDim.x) lut_rx[i] = 1.0f * ((float)i - K2) / K0;
  for (int i = threadIdx.x; i < H; i += blockDim.x) lut_ry[i] = 1.0f * ((float)i - K3) / K1;
  float T[12];
#pragma unroll
  for (int k = 0; k < 12; k++) T[k] = Tgc_in[k];
  const float Cx = Tcg_in[3], Cy = Tcg_in[7], Cz = Tcg_in[11];
  const float mu = s->mu, max_w = s->max_w;
  const float K[4] = {K0, K1, K2, K3};
  __syncthreads();

  typedef typename S::word word;
  constexpr int kPerVec = 16 / sizeof(word);
  constexpr int kVecs = kBrickVox / kPerVec;  // 16-byte vectors per brick
  const int lane = threadIdx.x & 31;
  const int gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t count = *((volatile uint32_t*)s->brick_count);
  const int nb0 = s->nb[0], nb1 = s->nb[1];
  word* vol = reinterpret_cast<word*>(s->vol);

  for (uint32_t i = gwarp; i < count; i += nwarps) {
    const uint32_t b = s->brick_list[i];
    int nupd = 0;
    const int bx = (int)(b % (uint32_t)nb0), by = (int)((b / (uint32_t)nb0) % (uint32_t)nb1),
              bz = (int)(b / ((uint32_t)nb0 * (uint32_t)nb1));
    uint4* bv = reinterpret_cast<uint4*>(vol + (size_t)b * kBrickVox);
#pragma unroll 1
    for (int k = 0; k < kVecs / 32; k++) {
      const int vi = k * 32 + lane;
      uint4 raw = bv[vi];
      word wv[kPerVec];
      memcpy(wv, &raw, 16);
      bool changed = false;
#pragma unroll
      for (int e = 0; e < kPerVec; e++) {
        const int li = vi * kPerVec + e;
        const int xc = bx * 8 + (li & 7), yc = by * 8 + ((li >> 3) & 7), zc = bz * 8 + (li >> 6);
        float told;
        uint32_t wold;
        S::decode(wv[e], told, wold);
        const float oldW = (float)wold;
        if (oldW >= max_w) continue;
        F3 pg = f3(lut_p[0][xc], lut_p[1][yc], lut_p[2][zc]);
        F3 pc = transform(pg, T);
        float u, v;
        project(pc, K, u, v);
        int x = __float2int_rn(u), y = __float2int_rn(v);
        if (x < 0 || x > W - 1 || y < 0 || y > H - 1) continue;
        float dm = __ldg(depth + (size_t)y * W + x);
        if (!(dm > 0.0f)) continue;
        float rx = lut_rx[x], ry = lut_ry[y];
        float lam = 1.0f / sqrtf(rx * rx + ry * ry + 1.0f);
        F3 dc = f3(pg.x - Cx, pg.y - Cy, pg.z - Cz);
        float nrm = sqrtf(dc.x * dc.x + dc.y * dc.y + dc.z * dc.z);
        float sdf = dm - lam * nrm;
        if (sdf < -mu) continue;
        float ts = fminf(1.0f, sdf / mu);
        float newW = oldW + 1.0f;
        float inewW = 1.0f / newW;
        float tnew = (oldW * told + ts) * inewW;
        wv[e] = S::encode(tnew, (uint32_t)newW);
        changed = true;
        nupd++;
      }
      if (changed) {
        memcpy(&raw, wv, 16);
        bv[vi] = raw;
      }
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) nupd += __shfl_xor_sync(0xffffffffu, nupd, m);
    if (lane == 0) {
      s->brick_flag[b] = 0u;
      if (nupd) {
        atomicAdd(s->brick_count + 1, (uint32_t)nupd);
        // weights never decrease, so a brick that got an update stays occupied
        if (s->occ) atomicOr(s->occ + (b >> 5), 1u << (b & 31));
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

// recomputes the occupancy bits from the weights (after a volume import);
// one warp per brick
template <class S>
__global__ void k_occupancy(const typename S::word* vol, size_t nbr, uint32_t* occ) {
  const int lane = threadIdx.x & 31;
  const size_t gw = ((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const size_t nwarp = ((size_t)gridDim.x * blockDim.x) >> 5;
  for (size_t b = gw; b < nbr; b += nwarp) {
    bool any = false;
    for (int k = lane; k < kBrickVox; k += 32) {
      float t;
      uint32_t w;
      S::decode(vol[b * kBrickVox + k], t, w);
      any |= w != 0u;
    }
    const unsigned m = __ballot_sync(0xffffffffu, any);
    if (lane == 0 && m) atomicOr(occ + (b >> 5), 1u << (b & 31));
  }
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

}  // namespace

void launch_integrate(const SessionDev* d, const SessionDev& h, const float* depth, const float* Tgc,
                      const float* Tcg, bool gate, cudaStream_t st) {
  cudaMemsetAsync(h.brick_count, 0, 2 * sizeof(uint32_t), st);
  dim3 b(32, 8), g((h.lv[0].W + 31) / 32, (h.lv[0].H + 7) / 8);
  k_activate<<<g, b, 0, st>>>(d, depth, Tcg, gate ? 1 : 0);
  // persistent grid: enough warps to cover every SM several times over
  int blocks = sm_count() * 4;
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      k_integrate<StoreF16><<<blocks, kIntThreads, 0, st>>>(d, depth, Tgc, Tcg, gate ? 1 : 0);
      break;
    case VS_TSDF_FP32:
      k_integrate<StoreF32><<<blocks, kIntThreads, 0, st>>>(d, depth, Tgc, Tcg, gate ? 1 : 0);
      break;
    default:
      k_integrate<StoreI16><<<blocks, kIntThreads, 0, st>>>(d, depth, Tgc, Tcg, gate ? 1 : 0);
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

void launch_occupancy_rebuild(const SessionDev& h, cudaStream_t st) {
  const size_t nbr = (size_t)h.nb[0] * h.nb[1] * h.nb[2];
  cudaMemsetAsync(h.occ, 0, ((nbr + 31) / 32) * 4, st);
  const int blocks = sm_count() * 8;
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      k_occupancy<StoreF16><<<blocks, 256, 0, st>>>((const uint32_t*)h.vol, nbr, h.occ);
      break;
    case VS_TSDF_FP32:
      k_occupancy<StoreF32><<<blocks, 256, 0, st>>>((const uint2*)h.vol, nbr, h.occ);
      break;
    default:
      k_occupancy<StoreI16><<<blocks, 256, 0, st>>>((const uint32_t*)h.vol, nbr, h.occ);
      break;
  }
}

int integrate_max_dim() { return kMaxDimLut; }
int integrate_max_image() { return kMaxImgLut; }

}  // namespace vs
