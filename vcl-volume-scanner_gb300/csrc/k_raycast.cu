// TSDF ray casting into model depth / vertex / normal maps.
//
// Reference: g_rmi_Render_Maps_for_ICP, d_crtc_Cast_Ray_on_TSDF_Cube_NEW,
// d_gtvu / d_gtvi and d_csnt (STAC/Engine/GPU/z_yooji_cuda_tsdf_renderer.cu:
// 1069-1209, 466-635, 68-153, 288-464; host set-up :1642-1700).  The
// reference launches one 16x16-block grid per pyramid level; here one
// persistent launch covers every level of every session of a batch table
// (blocks take 16x8 tiles from an atomic work counter, so a slow tile near a
// surface does not hold up a whole grid row), each ray keeps its whole march
// state in registers, and every voxel read is one 32-bit word that carries
// both the TSDF value and the weight (one gather instead of the reference's
// separate float and uchar arrays).
//
// The reference's march loop has no iteration bound: a fine-search ray whose
// signed steps keep changing direction never leaves it.  The loop here ends
// after 4 * (2 r_cube / voxel) + 64 steps and reports no hit; the CPU oracle
// applies the same bound.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

constexpr int TX = 16, TY = 8;

struct RayArgs {
  const BatchTable* bt;
  unsigned* work;       // [0] next tile, [1] finished blocks; zero between launches
  int level;            // < 0: every level of every slot into the model maps
  // explicit poses and outputs of a one-level, one-slot call (reference layout)
  const float* Tgc;
  const float* Tcg;
  const float* center;  // device float[3]
  float light[3];
  int gate;
  float* out_depth;
  float* out_vtx3;
  float* out_nrm3;
  uint8_t* out_img;
};

// Volume reads.  A brick whose occupancy bit is clear has weight 0 in every
// voxel (weights only grow), so its voxels answer "no value" from a 32 KB
// bitmap that stays in L1 instead of a volume gather: free-space steps of the
// march cost no HBM traffic, with results identical to reading the voxel.
template <class S>
struct Vol {
  const typename S::word* v;
  const uint32_t* occ;
  int dim[3];
  int nb[3];
  __device__ inline bool occupied(int x, int y, int z) const {
    const uint32_t b = ((uint32_t)(z >> 3) * (uint32_t)nb[1] + (uint32_t)(y >> 3)) * (uint32_t)nb[0] + (uint32_t)(x >> 3);
    return (__ldg(occ + (b >> 5)) >> (b & 31)) & 1u;
  }
  // d_gtvu_Get_TSDF_Value_Uninterpolated: nearest voxel (ROUNDF), weight > 0
  __device__ inline bool gtvu(F3 p, float& out) const {
    out = 1.0f;
    if (isnan(p.x) || isnan(p.y) || isnan(p.z)) return false;
    int x = roundf_ref(p.x), y = roundf_ref(p.y), z = roundf_ref(p.z);
    if (x < 0 || x >= dim[0] || y < 0 || y >= dim[1] || z < 0 || z >= dim[2]) return false;
    if (!occupied(x, y, z)) return false;
    float t;
    uint32_t w;
    S::decode(__ldg(v + brick_word_index(x, y, z, nb)), t, w);
    if (w == 0u) return false;
    out = t;
    return true;
  }
  __device__ inline bool at(int x, int y, int z, float& out) const {
    if (x < 0 || x >= dim[0] || y < 0 || y >= dim[1] || z < 0 || z >= dim[2]) return false;
    if (!occupied(x, y, z)) return false;
    float t;
    uint32_t w;
    S::decode(__ldg(v + brick_word_index(x, y, z, nb)), t, w);
    if (w == 0u) return false;
    out = t;
    return true;
  }
  // d_gtvi_Get_TSDF_Value_Interpolated (offset = floor, see the oracle)
  __device__ inline bool gtvi(F3 p, float& out) const {
    out = 1.0f;
    if (isnan(p.x) || isnan(p.y) || isnan(p.z)) return false;
    float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
    int ox = (int)fx, oy = (int)fy, oz = (int)fz;
    float rx = p.x - fx, ry = p.y - fy, rz = p.z - fz;
    float f0, f1, f2, f3_, b0, b1, b2, b3;
    if (!at(ox, oy, oz, f0) || !at(ox + 1, oy, oz, f1) || !at(ox, oy + 1, oz, f2) || !at(ox + 1, oy + 1, oz, f3_))
      return false;
    if (!at(ox, oy, oz + 1, b0) || !at(ox + 1, oy, oz + 1, b1) || !at(ox, oy + 1, oz + 1, b2) ||
        !at(ox + 1, oy + 1, oz + 1, b3))
      return false;
    float inf = (1.0f - ry) * ((1.0f - rx) * f0 + rx * f1) + ry * ((1.0f - rx) * f2 + rx * f3_);
    float inb = (1.0f - ry) * ((1.0f - rx) * b0 + rx * b1) + ry * ((1.0f - rx) * b2 + rx * b3);
    out = (1.0f - rz) * inf + rz * inb;
    return true;
  }
};

// d_csnt_Compute_Surface_Normal_from_TSDF: gradient of the trilinear field from
// a 4 + 12 + 12 + 4 voxel stencil
template <class S>
__device__ bool surface_normal(const Vol<S>& V, const SessionDev& s, F3 p3d, F3& nout) {
  F3 vox;
  if (!pos_in_voxel(p3d, s, vox)) return false;
  if (isnan(vox.x) || isnan(vox.y) || isnan(vox.z)) return false;
  float fx = floorf(vox.x), fy = floorf(vox.y), fz = floorf(vox.z);
  const int ox = (int)fx, oy = (int)fy, oz = (int)fz;
  const float rx = vox.x - fx, ry = vox.y - fy, rz = vox.z - fz;
  const int dx1[4] = {0, 1, 0, 1}, dy1[4] = {0, 0, 1, 1};
  const int dx2[12] = {0, 1, -1, 0, 1, 2, -1, 0, 1, 2, 0, 1};
  const int dy2[12] = {-1, -1, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2};
  float fm[4], fr[12], bk[12], bm[4];
#pragma unroll
  for (int i = 0; i < 4; i++)
    if (!V.at(ox + dx1[i], oy + dy1[i], oz - 1, fm[i])) return false;
#pragma unroll
  for (int i = 0; i < 12; i++)
    if (!V.at(ox + dx2[i], oy + dy2[i], oz, fr[i])) return false;
#pragma unroll
  for (int i = 0; i < 12; i++)
    if (!V.at(ox + dx2[i], oy + dy2[i], oz + 1, bk[i])) return false;
#pragma unroll
  for (int i = 0; i < 4; i++)
    if (!V.at(ox + dx1[i], oy + dy1[i], oz + 2, bm[i])) return false;
  float a4[4], b4[4], a2[2], b2[2], gx, gy, gz;
  a4[0] = (1.0f - rz) * fr[2] + rz * bk[2];
  a4[1] = (1.0f - rz) * fr[3] + rz * bk[3];
  a4[2] = (1.0f - rz) * fr[4] + rz * bk[4];
  a4[3] = (1.0f - rz) * fr[5] + rz * bk[5];
  b4[0] = (1.0f - rz) * fr[6] + rz * bk[6];
  b4[1] = (1.0f - rz) * fr[7] + rz * bk[7];
  b4[2] = (1.0f - rz) * fr[8] + rz * bk[8];
  b4[3] = (1.0f - rz) * fr[9] + rz * bk[9];
  a2[0] = (1.0f - rx) * a4[0] + rx * a4[1];
  a2[1] = (1.0f - rx) * b4[0] + rx * b4[1];
  b2[0] = (1.0f - rx) * a4[2] + rx * a4[3];
  b2[1] = (1.0f - rx) * b4[2] + rx * b4[3];
  gx = (1.0f - ry) * b2[0] + ry * b2[1];
  gx -= (1.0f - ry) * a2[0] + ry * a2[1];
  a4[0] = (1.0f - rz) * fr[0] + rz * bk[0];
  a4[1] = (1.0f - rz) * fr[3] + rz * bk[3];
  a4[2] = (1.0f - rz) * fr[7] + rz * bk[7];
  a4[3] = (1.0f - rz) * fr[10] + rz * bk[10];
  b4[0] = (1.0f - rz) * fr[1] + rz * bk[1];
  b4[1] = (1.0f - rz) * fr[4] + rz * bk[4];
  b4[2] = (1.0f - rz) * fr[8] + rz * bk[8];
  b4[3] = (1.0f - rz) * fr[11] + rz * bk[11];
  a2[0] = (1.0f - ry) * a4[0] + ry * a4[1];
  a2[1] = (1.0f - ry) * b4[0] + ry * b4[1];
  b2[0] = (1.0f - ry) * a4[2] + ry * a4[3];
  b2[1] = (1.0f - ry) * b4[2] + ry * b4[3];
  gy = (1.0f - rx) * b2[0] + rx * b2[1];
  gy -= (1.0f - rx) * a2[0] + rx * a2[1];
  a4[0] = (1.0f - ry) * fm[0] + ry * fm[2];
  a4[1] = (1.0f - ry) * fr[3] + ry * fr[7];
  a4[2] = (1.0f - ry) * bk[3] + ry * bk[7];
  a4[3] = (1.0f - ry) * bm[0] + ry * bm[2];
  b4[0] = (1.0f - ry) * fm[1] + ry * fm[3];
  b4[1] = (1.0f - ry) * fr[4] + ry * fr[8];
  b4[2] = (1.0f - ry) * bk[4] + ry * bk[8];
  b4[3] = (1.0f - ry) * bm[1] + ry * bm[3];
  a2[0] = (1.0f - rz) * a4[0] + rz * a4[1];
  a2[1] = (1.0f - rz) * b4[0] + rz * b4[1];
  b2[0] = (1.0f - rz) * a4[2] + rz * a4[3];
  b2[1] = (1.0f - rz) * b4[2] + rz * b4[3];
  gz = (1.0f - rx) * b2[0] + rx * b2[1];
  gz -= (1.0f - rx) * a2[0] + rx * a2[1];
  if (gx == 0.0f && gy == 0.0f && gz == 0.0f) return false;
  nout = normalised(f3(gx, gy, gz));
  return true;
}

template <class S>
__device__ bool cast_ray(const Vol<S>& V, const SessionDev& s, const float* K, float px, float py,
                         const float* Tcg, F3 cam, F3 ncc, float dist_cc, float theta_max, F3& p3d) {
  enum { COARSE, FINE, BEHIND };
  const float dmin = dist_cc - s.r_cube, dmax = dist_cc + s.r_cube;
  F3 pe = transform(back_project(px, py, K, dmax), Tcg);
  F3 rd = normalised(sub(pe, cam));
  float theta = acosf(dot(rd, ncc));
  if (theta > theta_max) return false;
  F3 ps = add(cam, scale(dmin, rd));
  const float step_scale = 0.9f * s.mu * s.vox_inv;
  const float total_max = 2.0f * s.r_cube * s.vox_inv;
  float step, total = 0.0f, tsdf;
  F3 vs;
  pos_in_voxel(ps, s, vs);
  int state;
  if (!V.gtvu(vs, tsdf))
    state = COARSE;
  else if (tsdf >= 0.0f)
    state = FINE;
  else
    return false;
  const int cap = 4 * (int)total_max + 64;
  int it = 0;
  while (state != BEHIND) {
    if (++it > cap) return false;
    if (state == COARSE)
      step = step_scale;
    else
      step = (tsdf > 0.0f) ? fmaxf(step_scale * tsdf, 1.0f) : fminf(step_scale * tsdf, -1.0f);
    vs = add(vs, scale(step, rd));
    total += step;
    if (total > total_max) break;
    V.gtvu(vs, tsdf);
    if (tsdf > -1.0f && tsdf < 1.0f) {
      V.gtvi(vs, tsdf);
      if (tsdf < 0.0f) {
        if (state == COARSE) break;
        state = BEHIND;
      } else if (tsdf == 0.0f) {
        p3d = pos_in_world(vs, s);
        return true;
      } else if (state == COARSE) {
        state = FINE;
      }
    }
  }
  if (state == BEHIND) {
    step = step_scale * tsdf;
    vs = add(vs, scale(step, rd));
    V.gtvi(vs, tsdf);
    step = step_scale * tsdf;
    vs = add(vs, scale(step, rd));
    p3d = pos_in_world(vs, s);
    return true;
  }
  return false;
}

__device__ inline int ray_tiles(const SessionDev& s, int l) {
  return ((s.lv[l].W + TX - 1) / TX) * ((s.lv[l].H + TY - 1) / TY);
}

template <class S>
__device__ void raycast_tile(const RayArgs& a, const SessionDev& s, int l, int t) {
  if (a.gate && s.pose->failed) return;
  const int w = s.lv[l].W, h = s.lv[l].H;
  const int tw = (w + TX - 1) / TX;
  const int x = (t % tw) * TX + threadIdx.x, y = (t / tw) * TY + threadIdx.y;
  if (x >= w || y >= h) return;
  Vol<S> V;
  V.v = reinterpret_cast<const typename S::word*>(s.vol);
  V.occ = s.occ;
  for (int k = 0; k < 3; k++) V.dim[k] = s.dim[k], V.nb[k] = s.nb[k];
  const bool ext = a.level >= 0;
  const float* Tgc_in = ext ? a.Tgc : s.pose->Tgc;
  const float* Tcg_in = ext ? a.Tcg : s.pose->Tcg;
  const float* cen = ext ? a.center : s.pose->center;
  float Tgc[12], Tcg[12], K[4];
#pragma unroll
  for (int k = 0; k < 12; k++) Tgc[k] = Tgc_in[k], Tcg[k] = Tcg_in[k];
#pragma unroll
  for (int k = 0; k < 4; k++) K[k] = s.lv[l].K[k];
  const F3 cam = f3(cen[0], cen[1], cen[2]);
  // host-side set-up of rmi_Render_Maps_for_ICP (:1667-1675)
  const F3 cc = f3(s.cube_center[0], s.cube_center[1], s.cube_center[2]);
  const F3 vcc = sub(cc, cam);
  const F3 ncc = normalised(vcc);
  const float dist_cc = length(vcc);
  const float theta_max = asinf(s.r_cube / dist_cc);

  F3 pg, sn;
  bool valid = cast_ray(V, s, K, (float)x, (float)y, Tcg, cam, ncc, dist_cc, theta_max, pg);
  if (valid) valid = surface_normal(V, s, pg, sn);
  const size_t idx = (size_t)y * w + x;
  float dep = 0.0f, img = 0.0f;
  F3 pc = f3(-100.0f, -100.0f, -100.0f), sc = f3(-100.0f, -100.0f, -100.0f);
  if (valid) {
    pc = transform(pg, Tgc);
    dep = pc.z;
    sc = rotate(sn, Tgc);
    float ang = sc.x * a.light[0] + sc.y * a.light[1] + sc.z * a.light[2];
    img = fmaxf(0.0f, fminf(255.0f, (0.8f * ang + 0.2f) * 255.0f));
  }
  if (ext) {
    a.out_depth[idx] = dep;
    a.out_vtx3[3 * idx] = pc.x;
    a.out_vtx3[3 * idx + 1] = pc.y;
    a.out_vtx3[3 * idx + 2] = pc.z;
    a.out_nrm3[3 * idx] = sc.x;
    a.out_nrm3[3 * idx + 1] = sc.y;
    a.out_nrm3[3 * idx + 2] = sc.z;
    if (a.out_img) a.out_img[idx] = (uint8_t)img;
  } else {
    float vw = valid ? 1.0f : 0.0f;
    s.m_depth[l][idx] = dep;
    s.m_vtx[l][idx] = make_float4(pc.x, pc.y, pc.z, vw);
    s.m_nrm[l][idx] = make_float4(sc.x, sc.y, sc.z, vw);
    s.m_img[l][idx] = (uint8_t)img;
  }
}

template <class S>
__global__ void __launch_bounds__(TX* TY) k_raycast(RayArgs a) {
  __shared__ int s_item;
  const BatchTable* __restrict__ bt = a.bt;
  const int n = bt->n;
  const int total = (a.level >= 0) ? ray_tiles(*bt->s[0], a.level) : bt->ray[n];
  const bool lead = threadIdx.x == 0 && threadIdx.y == 0;
  for (;;) {
    if (lead) s_item = (int)atomicAdd(a.work, 1u);
    __syncthreads();
    const int item = s_item;
    __syncthreads();  // every thread has the item before the next fetch
    if (item >= total) break;
    if (a.level >= 0) {
      raycast_tile<S>(a, *bt->s[0], a.level, item);
    } else {
      int t;
      const int slot = find_slot(bt->ray, n, item, t);
      const SessionDev& s = *bt->s[slot];
      int l = 0;
      for (; l < s.levels - 1; l++) {
        const int nt = ray_tiles(s, l);
        if (t < nt) break;
        t -= nt;
      }
      raycast_tile<S>(a, s, l, t);
    }
  }
  // the last block to finish clears the counters for the next launch
  if (lead) {
    __threadfence();
    if (atomicAdd(a.work + 1, 1u) == gridDim.x - 1) {
      a.work[0] = 0u;
      a.work[1] = 0u;
      __threadfence();
    }
  }
}

__global__ void k_maps_export(const float4* __restrict__ mv, const float4* __restrict__ mn,
                              const float4* __restrict__ iv, const float4* __restrict__ in, size_t n,
                              float* v3, float* n3, float* iv3, float* in3) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (v3) {
      float4 a = mv[i];
      v3[3 * i] = a.x, v3[3 * i + 1] = a.y, v3[3 * i + 2] = a.z;
    }
    if (n3) {
      float4 a = mn[i];
      n3[3 * i] = a.x, n3[3 * i + 1] = a.y, n3[3 * i + 2] = a.z;
    }
    if (iv3) {
      float4 a = iv[i];
      iv3[3 * i] = a.x, iv3[3 * i + 1] = a.y, iv3[3 * i + 2] = a.z;
    }
    if (in3) {
      float4 a = in[i];
      in3[3 * i] = a.x, in3[3 * i + 1] = a.y, in3[3 * i + 2] = a.z;
    }
  }
}

}  // namespace

int raycast_grid() {
  static int g = 0;
  if (!g) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_raycast<StoreI16>, TX * TY, 0) != cudaSuccess ||
        per_sm < 1)
      per_sm = 4;
    g = sm_count() * per_sm;
  }
  return g;
}

void launch_raycast(const BatchTable* bt, int tsdf_type, int level, const float* Tgc, const float* Tcg,
                    const float* center, float lx, float ly, float lz, bool gate, float* out_depth, float* out_vtx3,
                    float* out_nrm3, uint8_t* out_img, cudaStream_t st) {
  RayArgs a;
  a.bt = bt;
  a.work = const_cast<unsigned*>(bt->work);
  a.level = level;
  a.Tgc = Tgc;
  a.Tcg = Tcg;
  a.center = center;
  a.light[0] = lx;
  a.light[1] = ly;
  a.light[2] = lz;
  a.gate = gate ? 1 : 0;
  a.out_depth = out_depth;
  a.out_vtx3 = out_vtx3;
  a.out_nrm3 = out_nrm3;
  a.out_img = out_img;
  const int grid = raycast_grid();
  dim3 blk(TX, TY);
  switch (tsdf_type) {
    case VS_TSDF_FP16:
      k_raycast<StoreF16><<<grid, blk, 0, st>>>(a);
      break;
    case VS_TSDF_FP32:
      k_raycast<StoreF32><<<grid, blk, 0, st>>>(a);
      break;
    default:
      k_raycast<StoreI16><<<grid, blk, 0, st>>>(a);
      break;
  }
}

void launch_maps_export(const SessionDev& h, int level, float* vtx3, float* nrm3, float* ivtx3, float* inrm3,
                        cudaStream_t st) {
  size_t n = (size_t)h.lv[level].W * h.lv[level].H;
  k_maps_export<<<(int)((n + 255) / 256), 256, 0, st>>>(h.m_vtx[level], h.m_nrm[level], h.in_vtx[level],
                                                         h.in_nrm[level], n, vtx3, nrm3, ivtx3, inrm3);
}

}  // namespace vs
