// TSDF ray casting into model depth / vertex / normal maps.
//
// Reference: g_rmi_Render_Maps_for_ICP, d_crtc_Cast_Ray_on_TSDF_Cube_NEW,
// d_gtvu / d_gtvi and d_csnt (STAC/Engine/GPU/z_yooji_cuda_tsdf_renderer.cu:
// 1069-1209, 466-635, 68-153, 288-464; host set-up :1642-1700).  The
// reference launches one 16x16-block grid per pyramid level; here one
// persistent launch (k_ray_fused) covers every level of every session of a
// batch table, marching each ray to its surface point and computing the
// surface normal and the maps there.  Colour ray-casts, whose shading needs
// more registers, run as two launches: k_ray_march writes the surface points
// to a hit buffer and k_ray_shade shades them.  Each warp takes 8x4-ray tiles
// from an atomic work counter, so a slow tile near a surface holds up neither
// a grid row nor the other warps of its block.  A ray keeps its whole march
// state in registers, and every voxel read is one 32-bit word that carries
// both the TSDF value and the weight (one gather instead of the reference's
// separate float and uchar arrays).  Before the march, the distance field of
// the band sub-cubes is rebuilt (k_band_xy, k_band_z), which lets the march
// jump through free space.
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

constexpr int kRayThreads = 128;  // a warp's 32 rays form a (1 << lx) x (32 >> lx) tile

struct RayArgs {
  const BatchTable* bt;
  unsigned* work;       // [0] next tile, [1] finished warps; zero between launches
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
  uint8_t* out_rgb;     // planar colour image (NULL: none)
  int mode;             // kRay* bits of the external render variants (0: the ICP maps)
};

// Volume reads.  Every voxel read is one word (TSDF value and weight); a
// voxel never written holds weight 0 and reads "no value".  Free space is
// skipped through the band distance field, so the samples the march does take
// lie near band bricks, where a separate occupancy test would only add
// instructions.
template <class S>
struct Vol {
  const typename S::word* v;
  const uint8_t* bdist;  // distance in bricks to the nearest band brick
  int dim[3];
  uint32_t nbx, nbxy;  // bricks per row / per slab
  uint32_t sy, sz;  // word strides of one brick row / one brick slab: 512 nb[0], 512 nb[0] nb[1]
  // The word index of voxel (x, y, z) >= 0 is the sum of one term per axis
  // (brick part + offset inside the brick), in 32 bits (volumes of at most
  // 1024^3 voxels have fewer than 2^30 words).  Stencils compute each axis
  // term once and add them.
  __device__ inline uint32_t wx(int x) const { return (((uint32_t)x >> 3) << 9) + ((uint32_t)x & 7u); }
  __device__ inline uint32_t wy(int y) const { return ((uint32_t)y >> 3) * sy + (((uint32_t)y & 7u) << 3); }
  __device__ inline uint32_t wz(int z) const { return ((uint32_t)z >> 3) * sz + (((uint32_t)z & 7u) << 6); }
  // the value of word i, and whether its weight is > 0
  __device__ inline bool word_ok(uint32_t i, float& t) const {
    uint32_t w;
    S::decode(__ldg(v + i), t, w);
    return w != 0u;
  }
  // Free-space run: how many of the next steps p + k inc (k = 1..m) are
  // certain to read TSDF 1 ("no value", or a voxel whose value is 1) -
  // outside the volume, or inside the box of bricks that holds no band brick
  // (the bricks within Chebyshev distance bdist - 1 of a position's brick) -
  // so that the march only has to advance the position for them.  Boxes are
  // chained: the step after a box joins the run when it certainly reads 1
  // too, and the next box starts there.  The bounds are pulled in by 0.05
  // voxel, far more than the rounding of a position p + k inc (one product
  // and one sum: under 1e-3 voxel wherever both p and the position lie within
  // 2048 voxels of the volume) or of the approximate reciprocals of the
  // increment, so a step counted here reads 1 however its position rounds.  A negative result -k
  // says p lies in a band brick that the ray leaves after about k steps; the
  // caller need not ask again before then (asking late only delays a run, it
  // never changes a sample).  A NaN coordinate fails every comparison below
  // and gives 0.
  static constexpr int kMaxRun = 4096;
  static constexpr int kMaxBoxes = 2;
  __device__ inline int free_run(F3 p, F3 inc) const {
    const float d = 0.05f;
    const float pa[3] = {p.x, p.y, p.z}, ia[3] = {inc.x, inc.y, inc.z};
    const float ra[3] = {__fdividef(1.0f, inc.x), __fdividef(1.0f, inc.y), __fdividef(1.0f, inc.z)};
    int run = 0;
    for (int j = 0; j < kMaxBoxes; j++) {
      // q: step `run` (j = 0: the current sample, which read 1; after that
      // the step following the last box, a candidate for the run)
      float q[3];
#pragma unroll
      for (int a = 0; a < 3; a++) q[a] = j == 0 ? pa[a] : (float)run * ia[a] + pa[a];
      // a coordinate is in range iff -0.5 < q < dim - 0.5 (gtvu rounds with ROUNDF)
      bool inside = true;
#pragma unroll
      for (int a = 0; a < 3; a++) inside &= q[a] > -0.5f && q[a] < (float)dim[a] - 0.5f;
      float t;
      bool band = false, sure = false;  // sure: q reads 1 however it rounds
      if (!inside) {
        // outside until every coordinate that is out of range has come in
        t = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; a++) {
          const float hi = (float)dim[a] - 0.5f;
          if (q[a] <= -0.5f) {
            t = fmaxf(t, ia[a] > 0.0f ? (-0.5f - d - q[a]) * ra[a] : 1e30f);
            sure |= q[a] < -0.5f - d;
          } else if (q[a] >= hi) {
            t = fmaxf(t, ia[a] < 0.0f ? (hi + d - q[a]) * ra[a] : 1e30f);
            sure |= q[a] > hi + d;
          }
        }
      } else {
        // inside: every coordinate > -0.5, where ROUNDF is (int)(q + 0.5);
        // brick b holds the nearest voxel, and the box of bricks b - h ..
        // b + h (h = bdist - 1) holds no band brick; in a band brick (bdist
        // 0) the box is the brick itself
        const int b[3] = {(int)(q[0] + 0.5f) >> 3, (int)(q[1] + 0.5f) >> 3, (int)(q[2] + 0.5f) >> 3};
        const int dist = __ldg(bdist + (uint32_t)b[2] * nbxy + (uint32_t)b[1] * nbx + (uint32_t)b[0]);
        band = dist == 0;
        sure = !band;
        const int h = band ? 0 : dist - 1;
        t = 1e30f;
#pragma unroll
        for (int a = 0; a < 3; a++) {
          const float lo = (float)((b[a] - h) * 8) - 0.5f, hi = (float)((b[a] + h + 1) * 8) - 0.5f;
          sure &= q[a] > lo + d && q[a] < hi - d;
          if (ia[a] > 0.0f)
            t = fminf(t, (hi - d - q[a]) * ra[a]);
          else if (ia[a] < 0.0f)
            t = fminf(t, (lo + d - q[a]) * ra[a]);
        }
      }
      if (j > 0 && !sure) return run - 1;
      // steps k >= 1 from q with k < t
      t = fminf(t, (float)(kMaxRun + 1));
      const int m = (int)ceilf(t) - 1;
      if (j == 0 && band) return m > 0 ? -m : 0;
      run += m > 0 ? m : 0;
      if (run >= kMaxRun) return run;
      run++;  // the next candidate
    }
    return run - 1;
  }

  // d_gtvu_Get_TSDF_Value_Uninterpolated: nearest voxel (ROUNDF), weight > 0.
  // ROUNDF(p) is negative for every p <= -0.5 and equals (int)(p + 0.5) for
  // every p > -0.5 (both branches give 0 on (-0.5, 0)), so one comparison per
  // coordinate decides the lower bound, and a NaN coordinate fails it too.
  __device__ inline bool gtvu(F3 p, float& out) const {
    out = 1.0f;
    if (!(p.x > -0.5f && p.y > -0.5f && p.z > -0.5f)) return false;
    const int x = (int)(p.x + 0.5f), y = (int)(p.y + 0.5f), z = (int)(p.z + 0.5f);
    if (x >= dim[0] || y >= dim[1] || z >= dim[2]) return false;
    const uint32_t i = wx(x) + wy(y) + wz(z);
    float t;
    if (!word_ok(i, t)) return false;
    out = t;
    return true;
  }
  // d_gtvi_Get_TSDF_Value_Interpolated (offset = floor, see the oracle); the
  // eight reads have no side effects, so reading all of them before the
  // validity test gives the short-circuit form's result
  __device__ inline bool gtvi(F3 p, float& out) const {
    out = 1.0f;
    if (isnan(p.x) || isnan(p.y) || isnan(p.z)) return false;
    float fx = floorf(p.x), fy = floorf(p.y), fz = floorf(p.z);
    int ox = (int)fx, oy = (int)fy, oz = (int)fz;
    float rx = p.x - fx, ry = p.y - fy, rz = p.z - fz;
    // the eight corners are in range iff both values of every axis are; an
    // out-of-range value is clamped for its (discarded) read
    bool ok = ox >= 0 && ox + 1 < dim[0] && oy >= 0 && oy + 1 < dim[1] && oz >= 0 && oz + 1 < dim[2];
    const int cx = min(max(ox, 0), dim[0] - 2), cy = min(max(oy, 0), dim[1] - 2), cz = min(max(oz, 0), dim[2] - 2);
    const uint32_t x0 = wx(cx), x1 = wx(cx + 1), y0 = wy(cy), y1 = wy(cy + 1), z0 = wz(cz), z1 = wz(cz + 1);
    float f0, f1, f2, f3_, b0, b1, b2, b3;
    ok &= word_ok(z0 + y0 + x0, f0);
    ok &= word_ok(z0 + y0 + x1, f1);
    ok &= word_ok(z0 + y1 + x0, f2);
    ok &= word_ok(z0 + y1 + x1, f3_);
    ok &= word_ok(z1 + y0 + x0, b0);
    ok &= word_ok(z1 + y0 + x1, b1);
    ok &= word_ok(z1 + y1 + x0, b2);
    ok &= word_ok(z1 + y1 + x1, b3);
    if (!ok) return false;
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
  // all 32 reads are issued before any validity test (no side effects, so
  // the result equals the reference's read-and-return-early order).  The
  // stencil spans o - 1 .. o + 2 on every axis and uses each of those values,
  // so it is in range iff o - 1 >= 0 and o + 2 < dim on all three axes.
  bool ok = ox >= 1 && ox + 2 < V.dim[0] && oy >= 1 && oy + 2 < V.dim[1] && oz >= 1 && oz + 2 < V.dim[2];
  const int cx = min(max(ox, 1), V.dim[0] - 3), cy = min(max(oy, 1), V.dim[1] - 3), cz = min(max(oz, 1), V.dim[2] - 3);
  uint32_t X[4], Y[4], Z[4];
#pragma unroll
  for (int k = 0; k < 4; k++) X[k] = V.wx(cx - 1 + k), Y[k] = V.wy(cy - 1 + k), Z[k] = V.wz(cz - 1 + k);
  float fm[4], fr[12], bk[12], bm[4];
#pragma unroll
  for (int i = 0; i < 4; i++) ok &= V.word_ok(Z[0] + Y[1 + dy1[i]] + X[1 + dx1[i]], fm[i]);
#pragma unroll
  for (int i = 0; i < 12; i++) ok &= V.word_ok(Z[1] + Y[1 + dy2[i]] + X[1 + dx2[i]], fr[i]);
#pragma unroll
  for (int i = 0; i < 12; i++) ok &= V.word_ok(Z[2] + Y[1 + dy2[i]] + X[1 + dx2[i]], bk[i]);
#pragma unroll
  for (int i = 0; i < 4; i++) ok &= V.word_ok(Z[3] + Y[1 + dy1[i]] + X[1 + dx1[i]], bm[i]);
  if (!ok) return false;
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
                         const float* Tcg, F3 cam, float dmin, float dmax, bool cone, F3 ncc, float theta_max,
                         F3& p3d) {
  enum { COARSE, FINE, BEHIND };
  F3 pe = transform(back_project(px, py, K, dmax), Tcg);
  F3 rd = normalised(sub(pe, cam));
  if (cone) {
    float theta = acosf(dot(rd, ncc));
    if (theta > theta_max) return false;
  }
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
  int recheck = 0;  // full steps before the next free-space test
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
    if (tsdf == 1.0f && state != BEHIND && --recheck < 0) {
      // While samples read TSDF 1 (no value, or a voxel whose value is 1) the
      // state and the step stay as they are, so the `run` steps of a
      // free-space run are taken at once: p + run * inc and total + run * sn.
      // The step-by-step sums of the reference round after every step; the
      // jump rounds once, so the position after a run of m steps differs
      // from theirs by at most about m / 2 ulps of the voxel coordinate
      // (under 1e-2 voxel for runs of a few hundred steps and coordinates
      // below 1024), which moves the later samples and the surface point by
      // far less than the 1 mm ray-cast tolerance.
      const float sn = (state == COARSE) ? step_scale : fmaxf(step_scale * tsdf, 1.0f);
      const F3 inc = scale(sn, rd);
      int m = V.free_run(vs, inc);
      if (m < 0) {
        recheck = -m;
        m = 0;
      }
      // the loop above would stop at iteration cap + 1: run at most cap - it
      // steps here, then stop as it would.  total only grows (sn > 0), so it
      // passed total_max inside the run iff it is past it at the end, and the
      // ray then ends without a hit whichever step it was.
      const bool capped = m > cap - it;
      const int run = capped ? cap - it : m;
      if (run > 0) {
        const float fr = (float)run;
        vs = add(vs, scale(fr, inc));
        total += fr * sn;
      }
      if (total > total_max) return false;
      it += run;
      if (capped) return false;
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

__device__ inline int ray_tiles(const SessionDev& s, int l, int rx, int ry) {
  return ((s.lv[l].W + rx - 1) / rx) * ((s.lv[l].H + ry - 1) / ry);
}

// Hands the calling warp ray tiles until none are left and calls
// f(session, level, x, y) for each lane's pixel inside its level.  The last
// warp to finish clears the counters for the next launch.
template <class F>
__device__ inline void for_each_ray_tile(const RayArgs& a, F&& f) {
  const BatchTable* __restrict__ bt = a.bt;
  const int lane = threadIdx.x & 31;
  const int n = bt->n;
  const int lx = bt->ray_lx, rx = 1 << lx, ry = 32 >> lx;
  const int total = (a.level >= 0) ? ray_tiles(*bt->s[0], a.level, rx, ry) : bt->ray[n];
  for (;;) {
    int item = 0;
    if (lane == 0) item = (int)atomicAdd(a.work, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) break;
    int t, l, slot;
    if (a.level >= 0) {
      slot = 0;
      l = a.level;
      t = item;
    } else {
      slot = find_slot(bt->ray, n, item, t);
      const SessionDev& s = *bt->s[slot];
      l = 0;
      for (; l < s.levels - 1; l++) {
        const int nt = ray_tiles(s, l, rx, ry);
        if (t < nt) break;
        t -= nt;
      }
    }
    const SessionDev& s = *bt->s[slot];
    if (a.gate && s.pose->failed) continue;
    const int tw = (s.lv[l].W + rx - 1) / rx;
    const int x = (t % tw) * rx + (lane & (rx - 1)), y = (t / tw) * ry + (lane >> lx);
    if (x < s.lv[l].W && y < s.lv[l].H) f(s, l, x, y);
  }
  if (lane == 0) {
    __threadfence();
    const unsigned warps = gridDim.x * (blockDim.x >> 5);
    if (atomicAdd(a.work + 1, 1u) == warps - 1) {
      a.work[0] = 0u;
      a.work[1] = 0u;
      __threadfence();
    }
  }
}

// offset of level l's pixels in the per-session hit buffer
__device__ inline size_t hit_offset(const SessionDev& s, int l) {
  size_t o = 0;
  for (int k = 0; k < l; k++) o += (size_t)s.lv[k].W * s.lv[k].H;
  return o;
}

template <class S>
__device__ inline Vol<S> volume_of(const SessionDev& s) {
  Vol<S> V;
  V.v = reinterpret_cast<const typename S::word*>(s.vol);
  V.bdist = s.bdist;
  for (int k = 0; k < 3; k++) V.dim[k] = s.dim[k];
  V.nbx = (uint32_t)s.nb[0];
  V.nbxy = (uint32_t)s.nb[0] * (uint32_t)s.nb[1];
  V.sy = (uint32_t)s.nb[0] << 9;
  V.sz = ((uint32_t)s.nb[0] * (uint32_t)s.nb[1]) << 9;
  return V;
}

// Band distance field (the Chebyshev distance transform of the band bricks,
// saturating at kBandReach + 1), separable: the distance along x to the
// nearest band brick of the row, then per brick the minimum over its column
// of max(|dy|, x distance), then the same along z.  Each pass holds one plane
// of bricks in shared memory and evaluates its 2 kBandReach + 1 window
// without data-dependent exits, so the reads of a brick's window are
// independent.
constexpr int kBandSat = kBandReach + 1;
constexpr int kBandThreads = 1024;

// d(i) = min over |k| <= kBandReach of max(|k|, in[i + k * stride]), for
// positions inside [0, n) along the pass's axis (c: the brick's coordinate)
__device__ inline int band_window(const uint8_t* in, int i, int c, int n, int stride) {
  int d = in[i];
#pragma unroll
  for (int k = 1; k <= kBandReach; k++) {
    const int lo = c - k >= 0 ? in[i - k * stride] : kBandSat;
    const int hi = c + k < n ? in[i + k * stride] : kBandSat;
    d = min(d, max(k, min(lo, hi)));
  }
  return d;
}

// i / n for 0 <= i < 2^14 and 1 <= n <= 128 without an integer division:
// (i + 0.5) / n lies at least 0.5 / n from every integer, far more than the
// float rounding of (i + 0.5) * (1 / n)
__device__ inline int small_div(int i, float inv_n) { return (int)(((float)i + 0.5f) * inv_n); }

// x and y passes, one block per z slab of a session: band flags (0 / 1) ->
// x distances -> xy distances
__global__ void __launch_bounds__(kBandThreads) k_band_xy(const BatchTable* __restrict__ bt) {
  __shared__ uint8_t sb[kMaxBricksAxis * kMaxBricksAxis];
  __shared__ uint8_t sx[kMaxBricksAxis * kMaxBricksAxis];
  const int n = bt->n;
  const int total = bt->slab[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int z;
    const SessionDev* __restrict__ s = bt->s[find_slot(bt->slab, n, item, z)];
    const int nb0 = s->nb[0], nb1 = s->nb[1], np = nb0 * nb1;
    const float inv0 = 1.0f / (float)nb0;
    const uint8_t* __restrict__ band = s->band + (size_t)z * np;
    __syncthreads();  // the previous slab's reads of sb / sx are done
    // a band brick is at distance 0, any other at "not yet found"
    for (int i = threadIdx.x; i < np; i += blockDim.x) sb[i] = band[i] ? 0 : kBandSat;
    __syncthreads();
    for (int i = threadIdx.x; i < np; i += blockDim.x)
      sx[i] = (uint8_t)band_window(sb, i, i - small_div(i, inv0) * nb0, nb0, 1);
    __syncthreads();
    uint8_t* __restrict__ out = s->btmp + (size_t)z * np;
    for (int i = threadIdx.x; i < np; i += blockDim.x)
      out[i] = (uint8_t)band_window(sx, i, small_div(i, inv0), nb1, nb0);
  }
}

// z pass, one block per y row of a session: the x-z plane of xy distances in
// shared memory -> distances
__global__ void __launch_bounds__(kBandThreads) k_band_z(const BatchTable* __restrict__ bt) {
  __shared__ uint8_t sp[kMaxBricksAxis * kMaxBricksAxis];
  const int n = bt->n;
  const int total = bt->brow[n];
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    int y;
    const SessionDev* __restrict__ s = bt->s[find_slot(bt->brow, n, item, y)];
    const int nb0 = s->nb[0], nb2 = s->nb[2], np = nb0 * s->nb[1], nq = nb0 * nb2;
    const float inv0 = 1.0f / (float)nb0;
    __syncthreads();  // the previous row's reads of sp are done
    // plane element (x, z) at z * nb0 + x; brick z * np + y * nb0 + x
    for (int i = threadIdx.x; i < nq; i += blockDim.x) {
      const int z = small_div(i, inv0);
      sp[i] = s->btmp[(size_t)z * (np - nb0) + (size_t)y * nb0 + i];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nq; i += blockDim.x) {
      const int z = small_div(i, inv0);
      s->bdist[(size_t)z * (np - nb0) + (size_t)y * nb0 + i] = (uint8_t)band_window(sp, i, z, nb2, nb0);
    }
  }
}

#ifndef VS_RAY_MIN_BLOCKS
#define VS_RAY_MIN_BLOCKS 8  // resident 128-thread blocks per SM the register allocation must allow
#endif
#ifndef VS_SHADE_MIN_BLOCKS
#define VS_SHADE_MIN_BLOCKS 8
#endif

// the ray of pixel (x, y) of level l to its surface point pg (global
// coordinates); false: no hit
template <class S, bool SCENE>
__device__ inline bool march_ray(const RayArgs& a, const Vol<S>& V, const SessionDev& s, int l, int x, int y, F3& pg) {
  const bool ext = a.level >= 0;
  const float* Tcg_in = ext ? a.Tcg : s.pose->Tcg;
  const float* cen = ext ? a.center : s.pose->center;
  float Tcg[12], K[4];
#pragma unroll
  for (int k = 0; k < 12; k++) Tcg[k] = Tcg_in[k];
#pragma unroll
  for (int k = 0; k < 4; k++) K[k] = s.lv[l].K[k];
  const F3 cam = f3(cen[0], cen[1], cen[2]);
  // host-side set-up of rmi_Render_Maps_for_ICP (:1667-1675)
  const F3 cc = f3(s.cube_center[0], s.cube_center[1], s.cube_center[2]);
  const F3 vcc = sub(cc, cam);
  const F3 ncc = normalised(vcc);
  const float dist_cc = length(vcc);
  const float theta_max = asinf(s.r_cube / dist_cc);
  // object mode (d_crtc_NEW, :466-635): the segment of the ray through the
  // cube's bounding sphere inside its view cone; scene mode (d_crtcs,
  // :908-1066): from the camera centre to 2 r_cube, no cone
  const float dmin = SCENE ? 0.0f : dist_cc - s.r_cube;
  const float dmax = SCENE ? 2.0f * s.r_cube : dist_cc + s.r_cube;
  return cast_ray(V, s, K, (float)x, (float)y, Tcg, cam, dmin, dmax, !SCENE, ncc, theta_max, pg);
}

// phase 1: march every ray to its surface point (global coordinates; w = 1
// hit, 0 none) in the session's hit buffer
template <class S, bool SCENE>
__global__ void __launch_bounds__(kRayThreads, VS_RAY_MIN_BLOCKS) k_ray_march(RayArgs a) {
  for_each_ray_tile(a, [&](const SessionDev& s, int l, int x, int y) {
    F3 pg;
    const bool hit = march_ray<S, SCENE>(a, volume_of<S>(s), s, l, x, y, pg);
    s.ray_hit[hit_offset(s, l) + (size_t)y * s.lv[l].W + x] =
        hit ? make_float4(pg.x, pg.y, pg.z, 1.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  });
}

// d_grvi_Get_RGB_Value_Interpolated (z_yooji_cuda_tsdf_renderer.cu:232-284):
// trilinear colour of the eight voxels around the hit, every one in range with
// weight > 0 (d_grvu, :194-229), rounded to 8 bits as InfiniTAM's toUChar
// (round half away from zero, clamp to 0..255); 0 when a neighbour fails.
// The 16 reads (weights and colours) are issued before any test.
template <class S>
__device__ uint32_t trilinear_color(const Vol<S>& V, const SessionDev& s, F3 pg) {
  F3 v;
  pos_in_voxel(pg, s, v);
  if (isnan(v.x) || isnan(v.y) || isnan(v.z)) return 0u;
  const float fx = floorf(v.x), fy = floorf(v.y), fz = floorf(v.z);
  const int ox = (int)fx, oy = (int)fy, oz = (int)fz;
  const float rx = v.x - fx, ry = v.y - fy, rz = v.z - fz;
  float tdummy;
  bool ok = ox >= 0 && ox + 1 < V.dim[0] && oy >= 0 && oy + 1 < V.dim[1] && oz >= 0 && oz + 1 < V.dim[2];
  const int cx = min(max(ox, 0), V.dim[0] - 2), cy = min(max(oy, 0), V.dim[1] - 2), cz = min(max(oz, 0), V.dim[2] - 2);
  const uint32_t X[2] = {V.wx(cx), V.wx(cx + 1)}, Y[2] = {V.wy(cy), V.wy(cy + 1)}, Z[2] = {V.wz(cz), V.wz(cz + 1)};
  uint32_t c[8];
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t w = Z[i >> 2] + Y[(i >> 1) & 1] + X[i & 1];
    ok &= V.word_ok(w, tdummy);
    c[i] = __ldg(s.col + w);
  }
  if (!ok) return 0u;
  uint32_t out[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    float f[4], b[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      f[i] = (float)rgb_channel(c[i], k);
      b[i] = (float)rgb_channel(c[4 + i], k);
    }
    const float inf = (1.0f - ry) * ((1.0f - rx) * f[0] + rx * f[1]) + ry * ((1.0f - rx) * f[2] + rx * f[3]);
    const float inb = (1.0f - ry) * ((1.0f - rx) * b[0] + rx * b[1]) + ry * ((1.0f - rx) * b[2] + rx * b[3]);
    const float val = (1.0f - rz) * inf + rz * inb;
    const float rounded = (val < 0.0f) ? (val - 0.5f) : (val + 0.5f);
    out[k] = (uint32_t)(uint8_t)fmaxf(0.0f, fminf(255.0f, rounded));
  }
  return pack_rgb(out[0], out[1], out[2]);
}

// d_grvu_Get_RGB_Value_Uninterpolated (z_yooji_cuda_tsdf_renderer.cu:155-229)
// for the scene maps: the colour of the nearest voxel (ROUNDF) if it is in
// range with weight > 0, else 0.  (The reference's scene image writes the green
// channel into the red plane, marked there as temporary; the true colour is
// written here.)
template <class S>
__device__ uint32_t nearest_color(const Vol<S>& V, const SessionDev& s, F3 pg) {
  F3 v;
  pos_in_voxel(pg, s, v);
  if (isnan(v.x) || isnan(v.y) || isnan(v.z)) return 0u;
  const int x = roundf_ref(v.x), y = roundf_ref(v.y), z = roundf_ref(v.z);
  if (x < 0 || x >= V.dim[0] || y < 0 || y >= V.dim[1] || z < 0 || z >= V.dim[2]) return 0u;
  const uint32_t w = V.wx(x) + V.wy(y) + V.wz(z);
  float t;
  if (!V.word_ok(w, t)) return 0u;
  return __ldg(s.col + w);
}

// surface normal of a hit (d_csnt), camera-frame vertex and normal, shading,
// colour, into the model maps or the external outputs
template <class S, bool COLOR>
__device__ inline void shade_ray(const RayArgs& a, const Vol<S>& V, const SessionDev& s, int l, int x, int y,
                                 bool hit, F3 pg) {
  const bool ext = a.level >= 0;
  const size_t idx = (size_t)y * s.lv[l].W + x;
  F3 sn;
  bool valid = hit;
  if (valid) valid = surface_normal(V, s, pg, sn);
  float dep = 0.0f, img = 0.0f;
  uint32_t rgb = 0u;
  F3 pc = f3(-100.0f, -100.0f, -100.0f), sc = f3(-100.0f, -100.0f, -100.0f);
  if (valid) {
    if (COLOR && s.col) rgb = (a.mode & kRayNearestColor) ? nearest_color(V, s, pg) : trilinear_color(V, s, pg);
    const float* Tgc_in = ext ? a.Tgc : s.pose->Tgc;
    float Tgc[12];
#pragma unroll
    for (int k = 0; k < 12; k++) Tgc[k] = Tgc_in[k];
    pc = transform(pg, Tgc);
    dep = pc.z;
    sc = (a.mode & kRayGlobalNormals) ? sn : rotate(sn, Tgc);
    float ang = sc.x * a.light[0] + sc.y * a.light[1] + sc.z * a.light[2];
    img = fmaxf(0.0f, fminf(255.0f, (0.8f * ang + 0.2f) * 255.0f));
  }
  if (ext) {
    if (!valid && (a.mode & kRayWhiteBackground)) rgb = 0x00ffffffu;
    a.out_depth[idx] = dep;
    if (a.out_vtx3) {
      a.out_vtx3[3 * idx] = pc.x;
      a.out_vtx3[3 * idx + 1] = pc.y;
      a.out_vtx3[3 * idx + 2] = pc.z;
    }
    a.out_nrm3[3 * idx] = sc.x;
    a.out_nrm3[3 * idx + 1] = sc.y;
    a.out_nrm3[3 * idx + 2] = sc.z;
    if (a.out_img) a.out_img[idx] = (uint8_t)img;
    if (COLOR && a.out_rgb) {
      const size_t plane = (size_t)s.lv[l].W * s.lv[l].H;
      a.out_rgb[idx] = (uint8_t)rgb_channel(rgb, 0);
      a.out_rgb[plane + idx] = (uint8_t)rgb_channel(rgb, 1);
      a.out_rgb[2 * plane + idx] = (uint8_t)rgb_channel(rgb, 2);
    }
  } else {
    const float vw = valid ? 1.0f : 0.0f;
    s.m_depth[l][idx] = dep;
    s.m_vtx[l][idx] = make_float4(pc.x, pc.y, pc.z, vw);
    s.m_nrm[l][idx] = make_float4(sc.x, sc.y, sc.z, vw);
    s.m_img[l][idx] = (uint8_t)img;
    if (COLOR && s.col) s.m_rgb[l][idx] = rgb;
  }
}

// phase 2: the maps of every ray from its surface point in the hit buffer
template <class S, bool COLOR>
__global__ void __launch_bounds__(kRayThreads, VS_SHADE_MIN_BLOCKS) k_ray_shade(RayArgs a) {
  for_each_ray_tile(a, [&](const SessionDev& s, int l, int x, int y) {
    const float4 h = s.ray_hit[hit_offset(s, l) + (size_t)y * s.lv[l].W + x];
    shade_ray<S, COLOR>(a, volume_of<S>(s), s, l, x, y, h.w != 0.0f, f3(h.x, h.y, h.z));
  });
}

#ifndef VS_FUSED_MIN_BLOCKS
#define VS_FUSED_MIN_BLOCKS 8
#endif

// both phases in one pass, without the hit buffer (every ray-cast without
// colour)
template <class S, bool SCENE>
__global__ void __launch_bounds__(kRayThreads, VS_FUSED_MIN_BLOCKS) k_ray_fused(RayArgs a) {
  for_each_ray_tile(a, [&](const SessionDev& s, int l, int x, int y) {
    const Vol<S> V = volume_of<S>(s);
    F3 pg;
    const bool hit = march_ray<S, SCENE>(a, V, s, l, x, y, pg);
    shade_ray<S, false>(a, V, s, l, x, y, hit, pg);
  });
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

template <class K>
int max_per_sm(K kernel) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kRayThreads, 0) != cudaSuccess || per_sm < 1)
    per_sm = 4;
  return per_sm;
}

template <class S>
int ray_max_per_sm(bool shade) {
  static const int m = max_per_sm(k_ray_march<S, false>);
  static const int h = max_per_sm(k_ray_shade<S, false>);
  return shade ? h : m;
}

int grid_of(int want, int most) { return sm_count() * ((want > 0 && want < most) ? want : most); }

template <class S>
void launch_ray_phases(const RayArgs& a0, const LaunchShape& shape, bool color, cudaStream_t st) {
  RayArgs a = a0;
  k_band_xy<<<sm_count() * 2, kBandThreads, 0, st>>>(a.bt);
  k_band_z<<<sm_count() * 2, kBandThreads, 0, st>>>(a.bt);
  if (!color) {
    static const int most_fused = max_per_sm(k_ray_fused<S, false>);
    if (a.mode & kRayScene)
      k_ray_fused<S, true><<<grid_of(shape.march_blocks_per_sm, most_fused), kRayThreads, 0, st>>>(a);
    else
      k_ray_fused<S, false><<<grid_of(shape.march_blocks_per_sm, most_fused), kRayThreads, 0, st>>>(a);
    return;
  }
  if (a.mode & kRayScene)
    k_ray_march<S, true><<<grid_of(shape.march_blocks_per_sm, ray_max_per_sm<S>(false)), kRayThreads, 0, st>>>(a);
  else
    k_ray_march<S, false><<<grid_of(shape.march_blocks_per_sm, ray_max_per_sm<S>(false)), kRayThreads, 0, st>>>(a);
  a.work = a0.work + 4;
  static const int most_color = max_per_sm(k_ray_shade<S, true>);
  if (color)
    k_ray_shade<S, true><<<grid_of(shape.shade_blocks_per_sm, most_color), kRayThreads, 0, st>>>(a);
  else
    k_ray_shade<S, false><<<grid_of(shape.shade_blocks_per_sm, ray_max_per_sm<S>(true)), kRayThreads, 0, st>>>(a);
}

void launch_raycast(const BatchTable* bt, int tsdf_type, int level, const float* Tgc, const float* Tcg,
                    const float* center, float lx, float ly, float lz, bool gate, float* out_depth, float* out_vtx3,
                    float* out_nrm3, uint8_t* out_img, cudaStream_t st, const LaunchShape& shape, uint8_t* out_rgb,
                    bool color, int mode) {
  RayArgs a;
  a.bt = bt;
  a.work = const_cast<unsigned*>(bt->work);  // [0..1] march, [4..5] shade
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
  a.out_rgb = out_rgb;
  a.mode = mode;
  switch (tsdf_type) {
    case VS_TSDF_FP16:
      launch_ray_phases<StoreF16>(a, shape, color, st);
      break;
    case VS_TSDF_FP32:
      launch_ray_phases<StoreF32>(a, shape, color, st);
      break;
    default:
      launch_ray_phases<StoreI16>(a, shape, color, st);
      break;
  }
}

int ray_max_blocks_per_sm(int tsdf_type, bool shade) {
  switch (tsdf_type) {
    case VS_TSDF_FP16:
      return ray_max_per_sm<StoreF16>(shade);
    case VS_TSDF_FP32:
      return ray_max_per_sm<StoreF32>(shade);
    default:
      return ray_max_per_sm<StoreI16>(shade);
  }
}

void launch_maps_export(const SessionDev& h, int level, float* vtx3, float* nrm3, float* ivtx3, float* inrm3,
                        cudaStream_t st) {
  size_t n = (size_t)h.lv[level].W * h.lv[level].H;
  k_maps_export<<<(int)((n + 255) / 256), 256, 0, st>>>(h.m_vtx[level], h.m_nrm[level], h.in_vtx[level],
                                                         h.in_nrm[level], n, vtx3, nrm3, ivtx3, inrm3);
}

}  // namespace vs
