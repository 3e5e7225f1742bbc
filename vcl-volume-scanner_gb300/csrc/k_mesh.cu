// Surface extraction (marching tetrahedra) and sub-cube gather / scatter for
// snapshots.
//
// The reference meshes its silhouette volumes with marching cubes
// (STAC/VCL_3DO/z_Utility_Mesh_Generation.cpp:878-1437, on uchar volumes);
// the TSDF it scans is exported through a closed writer.  Here the zero level
// set of the TSDF itself is extracted on the device, one warp per sub-cube
// that holds data, by marching tetrahedra: a cell of 2x2x2 voxels whose
// corners all have weight > 0 is split into six tetrahedra around its
// (0,0,0)-(1,1,1) diagonal (the same split in every cell, so neighbouring
// cells meet on the same face diagonals and the surface closes), and each
// tetrahedron gives 0, 1 or 2 triangles from the signs of its corners.  No case
// table is needed.
#include <cuda_runtime.h>
#include <stdint.h>

#include "vs_internal.cuh"

namespace vs {
namespace {

// cube corner c = (c & 1, (c >> 1) & 1, c >> 2); the six tetrahedra share
// corners 0 and 7, the other two walk the cycle 1 3 2 6 4 5 (each step flips
// one coordinate)
__constant__ int kTetra[6][4] = {{0, 7, 1, 3}, {0, 7, 3, 2}, {0, 7, 2, 6}, {0, 7, 6, 4}, {0, 7, 4, 5}, {0, 7, 5, 1}};

struct MeshOut {
  float* xyz;       // 9 floats per triangle
  uint8_t* rgb;     // 9 bytes per triangle, or NULL
  uint64_t capacity;
  unsigned long long* count;
};

struct EdgeV {
  F3 p;        // world position
  float c[3];  // colour
};

// zero crossing on the edge a-b (voxel coordinates pa, pb; TSDF va < 0 <= vb
// or the other way round), in world coordinates
__device__ inline EdgeV edge_vertex(const SessionDev& s, F3 pa, F3 pb, float va, float vb, const float* ca,
                                    const float* cb) {
  const float t = (0.0f - va) / (vb - va);
  const F3 pv = f3(pa.x + t * (pb.x - pa.x), pa.y + t * (pb.y - pa.y), pa.z + t * (pb.z - pa.z));
  EdgeV e;
  e.p = pos_in_world(pv, s);
#pragma unroll
  for (int k = 0; k < 3; k++) e.c[k] = ca[k] + t * (cb[k] - ca[k]);
  return e;
}

__device__ inline void emit(const MeshOut& o, const EdgeV& a, const EdgeV& b, const EdgeV& c, F3 inside,
                            F3 outside) {
  // face free space: the normal points from the inside corners to the outside ones
  const F3 u = sub(b.p, a.p), v = sub(c.p, a.p);
  const F3 n = f3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
  const bool flip = dot(n, sub(outside, inside)) < 0.0f;
  const EdgeV* t[3] = {&a, flip ? &c : &b, flip ? &b : &c};
  const unsigned long long i = atomicAdd(o.count, 1ull);
  if (i >= o.capacity) return;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    o.xyz[9 * i + 3 * k] = t[k]->p.x;
    o.xyz[9 * i + 3 * k + 1] = t[k]->p.y;
    o.xyz[9 * i + 3 * k + 2] = t[k]->p.z;
    if (o.rgb)
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        const float x = t[k]->c[ch] + 0.5f;
        o.rgb[9 * i + 3 * k + ch] = (uint8_t)fminf(255.0f, fmaxf(0.0f, x));
      }
  }
}

template <class S>
__global__ void __launch_bounds__(256) k_mesh(const SessionDev* __restrict__ sd, const uint32_t* __restrict__ bricks,
                                              int nbricks, MeshOut o) {
  const SessionDev& s = *sd;
  const typename S::word* vol = reinterpret_cast<const typename S::word*>(s.vol);
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = (gridDim.x * blockDim.x) >> 5;
  for (int i = gw; i < nbricks; i += nw) {
    const uint32_t b = bricks[i];
    const int bx = (int)(b % (uint32_t)s.nb[0]), by = (int)((b / (uint32_t)s.nb[0]) % (uint32_t)s.nb[1]),
              bz = (int)(b / ((uint32_t)s.nb[0] * (uint32_t)s.nb[1]));
    for (int cidx = lane; cidx < kBrickVox; cidx += 32) {
      const int x = bx * 8 + (cidx & 7), y = by * 8 + ((cidx >> 3) & 7), z = bz * 8 + (cidx >> 6);
      if (x + 1 >= s.dim[0] || y + 1 >= s.dim[1] || z + 1 >= s.dim[2]) continue;
      float v[8], col[8][3];
      bool ok = true;
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const int cx = x + (c & 1), cy = y + ((c >> 1) & 1), cz = z + (c >> 2);
        const size_t wi = brick_word_index(cx, cy, cz, s.nb);
        uint32_t w;
        S::decode(vol[wi], v[c], w);
        ok &= w != 0u;
        const uint32_t cw = s.col ? s.col[wi] : 0u;
#pragma unroll
        for (int k = 0; k < 3; k++) col[c][k] = (float)rgb_channel(cw, k);
      }
      if (!ok) continue;
      unsigned neg = 0u;
#pragma unroll
      for (int c = 0; c < 8; c++) neg |= (v[c] < 0.0f ? 1u : 0u) << c;
      if (neg == 0u || neg == 0xffu) continue;
      for (int t = 0; t < 6; t++) {
        int in[4], out[4], ni = 0, no = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const int c = kTetra[t][k];
          if ((neg >> c) & 1u)
            in[ni++] = c;
          else
            out[no++] = c;
        }
        if (ni == 0 || no == 0) continue;
        auto P = [&](int c) { return f3((float)(x + (c & 1)), (float)(y + ((c >> 1) & 1)), (float)(z + (c >> 2))); };
        auto E = [&](int a, int c) { return edge_vertex(s, P(a), P(c), v[a], v[c], col[a], col[c]); };
        // centroids of the inside and outside corners (world) orient the faces
        F3 ci = f3(0, 0, 0), co = f3(0, 0, 0);
        for (int k = 0; k < ni; k++) ci = add(ci, P(in[k]));
        for (int k = 0; k < no; k++) co = add(co, P(out[k]));
        ci = scale(1.0f / (float)ni, ci);
        co = scale(1.0f / (float)no, co);
        if (ni == 1 || no == 1) {
          const int lone = (ni == 1) ? in[0] : out[0];
          const int* rest = (ni == 1) ? out : in;
          emit(o, E(lone, rest[0]), E(lone, rest[1]), E(lone, rest[2]), ci, co);
        } else {
          const EdgeV e00 = E(in[0], out[0]), e01 = E(in[0], out[1]), e11 = E(in[1], out[1]), e10 = E(in[1], out[0]);
          emit(o, e00, e01, e11, ci, co);
          emit(o, e00, e11, e10, ci, co);
        }
      }
    }
  }
}

// sub-cube gather / scatter: words of the listed bricks <-> a packed buffer
template <class W>
__global__ void k_bricks_copy(W* vol, const uint32_t* __restrict__ bricks, int n, W* packed, int to_packed) {
  const size_t total = (size_t)n * kBrickVox;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const size_t src = (size_t)bricks[i / kBrickVox] * kBrickVox + (i % kBrickVox);
    if (to_packed)
      packed[i] = vol[src];
    else
      vol[src] = packed[i];
  }
}

}  // namespace

void launch_mesh(const SessionDev& h, const SessionDev* d, const uint32_t* bricks, int n, float* xyz, uint8_t* rgb,
                 uint64_t capacity, unsigned long long* count, cudaStream_t st) {
  MeshOut o;
  o.xyz = xyz;
  o.rgb = rgb;
  o.capacity = capacity;
  o.count = count;
  const int blocks = (n + 7) / 8 < sm_count() * 8 ? (n + 7) / 8 : sm_count() * 8;
  if (blocks < 1) return;
  switch (h.tsdf_type) {
    case VS_TSDF_FP16:
      k_mesh<StoreF16><<<blocks, 256, 0, st>>>(d, bricks, n, o);
      break;
    case VS_TSDF_FP32:
      k_mesh<StoreF32><<<blocks, 256, 0, st>>>(d, bricks, n, o);
      break;
    default:
      k_mesh<StoreI16><<<blocks, 256, 0, st>>>(d, bricks, n, o);
      break;
  }
}

void launch_bricks_copy(const SessionDev& h, const uint32_t* bricks, int n, void* packed_vol, uint32_t* packed_col,
                        bool to_packed, cudaStream_t st) {
  if (n <= 0) return;
  const int blocks = sm_count() * 8;
  if (voxel_bytes(h.tsdf_type) == 8)
    k_bricks_copy<uint2><<<blocks, 256, 0, st>>>(reinterpret_cast<uint2*>(h.vol), bricks, n,
                                                 reinterpret_cast<uint2*>(packed_vol), to_packed ? 1 : 0);
  else
    k_bricks_copy<uint32_t><<<blocks, 256, 0, st>>>(reinterpret_cast<uint32_t*>(h.vol), bricks, n,
                                                    reinterpret_cast<uint32_t*>(packed_vol), to_packed ? 1 : 0);
  if (h.col && packed_col)
    k_bricks_copy<uint32_t><<<blocks, 256, 0, st>>>(h.col, bricks, n, packed_col, to_packed ? 1 : 0);
}

}  // namespace vs
