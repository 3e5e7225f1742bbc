// Snapshot / resume and mesh export (vs_session_save / vs_session_load,
// vs_extract_mesh, vs_save_mesh_ply in include/vs.h), and the host side of the
// depth -> colour registration (vs_warp_depth_*).
//
// Snapshot file (little-endian, this library's own format; the reference's
// .vcl writer is closed):
//   char     magic[8]      "VSSNAP01"
//   uint32   header_bytes  size of vs_config that follows
//   vs_config cfg
//   double   T_gc[16]      FP64 master pose
//   int32    frame, tracked
//   uint64   n             sub-cubes holding data (occupancy bit set)
//   uint32   index[n]      ascending
//   words    n * 512 TSDF words (4 bytes, 8 for the FP32 storage)
//   uint32   n * 512 colour words (sessions with colour only)
//   uint64   m             sub-cubes the last integration flagged (optional)
//   uint32   flagged[m]    ascending
// Only sub-cubes whose occupancy bit is set carry data; every other voxel is in
// its initial state.  Loading creates a session with the saved configuration,
// scatters the sub-cubes, rebuilds the occupancy levels, restores the pose and
// the flagged set (what a valid-volume carving visits), and ray-casts the
// model maps from the pose, which is what the saved session's next frame would
// read.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "vs.h"
#include "vs_host.h"
#include "vs_internal.cuh"

namespace vs {
void launch_mesh(const SessionDev& h, const SessionDev* d, const uint32_t* bricks, int n, float* xyz, uint8_t* rgb,
                 uint64_t capacity, unsigned long long* count, cudaStream_t st);
void launch_bricks_copy(const SessionDev& h, const uint32_t* bricks, int n, void* packed_vol, uint32_t* packed_col,
                        bool to_packed, cudaStream_t st);
template <class T>
void launch_warp_depth(const T* in, int wd, int hd, const float* Kd, const float* T_rgb_d, const float* Kr, int wr,
                       int hr, float scale, unsigned* scratch, T* out, cudaStream_t st);
}  // namespace vs

using namespace vs;

namespace {

const char kMagic[8] = {'V', 'S', 'S', 'N', 'A', 'P', '0', '1'};

// ascending indices of the sub-cubes whose occupancy bit is set
int occupied_bricks(vs_session* s, std::vector<uint32_t>& out) {
  const size_t nbr = (size_t)s->h.nb[0] * s->h.nb[1] * s->h.nb[2];
  std::vector<uint32_t> bits((nbr + 31) / 32);
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e == cudaSuccess) e = cudaMemcpy(bits.data(), s->h.occ, bits.size() * 4, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail_code(e, "occupancy read");
  out.clear();
  for (size_t wi = 0; wi < bits.size(); wi++)
    for (uint32_t m = bits[wi]; m; m &= m - 1) out.push_back((uint32_t)(wi * 32 + __builtin_ctz(m)));
  return VS_OK;
}

// ascending indices of the sub-cubes flagged by the last integration
// (flag == activation stamp != 0)
int flagged_bricks(vs_session* s, std::vector<uint32_t>& out) {
  const size_t nbr = (size_t)s->h.nb[0] * s->h.nb[1] * s->h.nb[2];
  std::vector<uint32_t> flags(nbr);
  uint32_t cnt[4];
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e == cudaSuccess) e = cudaMemcpy(flags.data(), s->h.brick_flag, nbr * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(cnt, s->h.brick_count, sizeof(cnt), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail_code(e, "sub-cube flags read");
  out.clear();
  if (cnt[2] == 0u) return VS_OK;
  for (size_t b = 0; b < nbr; b++)
    if (flags[b] == cnt[2]) out.push_back((uint32_t)b);
  return VS_OK;
}

struct DevBuf {
  void* p = nullptr;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
};

bool write_all(FILE* f, const void* p, size_t n) { return n == 0 || fwrite(p, 1, n, f) == n; }
bool read_all(FILE* f, void* p, size_t n) { return n == 0 || fread(p, 1, n, f) == n; }

}  // namespace

extern "C" {

int vs_session_config(vs_session* s, vs_config* out) {
  if (!s || !out) return fail_code(VS_ERR_ARG, "null argument");
  *out = s->cfg;
  return VS_OK;
}

int vs_session_save(vs_session* s, const char* path) {
  if (!s || !path) return fail_code(VS_ERR_ARG, "null argument");
  std::vector<uint32_t> list, flagged;
  int rc = occupied_bricks(s, list);
  if (rc == VS_OK) rc = flagged_bricks(s, flagged);
  if (rc) return rc;
  vs_config cfg = s->cfg;
  double T[16];
  int info[4];
  rc = vs_get_pose(s, nullptr, T, info);
  if (rc) return rc;
  const size_t n = list.size(), wb = voxel_bytes(s->h.tsdf_type);
  std::vector<unsigned char> words(n * kBrickVox * wb);
  std::vector<uint32_t> cols(s->h.col ? n * kBrickVox : 0);
  if (n) {
    DevBuf dl, dv, dc;
    cudaError_t e = cudaMalloc(&dl.p, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dv.p, words.size());
    if (e == cudaSuccess && !cols.empty()) e = cudaMalloc(&dc.p, cols.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(dl.p, list.data(), n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      launch_bricks_copy(s->h, (const uint32_t*)dl.p, (int)n, dv.p, (uint32_t*)dc.p, true, s->stream);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess) e = cudaMemcpy(words.data(), dv.p, words.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && !cols.empty()) e = cudaMemcpy(cols.data(), dc.p, cols.size() * 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail_code(e, "snapshot gather");
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail_code(VS_ERR_ARG, std::string("cannot open ") + path);
  const uint32_t hb = (uint32_t)sizeof(vs_config);
  const int32_t fr = info[3], tr = info[0];
  const uint64_t n64 = n;
  bool ok = write_all(f, kMagic, 8) && write_all(f, &hb, 4) && write_all(f, &cfg, sizeof(cfg)) &&
            write_all(f, T, sizeof(T)) && write_all(f, &fr, 4) && write_all(f, &tr, 4) && write_all(f, &n64, 8) &&
            write_all(f, list.data(), n * 4) && write_all(f, words.data(), words.size()) &&
            write_all(f, cols.data(), cols.size() * 4);
  const uint64_t m64 = flagged.size();
  ok = ok && write_all(f, &m64, 8) && write_all(f, flagged.data(), flagged.size() * 4);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail_code(VS_ERR_ARG, std::string("write failed: ") + path);
  return VS_OK;
}

int vs_session_load(const char* path, vs_session** out) {
  if (!path || !out) return fail_code(VS_ERR_ARG, "null argument");
  *out = nullptr;
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail_code(VS_ERR_ARG, std::string("cannot open ") + path);
  char magic[8];
  uint32_t hb = 0;
  vs_config cfg;
  double T[16];
  int32_t fr = 0, tr = 0;
  uint64_t n = 0;
  bool ok = read_all(f, magic, 8) && std::memcmp(magic, kMagic, 8) == 0 && read_all(f, &hb, 4) &&
            hb == sizeof(vs_config) && read_all(f, &cfg, sizeof(cfg)) && read_all(f, T, sizeof(T)) &&
            read_all(f, &fr, 4) && read_all(f, &tr, 4) && read_all(f, &n, 8);
  if (!ok) {
    std::fclose(f);
    return fail_code(VS_ERR_ARG, std::string("not a snapshot of this library: ") + path);
  }
  const size_t nbr = (size_t)(cfg.dim[0] / 8) * (cfg.dim[1] / 8) * (cfg.dim[2] / 8);
  if (n > nbr || cfg.dim[0] <= 0 || cfg.dim[1] <= 0 || cfg.dim[2] <= 0) {
    std::fclose(f);
    return fail_code(VS_ERR_ARG, "corrupt snapshot header");
  }
  const size_t wb = voxel_bytes(cfg.tsdf_type);
  std::vector<uint32_t> list(n);
  std::vector<unsigned char> words(n * kBrickVox * wb);
  std::vector<uint32_t> cols(cfg.color ? n * kBrickVox : 0);
  ok = read_all(f, list.data(), n * 4) && read_all(f, words.data(), words.size()) &&
       read_all(f, cols.data(), cols.size() * 4);
  // the flagged set is optional (absent: nothing flagged)
  std::vector<uint32_t> flagged;
  uint64_t m = 0;
  if (ok && read_all(f, &m, 8)) {
    if (m > nbr) ok = false;
    if (ok) {
      flagged.resize(m);
      ok = read_all(f, flagged.data(), m * 4);
    }
  }
  std::fclose(f);
  if (!ok) return fail_code(VS_ERR_ARG, "truncated snapshot");
  for (uint64_t i = 0; i < n; i++)
    if (list[i] >= nbr || (i && list[i] <= list[i - 1])) return fail_code(VS_ERR_ARG, "corrupt sub-cube index list");
  for (uint64_t i = 0; i < m; i++)
    if (flagged[i] >= nbr || (i && flagged[i] <= flagged[i - 1]))
      return fail_code(VS_ERR_ARG, "corrupt flagged sub-cube list");
  vs_session* s = nullptr;
  int rc = vs_session_create(&cfg, &s);
  if (rc) return rc;
  // frees the half-built session; m replaces the error message when given
  auto bail = [&](int code, const std::string& m) {
    vs_session_destroy(s);
    return m.empty() ? code : fail_code(code, m);
  };
  if (n) {
    DevBuf dl, dv, dc;
    cudaError_t e = cudaMalloc(&dl.p, n * 4);
    if (e == cudaSuccess) e = cudaMalloc(&dv.p, words.size());
    if (e == cudaSuccess && !cols.empty()) e = cudaMalloc(&dc.p, cols.size() * 4);
    if (e == cudaSuccess) e = cudaMemcpy(dl.p, list.data(), n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dv.p, words.data(), words.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && !cols.empty()) e = cudaMemcpy(dc.p, cols.data(), cols.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
      launch_bricks_copy(s->h, (const uint32_t*)dl.p, (int)n, dv.p, (uint32_t*)dc.p, false, s->stream);
      launch_occupancy_rebuild(s->h, s->d, s->stream);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) return bail(cuda_fail_code(e, "snapshot scatter"), "");
  }
  if (m) {
    // activation stamp 1, and flag 1 on the flagged sub-cubes
    std::vector<uint32_t> flags(nbr, 0u);
    for (uint32_t b : flagged) flags[b] = 1u;
    const uint32_t stamp = 1u;
    cudaError_t e = cudaMemcpy(s->h.brick_flag, flags.data(), nbr * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(s->h.brick_count + 2, &stamp, 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return bail(cuda_fail_code(e, "snapshot flags"), "");
  }
  rc = vs_set_pose(s, T);
  if (rc) return bail(rc, "");
  // frame counter and tracking flag as saved
  Pose head;
  cudaError_t e = cudaMemcpy(&head, s->h.pose, kPoseHeadBytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) {
    head.frame = fr;
    head.tracked = tr;
    e = cudaMemcpy(s->h.pose, &head, kPoseHeadBytes, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return bail(cuda_fail_code(e, "snapshot pose"), "");
  // the model maps the next frame's ICP reads
  rc = vs_stage_raycast(s);
  if (rc == VS_OK) rc = vs_session_sync(s);
  if (rc) return bail(rc, "");
  *out = s;
  return VS_OK;
}

int vs_extract_mesh(vs_session* s, float* xyz_host, uint8_t* rgb_host, uint64_t capacity, uint64_t* n_triangles) {
  if (!s || !n_triangles) return fail_code(VS_ERR_ARG, "null argument");
  if (capacity && !xyz_host) return fail_code(VS_ERR_ARG, "null output with a non-zero capacity");
  std::vector<uint32_t> list;
  int rc = occupied_bricks(s, list);
  if (rc) return rc;
  DevBuf dl, dx, dc, dn;
  cudaError_t e = cudaMalloc(&dn.p, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemset(dn.p, 0, sizeof(unsigned long long));
  if (e == cudaSuccess && !list.empty()) e = cudaMalloc(&dl.p, list.size() * 4);
  if (e == cudaSuccess && !list.empty()) e = cudaMemcpy(dl.p, list.data(), list.size() * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && capacity) e = cudaMalloc(&dx.p, capacity * 9 * sizeof(float));
  if (e == cudaSuccess && capacity && rgb_host) e = cudaMalloc(&dc.p, capacity * 9);
  if (e != cudaSuccess) return cuda_fail_code(e, "mesh buffers");
  launch_mesh(s->h, s->d, (const uint32_t*)dl.p, (int)list.size(), (float*)dx.p, (uint8_t*)dc.p, capacity,
              (unsigned long long*)dn.p, s->stream);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  unsigned long long total = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&total, dn.p, sizeof(total), cudaMemcpyDeviceToHost);
  const uint64_t m = total < capacity ? total : capacity;
  if (e == cudaSuccess && m) e = cudaMemcpy(xyz_host, dx.p, m * 9 * sizeof(float), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && m && rgb_host) e = cudaMemcpy(rgb_host, dc.p, m * 9, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail_code(e, "mesh extraction");
  *n_triangles = total;
  return VS_OK;
}

int vs_save_mesh_ply(vs_session* s, const char* path) {
  if (!s || !path) return fail_code(VS_ERR_ARG, "null argument");
  uint64_t n = 0;
  int rc = vs_extract_mesh(s, nullptr, nullptr, 0, &n);
  if (rc) return rc;
  std::vector<float> xyz(n * 9);
  const bool color = s->h.col != nullptr;
  std::vector<uint8_t> rgb(color ? n * 9 : 0);
  uint64_t got = 0;
  rc = vs_extract_mesh(s, xyz.data(), color ? rgb.data() : nullptr, n, &got);
  if (rc) return rc;
  n = got < n ? got : n;
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail_code(VS_ERR_ARG, std::string("cannot open ") + path);
  std::string hdr = "ply\nformat binary_little_endian 1.0\nelement vertex " + std::to_string(3 * n) +
                    "\nproperty float x\nproperty float y\nproperty float z\n";
  if (color) hdr += "property uchar red\nproperty uchar green\nproperty uchar blue\n";
  hdr += "element face " + std::to_string(n) + "\nproperty list uchar int vertex_indices\nend_header\n";
  bool ok = write_all(f, hdr.data(), hdr.size());
  for (uint64_t v = 0; ok && v < 3 * n; v++) {
    ok = write_all(f, &xyz[3 * v], 12);
    if (ok && color) ok = write_all(f, &rgb[3 * v], 3);
  }
  for (uint64_t t = 0; ok && t < n; t++) {
    const uint8_t three = 3;
    const int32_t idx[3] = {(int32_t)(3 * t), (int32_t)(3 * t + 1), (int32_t)(3 * t + 2)};
    ok = write_all(f, &three, 1) && write_all(f, idx, 12);
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return fail_code(VS_ERR_ARG, std::string("write failed: ") + path);
  return VS_OK;
}

}  // extern "C"

// ---- depth -> colour registration (k_register.cu) ----------------------------

static int warp_checks(const void* in, int wd, int hd, const float* Kd, const float* T, const float* Kr, int wr,
                       int hr, const void* out) {
  if (!in || !Kd || !T || !Kr || !out) return fail_code(VS_ERR_ARG, "null argument");
  if (wd < 1 || hd < 1 || wr < 1 || hr < 1 || wd > 8192 || hd > 8192 || wr > 8192 || hr > 8192)
    return fail_code(VS_ERR_ARG, "image size out of range (1..8192)");
  if (Kd[0] == 0 || Kd[1] == 0 || Kr[0] == 0 || Kr[1] == 0) return fail_code(VS_ERR_ARG, "focal length is zero");
  return VS_OK;
}

template <class T>
static int warp_run(const T* in, int wd, int hd, const float* Kd, const float* Tm, const float* Kr, int wr, int hr,
                    float scale, T* out, void* stream) {
  unsigned* scratch = nullptr;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&scratch), (size_t)wr * hr * 4, st);
  if (e != cudaSuccess) return cuda_fail_code(e, "warp scratch");
  launch_warp_depth<T>(in, wd, hd, Kd, Tm, Kr, wr, hr, scale, scratch, out, st);
  e = cudaGetLastError();
  cudaError_t e2 = cudaFreeAsync(scratch, st);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail_code(e, "depth warp");
  return VS_OK;
}

extern "C" {

int vs_warp_depth_to_color(const float* depth_dev, int w_d, int h_d, const float* K_d, const float* T_rgb_wrt_d,
                           const float* K_rgb, int w_rgb, int h_rgb, float* depth_rgb_dev, void* stream) {
  int rc = warp_checks(depth_dev, w_d, h_d, K_d, T_rgb_wrt_d, K_rgb, w_rgb, h_rgb, depth_rgb_dev);
  if (rc) return rc;
  return warp_run<float>(depth_dev, w_d, h_d, K_d, T_rgb_wrt_d, K_rgb, w_rgb, h_rgb, 1.0f, depth_rgb_dev, stream);
}

int vs_warp_depth_mm_to_color(const uint16_t* depth_mm_dev, int w_d, int h_d, float depth_scale, const float* K_d,
                              const float* T_rgb_wrt_d, const float* K_rgb, int w_rgb, int h_rgb,
                              uint16_t* depth_mm_rgb_dev, void* stream) {
  int rc = warp_checks(depth_mm_dev, w_d, h_d, K_d, T_rgb_wrt_d, K_rgb, w_rgb, h_rgb, depth_mm_rgb_dev);
  if (rc) return rc;
  if (!(depth_scale > 0)) return fail_code(VS_ERR_ARG, "depth_scale must be > 0");
  return warp_run<uint16_t>(depth_mm_dev, w_d, h_d, K_d, T_rgb_wrt_d, K_rgb, w_rgb, h_rgb, depth_scale,
                            depth_mm_rgb_dev, stream);
}

}  // extern "C"
