// Host layer and C ABI (include/vs.h): session lifecycle, the per-frame CUDA
// graph, the reference-shaped stage entry points and state access.
//
// A session replaces what the reference keeps in per-file __constant__
// globals and in its device containers (GKvObjectCube, GKvTrackingState,
// GKvRgbdFrame, STAC/Object/GPU/*): every buffer is allocated once at
// creation, described by one SessionDev record in device memory, and reused
// for every frame.  The per-frame path (so_Scan_Object,
// STAC/Engine/CPU/z_yooji_object_scanner.cpp:472-629) is captured once into a
// CUDA graph and replayed.
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "vs.h"
#include "vs_host.h"
#include "vs_internal.cuh"

namespace vs {
void launch_volume_slab(const SessionDev& h, bool do_export, int z0, int nz, float* tsdf, uint16_t* w,
                        cudaStream_t st);
void configure_filter_kernels();
int integrate_max_dim();
int integrate_max_image();
}  // namespace vs

using namespace vs;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return VS_ERR_CUDA;
}
#define VS_CU(call)                                   \
  do {                                                \
    cudaError_t e_ = (call);                          \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
  } while (0)

int check_config(const vs_config* c) {
  if (!c) return fail(VS_ERR_ARG, "null config");
  if (c->levels < 1 || c->levels > kMaxLevels) return fail(VS_ERR_ARG, "levels must be 1..3");
  if (c->width < 8 || c->height < 8 || c->width > integrate_max_image() || c->height > integrate_max_image())
    return fail(VS_ERR_ARG, "image size out of range (8..2048)");
  if ((c->width >> (c->levels - 1)) < 4 || (c->height >> (c->levels - 1)) < 4)
    return fail(VS_ERR_ARG, "top pyramid level smaller than 4 pixels");
  for (int k = 0; k < 3; k++)
    if (c->dim[k] < 8 || c->dim[k] % 8 || c->dim[k] > integrate_max_dim())
      return fail(VS_ERR_ARG, "volume dims must be multiples of 8 in 8..1024");
  if (!(c->voxel_size > 0) || !(c->mu > 0) || !(c->max_w >= 1) || c->max_w > 65535.0f)
    return fail(VS_ERR_ARG, "voxel_size, mu must be > 0 and max_w in 1..65535");
  if (!(c->th_icp > 0)) return fail(VS_ERR_ARG, "th_icp must be > 0");
  if (c->fx == 0 || c->fy == 0) return fail(VS_ERR_ARG, "focal length is zero");
  if (c->tsdf_type < 0 || c->tsdf_type > 2) return fail(VS_ERR_ARG, "bad tsdf_type");
  if (c->reduce_mode < 0 || c->reduce_mode > 2) return fail(VS_ERR_ARG, "bad reduce_mode");
  for (int l = 0; l < kMaxLevels; l++)
    if (c->icp_iters[l] < 0 || c->icp_iters[l] > 100) return fail(VS_ERR_ARG, "icp_iters must be 0..100");
  if (c->color != 0 && c->color != 1) return fail(VS_ERR_ARG, "color must be 0 or 1");
  return VS_OK;
}

// level geometry and cube constants, in the reference's float arithmetic
void fill_geometry(const vs_config* c, SessionDev& h) {
  float fx = c->fx, fy = c->fy, px = c->cx, py = c->cy;
  int w = c->width, hh = c->height;
  for (int k = 0; k < kMaxLevels; k++) {
    h.lv[k].W = w;
    h.lv[k].H = hh;
    h.lv[k].K[0] = fx;
    h.lv[k].K[1] = fy;
    h.lv[k].K[2] = px;
    h.lv[k].K[3] = py;
    // z_yooji_cuda_pose_tracker.cu:770, z_yooji_cuda_tsdf_renderer.cu:1617
    fx = 0.5f * fx;
    fy = 0.5f * fy;
    px = 0.5f * (px - 0.5f);
    py = 0.5f * (py - 0.5f);
    w /= 2;
    hh /= 2;
  }
  h.levels = c->levels;
  for (int k = 0; k < 3; k++) {
    h.dim[k] = c->dim[k];
    h.nb[k] = c->dim[k] / 8;
    h.origin[k] = c->origin[k];
  }
  h.vox = c->voxel_size;
  h.vox_inv = 1.0f / c->voxel_size;  // z_yooji_cuda_volume_integrator.cu:847
  h.mu = c->mu;
  h.max_w = c->max_w;
  for (int k = 0; k < 3; k++) h.cube_center[k] = h.origin[k] + (float)h.dim[k] * h.vox / 2.0f;
  F3 d = f3(h.origin[0] - h.cube_center[0], h.origin[1] - h.cube_center[1], h.origin[2] - h.cube_center[2]);
  h.r_cube = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
  h.th_icp = c->th_icp;
  h.cos_normal = c->cos_normal;
  for (int k = 0; k < kMaxLevels; k++) h.iters[k] = c->icp_iters[k];
  h.reduce_mode = c->reduce_mode;
  h.tsdf_type = c->tsdf_type;
  h.depth_scale = c->depth_scale;
  // cGaussian (updateGaussian, z_yooji_cuda_img_proc.cu:275-286), delta 4, radius 2
  const float delta = 4.0f;
  for (int i = 0; i < 5; i++) {
    float x = (float)(i - 2);
    h.gauss[i] = std::exp(-(x * x) / (2 * delta * delta));
  }
}

template <class T>
int alloc(vs_session* s, T** p, size_t bytes) {
  void* q = nullptr;
  cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    g_err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
    return VS_ERR_MEMORY;
  }
  s->allocs.push_back(q);
  *p = reinterpret_cast<T*>(q);
  return VS_OK;
}

size_t volume_bytes(const vs_config* c) {
  return (size_t)c->dim[0] * c->dim[1] * c->dim[2] * voxel_bytes(c->tsdf_type);
}

void free_all(vs_session* s) {
  for (auto& e : s->ev)
    if (e) cudaEventDestroy(e), e = nullptr;
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->exec = nullptr;
  s->graph = nullptr;
  for (void* p : s->allocs) cudaFree(p);
  s->allocs.clear();
  if (s->host_pose) cudaFreeHost(s->host_pose);
  s->host_pose = nullptr;
  if (s->stream) cudaStreamDestroy(s->stream);
  s->stream = nullptr;
}

int reset_state(vs_session* s) {
  launch_volume_init(s->h, s->stream);
  VS_CU(cudaGetLastError());
  VS_CU(cudaMemsetAsync(s->h.brick_flag, 0, sizeof(uint32_t) * (size_t)s->h.nb[0] * s->h.nb[1] * s->h.nb[2],
                        s->stream));
  VS_CU(cudaMemsetAsync(s->h.brick_count, 0, 4 * sizeof(uint32_t), s->stream));
  launch_occupancy_clear(s->h, s->stream);
  VS_CU(cudaGetLastError());
  VS_CU(cudaMemsetAsync(s->h.icp_counter, 0, sizeof(unsigned), s->stream));
  Pose p;
  std::memset(&p, 0, sizeof(p));
  for (int i = 0; i < 16; i++) {
    double v = (i % 5 == 0) ? 1.0 : 0.0;
    p.T_gc[i] = p.T12[i] = v;
    p.Tgc[i] = p.Tcg[i] = p.T21[i] = (float)v;
  }
  p.tracked = 1;
  *s->host_pose = p;
  VS_CU(cudaMemcpyAsync(s->h.pose, s->host_pose, sizeof(Pose), cudaMemcpyHostToDevice, s->stream));
  if (s->h.col) {
    const size_t n0 = (size_t)s->h.lv[0].W * s->h.lv[0].H;
    VS_CU(cudaMemsetAsync(s->h.col, 0, (size_t)s->h.nb[0] * s->h.nb[1] * s->h.nb[2] * kBrickVox * 4, s->stream));
    VS_CU(cudaMemsetAsync(s->h.rgb_in, 0, n0 * 3, s->stream));
    VS_CU(cudaMemsetAsync(s->h.rgb_packed, 0, n0 * 4, s->stream));
    for (int l = 0; l < s->h.levels; l++)
      VS_CU(cudaMemsetAsync(s->h.m_rgb[l], 0, (size_t)s->h.lv[l].W * s->h.lv[l].H * 4, s->stream));
  }
  // model maps start invalid (depth 0, vertex / normal -100)
  for (int l = 0; l < s->h.levels; l++) {
    size_t n = (size_t)s->h.lv[l].W * s->h.lv[l].H;
    VS_CU(cudaMemsetAsync(s->h.m_depth[l], 0, n * 4, s->stream));
    VS_CU(cudaMemsetAsync(s->h.m_img[l], 0, n, s->stream));
    std::vector<float4> inv(n, make_float4(-100.0f, -100.0f, -100.0f, 0.0f));
    VS_CU(cudaMemcpy(s->h.m_vtx[l], inv.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    VS_CU(cudaMemcpy(s->h.m_nrm[l], inv.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    VS_CU(cudaMemcpy(s->h.in_vtx[l], inv.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
    VS_CU(cudaMemcpy(s->h.in_nrm[l], inv.data(), n * sizeof(float4), cudaMemcpyHostToDevice));
  }
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

// the per-frame sequence (recorded into the graph); with stage timing on,
// event-record nodes separate filter / track / integrate / ray-cast
void record_frame(vs_session* s, cudaStream_t st) {
  const SessionDev& h = s->h;
  auto mark = [&](int i) {
    if (s->timing) cudaEventRecordWithFlags(s->ev[i], st, cudaEventRecordExternal);
  };
  mark(0);
  launch_filter(s->tab, st);
  if (h.cos_normal > -2.0f) launch_input_maps(s->tab, st);
  mark(1);
  launch_icp(s->tab, h.levels, h.iters, h.reduce_mode, st, true, nullptr);
  mark(2);
  const bool color = h.col != nullptr;
  launch_integrate(s->tab, h.tsdf_type, nullptr, nullptr, nullptr, true, st, color);
  mark(3);
  launch_raycast(s->tab, h.tsdf_type, -1, nullptr, nullptr, nullptr, 0.0f, 0.0f, -1.0f, true, nullptr, nullptr,
                 nullptr, nullptr, st, LaunchShape(), nullptr, color);
  mark(4);
}

int build_graph(vs_session* s) {
  if (s->exec) return VS_OK;
  VS_CU(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  record_frame(s, s->stream);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  s->graph = g;
  VS_CU(cudaGraphInstantiate(&s->exec, g, 0));
  return VS_OK;
}

std::once_flag g_once;

}  // namespace

namespace vs {
// lets other translation units report through vs_last_error()
void set_error(const char* msg) { g_err = msg; }
int fail_code(int code, const std::string& msg) { return fail(code, msg); }
int cuda_fail_code(cudaError_t e, const char* what) { return cuda_fail(e, what); }
}  // namespace vs

extern "C" {

void vs_config_default(vs_config* c, int width, int height) {
  std::memset(c, 0, sizeof(*c));
  c->width = width;
  c->height = height;
  c->fx = c->fy = 525.0f;
  c->cx = 0.5f * width - 0.5f;
  c->cy = 0.5f * height - 0.5f;
  c->levels = 3;
  c->dim[0] = c->dim[1] = c->dim[2] = 256;
  c->voxel_size = 1.0f / 256.0f;
  c->origin[0] = -0.5f;
  c->origin[1] = -0.5f;
  c->origin[2] = 0.5f;
  c->mu = 0.03f;
  c->max_w = 100.0f;
  c->th_icp = 0.1f * 0.1f;
  c->cos_normal = -3.0f;
  c->icp_iters[0] = 10;
  c->icp_iters[1] = 5;
  c->icp_iters[2] = 4;
  c->reduce_mode = VS_REDUCE_KAHAN;
  c->tsdf_type = VS_TSDF_INT16;
  c->depth_scale = 0.001f;
  c->color = 0;
}

const char* vs_last_error(void) { return g_err.c_str(); }

int vs_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

size_t vs_session_bytes(const vs_config* c) {
  if (check_config(c) != VS_OK) return 0;
  size_t b = volume_bytes(c);
  size_t nbr = (size_t)(c->dim[0] / 8) * (c->dim[1] / 8) * (c->dim[2] / 8);
  b += 2 * nbr * 4 + ((nbr + 31) / 32) * 4 + 3 * nbr + 64;
  int w = c->width, h = c->height;
  b += (size_t)w * h * (2 + 4 + 4);
  for (int l = 0; l < c->levels; l++) {
    size_t n = (size_t)(w >> l) * (h >> l);
    b += n * (4 + 16 + 16 + 1 + 4 + 16 + 16 + 1) + 2 * (size_t)(h >> l) * (((w >> l) + 31) / 32) * 4;
  }
  b += (size_t)kIcpMaxBlocks * kPartials * 16 + sizeof(Pose) + sizeof(SessionDev) + sizeof(BatchTable) + 64;
  b += (size_t)(c->dim[0] + c->dim[1] + c->dim[2] + w + h) * 4;
  for (int l = 0; l < c->levels; l++) b += (size_t)(w >> l) * (h >> l) * 16;  // ray-cast hit points
  b += (size_t)w * h * (4 + 8);                                                // ray-scale map, {depth, scale} map
  if (c->color) {
    b += (size_t)c->dim[0] * c->dim[1] * c->dim[2] * 4 + (size_t)w * h * (3 + 4);  // colour volume and frame
    for (int l = 0; l < c->levels; l++) b += (size_t)(w >> l) * (h >> l) * 4;      // colour maps
  }
  return b;
}

int vs_session_create(const vs_config* cfg, vs_session** out) {
  if (!out) return fail(VS_ERR_ARG, "null output");
  *out = nullptr;
  int rc = check_config(cfg);
  if (rc) return rc;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(VS_ERR_CUDA, "no CUDA device available");
  std::call_once(g_once, [] { configure_filter_kernels(); });
  vs_session* s = new vs_session;
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  std::memset(&s->h, 0, sizeof(s->h));
  fill_geometry(cfg, s->h);
  SessionDev& h = s->h;
  e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete s;
    return cuda_fail(e, "cudaStreamCreate");
  }
  e = cudaMallocHost(&s->host_pose, sizeof(Pose));
  if (e != cudaSuccess) {
    free_all(s);
    delete s;
    return cuda_fail(e, "cudaMallocHost");
  }
  const size_t nbr = (size_t)h.nb[0] * h.nb[1] * h.nb[2];
  const size_t n0 = (size_t)h.lv[0].W * h.lv[0].H;
  rc = 0;
  rc |= alloc(s, &h.vol, volume_bytes(cfg));
  rc |= alloc(s, &h.brick_flag, nbr * 4);
  rc |= alloc(s, &h.brick_list, nbr * 4);
  rc |= alloc(s, &h.brick_count, 64);
  rc |= alloc(s, &h.occ, occupancy_words(h) * 4);
  rc |= alloc(s, &h.band, nbr);
  rc |= alloc(s, &h.bdist, nbr);
  rc |= alloc(s, &h.btmp, nbr);
  rc |= alloc(s, &h.depth_mm, n0 * 2);
  rc |= alloc(s, &h.depth_raw, n0 * 4);
  rc |= alloc(s, &s->stage_f, n0 * 4);
  rc |= alloc(s, &s->dev_small, 64);
  for (int l = 0; l < h.levels; l++) {
    size_t n = (size_t)h.lv[l].W * h.lv[l].H;
    rc |= alloc(s, &h.depth[l], n * 4);
    rc |= alloc(s, &h.in_vtx[l], n * 16);
    rc |= alloc(s, &h.in_nrm[l], n * 16);
    rc |= alloc(s, &h.in_code[l], n);
    rc |= alloc(s, &h.in_amask[l], (size_t)h.lv[l].H * ((h.lv[l].W + 31) / 32) * 4);
    rc |= alloc(s, &h.in_rmask[l], (size_t)h.lv[l].H * ((h.lv[l].W + 31) / 32) * 4);
    rc |= alloc(s, &h.m_depth[l], n * 4);
    rc |= alloc(s, &h.m_vtx[l], n * 16);
    rc |= alloc(s, &h.m_nrm[l], n * 16);
    rc |= alloc(s, &h.m_img[l], n);
  }
  rc |= alloc(s, &h.partials, (size_t)kIcpMaxBlocks * kPartials * 16);
  rc |= alloc(s, &h.icp_counter, 64);
  rc |= alloc(s, &h.pose, sizeof(Pose));
  rc |= alloc(s, &h.lut_vox, (size_t)(h.dim[0] + h.dim[1] + h.dim[2]) * 4);
  rc |= alloc(s, &h.lut_ray, (size_t)(h.lv[0].W + h.lv[0].H) * 4);
  rc |= alloc(s, &h.lam_map, n0 * 4);
  rc |= alloc(s, &h.dl_map, n0 * 8);
  if (cfg->color) {
    rc |= alloc(s, &h.col, nbr * kBrickVox * 4);
    rc |= alloc(s, &h.rgb_in, n0 * 3);
    rc |= alloc(s, &h.rgb_packed, n0 * 4);
    for (int l = 0; l < h.levels; l++) rc |= alloc(s, &h.m_rgb[l], (size_t)h.lv[l].W * h.lv[l].H * 4);
  }
  {  // the hit buffer between the two launches of a colour ray-cast (a batch with a colour
     // session runs them for every session of the batch)
    size_t npx = 0;
    for (int l = 0; l < h.levels; l++) npx += (size_t)h.lv[l].W * h.lv[l].H;
    rc |= alloc(s, &h.ray_hit, npx * sizeof(float4));
  }
  rc |= alloc(s, &s->d, sizeof(SessionDev));
  rc |= alloc(s, &s->tab, sizeof(BatchTable));
  if (rc) {
    std::string m = g_err;
    free_all(s);
    delete s;
    return fail(VS_ERR_MEMORY, m);
  }
  e = cudaMemcpy(s->d, &h, sizeof(SessionDev), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    BatchTable t;
    const SessionDev* hr = &h;
    const SessionDev* dr = s->d;
    fill_batch_table(t, &hr, &dr, 1);
    e = cudaMemcpy(s->tab, &t, sizeof(BatchTable), cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {
    launch_session_tables(h, s->d, s->stream);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    free_all(s);
    delete s;
    return cuda_fail(e, "session record set-up");
  }
  rc = reset_state(s);
  if (rc) {
    std::string m = g_err;
    free_all(s);
    delete s;
    return fail(rc, m);
  }
  *out = s;
  return VS_OK;
}

int vs_session_destroy(vs_session* s) {
  if (!s) return VS_OK;
  cudaStreamSynchronize(s->stream);
  free_all(s);
  delete s;
  return VS_OK;
}

int vs_session_reset(vs_session* s) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaStreamSynchronize(s->stream));
  return reset_state(s);
}

int vs_session_sync(vs_session* s) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

// ---- reference-shaped stage entry points ----------------------------------

int vs_bilateral_filter_depth(vs_session* s, float* out_dev, const float* in_host, int ww, int hh) {
  if (!s || !out_dev || !in_host) return fail(VS_ERR_ARG, "null argument");
  if (ww != s->h.lv[0].W || hh != s->h.lv[0].H) return fail(VS_ERR_ARG, "size differs from the session");
  VS_CU(cudaMemcpyAsync(s->stage_f, in_host, (size_t)ww * hh * 4, cudaMemcpyHostToDevice, s->stream));
  launch_bilateral_float(s->h, s->stage_f, out_dev, s->stream);
  VS_CU(cudaGetLastError());
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_bilateral_filter_depth_host(vs_session* s, float* out_host, const float* in_host, int ww, int hh) {
  if (!s || !out_host || !in_host) return fail(VS_ERR_ARG, "null argument");
  if (ww != s->h.lv[0].W || hh != s->h.lv[0].H) return fail(VS_ERR_ARG, "size differs from the session");
  VS_CU(cudaMemcpyAsync(s->stage_f, in_host, (size_t)ww * hh * 4, cudaMemcpyHostToDevice, s->stream));
  launch_bilateral_float(s->h, s->stage_f, s->h.depth[0], s->stream);
  VS_CU(cudaGetLastError());
  VS_CU(cudaMemcpyAsync(out_host, s->h.depth[0], (size_t)ww * hh * 4, cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_track_pose(vs_session* s, const float* init_T01_dev, int* tracked) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  launch_icp(s->tab, s->h.levels, s->h.iters, s->h.reduce_mode, s->stream, false, init_T01_dev);
  VS_CU(cudaGetLastError());
  VS_CU(cudaMemcpyAsync(s->host_pose, s->h.pose, sizeof(Pose), cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  if (tracked) *tracked = s->host_pose->failed ? 0 : 1;
  return VS_OK;
}

int vs_integrate_depth(vs_session* s, const float* depth_dev, int ww, int hh, const float* T_gc_dev,
                       const float* T_cg_dev) {
  if (!s || !depth_dev || !T_gc_dev || !T_cg_dev) return fail(VS_ERR_ARG, "null argument");
  if (ww != s->h.lv[0].W || hh != s->h.lv[0].H) return fail(VS_ERR_ARG, "size differs from the session");
  launch_integrate(s->tab, s->h.tsdf_type, depth_dev, T_gc_dev, T_cg_dev, false, s->stream, false);
  VS_CU(cudaGetLastError());
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_integrate_depth_color(vs_session* s, const float* depth_dev, const uint8_t* img_color_dev, int ww, int hh,
                             const float* T_gc_dev, const float* T_cg_dev) {
  if (!s || !depth_dev || !img_color_dev || !T_gc_dev || !T_cg_dev) return fail(VS_ERR_ARG, "null argument");
  if (!s->h.col) return fail(VS_ERR_STATE, "session has no colour volume (cfg.color = 0)");
  if (ww != s->h.lv[0].W || hh != s->h.lv[0].H) return fail(VS_ERR_ARG, "size differs from the session");
  launch_pack_color(s->h, img_color_dev, s->stream);
  launch_integrate(s->tab, s->h.tsdf_type, depth_dev, T_gc_dev, T_cg_dev, false, s->stream, true);
  VS_CU(cudaGetLastError());
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_render_maps(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                   const float* cam_cen, const float* light, int level, float* depth_dev, float* vtx_dev,
                   float* nrm_dev, uint8_t* img_dev) {
  if (!s || !T_gc_dev || !T_cg_dev || !cam_cen || !light || !depth_dev || !vtx_dev || !nrm_dev)
    return fail(VS_ERR_ARG, "null argument");
  if (level < 0 || level >= s->h.levels) return fail(VS_ERR_ARG, "bad level");
  if (ww != s->h.lv[level].W || hh != s->h.lv[level].H) return fail(VS_ERR_ARG, "size differs from the level");
  VS_CU(cudaMemcpyAsync(s->dev_small, cam_cen, 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  launch_raycast(s->tab, s->h.tsdf_type, level, T_gc_dev, T_cg_dev, s->dev_small, light[0], light[1], light[2],
                 false, depth_dev, vtx_dev, nrm_dev, img_dev, s->stream);
  VS_CU(cudaGetLastError());
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_render_maps_color(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                         const float* cam_cen, const float* light, int level, float* depth_dev, float* vtx_dev,
                         float* nrm_dev, uint8_t* img_dev, uint8_t* rgb_dev) {
  if (!s || !T_gc_dev || !T_cg_dev || !cam_cen || !light || !depth_dev || !vtx_dev || !nrm_dev || !rgb_dev)
    return fail(VS_ERR_ARG, "null argument");
  if (!s->h.col) return fail(VS_ERR_STATE, "session has no colour volume (cfg.color = 0)");
  if (level < 0 || level >= s->h.levels) return fail(VS_ERR_ARG, "bad level");
  if (ww != s->h.lv[level].W || hh != s->h.lv[level].H) return fail(VS_ERR_ARG, "size differs from the level");
  VS_CU(cudaMemcpyAsync(s->dev_small, cam_cen, 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  launch_raycast(s->tab, s->h.tsdf_type, level, T_gc_dev, T_cg_dev, s->dev_small, light[0], light[1], light[2],
                 false, depth_dev, vtx_dev, nrm_dev, img_dev, s->stream, LaunchShape(), rgb_dev, true);
  VS_CU(cudaGetLastError());
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

// the ray-cast variants that write external outputs only
static int render_variant(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                          const float* cam_cen, const float* light, int level, float* depth_dev, float* vtx_dev,
                          float* nrm_dev, uint8_t* img_dev, uint8_t* rgb_dev, int mode) {
  if (!s || !T_gc_dev || !T_cg_dev || !cam_cen || !light || !depth_dev || !nrm_dev || !img_dev)
    return fail(VS_ERR_ARG, "null argument");
  if (rgb_dev && !s->h.col) return fail(VS_ERR_STATE, "session has no colour volume (cfg.color = 0)");
  if (level < 0 || level >= s->h.levels) return fail(VS_ERR_ARG, "bad level");
  if (ww != s->h.lv[level].W || hh != s->h.lv[level].H) return fail(VS_ERR_ARG, "size differs from the level");
  VS_CU(cudaMemcpyAsync(s->dev_small, cam_cen, 3 * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  launch_raycast(s->tab, s->h.tsdf_type, level, T_gc_dev, T_cg_dev, s->dev_small, light[0], light[1], light[2],
                 false, depth_dev, vtx_dev, nrm_dev, img_dev, s->stream, LaunchShape(), rgb_dev, rgb_dev != nullptr,
                 mode);
  VS_CU(cudaGetLastError());
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_render_maps_scene(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                         const float* cam_cen, const float* light, float* depth_dev, float* vtx_dev, float* nrm_dev,
                         uint8_t* img_dev, uint8_t* rgb_dev) {
  if (!vtx_dev) return fail(VS_ERR_ARG, "null argument");
  return render_variant(s, ww, hh, T_gc_dev, T_cg_dev, cam_cen, light, 0, depth_dev, vtx_dev, nrm_dev, img_dev,
                        rgb_dev, kRayScene | kRayGlobalNormals | kRayNearestColor);
}

int vs_render_view_scene(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                         const float* cam_cen, const float* light, float* depth_dev, float* nrm_dev, uint8_t* img_dev,
                         uint8_t* rgb_dev) {
  return render_variant(s, ww, hh, T_gc_dev, T_cg_dev, cam_cen, light, 0, depth_dev, nullptr, nrm_dev, img_dev,
                        rgb_dev, kRayScene | kRayGlobalNormals);
}

int vs_render_view(vs_session* s, int ww, int hh, const float* T_gc_dev, const float* T_cg_dev,
                   const float* cam_cen, const float* light, int level, float* depth_dev, float* nrm_dev,
                   uint8_t* img_dev, uint8_t* rgb_dev) {
  return render_variant(s, ww, hh, T_gc_dev, T_cg_dev, cam_cen, light, level, depth_dev, nullptr, nrm_dev, img_dev,
                        rgb_dev, kRayGlobalNormals | kRayWhiteBackground);
}

int vs_update_valid_volume(vs_session* s, const uint8_t* vol_valid, int is_host, uint32_t* carved) {
  if (!s || !vol_valid) return fail(VS_ERR_ARG, "null argument");
  const size_t n = (size_t)s->h.dim[0] * s->h.dim[1] * s->h.dim[2];
  const uint8_t* v = vol_valid;
  uint8_t* tmp = nullptr;
  if (is_host) {
    VS_CU(cudaMallocAsync(reinterpret_cast<void**>(&tmp), n, s->stream));
    cudaError_t e = cudaMemcpyAsync(tmp, vol_valid, n, cudaMemcpyHostToDevice, s->stream);
    if (e != cudaSuccess) {
      cudaFreeAsync(tmp, s->stream);
      return cuda_fail(e, "cudaMemcpyAsync");
    }
    v = tmp;
  } else if (reinterpret_cast<uintptr_t>(vol_valid) % 8) {
    return fail(VS_ERR_ARG, "vol_valid must be 8-byte aligned");
  }
  unsigned* d_count = reinterpret_cast<unsigned*>(s->dev_small + 4);
  cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(unsigned), s->stream);
  if (e == cudaSuccess) {
    launch_carve(s->h, s->d, v, d_count, s->stream);
    e = cudaGetLastError();
  }
  unsigned c = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&c, d_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream);
  if (tmp) {
    const cudaError_t e2 = cudaFreeAsync(tmp, s->stream);
    if (e == cudaSuccess) e = e2;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_fail(e, "vs_update_valid_volume");
  if (carved) *carved = c;
  return VS_OK;
}

int vs_set_color_frame(vs_session* s, const uint8_t* img_color, int is_host) {
  if (!s || !img_color) return fail(VS_ERR_ARG, "null argument");
  if (!s->h.col) return fail(VS_ERR_STATE, "session has no colour volume (cfg.color = 0)");
  const size_t n = (size_t)s->h.lv[0].W * s->h.lv[0].H * 3;
  VS_CU(cudaMemcpyAsync(s->h.rgb_in, img_color, n, is_host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                        s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

static int color_transfer(vs_session* s, uint8_t* out, const uint8_t* in, int level) {
  if (!s->h.col) return fail(VS_ERR_STATE, "session has no colour volume (cfg.color = 0)");
  size_t n;
  if (level < 0)
    n = (size_t)s->h.dim[0] * s->h.dim[1] * s->h.dim[2] * 3;
  else
    n = (size_t)s->h.lv[level].W * s->h.lv[level].H * 3;
  VS_CU(cudaStreamSynchronize(s->stream));
  uint8_t* d = nullptr;
  VS_CU(cudaMalloc(&d, n));
  cudaError_t e = cudaSuccess;
  if (in) {
    e = cudaMemcpy(d, in, n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) launch_color_volume(s->h, false, d, s->stream);
  } else if (level < 0) {
    launch_color_volume(s->h, true, d, s->stream);
  } else {
    launch_color_map_export(s->h, level, d, s->stream);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e == cudaSuccess && out) e = cudaMemcpy(out, d, n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_fail(e, "colour transfer");
  return VS_OK;
}

int vs_get_color_volume(vs_session* s, uint8_t* rgb_host) {
  if (!s || !rgb_host) return fail(VS_ERR_ARG, "null argument");
  return color_transfer(s, rgb_host, nullptr, -1);
}

int vs_set_color_volume(vs_session* s, const uint8_t* rgb_host) {
  if (!s || !rgb_host) return fail(VS_ERR_ARG, "null argument");
  return color_transfer(s, nullptr, rgb_host, -1);
}

int vs_get_color_map(vs_session* s, int level, uint8_t* rgb_host) {
  if (!s || !rgb_host) return fail(VS_ERR_ARG, "null argument");
  if (level < 0 || level >= s->h.levels) return fail(VS_ERR_ARG, "bad level");
  return color_transfer(s, rgb_host, nullptr, level);
}

// ---- per-frame path --------------------------------------------------------

int vs_scan_frame(vs_session* s, const uint16_t* depth_mm_dev, void* stream) {
  if (!s || !depth_mm_dev) return fail(VS_ERR_ARG, "null argument");
  int rc = build_graph(s);
  if (rc) return rc;
  cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
  const size_t n0 = (size_t)s->h.lv[0].W * s->h.lv[0].H;
  if (depth_mm_dev != s->h.depth_mm)
    VS_CU(cudaMemcpyAsync(s->h.depth_mm, depth_mm_dev, n0 * 2, cudaMemcpyDeviceToDevice, st));
  VS_CU(cudaGraphLaunch(s->exec, st));
  return VS_OK;
}

int vs_scan_frame_host(vs_session* s, const uint16_t* depth_mm_host, float* T_gc_out, int* tracked) {
  if (!s || !depth_mm_host) return fail(VS_ERR_ARG, "null argument");
  int rc = build_graph(s);
  if (rc) return rc;
  const size_t n0 = (size_t)s->h.lv[0].W * s->h.lv[0].H;
  VS_CU(cudaMemcpyAsync(s->h.depth_mm, depth_mm_host, n0 * 2, cudaMemcpyHostToDevice, s->stream));
  VS_CU(cudaGraphLaunch(s->exec, s->stream));
  VS_CU(cudaMemcpyAsync(s->host_pose, s->h.pose, kPoseHeadBytes, cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  if (T_gc_out) std::memcpy(T_gc_out, s->host_pose->Tgc, 16 * sizeof(float));
  if (tracked) *tracked = s->host_pose->tracked;
  return VS_OK;
}

int vs_stage_filter(vs_session* s, const uint16_t* depth_mm_dev) {
  if (!s || !depth_mm_dev) return fail(VS_ERR_ARG, "null argument");
  const size_t n0 = (size_t)s->h.lv[0].W * s->h.lv[0].H;
  if (depth_mm_dev != s->h.depth_mm)
    VS_CU(cudaMemcpyAsync(s->h.depth_mm, depth_mm_dev, n0 * 2, cudaMemcpyDeviceToDevice, s->stream));
  launch_filter(s->tab, s->stream);
  if (s->h.cos_normal > -2.0f) launch_input_maps(s->tab, s->stream);
  VS_CU(cudaGetLastError());
  return VS_OK;
}
int vs_stage_track(vs_session* s) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  launch_icp(s->tab, s->h.levels, s->h.iters, s->h.reduce_mode, s->stream, true, nullptr);
  VS_CU(cudaGetLastError());
  return VS_OK;
}
int vs_stage_integrate(vs_session* s) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  launch_integrate(s->tab, s->h.tsdf_type, nullptr, nullptr, nullptr, true, s->stream, s->h.col != nullptr);
  VS_CU(cudaGetLastError());
  return VS_OK;
}
int vs_stage_raycast(vs_session* s) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  launch_raycast(s->tab, s->h.tsdf_type, -1, nullptr, nullptr, nullptr, 0.0f, 0.0f, -1.0f, true, nullptr, nullptr,
                 nullptr, nullptr, s->stream, LaunchShape(), nullptr, s->h.col != nullptr);
  VS_CU(cudaGetLastError());
  return VS_OK;
}

// ---- state access ----------------------------------------------------------

int vs_get_pose(vs_session* s, float* T_gc, double* T_gc_f64, int* info) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaMemcpyAsync(s->host_pose, s->h.pose, sizeof(Pose), cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  const Pose& p = *s->host_pose;
  if (T_gc) std::memcpy(T_gc, p.Tgc, sizeof(p.Tgc));
  if (T_gc_f64) std::memcpy(T_gc_f64, p.T_gc, sizeof(p.T_gc));
  if (info) {
    info[0] = p.tracked;
    info[1] = p.iters_run;
    info[2] = p.valid_count;
    info[3] = p.frame;
  }
  return VS_OK;
}

int vs_get_icp_system(vs_session* s, double* sums29, float* x6) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaMemcpyAsync(s->host_pose, s->h.pose, sizeof(Pose), cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  if (sums29) std::memcpy(sums29, s->host_pose->last_sums, sizeof(s->host_pose->last_sums));
  if (x6) std::memcpy(x6, s->host_pose->last_x, sizeof(s->host_pose->last_x));
  return VS_OK;
}

int vs_get_band(vs_session* s, uint8_t* band, uint8_t* dist) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  const size_t nbr = (size_t)s->h.nb[0] * s->h.nb[1] * s->h.nb[2];
  if (band) VS_CU(cudaMemcpyAsync(band, s->h.band, nbr, cudaMemcpyDeviceToHost, s->stream));
  if (dist) VS_CU(cudaMemcpyAsync(dist, s->h.bdist, nbr, cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  return VS_OK;
}

int vs_set_pose(vs_session* s, const double* T_gc_f64) {
  if (!s || !T_gc_f64) return fail(VS_ERR_ARG, "null argument");
  double* dT = nullptr;
  VS_CU(cudaMalloc(&dT, 16 * sizeof(double)));
  cudaError_t e = cudaMemcpy(dT, T_gc_f64, 16 * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    launch_pose_set(s->d, dT, s->stream);
    e = cudaStreamSynchronize(s->stream);
  }
  cudaFree(dT);
  if (e != cudaSuccess) return cuda_fail(e, "vs_set_pose");
  return VS_OK;
}

static int volume_transfer(vs_session* s, bool do_export, float* tsdf, uint16_t* w, const float* tsdf_in,
                           const uint16_t* w_in) {
  const int X = s->h.dim[0], Y = s->h.dim[1], Z = s->h.dim[2];
  const int slab = 64;
  const size_t plane = (size_t)X * Y;
  float* dt = nullptr;
  uint16_t* dw = nullptr;
  VS_CU(cudaMalloc(&dt, plane * slab * 4));
  cudaError_t e = cudaMalloc(&dw, plane * slab * 2);
  if (e != cudaSuccess) {
    cudaFree(dt);
    return cuda_fail(e, "cudaMalloc(volume staging)");
  }
  for (int z0 = 0; z0 < Z && e == cudaSuccess; z0 += slab) {
    int nz = (Z - z0 < slab) ? Z - z0 : slab;
    size_t n = plane * nz;
    if (do_export) {
      launch_volume_slab(s->h, true, z0, nz, tsdf ? dt : nullptr, w ? dw : nullptr, s->stream);
      if (tsdf) e = cudaMemcpyAsync(tsdf + plane * z0, dt, n * 4, cudaMemcpyDeviceToHost, s->stream);
      if (e == cudaSuccess && w) e = cudaMemcpyAsync(w + plane * z0, dw, n * 2, cudaMemcpyDeviceToHost, s->stream);
    } else {
      if (tsdf_in) e = cudaMemcpyAsync(dt, tsdf_in + plane * z0, n * 4, cudaMemcpyHostToDevice, s->stream);
      if (e == cudaSuccess && w_in) e = cudaMemcpyAsync(dw, w_in + plane * z0, n * 2, cudaMemcpyHostToDevice, s->stream);
      if (e == cudaSuccess)
        launch_volume_slab(s->h, false, z0, nz, tsdf_in ? dt : nullptr, w_in ? dw : nullptr, s->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  }
  if (e == cudaSuccess && !do_export) {
    launch_occupancy_rebuild(s->h, s->d, s->stream);
    e = cudaStreamSynchronize(s->stream);
  }
  cudaFree(dt);
  cudaFree(dw);
  if (e != cudaSuccess) return cuda_fail(e, "volume transfer");
  return VS_OK;
}

int vs_get_volume(vs_session* s, float* tsdf_host, uint16_t* weight_host) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaStreamSynchronize(s->stream));
  return volume_transfer(s, true, tsdf_host, weight_host, nullptr, nullptr);
}

int vs_set_volume(vs_session* s, const float* tsdf_host, const uint16_t* weight_host) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaStreamSynchronize(s->stream));
  return volume_transfer(s, false, nullptr, nullptr, tsdf_host, weight_host);
}

int vs_get_active_bricks(vs_session* s, uint32_t* count, uint32_t* bricks_host, uint32_t capacity) {
  if (!s || !count) return fail(VS_ERR_ARG, "null argument");
  uint32_t c = 0;
  VS_CU(cudaMemcpyAsync(&c, s->h.brick_count, 4, cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  *count = c;
  if (bricks_host && capacity) {
    uint32_t n = c < capacity ? c : capacity;
    VS_CU(cudaMemcpy(bricks_host, s->h.brick_list, (size_t)n * 4, cudaMemcpyDeviceToHost));
  }
  return VS_OK;
}

int vs_get_maps(vs_session* s, int level, float* mdepth, float* mvtx3, float* mnrm3, uint8_t* mimg,
                float* idepth, float* ivtx3, float* inrm3) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  if (level < 0 || level >= s->h.levels) return fail(VS_ERR_ARG, "bad level");
  const size_t n = (size_t)s->h.lv[level].W * s->h.lv[level].H;
  VS_CU(cudaStreamSynchronize(s->stream));
  if (mdepth) VS_CU(cudaMemcpy(mdepth, s->h.m_depth[level], n * 4, cudaMemcpyDeviceToHost));
  if (mimg) VS_CU(cudaMemcpy(mimg, s->h.m_img[level], n, cudaMemcpyDeviceToHost));
  if (idepth) VS_CU(cudaMemcpy(idepth, s->h.depth[level], n * 4, cudaMemcpyDeviceToHost));
  float* stage = nullptr;
  if (mvtx3 || mnrm3 || ivtx3 || inrm3) {
    VS_CU(cudaMalloc(&stage, n * 12 * 4));
    float* a = stage;
    float* b = stage + 3 * n;
    float* c = stage + 6 * n;
    float* d = stage + 9 * n;
    launch_maps_export(s->h, level, mvtx3 ? a : nullptr, mnrm3 ? b : nullptr, ivtx3 ? c : nullptr,
                       inrm3 ? d : nullptr, s->stream);
    cudaError_t e = cudaStreamSynchronize(s->stream);
    if (e == cudaSuccess && mvtx3) e = cudaMemcpy(mvtx3, a, n * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && mnrm3) e = cudaMemcpy(mnrm3, b, n * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && ivtx3) e = cudaMemcpy(ivtx3, c, n * 12, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && inrm3) e = cudaMemcpy(inrm3, d, n * 12, cudaMemcpyDeviceToHost);
    cudaFree(stage);
    if (e != cudaSuccess) return cuda_fail(e, "vs_get_maps");
  }
  return VS_OK;
}

int vs_set_stage_timing(vs_session* s, int enable) {
  if (!s) return fail(VS_ERR_ARG, "null session");
  VS_CU(cudaStreamSynchronize(s->stream));
  if (enable && !s->ev[0])
    for (auto& e : s->ev) VS_CU(cudaEventCreate(&e));
  if ((enable != 0) != s->timing) {
    s->timing = enable != 0;
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    s->exec = nullptr;
    s->graph = nullptr;
  }
  return VS_OK;
}

int vs_get_stage_times(vs_session* s, float* ms) {
  if (!s || !ms) return fail(VS_ERR_ARG, "null argument");
  if (!s->timing) return fail(VS_ERR_STATE, "stage timing is off");
  VS_CU(cudaEventSynchronize(s->ev[4]));
  for (int i = 0; i < 4; i++) VS_CU(cudaEventElapsedTime(ms + i, s->ev[i], s->ev[i + 1]));
  return VS_OK;
}

int vs_get_frame_stats(vs_session* s, uint32_t* stats) {
  if (!s || !stats) return fail(VS_ERR_ARG, "null argument");
  uint32_t c[2] = {0, 0};
  VS_CU(cudaMemcpyAsync(c, s->h.brick_count, sizeof(c), cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaMemcpyAsync(s->host_pose, s->h.pose, kPoseHeadBytes, cudaMemcpyDeviceToHost, s->stream));
  VS_CU(cudaStreamSynchronize(s->stream));
  stats[0] = c[0];
  stats[1] = c[1];
  stats[2] = (uint32_t)s->host_pose->iters_run;
  stats[3] = (uint32_t)s->host_pose->valid_count;
  return VS_OK;
}

int vs_kernels_per_frame(const vs_config* c) {
  if (check_config(c) != VS_OK) return -1;
  int n = 1 + (c->levels - 1);              // bilateral + pyramid levels
  if (c->cos_normal > -2.0f) n += 3;        // input maps: pre, row scan, post
  n += 2;                                   // ICP begin / finish
  for (int l = 0; l < c->levels; l++) n += c->icp_iters[l];
  n += 3;                                   // counter reset, activation, update
  n += 2;                                   // ray march + shading of every level
  return n;
}

int vs_get_input_raw(vs_session* s, float* depth_m_host) {
  if (!s || !depth_m_host) return fail(VS_ERR_ARG, "null argument");
  const size_t n = (size_t)s->h.lv[0].W * s->h.lv[0].H;
  VS_CU(cudaStreamSynchronize(s->stream));
  VS_CU(cudaMemcpy(depth_m_host, s->h.depth_raw, n * 4, cudaMemcpyDeviceToHost));
  return VS_OK;
}

int vs_get_device_buffer(vs_session* s, int which, void** ptr) {
  if (!s || !ptr) return fail(VS_ERR_ARG, "null argument");
  if (which == 0) {
    *ptr = s->h.depth_raw;
    return VS_OK;
  }
  if (which >= 1 && which <= s->h.levels) {
    *ptr = s->h.depth[which - 1];
    return VS_OK;
  }
  return fail(VS_ERR_ARG, "bad buffer id");
}

}  // extern "C"
