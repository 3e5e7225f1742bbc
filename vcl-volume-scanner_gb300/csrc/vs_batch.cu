// Batch runner (vs_batch_* in include/vs.h): several sessions advanced by one
// frame each, one launch per stage.
//
// The runner owns a device work table and captures the per-frame sequence
// once; the graph starts with a copy of the table from pinned host memory, so
// replaying it for another set of sessions only rewrites that host table.  Two
// pinned tables (and two graph instances, one reading each) alternate, so the
// host fills step k+1's table while step k runs; the host waits for step k-1
// before it reuses that step's buffers.  A step ends by gathering every
// slot's pose head into one buffer that a single copy brings to the host.
//
// The sessions are split into kIcpGroups groups (by pixel count), and each
// group's whole frame (filter, maps, ICP, integration, ray-cast) runs as its
// own launch sequence on a branch of the graph.  Every persistent launch ends
// with a tail in which a few blocks still run (for ICP: the blocks closing a
// session's iteration with a reduction and an FP64 solve; for the ray-cast:
// the last tiles); with several sequences in flight the other sequences'
// blocks fill the SMs that a tail leaves idle.  A session's work and sums do
// not depend on which sessions share its launches, so the split changes no
// result.  With stage timing on, the stages run one after another over the
// whole batch (ICP still on branches) so that each stage's time is its own.
//
// The graph depends only on the schedule it was captured for: the deepest
// pyramid and the largest ICP iteration count per level among the sessions,
// whether any session needs input normal maps, the reduction mode and the
// TSDF storage.  Sessions with fewer levels or iterations skip the extra
// launches on the device; a step that needs a longer schedule recaptures.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <cstring>
#include <string>

#include "vs.h"
#include "vs_host.h"
#include "vs_internal.cuh"

using namespace vs;

namespace {

struct Schedule {
  int levels = 0;
  int iters[kMaxLevels] = {0, 0, 0};
  int inmaps = 0;
  int reduce_mode = -1;
  int tsdf_type = -1;
  int timing = 0;
  int color = 0;  // some session keeps a colour volume
  bool covers(const Schedule& o) const {
    if (o.reduce_mode != reduce_mode || o.tsdf_type != tsdf_type || o.timing != timing) return false;
    if (o.levels > levels || (o.inmaps && !inmaps) || (o.color && !color)) return false;
    for (int l = 0; l < kMaxLevels; l++)
      if (o.iters[l] > iters[l]) return false;
    return true;
  }
};

constexpr int kRing = 2;
#ifndef VS_ICP_GROUPS
#define VS_ICP_GROUPS 2
#endif
constexpr int kIcpGroups = VS_ICP_GROUPS;  // concurrent per-frame launch sequences

}  // namespace

struct vs_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  BatchTable* d_tab = nullptr;
  BatchTable* d_grp = nullptr;                 // kIcpGroups tables: the ICP groups
  void* d_heads = nullptr;                     // kMaxSlots pose heads
  BatchTable* h_tab[kRing] = {nullptr, nullptr};  // pinned
  BatchTable* h_grp[kRing] = {nullptr, nullptr};  // pinned, kIcpGroups each
  cudaStream_t side[kIcpGroups] = {};         // graph branches of ICP groups 1..
  cudaEvent_t fork = nullptr, join[kIcpGroups] = {};
  unsigned char* h_heads[kRing] = {nullptr, nullptr};  // pinned
  cudaEvent_t done[kRing] = {nullptr, nullptr};
  bool used[kRing] = {false, false};
  cudaGraphExec_t exec[kRing] = {nullptr, nullptr};
  Schedule sched;
  LaunchShape shape;                           // ray-cast launch shape (autotuned)
  int ring = 0;
  int last = -1;                               // ring slot of the last step
  int kernels = 0;
  bool timing = false;
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

namespace {

void drop_graphs(vs_batch* b) {
  for (auto& e : b->exec)
    if (e) cudaGraphExecDestroy(e), e = nullptr;
}

// one group's per-frame chain on one stream
void record_chain(vs_batch* b, const BatchTable* t, cudaStream_t st) {
  const Schedule& k = b->sched;
  launch_filter(t, st, b->shape.bil_rows);
  if (k.inmaps) launch_input_maps(t, st);
  launch_icp(t, k.levels, k.iters, k.reduce_mode, st, true, nullptr);
  launch_integrate(t, k.tsdf_type, nullptr, nullptr, nullptr, true, st, k.color != 0, b->shape.integrate_blocks_per_sm);
  launch_raycast(t, k.tsdf_type, -1, nullptr, nullptr, nullptr, 0.0f, 0.0f, -1.0f, true, nullptr, nullptr, nullptr,
                 nullptr, st, b->shape, nullptr, k.color != 0);
}

void record_step(vs_batch* b, int r, cudaStream_t st) {
  const Schedule& k = b->sched;
  auto mark = [&](int i) {
    if (k.timing) cudaEventRecordWithFlags(b->ev[i], st, cudaEventRecordExternal);
  };
  cudaMemcpyAsync(b->d_tab, b->h_tab[r], sizeof(BatchTable), cudaMemcpyHostToDevice, st);
  cudaMemcpyAsync(b->d_grp, b->h_grp[r], kIcpGroups * sizeof(BatchTable), cudaMemcpyHostToDevice, st);
  if (!k.timing) {
    // every group's whole frame on its own branch
    cudaEventRecord(b->fork, st);
    for (int g = 1; g < kIcpGroups; g++) cudaStreamWaitEvent(b->side[g], b->fork, 0);
    record_chain(b, b->d_grp, st);
    for (int g = 1; g < kIcpGroups; g++) {
      record_chain(b, b->d_grp + g, b->side[g]);
      cudaEventRecord(b->join[g], b->side[g]);
      cudaStreamWaitEvent(st, b->join[g], 0);
    }
  } else {
    // stage timing: the stages one after another (ICP still on branches), so
    // that each stage's time is its own
    mark(0);
    launch_filter(b->d_tab, st, b->shape.bil_rows);
    if (k.inmaps) launch_input_maps(b->d_tab, st);
    mark(1);
    cudaEventRecord(b->fork, st);
    for (int g = 1; g < kIcpGroups; g++) cudaStreamWaitEvent(b->side[g], b->fork, 0);
    launch_icp(b->d_grp, k.levels, k.iters, k.reduce_mode, st, true, nullptr);
    for (int g = 1; g < kIcpGroups; g++) {
      launch_icp(b->d_grp + g, k.levels, k.iters, k.reduce_mode, b->side[g], true, nullptr);
      cudaEventRecord(b->join[g], b->side[g]);
      cudaStreamWaitEvent(st, b->join[g], 0);
    }
    mark(2);
    launch_integrate(b->d_tab, k.tsdf_type, nullptr, nullptr, nullptr, true, st, k.color != 0,
                     b->shape.integrate_blocks_per_sm);
    mark(3);
    launch_raycast(b->d_tab, k.tsdf_type, -1, nullptr, nullptr, nullptr, 0.0f, 0.0f, -1.0f, true, nullptr, nullptr,
                   nullptr, nullptr, st, b->shape, nullptr, k.color != 0);
    mark(4);
  }
  launch_gather_heads(b->d_tab, b->d_heads, st);
  cudaMemcpyAsync(b->h_heads[r], b->d_heads, kMaxSlots * kPoseHeadBytes, cudaMemcpyDeviceToHost, st);
}

int build_graphs(vs_batch* b) {
  drop_graphs(b);
  for (int r = 0; r < kRing; r++) {
    cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail_code(e, "cudaStreamBeginCapture");
    record_step(b, r, b->stream);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return cuda_fail_code(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&b->exec[r], g, 0);
    size_t nn = 0;
    if (e == cudaSuccess && r == 0) {
      // kernels per step, for vs_batch_kernels_per_step
      cudaGraphGetNodes(g, nullptr, &nn);
      std::vector<cudaGraphNode_t> nodes(nn);
      cudaGraphGetNodes(g, nodes.data(), &nn);
      int kc = 0;
      for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) kc++;
      }
      b->kernels = kc;
    }
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail_code(e, "cudaGraphInstantiate");
  }
  return VS_OK;
}

int check_sessions(vs_batch* b, vs_session* const* ss, int n, Schedule& k) {
  if (n < 1 || n > kMaxSlots) return fail_code(VS_ERR_ARG, "batch size must be 1.." + std::to_string(kMaxSlots));
  for (int i = 0; i < n; i++) {
    const vs_session* s = ss[i];
    if (!s) return fail_code(VS_ERR_ARG, "null session in batch");
    if (s->device != b->device) return fail_code(VS_ERR_ARG, "sessions of a batch must share the runner's device");
    for (int j = 0; j < i; j++)
      if (ss[j] == s) return fail_code(VS_ERR_ARG, "a session appears twice in one batch");
    const SessionDev& h = s->h;
    if (i == 0) {
      k.reduce_mode = h.reduce_mode;
      k.tsdf_type = h.tsdf_type;
    } else if (h.reduce_mode != k.reduce_mode || h.tsdf_type != k.tsdf_type) {
      return fail_code(VS_ERR_ARG, "sessions of a batch must share reduce_mode and tsdf_type");
    }
    if (h.levels > k.levels) k.levels = h.levels;
    for (int l = 0; l < h.levels; l++)
      if (h.iters[l] > k.iters[l]) k.iters[l] = h.iters[l];
    if (h.cos_normal > -2.0f) k.inmaps = 1;
    if (h.col) k.color = 1;
  }
  k.timing = b->timing ? 1 : 0;
  return VS_OK;
}

// fills the next ring slot's table and launches.  frames (may be NULL): per
// session the frame its ingest reads in place (device memory or device-
// addressable pinned host memory; a NULL entry: the session's own buffer)
int launch_step(vs_batch* b, vs_session* const* ss, int n, const Schedule& k, cudaStream_t st, int r,
                const uint16_t* const* frames = nullptr) {
  if (!b->exec[0] || !b->sched.covers(k)) {
    Schedule m = k;
    if (b->exec[0] && b->sched.reduce_mode == k.reduce_mode && b->sched.tsdf_type == k.tsdf_type &&
        b->sched.timing == k.timing) {
      m.levels = std::max(m.levels, b->sched.levels);
      m.inmaps |= b->sched.inmaps;
      m.color |= b->sched.color;
      for (int l = 0; l < kMaxLevels; l++) m.iters[l] = std::max(m.iters[l], b->sched.iters[l]);
    }
    // the graphs read both ring buffers: let in-flight steps finish first
    cudaError_t e = cudaStreamSynchronize(b->stream);
    if (e == cudaSuccess && st != b->stream) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail_code(e, "batch schedule change");
    b->sched = m;
    int rc = build_graphs(b);
    if (rc) return rc;
  }
  const SessionDev* hr[kMaxSlots];
  const SessionDev* dr[kMaxSlots];
  for (int i = 0; i < n; i++) {
    hr[i] = &ss[i]->h;
    dr[i] = ss[i]->d;
  }
  fill_batch_table(*b->h_tab[r], hr, dr, n, b->shape.ray_lx, b->shape.bil_rows);
  for (int i = 0; i < n; i++) b->h_tab[r]->frame[i] = frames ? frames[i] : nullptr;
  // ICP groups: largest sessions first, each to the group with fewer pixels
  int order[kMaxSlots];
  for (int i = 0; i < n; i++) order[i] = i;
  auto px = [&](int i) { return (long long)hr[i]->lv[0].W * hr[i]->lv[0].H; };
  std::stable_sort(order, order + n, [&](int a, int c) { return px(a) > px(c); });
  const SessionDev* gh[kIcpGroups][kMaxSlots];
  const SessionDev* gd[kIcpGroups][kMaxSlots];
  const uint16_t* gf[kIcpGroups][kMaxSlots];
  int gn[kIcpGroups] = {0};
  long long load[kIcpGroups] = {0};
  for (int q = 0; q < n; q++) {
    const int i = order[q];
    int g = 0;
    for (int j = 1; j < kIcpGroups; j++)
      if (load[j] < load[g]) g = j;
    gh[g][gn[g]] = hr[i];
    gd[g][gn[g]] = dr[i];
    gf[g][gn[g]] = frames ? frames[i] : nullptr;
    gn[g]++;
    load[g] += px(i);
  }
  for (int g = 0; g < kIcpGroups; g++) {
    fill_batch_table(b->h_grp[r][g], gh[g], gd[g], gn[g], b->shape.ray_lx, b->shape.bil_rows);
    for (int j = 0; j < gn[g]; j++) b->h_grp[r][g].frame[j] = gf[g][j];
  }
  cudaError_t e = cudaGraphLaunch(b->exec[r], st);
  if (e == cudaSuccess) e = cudaEventRecord(b->done[r], st);
  if (e != cudaSuccess) return cuda_fail_code(e, "batch step launch");
  b->used[r] = true;
  b->last = r;
  b->ring = (r + 1) % kRing;
  return VS_OK;
}

// waits until the ring slot's previous step no longer needs its host buffers
int claim_slot(vs_batch* b, int& r) {
  r = b->ring;
  if (b->used[r]) {
    cudaError_t e = cudaEventSynchronize(b->done[r]);
    if (e != cudaSuccess) return cuda_fail_code(e, "batch ring wait");
  }
  return VS_OK;
}

void free_batch(vs_batch* b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  drop_graphs(b);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e), e = nullptr;
  for (int r = 0; r < kRing; r++) {
    if (b->done[r]) cudaEventDestroy(b->done[r]);
    if (b->h_tab[r]) cudaFreeHost(b->h_tab[r]);
    if (b->h_grp[r]) cudaFreeHost(b->h_grp[r]);
    if (b->h_heads[r]) cudaFreeHost(b->h_heads[r]);
  }
  if (b->d_tab) cudaFree(b->d_tab);
  if (b->d_grp) cudaFree(b->d_grp);
  if (b->fork) cudaEventDestroy(b->fork);
  for (int g = 1; g < kIcpGroups; g++) {
    if (b->join[g]) cudaEventDestroy(b->join[g]);
    if (b->side[g]) cudaStreamDestroy(b->side[g]);
  }
  if (b->d_heads) cudaFree(b->d_heads);
  if (b->stream) cudaStreamDestroy(b->stream);
}

}  // namespace

namespace vs {

// host frames -> one step, without waiting; the ring slot tells the caller
// where the step's pose heads land and which event marks its end
int batch_launch_host(vs_batch* b, vs_session* const* ss, int n, const uint16_t* const* frames_host, int* ring) {
  Schedule k;
  int rc = check_sessions(b, ss, n, k);
  if (rc) return rc;
  int r = 0;
  rc = claim_slot(b, r);
  if (rc) return rc;
  for (int i = 0; i < n; i++) {
    const SessionDev& h = ss[i]->h;
    cudaError_t e = cudaMemcpyAsync(h.depth_mm, frames_host[i], (size_t)h.lv[0].W * h.lv[0].H * 2,
                                    cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return cuda_fail_code(e, "batch frame upload");
  }
  rc = launch_step(b, ss, n, k, b->stream, r);
  if (rc) return rc;
  *ring = r;
  return VS_OK;
}

const unsigned char* batch_heads(const vs_batch* b, int r) { return b->h_heads[r]; }
cudaEvent_t batch_done(const vs_batch* b, int r) { return b->done[r]; }

}  // namespace vs

extern "C" {

int vs_batch_create(vs_batch** out) {
  if (!out) return fail_code(VS_ERR_ARG, "null output");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail_code(VS_ERR_CUDA, "no CUDA device available");
  vs_batch* b = new vs_batch;
  cudaGetDevice(&b->device);
  cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  for (int g = 1; g < kIcpGroups && e == cudaSuccess; g++) {
    e = cudaStreamCreateWithFlags(&b->side[g], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join[g], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaMalloc(&b->d_tab, sizeof(BatchTable));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_grp, kIcpGroups * sizeof(BatchTable));
  if (e == cudaSuccess) e = cudaMemset(b->d_grp, 0, kIcpGroups * sizeof(BatchTable));
  if (e == cudaSuccess) e = cudaMalloc(&b->d_heads, kMaxSlots * kPoseHeadBytes);
  for (int r = 0; r < kRing && e == cudaSuccess; r++) {
    e = cudaMallocHost(&b->h_tab[r], sizeof(BatchTable));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_heads[r], kMaxSlots * kPoseHeadBytes);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_grp[r], kIcpGroups * sizeof(BatchTable));
    if (e == cudaSuccess) std::memset(b->h_grp[r], 0, kIcpGroups * sizeof(BatchTable));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done[r], cudaEventDisableTiming);
    if (e == cudaSuccess) std::memset(b->h_tab[r], 0, sizeof(BatchTable));
  }
  if (e != cudaSuccess) {
    free_batch(b);
    delete b;
    return cuda_fail_code(e, "vs_batch_create");
  }
  *out = b;
  return VS_OK;
}

int vs_batch_destroy(vs_batch* b) {
  if (!b) return VS_OK;
  free_batch(b);
  delete b;
  return VS_OK;
}

int vs_batch_step(vs_batch* b, vs_session* const* sessions, int n, const uint16_t* const* depth_mm_dev,
                  void* stream) {
  if (!b || !sessions) return fail_code(VS_ERR_ARG, "null argument");
  Schedule k;
  int rc = check_sessions(b, sessions, n, k);
  if (rc) return rc;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : b->stream;
  int r = 0;
  rc = claim_slot(b, r);
  if (rc) return rc;
  // the ingest reads each device frame in place: no copy into the session
  return launch_step(b, sessions, n, k, st, r, depth_mm_dev);
}

int vs_batch_step_host(vs_batch* b, vs_session* const* sessions, int n, const uint16_t* const* depth_mm_host,
                       float* T_gc_out, int* tracked_out) {
  if (!b || !sessions || !depth_mm_host) return fail_code(VS_ERR_ARG, "null argument");
  Schedule k;
  int rc = check_sessions(b, sessions, n, k);
  if (rc) return rc;
  int r = 0;
  rc = claim_slot(b, r);
  if (rc) return rc;
  // pinned host frames are read in place by the ingest (the step reads them
  // over the host link while it runs, and this call returns only after the
  // step); pageable ones are copied into the session first
  const uint16_t* direct[kMaxSlots];
  for (int i = 0; i < n; i++) {
    if (!depth_mm_host[i]) return fail_code(VS_ERR_ARG, "null host frame");
    direct[i] = nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, depth_mm_host[i]) == cudaSuccess && a.type == cudaMemoryTypeHost &&
        a.devicePointer) {
      direct[i] = static_cast<const uint16_t*>(a.devicePointer);
      continue;
    }
    cudaGetLastError();  // a pageable pointer may leave an error behind
    const SessionDev& h = sessions[i]->h;
    cudaError_t e = cudaMemcpyAsync(h.depth_mm, depth_mm_host[i], (size_t)h.lv[0].W * h.lv[0].H * 2,
                                    cudaMemcpyHostToDevice, b->stream);
    if (e != cudaSuccess) return cuda_fail_code(e, "batch frame upload");
  }
  rc = launch_step(b, sessions, n, k, b->stream, r, direct);
  if (rc) return rc;
  cudaError_t e = cudaEventSynchronize(b->done[r]);
  if (e != cudaSuccess) return cuda_fail_code(e, "batch step");
  for (int i = 0; i < n; i++) {
    const Pose* p = reinterpret_cast<const Pose*>(b->h_heads[r] + (size_t)i * kPoseHeadBytes);
    if (T_gc_out) std::memcpy(T_gc_out + 16 * i, p->Tgc, 16 * sizeof(float));
    if (tracked_out) tracked_out[i] = p->tracked;
  }
  return VS_OK;
}

int vs_batch_sync(vs_batch* b) {
  if (!b) return fail_code(VS_ERR_ARG, "null batch");
  for (int r = 0; r < kRing; r++)
    if (b->used[r]) {
      cudaError_t e = cudaEventSynchronize(b->done[r]);
      if (e != cudaSuccess) return cuda_fail_code(e, "vs_batch_sync");
    }
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return cuda_fail_code(e, "vs_batch_sync");
  return VS_OK;
}

int vs_batch_set_stage_timing(vs_batch* b, int enable) {
  if (!b) return fail_code(VS_ERR_ARG, "null batch");
  int rc = vs_batch_sync(b);
  if (rc) return rc;
  if (enable && !b->ev[0])
    for (auto& e : b->ev) {
      cudaError_t c = cudaEventCreate(&e);
      if (c != cudaSuccess) return cuda_fail_code(c, "cudaEventCreate");
    }
  b->timing = enable != 0;
  return VS_OK;
}

int vs_batch_get_stage_times(vs_batch* b, float* ms) {
  if (!b || !ms) return fail_code(VS_ERR_ARG, "null argument");
  if (!b->timing || !b->sched.timing || b->last < 0) return fail_code(VS_ERR_STATE, "stage timing is off or no step ran");
  cudaError_t e = cudaEventSynchronize(b->ev[4]);
  for (int i = 0; i < 4 && e == cudaSuccess; i++) e = cudaEventElapsedTime(ms + i, b->ev[i], b->ev[i + 1]);
  if (e != cudaSuccess) return cuda_fail_code(e, "vs_batch_get_stage_times");
  return VS_OK;
}

int vs_batch_kernels_per_step(vs_batch* b) {
  if (!b) return -1;
  return b->exec[0] ? b->kernels : -1;
}

int vs_batch_get_launch_shape(vs_batch* b, vs_launch_shape* out) {
  if (!b || !out) return fail_code(VS_ERR_ARG, "null argument");
  out->ray_tile_log2 = b->shape.ray_lx;
  out->march_blocks_per_sm = b->shape.march_blocks_per_sm;
  out->shade_blocks_per_sm = b->shape.shade_blocks_per_sm;
  out->bilateral_rows = b->shape.bil_rows;
  out->integrate_blocks_per_sm = b->shape.integrate_blocks_per_sm;
  return VS_OK;
}

int vs_batch_set_launch_shape(vs_batch* b, const vs_launch_shape* in) {
  if (!b || !in) return fail_code(VS_ERR_ARG, "null argument");
  if (in->ray_tile_log2 < 0 || in->ray_tile_log2 > 5 || in->march_blocks_per_sm < 0 || in->shade_blocks_per_sm < 0 ||
      in->march_blocks_per_sm > 32 || in->shade_blocks_per_sm > 32 || in->integrate_blocks_per_sm < 0 ||
      in->integrate_blocks_per_sm > 32 ||
      (in->bilateral_rows != 0 && in->bilateral_rows != 4 && in->bilateral_rows != 8 && in->bilateral_rows != 16))
    return fail_code(VS_ERR_ARG, "launch shape out of range");
  int rc = vs_batch_sync(b);
  if (rc) return rc;
  b->shape.ray_lx = in->ray_tile_log2;
  b->shape.march_blocks_per_sm = in->march_blocks_per_sm;
  b->shape.shade_blocks_per_sm = in->shade_blocks_per_sm;
  b->shape.bil_rows = in->bilateral_rows ? in->bilateral_rows : 8;
  b->shape.integrate_blocks_per_sm = in->integrate_blocks_per_sm;
  drop_graphs(b);  // recaptured with the new grids at the next step
  return VS_OK;
}

// Times three stages of these sessions under their candidate launch shapes
// and keeps the fastest of each: the ray-cast (ray tile, march and shading
// grids), the filter (rows of the bilateral / activation tile) and the
// integration (update grid).  None of the shapes changes a result, and none
// of the timing runs changes a session's state: the ray-cast and the filter
// rewrite their outputs with the values the last step gave them, and the
// integration runs as a dry run (every voxel computed, none stored; its
// activation lists the same sub-cubes again).
namespace {

int time_launches(cudaStream_t st, int reps, cudaEvent_t e0, cudaEvent_t e1, const std::function<void()>& f,
                  float* ms) {
  cudaError_t e = cudaSuccess;
  for (int r = 0; r <= reps && e == cudaSuccess; r++) {
    if (r == 1) e = cudaEventRecord(e0, st);
    f();
    if (e == cudaSuccess) e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(e1, st);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, e0, e1);
  *ms /= (float)reps;
  return e == cudaSuccess ? VS_OK : cuda_fail_code(e, "vs_batch_autotune");
}

}  // namespace

int vs_batch_autotune(vs_batch* b, vs_session* const* sessions, int n, int reps, vs_launch_shape* best,
                      float* best_ms) {
  if (!b || !sessions) return fail_code(VS_ERR_ARG, "null argument");
  Schedule k;
  int rc = check_sessions(b, sessions, n, k);
  if (rc) return rc;
  if (reps < 1) reps = 3;
  rc = vs_batch_sync(b);
  if (rc) return rc;
  const SessionDev* hr[kMaxSlots];
  const SessionDev* dr[kMaxSlots];
  for (int i = 0; i < n; i++) {
    hr[i] = &sessions[i]->h;
    dr[i] = sessions[i]->d;
  }
  const int most_m = ray_max_blocks_per_sm(k.tsdf_type, false), most_s = ray_max_blocks_per_sm(k.tsdf_type, true);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e != cudaSuccess) return cuda_fail_code(e, "vs_batch_autotune");
  LaunchShape win = b->shape;
  float win_ms = 1e30f;
  BatchTable* t = b->h_tab[0];
  auto upload = [&](int lx, int rows) {
    fill_batch_table(*t, hr, dr, n, lx, rows);
    return cudaMemcpyAsync(b->d_tab, t, sizeof(BatchTable), cudaMemcpyHostToDevice, b->stream);
  };
  // ray-cast: ray tile and march grid
  for (int lx = 1; lx <= 5 && rc == VS_OK; lx++) {
    if (upload(lx, win.bil_rows) != cudaSuccess) rc = cuda_fail_code(cudaGetLastError(), "vs_batch_autotune");
    const int mcands[3] = {most_m, (most_m * 3) / 4, most_m / 2};
    for (int c = 0; c < 3 && rc == VS_OK; c++) {
      if (mcands[c] < 1 || (c > 0 && mcands[c] == mcands[c - 1])) continue;
      LaunchShape sh = win;
      sh.ray_lx = lx;
      sh.march_blocks_per_sm = mcands[c];
      sh.shade_blocks_per_sm = most_s;
      float ms = 0.0f;
      rc = time_launches(b->stream, reps, e0, e1, [&] {
        launch_raycast(b->d_tab, k.tsdf_type, -1, nullptr, nullptr, nullptr, 0.0f, 0.0f, -1.0f, true, nullptr,
                       nullptr, nullptr, nullptr, b->stream, sh, nullptr, k.color != 0);
      }, &ms);
      if (rc == VS_OK && ms < win_ms) {
        win_ms = ms;
        win = sh;
      }
    }
  }
  // filter and integration: the first candidate is the default shape, and
  // another replaces it only when it is more than 3 % faster (the stages run
  // in well under a millisecond on the tuning sessions, where a closer call
  // is timing noise)
  constexpr float kMargin = 0.97f;
  // filter: rows of the bilateral (and activation) tile
  float fil_ms = 1e30f;
  const int rows_c[3] = {8, 4, 16};
  for (int c = 0; c < 3 && rc == VS_OK; c++) {
    if (upload(win.ray_lx, rows_c[c]) != cudaSuccess) rc = cuda_fail_code(cudaGetLastError(), "vs_batch_autotune");
    float ms = 0.0f;
    if (rc == VS_OK) rc = time_launches(b->stream, reps, e0, e1, [&] { launch_filter(b->d_tab, b->stream, rows_c[c]); }, &ms);
    if (rc == VS_OK && ms < (c == 0 ? 1e30f : kMargin * fil_ms)) {
      fil_ms = ms;
      win.bil_rows = rows_c[c];
    }
  }
  // integration: update grid, as dry runs
  if (rc == VS_OK && upload(win.ray_lx, win.bil_rows) != cudaSuccess)
    rc = cuda_fail_code(cudaGetLastError(), "vs_batch_autotune");
  float int_ms = 1e30f;
  const int ib_c[3] = {0, 3, 2};
  for (int c = 0; c < 3 && rc == VS_OK; c++) {
    float ms = 0.0f;
    rc = time_launches(b->stream, reps, e0, e1, [&] {
      launch_integrate(b->d_tab, k.tsdf_type, nullptr, nullptr, nullptr, true, b->stream, k.color != 0, ib_c[c], true);
    }, &ms);
    if (rc == VS_OK && ms < (c == 0 ? 1e30f : kMargin * int_ms)) {
      int_ms = ms;
      win.integrate_blocks_per_sm = ib_c[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  b->shape = win;
  drop_graphs(b);
  if (best) {
    best->ray_tile_log2 = win.ray_lx;
    best->march_blocks_per_sm = win.march_blocks_per_sm;
    best->shade_blocks_per_sm = win.shade_blocks_per_sm;
    best->bilateral_rows = win.bil_rows;
    best->integrate_blocks_per_sm = win.integrate_blocks_per_sm;
  }
  if (best_ms) *best_ms = win_ms;
  return VS_OK;
}

}  // extern "C"
