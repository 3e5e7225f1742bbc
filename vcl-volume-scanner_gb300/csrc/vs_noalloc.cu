// vs_integrate_depth_noalloc: TSDF integration into a caller-owned volume
// without any device allocation by this library.
//
// Some callers cannot call cudaMalloc: code that runs inside a host
// framework's own memory pool or arena (the pool owns every device byte, so a
// stray cudaMalloc breaks its accounting or is forbidden outright), real-time
// loops where an allocation can stall on the driver's lock at an unbounded
// cost, and processes that pre-size every buffer at start-up under a fixed
// memory budget.  vs_session_create allocates the volume and its scratch, so
// those callers get this entry point instead: they own the volume buffer and
// pass it in, and the only other device memory used is the fixed scratch
// array below.
//
// Scratch: g_noalloc_scratch is a file-scope __device__ array of
// kNoAllocScratchBytes (about 2 MiB), which every GPU that loads the library
// holds until the process exits.  It carries the kernel descriptor and its
// one-slot work table, the voxel-centre and ray tables, the per-sub-cube
// activation flags, the list of active sub-cubes and the counters, for
// volumes of up to kNoAllocMaxBricks 8^3 sub-cubes (512^3 voxels); larger
// volumes are rejected with VS_ERR_ARG.  In host code the
// array's name is only a host-side stand-in, never a device address: its
// address is obtained once per device with cudaGetSymbolAddress, on the first
// call made with that device current, and that first call should therefore
// come before any stream capture.  Every call shares the array and it keeps
// the last call's contents, so each call clears the flags and counters it
// needs zeroed; calls on one stream run in order, calls that overlap on the
// GPU (different streams, or different host threads) race on the scratch.
//
// The kernels are the session path's own activation and update kernels
// (k_integrate.cu), handed a descriptor that lives in the scratch array.  The
// descriptor and the work table reach the scratch as kernel arguments (one
// set-up kernel copies them and clears the flags), so no host buffer is read
// after the call returns.  The set-up of the per-call tables also rewrites
// the library's shared table of 1/w (w = 1..65535) with the same values
// every call; session integrations running meanwhile read identical numbers.
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "vs.h"
#include "vs_internal.cuh"

namespace vs {
int integrate_max_dim();
int integrate_max_image();
void set_error(const char* msg);  // read back through vs_last_error()
}  // namespace vs

using namespace vs;

namespace {

constexpr size_t kNoAllocMaxBricks = 262144;  // 512^3 voxels in 8^3 sub-cubes
constexpr size_t kDescBytes = 2048;           // SessionDev record, padded
constexpr size_t kTableBytes = 8192;          // one-slot BatchTable, padded
constexpr size_t kLutBytes = (3 * 1024 + 2 * 2048) * sizeof(float);  // voxel-centre and ray tables
constexpr size_t kCounterBytes = 256;
constexpr size_t kHeadBytes = kDescBytes + kTableBytes + kLutBytes + kCounterBytes;
constexpr size_t kNoAllocScratchBytes = kHeadBytes + 2 * kNoAllocMaxBricks * sizeof(uint32_t);
static_assert(sizeof(SessionDev) <= kDescBytes, "descriptor does not fit its scratch slot");
static_assert(sizeof(BatchTable) <= kTableBytes, "work table does not fit its scratch slot");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static_assert(sizeof(SessionDev) + sizeof(BatchTable) + 64 <= 32764, "set-up arguments exceed the parameter space");

// copies the call's descriptor and work table into the scratch and clears
// the activation flags of the volume's sub-cubes
__global__ void k_noalloc_setup(const SessionDev h, const BatchTable t, SessionDev* d, BatchTable* dt,
                                uint32_t* flags, uint32_t nbr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr uint32_t kHw = sizeof(SessionDev) / 4, kTw = sizeof(BatchTable) / 4;
  static_assert(sizeof(SessionDev) % 4 == 0 && sizeof(BatchTable) % 4 == 0, "word copies");
  if (i < kHw) reinterpret_cast<uint32_t*>(d)[i] = reinterpret_cast<const uint32_t*>(&h)[i];
  if (i < kTw) reinterpret_cast<uint32_t*>(dt)[i] = reinterpret_cast<const uint32_t*>(&t)[i];
  for (uint32_t k = i; k < nbr; k += gridDim.x * blockDim.x) flags[k] = 0u;
}

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

int fail(int code, const std::string& m) {
  set_error(m.c_str());
  return code;
}

// once per device, with that device current
int scratch_address(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(VS_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(VS_ERR_CUDA, "device index out of range");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(VS_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return VS_OK;
}

}  // namespace

extern "C" int vs_integrate_depth_noalloc(uint32_t* volume_dev, const int* dim, const float* origin,
                                          float voxel_size, float mu, float max_w, const float* map_depth_dev,
                                          int ww, int hh, const float* K, const float* T_gc_dev,
                                          const float* T_cg_dev, void* stream) {
  if (!volume_dev || !dim || !origin || !map_depth_dev || !K || !T_gc_dev || !T_cg_dev)
    return fail(VS_ERR_ARG, "null argument");
  if (reinterpret_cast<uintptr_t>(volume_dev) % 16)
    return fail(VS_ERR_ARG, "volume_dev must be 16-byte aligned (sub-cubes are read and written as 16-byte vectors)");
  for (int k = 0; k < 3; k++)
    if (dim[k] < 8 || dim[k] % 8 || dim[k] > integrate_max_dim())
      return fail(VS_ERR_ARG, "volume dims must be multiples of 8 in 8..1024");
  const size_t nbr = (size_t)(dim[0] / 8) * (dim[1] / 8) * (dim[2] / 8);
  if (nbr > kNoAllocMaxBricks)
    return fail(VS_ERR_ARG, "volume has " + std::to_string(nbr) + " sub-cubes; the allocation-free path holds at most " +
                                std::to_string(kNoAllocMaxBricks) + " (512^3 voxels)");
  if (ww < 8 || hh < 8 || ww > integrate_max_image() || hh > integrate_max_image())
    return fail(VS_ERR_ARG, "image size out of range (8..2048)");
  if (!(voxel_size > 0) || !(mu > 0) || !(max_w >= 1) || max_w > 65535.0f || K[0] == 0 || K[1] == 0)
    return fail(VS_ERR_ARG, "voxel_size, mu, max_w or focal length out of range");
  void* base = nullptr;
  int rc = scratch_address(&base);
  if (rc) return rc;
  unsigned char* sb = static_cast<unsigned char*>(base);
  SessionDev h;
  std::memset(&h, 0, sizeof(h));
  h.levels = 1;
  h.lv[0].W = ww;
  h.lv[0].H = hh;
  for (int k = 0; k < 4; k++) h.lv[0].K[k] = K[k];
  for (int k = 0; k < 3; k++) {
    h.dim[k] = dim[k];
    h.nb[k] = dim[k] / 8;
    h.origin[k] = origin[k];
  }
  h.vox = voxel_size;
  h.vox_inv = 1.0f / voxel_size;
  h.mu = mu;
  h.max_w = max_w;
  h.tsdf_type = VS_TSDF_INT16;
  h.vol = volume_dev;
  h.lut_vox = reinterpret_cast<float*>(sb + kDescBytes + kTableBytes);
  h.lut_ray = h.lut_vox + 3 * 1024;
  h.brick_count = reinterpret_cast<uint32_t*>(sb + kDescBytes + kTableBytes + kLutBytes);
  h.brick_flag = reinterpret_cast<uint32_t*>(sb + kHeadBytes);
  h.brick_list = h.brick_flag + kNoAllocMaxBricks;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  SessionDev* d = reinterpret_cast<SessionDev*>(sb);
  BatchTable* dt = reinterpret_cast<BatchTable*>(sb + kDescBytes);
  BatchTable t;
  const SessionDev* hr = &h;
  const SessionDev* dr = d;
  fill_batch_table(t, &hr, &dr, 1);
  k_noalloc_setup<<<512, 256, 0, st>>>(h, t, d, dt, h.brick_flag, (uint32_t)nbr);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VS_ERR_CUDA, std::string("scratch set-up: ") + cudaGetErrorString(e));
  launch_session_tables(h, d, st);
  // counters are cleared inside launch_integrate
  launch_integrate(dt, VS_TSDF_INT16, map_depth_dev, T_gc_dev, T_cg_dev, false, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(VS_ERR_CUDA, std::string("integrate launch: ") + cudaGetErrorString(e));
  return VS_OK;
}
