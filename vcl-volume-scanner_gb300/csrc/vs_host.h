// Host-side definitions shared by the C ABI translation units: the session
// object and the error helpers behind vs_last_error().
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "vs.h"
#include "vs_internal.cuh"

struct vs_session {
  vs_config cfg;
  vs::SessionDev h;          // host copy of the device record
  vs::SessionDev* d = nullptr;
  vs::BatchTable* tab = nullptr;     // the session alone: a one-slot table (device)
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void*> allocs;
  float* stage_f = nullptr;      // level-0 float staging (bfd input)
  float* dev_small = nullptr;    // 16 floats of scratch: [0..2] camera centre, [4] carve counter
  vs::Pose* host_pose = nullptr;     // pinned
  int device = 0;
  bool timing = false;           // stage events recorded inside the graph
  cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
};

namespace vs {
void set_error(const char* msg);  // read back through vs_last_error()
// records msg (or the CUDA error) and returns the code
int fail_code(int code, const std::string& msg);
int cuda_fail_code(cudaError_t e, const char* what);
// batch runner internals used by the server
int batch_launch_host(vs_batch* b, vs_session* const* ss, int n, const uint16_t* const* frames_host, int* ring);
const unsigned char* batch_heads(const vs_batch* b, int r);
cudaEvent_t batch_done(const vs_batch* b, int r);
}  // namespace vs
