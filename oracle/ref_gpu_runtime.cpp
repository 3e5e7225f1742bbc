// Host definitions behind ref_shim/gpu/ref_gpu_shim.h: the launch variables
// and the runtime calls on host memory (TEST INFRASTRUCTURE ONLY).
#include <set>

#include "ref_gpu_shim.h"

uint3_ threadIdx, blockIdx;
dim3 blockDim, gridDim;

// The reference's GKvVolume / GKvMatrix release() frees without clearing its
// pointer and runs again from the destructor; on a GPU the second cudaFree
// only returns an error.  Freeing here is likewise idempotent: only live
// allocations are freed.
static std::set<void*> g_live;
cudaError_t cudaMalloc(void** p, size_t n) {
  *p = std::calloc(n ? n : 1, 1);
  if (!*p) return 2;
  g_live.insert(*p);
  return 0;
}
cudaError_t cudaFree(void* p) {
  if (g_live.erase(p)) std::free(p);
  return 0;
}
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind) {
  if (n) std::memmove(d, s, n);
  return 0;
}
cudaError_t cudaMallocPitch(void** p, size_t* pitch, size_t wbytes, size_t h) {
  *pitch = wbytes;
  return cudaMalloc(p, wbytes * h);
}
cudaError_t cudaMemcpy2D(void* d, size_t dpitch, const void* s, size_t spitch, size_t wbytes, size_t h,
                         cudaMemcpyKind) {
  for (size_t r = 0; r < h; r++)
    std::memmove(static_cast<char*>(d) + r * dpitch, static_cast<const char*>(s) + r * spitch, wbytes);
  return 0;
}
cudaError_t cudaMemset(void* d, int v, size_t n) {
  std::memset(d, v, n);
  return 0;
}
cudaError_t cudaDeviceSynchronize() { return 0; }
cudaError_t cudaGetLastError() { return 0; }
const char* cudaGetErrorString(cudaError_t) { return "no error"; }
