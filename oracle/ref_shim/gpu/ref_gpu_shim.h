// Host stand-ins for the CUDA runtime, curand and InfiniTAM's ITMMath, so that
// the reference's GPU sources (STAC/Engine/GPU/*.cu) compile as plain host C++
// for the reference-pin harness oracle/ref_pin_gpu.cpp (TEST INFRASTRUCTURE
// ONLY; nothing here runs on a GPU).  The harness calls the reference's
// __device__ functions directly and runs its kernels as host loops over the
// launch grid (threadIdx / blockIdx below are the loop's variables).
//
// Arithmetic: the functions below are restatements, kept to what the pinned
// code uses.  __float2int_rn rounds half to even (as the CUDA intrinsic is
// documented); ITMMath's vectors are plain structs whose operators work
// component by component in the order ITMMath writes them.
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>

#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__ static
#define __forceinline__ inline
#define __align__(n)

using std::abs;
using std::sqrt;
typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;

struct dim3 {
  unsigned x = 1, y = 1, z = 1;
  dim3(unsigned a = 1, unsigned b = 1, unsigned c = 1) : x(a), y(b), z(c) {}
};
struct uint3_ {
  unsigned x = 0, y = 0, z = 0;
};
// the launch emulation sets these before each call of a kernel body
extern uint3_ threadIdx, blockIdx;
extern dim3 blockDim, gridDim;
struct int2 {
  int x, y;
};
struct int3 {
  int x, y, z;
};
struct float2 {
  float x, y;
};
struct float3 {
  float x, y, z;
};
struct float4 {
  float x, y, z, w;
};
// a barrier: a no-op for the one-thread-at-a-time loop, a switch back to the
// block's scheduler when the block runs as cooperative threads (below)
void __syncthreads();
inline int __float2int_rn(float x) { return (int)std::nearbyint(x); }  // default rounding mode: half to even
// IEEE round-to-nearest operations by their definition
inline float __fadd_rn(float a, float b) { return a + b; }
inline float __fmul_rn(float a, float b) { return a * b; }
inline float __fmaf_rn(float a, float b, float c) { return std::fma(a, b, c); }
inline float __int2float_rn(int x) { return (float)x; }
// the fast exponential's error bound is the GPU's own; on the host it is the
// correctly rounded expf of the C library (the oracle's choice as well)
inline float __expf(float x) { return std::exp(x); }

// _yooji_cuda_math.hpp:98 (GKvMatrix<T>::to_host) names an undeclared
// `out_vol`; MSVC never checks the uninstantiated template, GCC needs the name
// to exist.  Nothing here instantiates it.
static void* out_vol;

// The runtime on host memory: "device" buffers are host buffers, copies are
// memcpy, a symbol is the plain global of the same name.
typedef int cudaError_t;
typedef struct CUstream_st* cudaStream_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost, cudaMemcpyHostToDevice, cudaMemcpyDeviceToHost, cudaMemcpyDeviceToDevice };
struct cudaChannelFormatDesc {
  int x, y, z, w, f;
};
cudaError_t cudaMalloc(void**, size_t);
cudaError_t cudaFree(void*);
cudaError_t cudaMemcpy(void*, const void*, size_t, cudaMemcpyKind);
cudaError_t cudaMemset(void*, int, size_t);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaGetLastError();
const char* cudaGetErrorString(cudaError_t);
template <class T>
cudaError_t cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off = 0,
                               cudaMemcpyKind = cudaMemcpyHostToDevice) {
  std::memcpy(reinterpret_cast<char*>(&sym) + off, src, n);
  return 0;
}
template <class T>
cudaError_t cudaMemcpyFromSymbol(void* dst, const T& sym, size_t n, size_t off = 0,
                                 cudaMemcpyKind = cudaMemcpyDeviceToHost) {
  std::memcpy(dst, reinterpret_cast<const char*>(&sym) + off, n);
  return 0;
}
#define checkCudaErrors(x) (x)
// pitched buffers: the pitch is the row's own size (no alignment padding), so
// a texture bound with pitch 4 W (z_yooji_cuda_img_proc.cu:305) reads the rows
// the pitched copy wrote, the dense layout the filter means to use
cudaError_t cudaMallocPitch(void** p, size_t* pitch, size_t wbytes, size_t h);
cudaError_t cudaMemcpy2D(void* d, size_t dpitch, const void* s, size_t spitch, size_t wbytes, size_t h,
                         cudaMemcpyKind);

// CUDA 8 texture references, as far as the bilateral filter uses them.
// tex2D follows the texture-fetching rules of the CUDA C programming guide
// for unnormalised coordinates: point sampling reads texel (floor x, floor y);
// linear filtering reads the 2x2 texels around (x - 0.5, y - 0.5) with
// weights a, b of 8 fractional bits as (1-b)((1-a) T00 + a T10) +
// b((1-a) T01 + a T11); addresses clamp to the edge (wrap and mirror apply to
// normalised coordinates only).  At the integer coordinates the filter uses,
// a = b = 1/2 and every product is exact, so the tap is the mean of 2x2
// texels whatever precision the texture unit blends in.
enum cudaTextureReadMode { cudaReadModeElementType, cudaReadModeNormalizedFloat };
enum cudaTextureAddressMode { cudaAddressModeWrap, cudaAddressModeClamp, cudaAddressModeMirror, cudaAddressModeBorder };
enum cudaTextureFilterMode { cudaFilterModePoint, cudaFilterModeLinear };
template <class T, int D = 1, cudaTextureReadMode M = cudaReadModeElementType>
struct texture {
  int normalized = 0;
  cudaTextureFilterMode filterMode = cudaFilterModePoint;
  cudaTextureAddressMode addressMode[3] = {cudaAddressModeClamp, cudaAddressModeClamp, cudaAddressModeClamp};
  const char* base = nullptr;
  long w = 0, h = 0;
  size_t pitch = 0;
};
template <class T>
cudaChannelFormatDesc cudaCreateChannelDesc() {
  return cudaChannelFormatDesc{int(8 * sizeof(T)), 0, 0, 0, 2};
}
template <class T, int D, cudaTextureReadMode M>
cudaError_t cudaBindTexture2D(size_t* off, texture<T, D, M>& t, const void* p, const cudaChannelFormatDesc&, size_t w,
                              size_t h, size_t pitch) {
  if (off) *off = 0;
  t.base = static_cast<const char*>(p), t.w = (long)w, t.h = (long)h, t.pitch = pitch;
  return 0;
}
template <class T, int D, cudaTextureReadMode M>
cudaError_t cudaUnbindTexture(texture<T, D, M>& t) {
  t.base = nullptr;
  return 0;
}
template <class T, int D, cudaTextureReadMode M>
T tex2D(const texture<T, D, M>& t, float x, float y) {
  auto at = [&](long i, long j) {
    i = i < 0 ? 0 : (i >= t.w ? t.w - 1 : i);
    j = j < 0 ? 0 : (j >= t.h ? t.h - 1 : j);
    return *reinterpret_cast<const T*>(t.base + (size_t)j * t.pitch + (size_t)i * sizeof(T));
  };
  if (t.filterMode == cudaFilterModePoint) return at((long)std::floor(x), (long)std::floor(y));
  const float xb = x - 0.5f, yb = y - 0.5f, fi = std::floor(xb), fj = std::floor(yb);
  const float a = std::nearbyint((xb - fi) * 256.0f) / 256.0f, b = std::nearbyint((yb - fj) * 256.0f) / 256.0f;
  const long i = (long)fi, j = (long)fj;
  return (1.0f - b) * ((1.0f - a) * at(i, j) + a * at(i + 1, j)) + b * ((1.0f - a) * at(i, j + 1) + a * at(i + 1, j + 1));
}

// Kernels with barriers (vs_block_threads set by the harness around their
// launches) run each block as cooperative threads on their own stacks: every
// thread runs up to its next __syncthreads, then the next thread, round after
// round, so all threads of the block pass each barrier together.  Between two
// barriers the threads run in descending order of their linear index
// (x + y X + z X Y).  A tree step `if (c < i) s[c] += s[c + i]` then reads each
// s[c + i] after its own thread has finished every earlier step and before any
// later one, which is the lock-step result that a warp-synchronous tail with
// no barrier means to compute.
extern bool vs_block_threads;
void vs_run_block_threads(const dim3& b, void (*body)(void*), void* arg);

// a kernel launch `k<<<grid, block>>>(args)` becomes
// `vs_launch(grid, block, [&](auto&&... a) { k(a...); })(args)`: every thread
// of the grid runs the kernel body in turn (kernels without shared memory or
// barriers), or each block runs as cooperative threads (vs_block_threads)
template <class F>
struct VsLaunch {
  dim3 g, b;
  F f;
  template <class... A>
  void operator()(A&&... a) {
    gridDim = g;
    blockDim = b;
    auto body = [&]() { f(a...); };
    using B = decltype(body);
    for (unsigned bz = 0; bz < g.z; bz++)
      for (unsigned by = 0; by < g.y; by++)
        for (unsigned bx = 0; bx < g.x; bx++)
          if (vs_block_threads) {
            blockIdx.x = bx, blockIdx.y = by, blockIdx.z = bz;
            vs_run_block_threads(b, [](void* p) { (*static_cast<B*>(p))(); }, &body);
          } else
          for (unsigned tz = 0; tz < b.z; tz++)
            for (unsigned ty = 0; ty < b.y; ty++)
              for (unsigned tx = 0; tx < b.x; tx++) {
                blockIdx.x = bx, blockIdx.y = by, blockIdx.z = bz;
                threadIdx.x = tx, threadIdx.y = ty, threadIdx.z = tz;
                f(a...);
              }
  }
};
template <class F>
VsLaunch<F> vs_launch(dim3 g, dim3 b, F f) {
  return VsLaunch<F>{g, b, f};
}
inline dim3 vs_dim3(dim3 d) { return d; }
inline dim3 vs_dim3(int n) { return dim3((unsigned)n); }
#define vs_launch_any(g, b, f) vs_launch(vs_dim3(g), vs_dim3(b), f)
