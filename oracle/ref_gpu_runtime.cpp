// Host definitions behind ref_shim/gpu/ref_gpu_shim.h: the launch variables
// and the runtime calls on host memory (TEST INFRASTRUCTURE ONLY).
#include <ucontext.h>

#include <set>
#include <vector>

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

// ---- cooperative threads of one block (kernels with barriers) --------------
bool vs_block_threads = false;
namespace {
struct BlockThread {
  ucontext_t ctx;
  uint3_ tid;
  bool done;
};
constexpr size_t kStack = 256 * 1024;
ucontext_t g_sched;
std::vector<BlockThread> g_thr;
std::vector<std::vector<char>> g_stacks;
int g_cur = -1;
void (*g_body)(void*);
void* g_arg;
void thread_entry() {
  g_body(g_arg);
  g_thr[g_cur].done = true;  // returning resumes g_sched through uc_link
}
}  // namespace

void __syncthreads() {
  if (g_cur >= 0) swapcontext(&g_thr[g_cur].ctx, &g_sched);
}

void vs_run_block_threads(const dim3& b, void (*body)(void*), void* arg) {
  const int n = (int)(b.x * b.y * b.z);
  g_thr.resize(n);
  if ((int)g_stacks.size() < n) g_stacks.resize(n);
  g_body = body, g_arg = arg;
  for (int i = 0; i < n; i++) {
    BlockThread& t = g_thr[i];
    t.tid.x = i % b.x, t.tid.y = (i / b.x) % b.y, t.tid.z = i / (b.x * b.y);
    t.done = false;
    g_stacks[i].resize(kStack);
    getcontext(&t.ctx);
    t.ctx.uc_stack.ss_sp = g_stacks[i].data();
    t.ctx.uc_stack.ss_size = kStack;
    t.ctx.uc_link = &g_sched;
    makecontext(&t.ctx, thread_entry, 0);
  }
  for (bool running = true; running;) {
    running = false;
    for (int i = n - 1; i >= 0; i--) {
      if (g_thr[i].done) continue;
      threadIdx = g_thr[i].tid;
      g_cur = i;
      swapcontext(&g_sched, &g_thr[i].ctx);
      running |= !g_thr[i].done;
    }
  }
  g_cur = -1;
}
