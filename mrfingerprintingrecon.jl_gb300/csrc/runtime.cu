// Library runtime: the private per-device stream, the stream scope of the
// running entry point and the pool-backed device buffers (common.cuh).
#include <mutex>

#include "common.cuh"

namespace mrsr {

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
cudaStream_t g_lib[kMaxDevices] = {nullptr};
cudaEvent_t g_fence[kMaxDevices] = {nullptr};
thread_local cudaStream_t t_call = nullptr;
thread_local bool t_in_call = false;

int current_device() {
  int d = 0;
  if (cudaGetDevice(&d) != cudaSuccess || d < 0 || d >= kMaxDevices) return 0;
  return d;
}

// first use on a device: the private stream, and a pool that keeps up to
// 8 GiB of freed blocks for reuse and never makes one stream wait on another
// to hand a block over
void init_device(int d) {
  cudaStreamCreateWithFlags(&g_lib[d], cudaStreamNonBlocking);
  cudaEventCreateWithFlags(&g_fence[d], cudaEventDisableTiming);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, d) == cudaSuccess) {
    uint64_t keep = 8ull << 30;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    int no = 0;
    cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
  }
}
}  // namespace

cudaStream_t lib_stream() {
  const int d = current_device();
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_lib[d]) init_device(d);
  return g_lib[d];
}

cudaStream_t call_stream() { return t_in_call ? t_call : lib_stream(); }
bool in_call() { return t_in_call; }

int fence_lib_after(cudaStream_t s) {
  cudaStream_t ls = lib_stream();
  if (s == ls) return MRSR_OK;
  const int d = current_device();
  std::lock_guard<std::mutex> lock(g_mu);  // one fence event per device, reused under the lock
  MRSR_CHECK_CUDA(cudaEventRecord(g_fence[d], s));
  MRSR_CHECK_CUDA(cudaStreamWaitEvent(ls, g_fence[d], 0));
  return MRSR_OK;
}

int copy_h2d(void* dst, const void* src, size_t bytes) {
  cudaStream_t s = call_stream();
  MRSR_CHECK_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
  if (!t_in_call) MRSR_CHECK_CUDA(cudaStreamSynchronize(s));
  return MRSR_OK;
}

CallScope::CallScope(cudaStream_t st) : prev(t_call), prev_in(t_in_call) {
  t_call = st;
  t_in_call = true;
}
CallScope::~CallScope() {
  t_call = prev;
  t_in_call = prev_in;
}

void DevBuf::release() {
  if (!p) return;
  cudaStream_t ls = lib_stream();
  if (t_in_call) fence_lib_after(t_call);
  cudaFreeAsync(p, ls);
  p = nullptr;
  bytes = 0;
}

int DevBuf::alloc(size_t n) {
  release();
  if (n == 0) return MRSR_OK;
  cudaStream_t s = call_stream();
  cudaError_t e = cudaMallocAsync(&p, n, s);
  if (e == cudaSuccess && !t_in_call) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    set_error("device allocation of %zu bytes failed: %s", n, cudaGetErrorString(e));
    return MRSR_ERR_ALLOC;
  }
  bytes = n;
  return MRSR_OK;
}

}  // namespace mrsr
