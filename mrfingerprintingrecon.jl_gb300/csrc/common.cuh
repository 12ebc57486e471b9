// Shared helpers of the sm_103a subspace normal-operator library.
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/mrsr.h"

namespace mrsr {

// ---------------------------------------------------------------- errors ---
void set_error(const char* fmt, ...);
const char* get_error();

struct Status {
  int code;
};

#define MRSR_CHECK_CUDA(expr)                                                   \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) {                                                    \
      ::mrsr::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #expr,             \
                        cudaGetErrorString(_e));                                \
      return MRSR_ERR_CUDA;                                                     \
    }                                                                           \
  } while (0)

#define MRSR_REQUIRE(cond, code, ...)                                           \
  do {                                                                          \
    if (!(cond)) {                                                              \
      ::mrsr::set_error(__VA_ARGS__);                                           \
      return (code);                                                            \
    }                                                                           \
  } while (0)

#define MRSR_TRY(expr)                                                          \
  do {                                                                          \
    int _s = (expr);                                                            \
    if (_s != MRSR_OK) return _s;                                               \
  } while (0)

// Launch-error check right after a <<<>>> launch.
#define MRSR_LAUNCH_CHECK() MRSR_CHECK_CUDA(cudaGetLastError())

// ------------------------------------------------------ stream scopes ---
// Every entry point that takes a stream opens a CallScope on it.  Device
// memory comes from the stream-ordered pool (cudaMallocAsync) on the call's
// stream, so the library never calls cudaMalloc / cudaFree, which would
// synchronise the whole device and stall other streams' work.  A buffer is
// freed on the library's private stream after that stream has waited for the
// work that may still use it: the running call's stream (temporaries) or the
// owning operator's last use (see mrsr_normalop).
cudaStream_t lib_stream();          // private non-blocking stream of the current device
cudaStream_t call_stream();         // stream of the running entry point, else lib_stream()
bool in_call();
// lib_stream() waits for the work enqueued so far on `s`
int fence_lib_after(cudaStream_t s);
// host -> device copy ordered on call_stream() (pageable source may be freed on return)
int copy_h2d(void* dst, const void* src, size_t bytes);

struct CallScope {
  cudaStream_t prev;
  bool prev_in;
  explicit CallScope(cudaStream_t st);
  ~CallScope();
};
#define MRSR_CALL_SCOPE(st) ::mrsr::CallScope _mrsr_call_scope(st)

// ------------------------------------------------------- device buffers ---
// RAII owner of a device workspace from the stream-ordered pool.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release();
  int alloc(size_t n);
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// ------------------------------------------------------- fast division ---
// Division by a runtime constant d (0 <= n < 2^31): q = (umulhi(n, m) + n) >> s
// with s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1 (Granlund and
// Montgomery's round-up method, the 33-bit magic's top bit folded as "+ n").
struct FastDiv {
  uint32_t d = 1, m = 1, s = 0;
  FastDiv() = default;
  explicit FastDiv(uint32_t d_) : d(d_) {
    s = 0;
    while ((1ull << s) < d) ++s;
    m = (uint32_t)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const { return (__umulhi(n, m) + n) >> s; }
};

// ------------------------------------------------------ complex helpers ---
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse): sgn=-1 -> -i, sgn=+1 -> +i
__host__ __device__ __forceinline__ float2 cmul_i(float2 a, float sgn) { return make_float2(-sgn * a.y, sgn * a.x); }

__host__ __device__ __forceinline__ int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Storage conversion for the intermediate K-stack (float2, or half2 scaled by a per-line factor).
template <class S> struct Store;
template <> struct Store<float2> {
  static __device__ __forceinline__ float2 load(const float2* p, int64_t i, float) { return p[i]; }
  static __device__ __forceinline__ void store(float2* p, int64_t i, float2 v, float) { p[i] = v; }
  static constexpr bool scaled = false;
};
template <> struct Store<__half2> {
  static __device__ __forceinline__ float2 load(const __half2* p, int64_t i, float s) {
    float2 v = __half22float2(p[i]);
    return make_float2(v.x * s, v.y * s);
  }
  static __device__ __forceinline__ void store(__half2* p, int64_t i, float2 v, float inv_s) {
    p[i] = __floats2half2_rn(v.x * inv_s, v.y * inv_s);
  }
  static constexpr bool scaled = true;
};

}  // namespace mrsr
