// Conjugate gradients on a normal operator, as IterativeSolvers.jl 0.9 `cg`
// runs it (x0 = 0): per iteration
//   u = r + (|r|^2 / prev^2) u,  c = A u,  alpha = |r|^2 / <u, c>,
//   x += alpha u,  r -= alpha c,  prev = |r|,  |r| = norm(r)
// stopping once |r| <= max(reltol |b|, abstol) or after maxiter iterations.
// Vectors are ComplexF32.  Each thread sums the products of its few elements
// (about four) with float32 FMAs; everything above that (warp, block, grid) is
// float64, and alpha and beta are formed once, in float64, by the block that
// finishes a reduction.  GB300's float64 rate is a small fraction of its float32
// rate, so no per-element work runs in float64.  Reductions are deterministic
// (per-block partials summed in a fixed order by the last block).  A device "done" flag makes iterations
// after convergence no-ops, so the host launches without synchronising.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "cg.cuh"
#include "normalop.cuh"

namespace mrsr {

constexpr int kCgThreads = 256;
constexpr int kCgBlocks = 1024;

struct CgState {
  double res;         // |r|
  double prev;        // previous |r| (1 before the first iteration)
  double tol;         // max(reltol |b|, abstol)
  double ar, ai;      // alpha (complex)
  int it;             // iterations done
  int maxiter;
  int done;
  unsigned int ticket;
  float beta;         // res^2 / prev^2 for the next direction update (0 before the first)
};

__device__ __forceinline__ double2 block_sum2(double2 v) {
  __shared__ double2 red[kCgThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_down_sync(0xffffffffu, v.x, o);
    v.y += __shfl_down_sync(0xffffffffu, v.y, o);
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double2 s = make_double2(0.0, 0.0);
  if (threadIdx.x == 0)
    for (int w = 0; w < kCgThreads / 32; ++w) {
      s.x += red[w].x;
      s.y += red[w].y;
    }
  return s;
}

// Block sum of each thread's float32 partials (the products of its few elements): the
// partials are widened to float64 and combined in float64 in a fixed order.  The result
// is valid in thread 0.
__device__ __forceinline__ double2 block_sum_f2(float2 v) { return block_sum2(make_double2(v.x, v.y)); }

// The last block to finish sums the per-block partials; returns true in that block's
// thread 0.  All its threads take part: thread t adds partials t, t + blockDim, ... in
// that order, then the block tree combines them, so the total does not depend on which
// block finished last or when (the reductions are deterministic run to run).
__device__ __forceinline__ bool last_block(CgState* st, double2* partial, double2 mine, double2* total) {
  __shared__ bool is_last;
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = mine;
    __threadfence();
    const unsigned t = atomicAdd(&st->ticket, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!is_last) return false;
  __threadfence();
  double2 s = make_double2(0.0, 0.0);
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
    const volatile double* p = reinterpret_cast<volatile double*>(partial + b);
    s.x += p[0];
    s.y += p[1];
  }
  s = block_sum2(s);
  if (threadIdx.x == 0) {
    *total = s;
    st->ticket = 0;
  }
  return threadIdx.x == 0;
}

// x = 0, r = b, u = 0, res = |b|
// Every vector kernel works on plane blockIdx.y of gridDim.y independent systems of n
// unknowns each (one system for a plain solve), each with its own state and partials.
__global__ void k_cg_init(const float2* b, float2* x, float2* r, float2* u, int64_t n, double reltol, double abstol,
                          int maxiter, CgState* st, double2* partial) {
  {
    const int64_t o = (int64_t)blockIdx.y * n;
    b += o; x += o; r += o; u += o;
    st += blockIdx.y;
    partial += (int64_t)blockIdx.y * gridDim.x;
  }
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = b[i];
    x[i] = make_float2(0.f, 0.f);
    r[i] = v;
    u[i] = make_float2(0.f, 0.f);
    acc = fmaf(v.x, v.x, fmaf(v.y, v.y, acc));
  }
  double2 s = block_sum_f2(make_float2(acc, 0.f));
  double2 tot;
  if (last_block(st, partial, s, &tot)) {
    const double res = sqrt(tot.x);
    st->res = res;
    st->prev = 1.0;
    st->beta = 0.f;
    st->tol = fmax(reltol * res, abstol);
    st->it = 0;
    st->maxiter = maxiter;
    st->done = (maxiter <= 0 || res <= st->tol) ? 1 : 0;
  }
}

// u = r + beta u with beta = res^2 / prev^2 (formed by the previous update, 0 at first)
__global__ void k_cg_dir(const float2* r, float2* u, int64_t n, const CgState* st) {
  r += (int64_t)blockIdx.y * n;
  u += (int64_t)blockIdx.y * n;
  st += blockIdx.y;
  if (st->done) return;
  const float b = st->beta;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 rv = r[i], uv = u[i];
    u[i] = make_float2(rv.x + b * uv.x, rv.y + b * uv.y);
  }
}

// alpha = res^2 / <u, c>  (<u, c> = sum conj(u) c)
__global__ void k_cg_alpha(const float2* u, const float2* c, int64_t n, CgState* st, double2* partial) {
  u += (int64_t)blockIdx.y * n;
  c += (int64_t)blockIdx.y * n;
  st += blockIdx.y;
  partial += (int64_t)blockIdx.y * gridDim.x;
  if (st->done) return;
  float re = 0.f, im = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = u[i], b = c[i];
    re = fmaf(a.x, b.x, fmaf(a.y, b.y, re));
    im = fmaf(a.x, b.y, fmaf(-a.y, b.x, im));
  }
  double2 s = block_sum_f2(make_float2(re, im));
  double2 tot;
  if (last_block(st, partial, s, &tot)) {
    const double r2 = st->res * st->res;
    const double den = tot.x * tot.x + tot.y * tot.y;
    // r2 / (tot.x + i tot.y)
    st->ar = den > 0.0 ? r2 * tot.x / den : 0.0;
    st->ai = den > 0.0 ? -r2 * tot.y / den : 0.0;
  }
}

// x += alpha u, r -= alpha c, then res = |r|, it += 1, done flag
__global__ void k_cg_update(float2* x, float2* r, const float2* u, const float2* c, int64_t n, CgState* st,
                            double2* partial) {
  {
    const int64_t o = (int64_t)blockIdx.y * n;
    x += o; r += o; u += o; c += o;
    st += blockIdx.y;
    partial += (int64_t)blockIdx.y * gridDim.x;
  }
  if (st->done) return;
  const float ar = (float)st->ar, ai = (float)st->ai;
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 uv = u[i], cv = c[i];
    float2 xv = x[i], rv = r[i];
    xv.x += ar * uv.x - ai * uv.y;
    xv.y += ar * uv.y + ai * uv.x;
    rv.x -= ar * cv.x - ai * cv.y;
    rv.y -= ar * cv.y + ai * cv.x;
    x[i] = xv;
    r[i] = rv;
    acc = fmaf(rv.x, rv.x, fmaf(rv.y, rv.y, acc));
  }
  double2 s = block_sum_f2(make_float2(acc, 0.f));
  double2 tot;
  if (last_block(st, partial, s, &tot)) {
    st->prev = st->res;
    st->res = sqrt(tot.x);
    st->beta = st->prev > 0.0 ? (float)(tot.x / (st->prev * st->prev)) : 0.f;
    st->it += 1;
    st->done = (st->res <= st->tol || st->it >= st->maxiter) ? 1 : 0;
  }
}

// about four elements per thread: the per-block partials and the final sum stay short
static unsigned vec_blocks(int64_t n) {
  return (unsigned)std::min<int64_t>(kCgBlocks, std::max<int64_t>(1, cdiv(n, 4 * kCgThreads)));
}

void CgWork::drop_graphs() {
  if (it8) cudaGraphExecDestroy(it8);
  if (it1) cudaGraphExecDestroy(it1);
  if (lo8) cudaGraphExecDestroy(lo8);
  if (lo1) cudaGraphExecDestroy(lo1);
  it8 = it1 = lo8 = lo1 = nullptr;
  lo_serial = 0;
}

CgWork::~CgWork() {
  drop_graphs();
  if (cap) cudaStreamDestroy(cap);
}

int CgWork::ensure(int64_t n_, int nseg_) {
  if (n == n_ && nseg == nseg_ && r.p) return MRSR_OK;
  drop_graphs();
  xw.release();  // cg_run allocates it at the new size
  n = n_;
  nseg = nseg_;
  MRSR_TRY(r.alloc(sizeof(float2) * n));
  MRSR_TRY(u.alloc(sizeof(float2) * n));
  MRSR_TRY(c.alloc(sizeof(float2) * n));
  MRSR_TRY(state.alloc(sizeof(CgState) * nseg));
  MRSR_TRY(partial.alloc(sizeof(double2) * kCgBlocks * nseg));
  MRSR_CHECK_CUDA(cudaMemsetAsync(state.p, 0, sizeof(CgState) * nseg, call_stream()));
  return MRSR_OK;
}

// one CG iteration on the workspace (iterate w.xw), enqueued on st
static int cg_iter_enqueue(mrsr_normalop* op, CgWork& w, cudaStream_t st) {
  const int64_t m = w.n / w.nseg;
  CgState* s = w.state.as<CgState>();
  double2* part = w.partial.as<double2>();
  const dim3 nb(vec_blocks(m), (unsigned)w.nseg);
  k_cg_dir<<<nb, kCgThreads, 0, st>>>(w.r.as<float2>(), w.u.as<float2>(), m, s);
  MRSR_LAUNCH_CHECK();
  MRSR_TRY(normalop_apply_internal(op, w.u.as<float2>(), w.c.as<float2>(), make_float2(1.f, 0.f),
                                   make_float2(0.f, 0.f), st));
  k_cg_alpha<<<nb, kCgThreads, 0, st>>>(w.u.as<float2>(), w.c.as<float2>(), m, s, part);
  MRSR_LAUNCH_CHECK();
  k_cg_update<<<nb, kCgThreads, 0, st>>>(w.xw.as<float2>(), w.r.as<float2>(), w.u.as<float2>(), w.c.as<float2>(), m,
                                         s, part);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// `iters` iterations recorded on the workspace's private stream into an executable graph
static int cg_capture(mrsr_normalop* op, CgWork& w, int iters, cudaGraphExec_t* out) {
  if (!w.cap) MRSR_CHECK_CUDA(cudaStreamCreateWithFlags(&w.cap, cudaStreamNonBlocking));
  MRSR_CHECK_CUDA(cudaStreamBeginCapture(w.cap, cudaStreamCaptureModeThreadLocal));
  int s = MRSR_OK;
  for (int k = 0; k < iters && s == MRSR_OK; ++k) s = cg_iter_enqueue(op, w, w.cap);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(w.cap, &g);
  if (s == MRSR_OK && e != cudaSuccess) {
    set_error("CG graph capture failed: %s", cudaGetErrorString(e));
    s = MRSR_ERR_CUDA;
  }
  if (s == MRSR_OK && cudaGraphInstantiate(out, g, 0) != cudaSuccess) {
    set_error("CG graph instantiation failed");
    s = MRSR_ERR_CUDA;
  }
  if (g) cudaGraphDestroy(g);
  return s;
}

int cg_run(mrsr_normalop* op, CgWork& w, const float2* b, float2* x, int maxiter, double reltol, double abstol,
           cudaStream_t st, int* iters, double* res, int nseg) {
  const int64_t n = op->geo.nimg() * op->geo.K;
  const int64_t m = n / nseg;  // unknowns per system
  MRSR_TRY(w.ensure(n, nseg));
  if (!w.xw.p) MRSR_TRY(w.xw.alloc(sizeof(float2) * n));
  CgState* s = w.state.as<CgState>();
  double2* part = w.partial.as<double2>();
  const dim3 nb(vec_blocks(m), (unsigned)nseg);
  k_cg_init<<<nb, kCgThreads, 0, st>>>(b, w.xw.as<float2>(), w.r.as<float2>(), w.u.as<float2>(), m, reltol, abstol,
                                       maxiter, s, part);
  MRSR_LAUNCH_CHECK();
  // The iterations run as graph launches of 8 (and single) iterations, recorded once per
  // workspace; between blocks of 8 the host reads the done flags when a tolerance is set,
  // so converged solves do not keep paying for applies.  Without a tolerance only an
  // exact zero residual ends a solve early, and the device's done flag already turns the
  // iterations after it into no-ops.
  if (maxiter >= 8 && !w.it8) MRSR_TRY(cg_capture(op, w, 8, &w.it8));
  if (maxiter % 8 != 0 && !w.it1) MRSR_TRY(cg_capture(op, w, 1, &w.it1));
  std::vector<CgState> h((size_t)nseg);
  auto all_done = [&]() {
    for (const CgState& v : h)
      if (!v.done) return false;
    return true;
  };
  const bool check = reltol > 0.0 || abstol > 0.0;
  int done_its = 0;
  while (done_its < maxiter) {
    const int nit = std::min(8, maxiter - done_its);
    if (nit == 8) {
      MRSR_CHECK_CUDA(cudaGraphLaunch(w.it8, st));
    } else {
      for (int k = 0; k < nit; ++k) MRSR_CHECK_CUDA(cudaGraphLaunch(w.it1, st));
    }
    done_its += nit;
    if (check && done_its < maxiter) {
      MRSR_CHECK_CUDA(cudaMemcpyAsync(h.data(), s, sizeof(CgState) * nseg, cudaMemcpyDeviceToHost, st));
      MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
      if (all_done()) break;
    }
  }
  MRSR_CHECK_CUDA(cudaMemcpyAsync(x, w.xw.p, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
  int dev_err = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(h.data(), s, sizeof(CgState) * nseg, cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&dev_err, op->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < nseg; ++i) {
    if (iters) iters[i] = h[i].it;
    if (res) res[i] = h[i].res;
  }
  return device_error_status(op, dev_err, st);
}

int cg_fixed_init_enqueue(mrsr_normalop* op, const float2* b, float2* x, int iters, cudaStream_t st) {
  CgWork& w = op->cg;
  const int64_t n = op->geo.nimg() * op->geo.K;
  MRSR_REQUIRE(w.n == n && w.nseg == 1 && w.r.p, MRSR_ERR_STATE, "CG work vectors are not allocated for this operator");
  k_cg_init<<<vec_blocks(n), kCgThreads, 0, st>>>(b, x, w.r.as<float2>(), w.u.as<float2>(), n, 0.0, 0.0, iters,
                                                  w.state.as<CgState>(), w.partial.as<double2>());
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int cg_fixed_iter_enqueue(mrsr_normalop* op, float2* x, cudaStream_t st, mrsr_normalop* apply_op) {
  CgWork& w = op->cg;
  if (!apply_op) apply_op = op;
  const int64_t n = op->geo.nimg() * op->geo.K;
  CgState* s = w.state.as<CgState>();
  double2* part = w.partial.as<double2>();
  const unsigned nb = vec_blocks(n);
  k_cg_dir<<<nb, kCgThreads, 0, st>>>(w.r.as<float2>(), w.u.as<float2>(), n, s);
  MRSR_LAUNCH_CHECK();
  MRSR_TRY(normalop_apply_internal(apply_op, w.u.as<float2>(), w.c.as<float2>(), make_float2(1.f, 0.f),
                                   make_float2(0.f, 0.f), st));
  k_cg_alpha<<<nb, kCgThreads, 0, st>>>(w.u.as<float2>(), w.c.as<float2>(), n, s, part);
  MRSR_LAUNCH_CHECK();
  k_cg_update<<<nb, kCgThreads, 0, st>>>(x, w.r.as<float2>(), w.u.as<float2>(), w.c.as<float2>(), n, s, part);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int cg_fixed_enqueue(mrsr_normalop* op, const float2* b, float2* x, int iters, cudaStream_t st) {
  MRSR_TRY(cg_fixed_init_enqueue(op, b, x, iters, st));
  for (int k = 0; k < iters; ++k) MRSR_TRY(cg_fixed_iter_enqueue(op, x, st));
  return MRSR_OK;
}

int cg_fixed_result(mrsr_normalop* op, int* iters, double* res) {
  MRSR_REQUIRE(op->cg.state.p, MRSR_ERR_STATE, "no CG has run on this operator");
  CgState h;
  int dev_err = 0;
  MRSR_CHECK_CUDA(cudaMemcpy(&h, op->cg.state.p, sizeof(CgState), cudaMemcpyDeviceToHost));
  MRSR_CHECK_CUDA(cudaMemcpy(&dev_err, op->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (iters) *iters = h.it;
  if (res) *res = h.res;
  return device_error_status(op, dev_err, call_stream());
}

// r = b - A x  (outer residual of the refinement, float32 operator)
__global__ void k_copy(const float2* a, float2* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = a[i];
}
__global__ void k_axpy(float2* y, const float2* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = x[i];
    float2 b = y[i];
    b.x += a.x;
    b.y += a.y;
    y[i] = b;
  }
}
__global__ void k_sub(float2* y, const float2* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = x[i];
    float2 b = y[i];
    b.x -= a.x;
    b.y -= a.y;
    y[i] = b;
  }
}
// |a|^2: per-block partials, then k_sum_parts adds them in block order (deterministic)
__global__ void k_norm2(const float2* a, int64_t n, double* part) {
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc = fmaf(a[i].x, a[i].x, fmaf(a[i].y, a[i].y, acc));
  double2 s = block_sum_f2(make_float2(acc, 0.f));
  if (threadIdx.x == 0) part[blockIdx.x] = s.x;
}
__global__ void k_sum_parts(const double* part, int nparts, double* out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += part[b];
    out[0] = s;
  }
}

}  // namespace mrsr

using namespace mrsr;

extern "C" int mrsr_cg(mrsr_normalop* op, const float* b, float* x, int maxiter, double reltol, double abstol,
                       int* iters_out, double* resnorm_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && b && x, MRSR_ERR_ARG, "NULL argument to mrsr_cg");
  MRSR_REQUIRE((const void*)b != (const void*)x, MRSR_ERR_ARG, "b and x must not alias");
  MRSR_REQUIRE(maxiter >= 0, MRSR_ERR_ARG, "maxiter must be >= 0");
  OpUse use{op, reinterpret_cast<cudaStream_t>(stream)};
  return cg_run(op, op->cg, reinterpret_cast<const float2*>(b), reinterpret_cast<float2*>(x), maxiter, reltol, abstol,
                reinterpret_cast<cudaStream_t>(stream), iters_out, resnorm_out);
}

extern "C" int mrsr_cg_stacked(mrsr_normalop* op, const float* b, float* x, int maxiter, double reltol, double abstol,
                               int* iters_out, double* resnorm_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && b && x, MRSR_ERR_ARG, "NULL argument to mrsr_cg_stacked");
  MRSR_REQUIRE((const void*)b != (const void*)x, MRSR_ERR_ARG, "b and x must not alias");
  MRSR_REQUIRE(maxiter >= 0, MRSR_ERR_ARG, "maxiter must be >= 0");
  MRSR_REQUIRE(lam_is_diag(op->lam_mode), MRSR_ERR_ARG,
               "mrsr_cg_stacked needs a stacked operator (mrsr_normalop_stack): the planes of any other "
               "operator are coupled by its kernel");
  OpUse use{op, reinterpret_cast<cudaStream_t>(stream)};
  return cg_run(op, op->cg, reinterpret_cast<const float2*>(b), reinterpret_cast<float2*>(x), maxiter, reltol, abstol,
                reinterpret_cast<cudaStream_t>(stream), iters_out, resnorm_out, op->geo.K);
}

extern "C" int mrsr_cg_refined(mrsr_normalop* op_lo, mrsr_normalop* op_hi, const float* b, float* x, int inner_iters,
                               int max_outer, double tol, int* outer_out, double* relres_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op_lo && op_hi && b && x, MRSR_ERR_ARG, "NULL argument to mrsr_cg_refined");
  MRSR_REQUIRE(op_lo->geo.nimg() == op_hi->geo.nimg() && op_lo->geo.K == op_hi->geo.K, MRSR_ERR_ARG,
               "operators of different sizes");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  OpUse use_lo{op_lo, st}, use_hi{op_hi, st};
  const int64_t n = op_hi->geo.nimg() * op_hi->geo.K;
  const float2* bb = reinterpret_cast<const float2*>(b);
  float2* xx = reinterpret_cast<float2*>(x);
  DevBuf r, d, nrm, part;
  MRSR_TRY(r.alloc(sizeof(float2) * n));
  MRSR_TRY(d.alloc(sizeof(float2) * n));
  MRSR_TRY(nrm.alloc(sizeof(double) * 2));
  const unsigned nb = vec_blocks(n);
  MRSR_TRY(part.alloc(sizeof(double) * nb));
  MRSR_CHECK_CUDA(cudaMemsetAsync(xx, 0, sizeof(float2) * n, st));
  k_norm2<<<nb, kCgThreads, 0, st>>>(bb, n, part.as<double>());
  MRSR_LAUNCH_CHECK();
  k_sum_parts<<<1, 32, 0, st>>>(part.as<double>(), (int)nb, nrm.as<double>());
  MRSR_LAUNCH_CHECK();
  double hn[2];
  MRSR_CHECK_CUDA(cudaMemcpyAsync(hn, nrm.p, sizeof(double), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  const double bnorm = std::sqrt(hn[0]);
  double relres = bnorm > 0 ? 1.0 : 0.0;
  int outer = 0;
  k_copy<<<nb, kCgThreads, 0, st>>>(bb, r.as<float2>(), n);
  MRSR_LAUNCH_CHECK();
  while (outer < max_outer && relres > tol) {
    int it = 0;
    double rr = 0;
    const double prev = relres;
    MRSR_TRY(cg_run(op_lo, op_lo->cg, r.as<float2>(), d.as<float2>(), inner_iters, 0.0, 0.0, st, &it, &rr));
    k_axpy<<<nb, kCgThreads, 0, st>>>(xx, d.as<float2>(), n);
    MRSR_LAUNCH_CHECK();
    // r = b - A_hi x
    k_copy<<<nb, kCgThreads, 0, st>>>(bb, r.as<float2>(), n);
    MRSR_LAUNCH_CHECK();
    MRSR_TRY(normalop_apply_internal(op_hi, xx, r.as<float2>(), make_float2(-1.f, 0.f), make_float2(1.f, 0.f), st));
    k_norm2<<<nb, kCgThreads, 0, st>>>(r.as<float2>(), n, part.as<double>());
    MRSR_LAUNCH_CHECK();
    k_sum_parts<<<1, 32, 0, st>>>(part.as<double>(), (int)nb, nrm.as<double>());
    MRSR_LAUNCH_CHECK();
    int dev_err = 0;
    MRSR_CHECK_CUDA(cudaMemcpyAsync(hn, nrm.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    MRSR_CHECK_CUDA(cudaMemcpyAsync(&dev_err, op_hi->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
    MRSR_TRY(device_error_status(op_hi, dev_err, st));
    relres = std::sqrt(hn[0]) / bnorm;
    ++outer;
    if (!(relres <= 2.0 * prev)) {
      // the correction doubled the float32 residual: at this level the inner operator's
      // rounding dominates and further steps only add error.  Undo the step and stop.
      // (CG minimises the error in the A-norm, so smaller rises of the residual's
      // 2-norm are normal and do not stop the loop.)
      k_sub<<<nb, kCgThreads, 0, st>>>(xx, d.as<float2>(), n);
      MRSR_LAUNCH_CHECK();
      relres = prev;
      break;
    }
  }
  if (outer_out) *outer_out = outer;
  if (relres_out) *relres_out = relres;
  return MRSR_OK;
}

// ---------------------------------------------------------------------------
// Relaxed mixed-precision CG.
//
// One CG recurrence (IterativeSolvers' iteration, x0 = 0) whose operator products switch
// from the float32 operator op_hi to the reduced-precision op_lo once the residual has
// fallen to ||r|| <= switch_relres ||b||.  The deviation of a CG iterate caused by an
// inexact product grows with the residual at the step where the product was taken
// (inexact Krylov theory: the tolerable product error at step k scales like 1 / ||r_k||),
// so the few large-residual steps run on the accurate operator and the many later steps
// on the fast one, and the iterate stays close to the float32 / float64 CG iterate of the
// same iteration count.  Restarted refinement (mrsr_cg_refined) instead converges to
// A_hi^-1 b, which on the kmask-truncated Toeplitz operator is far from a CG-k iterate.
// The vectors live in op_hi's CG workspace.
// ---------------------------------------------------------------------------
extern "C" int mrsr_cg_relaxed(mrsr_normalop* op_lo, mrsr_normalop* op_hi, const float* b, float* x, int maxiter,
                               double reltol, double abstol, double switch_relres, int* iters_out, int* hi_iters_out,
                               double* resnorm_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op_lo && op_hi && b && x, MRSR_ERR_ARG, "NULL argument to mrsr_cg_relaxed");
  MRSR_REQUIRE(op_lo != op_hi, MRSR_ERR_ARG, "mrsr_cg_relaxed needs two different operators");
  MRSR_REQUIRE(op_lo->geo.nimg() == op_hi->geo.nimg() && op_lo->geo.K == op_hi->geo.K, MRSR_ERR_ARG,
               "operators of different sizes");
  MRSR_REQUIRE(!lam_is_diag(op_hi->lam_mode) && !lam_is_diag(op_lo->lam_mode), MRSR_ERR_ARG,
               "mrsr_cg_relaxed solves one system; use mrsr_cg_stacked for stacked operators");
  MRSR_REQUIRE((const void*)b != (const void*)x, MRSR_ERR_ARG, "b and x must not alias");
  MRSR_REQUIRE(maxiter >= 0, MRSR_ERR_ARG, "maxiter must be >= 0");
  MRSR_REQUIRE(switch_relres >= 0.0, MRSR_ERR_ARG, "switch_relres must be >= 0");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  OpUse use_lo{op_lo, st}, use_hi{op_hi, st};
  CgWork& w = op_hi->cg;
  const int64_t n = op_hi->geo.nimg() * op_hi->geo.K;
  MRSR_TRY(w.ensure(n, 1));
  if (!w.xw.p) MRSR_TRY(w.xw.alloc(sizeof(float2) * n));
  CgState* s = w.state.as<CgState>();
  const unsigned nb = vec_blocks(n);
  k_cg_init<<<nb, kCgThreads, 0, st>>>(reinterpret_cast<const float2*>(b), w.xw.as<float2>(), w.r.as<float2>(),
                                       w.u.as<float2>(), n, reltol, abstol, maxiter, s, w.partial.as<double2>());
  MRSR_LAUNCH_CHECK();
  CgState h;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&h, s, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  const double bnorm = h.res;
  // phase 1: float32 products, one iteration at a time, the residual read back after each
  int done_its = 0, hi_its = 0;
  if (maxiter > 0 && h.res > switch_relres * bnorm && !h.done && !w.it1) MRSR_TRY(cg_capture(op_hi, w, 1, &w.it1));
  while (done_its < maxiter && !h.done && h.res > switch_relres * bnorm) {
    MRSR_CHECK_CUDA(cudaGraphLaunch(w.it1, st));
    ++done_its;
    ++hi_its;
    MRSR_CHECK_CUDA(cudaMemcpyAsync(&h, s, sizeof(CgState), cudaMemcpyDeviceToHost, st));
    MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  }
  // phase 2: reduced-precision products on the same recurrence, graphs of 8 and 1 iterations
  if (done_its < maxiter && !h.done) {
    if (w.lo_serial != op_lo->serial) {
      if (w.lo8) cudaGraphExecDestroy(w.lo8);
      if (w.lo1) cudaGraphExecDestroy(w.lo1);
      w.lo8 = w.lo1 = nullptr;
      w.lo_serial = op_lo->serial;
    }
    const int rest = maxiter - done_its;
    if (rest >= 8 && !w.lo8) MRSR_TRY(cg_capture(op_lo, w, 8, &w.lo8));
    if (rest % 8 != 0 && !w.lo1) MRSR_TRY(cg_capture(op_lo, w, 1, &w.lo1));
    const bool check = reltol > 0.0 || abstol > 0.0;
    while (done_its < maxiter) {
      const int nit = std::min(8, maxiter - done_its);
      if (nit == 8)
        MRSR_CHECK_CUDA(cudaGraphLaunch(w.lo8, st));
      else
        for (int k = 0; k < nit; ++k) MRSR_CHECK_CUDA(cudaGraphLaunch(w.lo1, st));
      done_its += nit;
      if (check && done_its < maxiter) {
        MRSR_CHECK_CUDA(cudaMemcpyAsync(&h, s, sizeof(CgState), cudaMemcpyDeviceToHost, st));
        MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
        if (h.done) break;
      }
    }
  }
  MRSR_CHECK_CUDA(cudaMemcpyAsync(x, w.xw.p, sizeof(float2) * n, cudaMemcpyDeviceToDevice, st));
  int err_hi = 0, err_lo = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&h, s, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&err_hi, op_hi->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&err_lo, op_lo->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  if (iters_out) *iters_out = h.it;
  if (hi_iters_out) *hi_iters_out = std::min(hi_its, h.it);
  if (resnorm_out) *resnorm_out = h.res;
  MRSR_TRY(device_error_status(op_hi, err_hi, st));
  return device_error_status(op_lo, err_lo, st);
}

// ---------------------------------------------------------------------------
// CG without device allocation.
//
// mrsr_cg allocates its three work vectors from the device's stream-ordered
// pool (cudaMallocAsync) on the first solve of an operator.  Some callers cannot allow that: a host framework that
// reserves device memory up front through its own pool (Julia's CUDA.jl, a
// serving process with a fixed memory budget) or a latency-critical loop that
// forbids allocation after start-up.  mrsr_cg_noalloc runs the same kernels
// with its work vectors in one statically sized device array that is part of
// this library: every GPU that loads the library holds kNoAllocScratchBytes
// (32 MiB) for as long as the process lives, and nothing is allocated per call.
// ---------------------------------------------------------------------------
namespace mrsr {

constexpr size_t kNoAllocScratchBytes = 32u << 20;
static __device__ __align__(256) unsigned char g_cg_scratch[kNoAllocScratchBytes];

static size_t noalloc_align(size_t x) { return (x + 255) & ~size_t(255); }

// Device address of g_cg_scratch on the current device.  In host code the
// symbol is only a host-side stand-in, never a device pointer, so the address
// is looked up once per device (with that device current) and cached.
static int noalloc_scratch(unsigned char** out) {
  static std::mutex mu;
  static unsigned char* addr[64] = {nullptr};
  int dev = 0;
  MRSR_CHECK_CUDA(cudaGetDevice(&dev));
  MRSR_REQUIRE(dev >= 0 && dev < 64, MRSR_ERR_DEVICE, "device ordinal %d out of range", dev);
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    MRSR_CHECK_CUDA(cudaGetSymbolAddress(&p, g_cg_scratch));
    addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = addr[dev];
  return MRSR_OK;
}

}  // namespace mrsr

extern "C" int mrsr_cg_noalloc(mrsr_normalop* op, const float* b, float* x, int maxiter, double reltol, double abstol,
                               int* iters_out, double* resnorm_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  using namespace mrsr;
  MRSR_REQUIRE(op && b && x, MRSR_ERR_ARG, "NULL argument to mrsr_cg_noalloc");
  MRSR_REQUIRE((const void*)b != (const void*)x, MRSR_ERR_ARG, "b and x must not alias");
  MRSR_REQUIRE(maxiter >= 0, MRSR_ERR_ARG, "maxiter must be >= 0");
  const int64_t n = op->geo.nimg() * op->geo.K;
  const size_t off_part = noalloc_align(sizeof(CgState));
  const size_t off_r = noalloc_align(off_part + sizeof(double2) * kCgBlocks);
  const size_t vec = noalloc_align(sizeof(float2) * (size_t)n);
  const size_t need = off_r + 3 * vec;
  MRSR_REQUIRE(need <= kNoAllocScratchBytes, MRSR_ERR_UNSUPPORTED,
               "mrsr_cg_noalloc: the problem needs %zu bytes of work space but the static scratch holds %zu "
               "(at most %lld unknowns); use mrsr_cg",
               need, kNoAllocScratchBytes, (long long)((kNoAllocScratchBytes - off_r) / (3 * sizeof(float2))));
  unsigned char* base = nullptr;
  MRSR_TRY(noalloc_scratch(&base));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  OpUse use{op, st};
  CgState* s = reinterpret_cast<CgState*>(base);
  double2* part = reinterpret_cast<double2*>(base + off_part);
  float2* r = reinterpret_cast<float2*>(base + off_r);
  float2* u = reinterpret_cast<float2*>(base + off_r + vec);
  float2* c = reinterpret_cast<float2*>(base + off_r + 2 * vec);
  // the scratch keeps the previous call's contents: the reduction ticket must start at zero
  MRSR_CHECK_CUDA(cudaMemsetAsync(s, 0, sizeof(CgState), st));
  const float2* bb = reinterpret_cast<const float2*>(b);
  float2* xx = reinterpret_cast<float2*>(x);
  const unsigned nb = vec_blocks(n);
  k_cg_init<<<nb, kCgThreads, 0, st>>>(bb, xx, r, u, n, reltol, abstol, maxiter, s, part);
  MRSR_LAUNCH_CHECK();
  // as in cg_run: without a tolerance only an exact zero residual ends a solve early, and
  // the device's done flag already turns the iterations after it into no-ops, so the host
  // reads the state back between blocks of 8 iterations only when a tolerance is set
  const bool check = reltol > 0.0 || abstol > 0.0;
  const int chunk = 8;
  CgState h;
  for (int it0 = 0; it0 < maxiter; it0 += chunk) {
    const int nit = std::min(chunk, maxiter - it0);
    for (int k = 0; k < nit; ++k) {
      k_cg_dir<<<nb, kCgThreads, 0, st>>>(r, u, n, s);
      MRSR_LAUNCH_CHECK();
      MRSR_TRY(normalop_apply_internal(op, u, c, make_float2(1.f, 0.f), make_float2(0.f, 0.f), st));
      k_cg_alpha<<<nb, kCgThreads, 0, st>>>(u, c, n, s, part);
      MRSR_LAUNCH_CHECK();
      k_cg_update<<<nb, kCgThreads, 0, st>>>(xx, r, u, c, n, s, part);
      MRSR_LAUNCH_CHECK();
    }
    if (check && it0 + nit < maxiter) {
      MRSR_CHECK_CUDA(cudaMemcpyAsync(&h, s, sizeof(CgState), cudaMemcpyDeviceToHost, st));
      MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
      if (h.done) break;
    }
  }
  int dev_err = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&h, s, sizeof(CgState), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&dev_err, op->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  if (iters_out) *iters_out = h.it;
  if (resnorm_out) *resnorm_out = h.res;
  return device_error_status(op, dev_err, st);
}

