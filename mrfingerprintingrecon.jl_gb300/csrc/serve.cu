// Pieces of the reconstruction server that live below the C ABI:
//
// * mrsr_normalop_share: a new operator on an existing operator's Toeplitz
//   kernel and kmask (held by reference count, never copied) with its own coil
//   maps and work stacks.  A server keeps one kernel per trajectory and basis
//   and makes a cheap operator per request from it.
// * mrsr_cg_batch_*: fixed-iteration CG solves of several independent systems
//   recorded once into one CUDA graph, one branch per system, so a batch is a
//   single graph launch and its solves overlap on the device.  With a float32
//   operator beside a fp16-storage one, each branch runs mixed-precision
//   iterative refinement with a fixed schedule instead.
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

#include "normalop.cuh"
#include "passes.cuh"

namespace mrsr {

constexpr int kVecThreads = 256;

static unsigned vec_grid(int64_t n) { return (unsigned)std::min<int64_t>(1024, std::max<int64_t>(1, cdiv(n, kVecThreads))); }

__global__ void k_sv_copy(const float2* a, float2* b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) b[i] = a[i];
}
__global__ void k_sv_zero(float2* a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = make_float2(0.f, 0.f);
}
__global__ void k_sv_add(float2* y, const float2* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = x[i];
    float2 b = y[i];
    y[i] = make_float2(b.x + a.x, b.y + a.y);
  }
}
// |a|^2, deterministic, in two launches: per-block partials (a thread's few squares in
// float32, then float64 across threads and warps), then one thread sums them in block
// order.  No per-element work runs in float64 (a small fraction of the float32 rate on
// GB300).
constexpr int kNormBlocks = 256;
static unsigned norm_grid(int64_t n) {
  return (unsigned)std::min<int64_t>(kNormBlocks, std::max<int64_t>(1, cdiv(n, 4 * kVecThreads)));
}
__global__ void k_sv_norm2_part(const float2* a, int64_t n, double* part) {
  __shared__ double wsum[kVecThreads / 32];
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    acc = fmaf(a[i].x, a[i].x, fmaf(a[i].y, a[i].y, acc));
  double d = acc;
  for (int o = 16; o > 0; o >>= 1) d += __shfl_down_sync(0xffffffffu, d, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = d;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < kVecThreads / 32; ++w) s += wsum[w];
    part[blockIdx.x] = s;
  }
}
__global__ void k_sv_norm2_fin(const double* part, int nparts, double* out) {
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += part[b];
    out[0] = s;
  }
}
static int sv_norm2(const float2* a, int64_t n, double* part, double* out, cudaStream_t st) {
  const unsigned g = norm_grid(n);
  k_sv_norm2_part<<<g, kVecThreads, 0, st>>>(a, n, part);
  MRSR_LAUNCH_CHECK();
  k_sv_norm2_fin<<<1, 32, 0, st>>>(part, (int)g, out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

}  // namespace mrsr

using namespace mrsr;

extern "C" int mrsr_normalop_share(const mrsr_normalop* src, const float* cmaps, int ncoils, int precision,
                                   mrsr_stream_t stream, mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(src, MRSR_ERR_ARG, "source operator is NULL");
  MRSR_REQUIRE(src->lam.p && src->kmask.p, MRSR_ERR_STATE, "source operator has no kernel");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  mrsr_normalop* op = new mrsr_normalop(src->store);
  const OpGeom& g = src->geo;
  int s = op_init_geometry(op, src->kind, g.ndims, g.n, g.K, cmaps ? ncoils : 1, precision);
  if (s == MRSR_OK) {
    op->lam_mode = src->lam_mode;
    op->P = src->P;
    op->nk = src->nk;
    op->TC = src->TC;
    op->FC = src->FC;
    s = op_set_cmaps(op, cmaps, st);
  }
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  mark_use(src, st);
  mark_use(op, st);
  *out = op;
  return MRSR_OK;
}

struct mrsr_cg_batch {
  struct Entry {
    mrsr_normalop* lo = nullptr;
    mrsr_normalop* hi = nullptr;
    const float2* b = nullptr;
    float2* x = nullptr;
    DevBuf r, d;   // refinement: outer residual and correction
    DevBuf part;   // refinement: per-block partial sums of a norm
  };
  std::unique_ptr<Entry[]> e;
  int ne = 0;
  DevBuf nrm;      // float64 |b|^2 and |r|^2 per entry (refinement)
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> ev;
  cudaGraph_t graph = nullptr;       // the whole schedule, or (looped) x = 0, r = b of every entry
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph_iter = nullptr;  // looped: `chunk` CG iterations of every entry
  cudaGraphExec_t exec_iter = nullptr;
  bool looped = false;
  int chunk = 1;                     // iterations per launch of graph_iter
  cudaStream_t last = nullptr;
  cudaEvent_t done = nullptr;  // recorded after each launch
  int inner = 0, outer = 0;
  int hi_iters = -1;  // >= 0: relaxed schedule (products on hi for the first hi_iters iterations)
  ~mrsr_cg_batch() {
    if (done) {
      cudaEventSynchronize(done);  // the graph and its vectors outlive its last launch
      cudaEventDestroy(done);
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (exec_iter) cudaGraphExecDestroy(exec_iter);
    if (graph_iter) cudaGraphDestroy(graph_iter);
    for (auto v : ev) cudaEventDestroy(v);
    for (auto s : branch) cudaStreamDestroy(s);
  }
};

namespace mrsr {

static int batch_branch(mrsr_cg_batch* bt, int i, cudaStream_t st) {
  mrsr_cg_batch::Entry& en = bt->e[i];
  const int64_t n = en.lo->geo.nimg() * en.lo->geo.K;
  const unsigned nb = vec_grid(n);
  if (!en.hi) return cg_fixed_enqueue(en.lo, en.b, en.x, bt->inner, st);
  if (bt->hi_iters >= 0) {
    // relaxed: one CG recurrence in hi's workspace, float32 products first
    MRSR_TRY(cg_fixed_init_enqueue(en.hi, en.b, en.x, bt->inner, st));
    for (int k = 0; k < bt->inner; ++k) MRSR_TRY(cg_fixed_iter_enqueue(en.hi, en.x, st, k < bt->hi_iters ? en.hi : en.lo));
    return MRSR_OK;
  }
  // refinement with a fixed schedule: x = 0, r = b; repeat: d = CG_lo(r), x += d, r = b - A_hi x
  double* nrm = bt->nrm.as<double>() + 2 * i;
  MRSR_TRY(sv_norm2(en.b, n, en.part.as<double>(), nrm, st));
  k_sv_zero<<<nb, kVecThreads, 0, st>>>(en.x, n);
  MRSR_LAUNCH_CHECK();
  k_sv_copy<<<nb, kVecThreads, 0, st>>>(en.b, en.r.as<float2>(), n);
  MRSR_LAUNCH_CHECK();
  for (int o = 0; o < bt->outer; ++o) {
    MRSR_TRY(cg_fixed_enqueue(en.lo, en.r.as<float2>(), en.d.as<float2>(), bt->inner, st));
    k_sv_add<<<nb, kVecThreads, 0, st>>>(en.x, en.d.as<float2>(), n);
    MRSR_LAUNCH_CHECK();
    k_sv_copy<<<nb, kVecThreads, 0, st>>>(en.b, en.r.as<float2>(), n);
    MRSR_LAUNCH_CHECK();
    MRSR_TRY(normalop_apply_internal(en.hi, en.x, en.r.as<float2>(), make_float2(-1.f, 0.f), make_float2(1.f, 0.f), st));
  }
  MRSR_TRY(sv_norm2(en.r.as<float2>(), n, en.part.as<double>(), nrm + 1, st));
  return MRSR_OK;
}

// Capture body(i, stream) of every entry as parallel branches of one graph.
template <class F>
static int batch_capture(mrsr_cg_batch* bt, F body, cudaGraph_t* graph, cudaGraphExec_t* exec) {
  const int n = bt->ne;
  // capture on a private stream so the caller's stream is never in capture mode
  cudaStream_t cap = bt->branch[0];
  MRSR_CHECK_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  int s = MRSR_OK;
  cudaError_t ce = cudaEventRecord(bt->ev[n], cap);
  for (int i = 1; i < n && ce == cudaSuccess; ++i) ce = cudaStreamWaitEvent(bt->branch[i], bt->ev[n], 0);
  for (int i = 0; i < n && ce == cudaSuccess && s == MRSR_OK; ++i) s = body(i, bt->branch[i]);
  for (int i = 1; i < n && ce == cudaSuccess && s == MRSR_OK; ++i) {
    ce = cudaEventRecord(bt->ev[i], bt->branch[i]);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(cap, bt->ev[i], 0);
  }
  cudaGraph_t g = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(cap, &g);
  if (s != MRSR_OK) {
    if (g) cudaGraphDestroy(g);
    return s;
  }
  if (ce != cudaSuccess || ee != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    set_error("graph capture of the CG batch failed: %s", cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    return MRSR_ERR_CUDA;
  }
  *graph = g;
  MRSR_CHECK_CUDA(cudaGraphInstantiate(exec, g, 0));
  return MRSR_OK;
}

static int batch_build(mrsr_cg_batch* bt, cudaStream_t st) {
  const int n = bt->ne;
  bt->branch.resize(n, nullptr);
  bt->ev.resize(n + 1, nullptr);
  for (int i = 0; i < n; ++i) MRSR_CHECK_CUDA(cudaStreamCreateWithFlags(&bt->branch[i], cudaStreamNonBlocking));
  for (int i = 0; i <= n; ++i) MRSR_CHECK_CUDA(cudaEventCreateWithFlags(&bt->ev[i], cudaEventDisableTiming));
  (void)st;
  bool plain = true;
  for (int i = 0; i < n; ++i) plain = plain && !bt->e[i].hi;
  if (!plain)  // refinement: the whole fixed schedule in one graph
    return batch_capture(
        bt, [&](int i, cudaStream_t s) { return batch_branch(bt, i, s); }, &bt->graph, &bt->exec);
  // plain CG: an init graph and a graph of `chunk` iterations launched until `inner` are
  // done.  Capture and instantiation cost grows with the node count (a 32-branch x
  // 100-iteration schedule: 19k nodes, ~50 ms to build, 4 ms to run), launches cost a
  // fixed overhead each, so chunks of about 2k nodes balance the two.  Iterations past
  // the limit return at once on the device.
  bt->looped = true;
  bt->chunk = std::max(1, std::min(bt->inner, 2048 / (6 * n)));
  MRSR_TRY(batch_capture(
      bt,
      [&](int i, cudaStream_t s) {
        const mrsr_cg_batch::Entry& en = bt->e[i];
        return cg_fixed_init_enqueue(en.lo, en.b, en.x, bt->inner, s);
      },
      &bt->graph, &bt->exec));
  return batch_capture(
      bt,
      [&](int i, cudaStream_t s) {
        for (int k = 0; k < bt->chunk; ++k) MRSR_TRY(cg_fixed_iter_enqueue(bt->e[i].lo, bt->e[i].x, s));
        return (int)MRSR_OK;
      },
      &bt->graph_iter, &bt->exec_iter);
}

}  // namespace mrsr

namespace mrsr {

static int batch_create(mrsr_normalop* const* ops_lo, mrsr_normalop* const* ops_hi, const float* const* b,
                        float* const* x, int n, int inner_iters, int outer_steps, int hi_iters, cudaStream_t st,
                        mrsr_cg_batch** out) {
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(ops_lo && b && x && n >= 1, MRSR_ERR_ARG, "empty or NULL batch");
  MRSR_REQUIRE(inner_iters >= 1, MRSR_ERR_ARG, "inner_iters must be >= 1");
  mrsr_cg_batch* bt = new mrsr_cg_batch();
  bt->inner = inner_iters;
  bt->outer = std::max(outer_steps, 1);
  bt->hi_iters = hi_iters;
  bt->e.reset(new mrsr_cg_batch::Entry[n]);
  bt->ne = n;
  int s = MRSR_OK;
  for (int i = 0; i < n && s == MRSR_OK; ++i) {
    mrsr_cg_batch::Entry& en = bt->e[i];
    en.lo = ops_lo[i];
    en.hi = ops_hi ? ops_hi[i] : nullptr;
    en.b = reinterpret_cast<const float2*>(b[i]);
    en.x = reinterpret_cast<float2*>(x[i]);
    if (!en.lo || !en.b || !en.x) {
      set_error("NULL operator or vector in batch entry %d", i);
      s = MRSR_ERR_ARG;
      break;
    }
    if ((const void*)en.b == (const void*)en.x) {
      set_error("b and x alias in batch entry %d", i);
      s = MRSR_ERR_ARG;
      break;
    }
    const int64_t nv = en.lo->geo.nimg() * en.lo->geo.K;
    if (en.hi && (en.hi->geo.nimg() != en.lo->geo.nimg() || en.hi->geo.K != en.lo->geo.K)) {
      set_error("batch entry %d: operators of different sizes", i);
      s = MRSR_ERR_ARG;
      break;
    }
    // branches run concurrently: no operator may appear twice (shared stacks / CG vectors)
    for (int j = 0; j < i && s == MRSR_OK; ++j) {
      const mrsr_cg_batch::Entry& o = bt->e[j];
      if (o.lo == en.lo || o.lo == en.hi || (o.hi && (o.hi == en.lo || o.hi == en.hi))) {
        set_error("batch entries %d and %d share an operator", j, i);
        s = MRSR_ERR_ARG;
      }
    }
    if (s != MRSR_OK) break;
    if (hi_iters >= 0) {
      if (!en.hi) {
        set_error("relaxed batch entry %d has no float32 operator", i);
        s = MRSR_ERR_ARG;
        break;
      }
      s = en.hi->cg.ensure(nv);  // the recurrence's vectors
      continue;
    }
    s = en.lo->cg.ensure(nv);
    if (s == MRSR_OK && en.hi) s = en.r.alloc(sizeof(float2) * nv);
    if (s == MRSR_OK && en.hi) s = en.d.alloc(sizeof(float2) * nv);
    if (s == MRSR_OK && en.hi) s = en.part.alloc(sizeof(double) * kNormBlocks);
  }
  if (s == MRSR_OK) s = bt->nrm.alloc(sizeof(double) * 2 * n);
  if (s == MRSR_OK) {
    const cudaError_t e = cudaMemsetAsync(bt->nrm.p, 0, sizeof(double) * 2 * n, st);
    if (e != cudaSuccess) {
      set_error("cudaMemset: %s", cudaGetErrorString(e));
      s = MRSR_ERR_CUDA;
    }
  }
  if (s == MRSR_OK && cudaEventCreateWithFlags(&bt->done, cudaEventDisableTiming) != cudaSuccess) {
    set_error("cudaEventCreate failed");
    s = MRSR_ERR_CUDA;
  }
  // work vectors were allocated on `st`; the graph's branches run on other streams
  if (s == MRSR_OK && cudaStreamSynchronize(st) != cudaSuccess) {
    set_error("cudaStreamSynchronize failed");
    s = MRSR_ERR_CUDA;
  }
  if (s == MRSR_OK) s = batch_build(bt, st);
  if (s != MRSR_OK) {
    delete bt;
    return s;
  }
  *out = bt;
  return MRSR_OK;
}

}  // namespace mrsr

extern "C" int mrsr_cg_batch_create(mrsr_normalop* const* ops_lo, mrsr_normalop* const* ops_hi,
                                    const float* const* b, float* const* x, int n, int inner_iters, int outer_steps,
                                    mrsr_stream_t stream, mrsr_cg_batch** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  return batch_create(ops_lo, ops_hi, b, x, n, inner_iters, outer_steps, -1, reinterpret_cast<cudaStream_t>(stream),
                      out);
}

extern "C" int mrsr_cg_batch_create_relaxed(mrsr_normalop* const* ops_lo, mrsr_normalop* const* ops_hi,
                                            const float* const* b, float* const* x, int n, int iters, int hi_iters,
                                            mrsr_stream_t stream, mrsr_cg_batch** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(ops_hi, MRSR_ERR_ARG, "a relaxed batch needs the float32 operators");
  MRSR_REQUIRE(hi_iters >= 0 && hi_iters <= iters, MRSR_ERR_ARG, "hi_iters must be in [0, iters]");
  return batch_create(ops_lo, ops_hi, b, x, n, iters, 1, hi_iters, reinterpret_cast<cudaStream_t>(stream), out);
}

extern "C" int mrsr_cg_batch_launch(mrsr_cg_batch* bt, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(bt && bt->exec, MRSR_ERR_ARG, "batch is NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  MRSR_CHECK_CUDA(cudaGraphLaunch(bt->exec, st));
  if (bt->looped)
    for (int k = 0; k < bt->inner; k += bt->chunk) MRSR_CHECK_CUDA(cudaGraphLaunch(bt->exec_iter, st));
  bt->last = st;
  MRSR_CHECK_CUDA(cudaEventRecord(bt->done, st));
  for (int i = 0; i < bt->ne; ++i) {
    MRSR_TRY(mark_use(bt->e[i].lo, st));
    if (bt->e[i].hi) MRSR_TRY(mark_use(bt->e[i].hi, st));
  }
  return MRSR_OK;
}

extern "C" int mrsr_cg_batch_result(mrsr_cg_batch* bt, int i, int* iters_out, double* resnorm_out) {
  MRSR_REQUIRE(bt, MRSR_ERR_ARG, "batch is NULL");
  MRSR_REQUIRE(i >= 0 && i < bt->ne, MRSR_ERR_ARG, "entry %d out of range", i);
  if (bt->last) MRSR_CHECK_CUDA(cudaEventSynchronize(bt->done));
  const mrsr_cg_batch::Entry& en = bt->e[i];
  if (!en.hi) {
    return cg_fixed_result(en.lo, iters_out, resnorm_out);
  }
  if (bt->hi_iters >= 0) {
    MRSR_TRY(cg_fixed_result(en.hi, iters_out, resnorm_out));
    int lo_err = 0;
    MRSR_CHECK_CUDA(cudaMemcpy(&lo_err, en.lo->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
    return device_error_status(en.lo, lo_err, call_stream());
  }
  double h[2];
  int dev_err[2] = {0, 0};
  MRSR_CHECK_CUDA(cudaMemcpy(h, bt->nrm.as<double>() + 2 * i, sizeof(h), cudaMemcpyDeviceToHost));
  MRSR_CHECK_CUDA(cudaMemcpy(&dev_err[0], en.lo->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
  MRSR_CHECK_CUDA(cudaMemcpy(&dev_err[1], en.hi->errflag.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (iters_out) *iters_out = bt->outer;
  if (resnorm_out) *resnorm_out = h[0] > 0 ? std::sqrt(h[1] / h[0]) : 0.0;
  MRSR_TRY(device_error_status(en.lo, dev_err[0], call_stream()));
  return device_error_status(en.hi, dev_err[1], call_stream());
}

extern "C" void mrsr_cg_batch_destroy(mrsr_cg_batch* bt) { delete bt; }
