// Conjugate-gradient workspace and driver (cg.cu).
#pragma once
#include "common.cuh"

struct mrsr_normalop;

namespace mrsr {

struct CgWork {
  int64_t n = 0;
  int nseg = 0;     // independent systems (planes of n / nseg unknowns each)
  DevBuf r, u, c;   // residual, direction, A*direction
  DevBuf xw;        // the iterate of cg_run (copied to the caller's x at the end)
  DevBuf state;     // device CgState per system (float64 scalars, iteration count, done flag)
  DevBuf partial;   // per-block float64 partial sums, per system
  // cg_run's iterations recorded once per workspace as CUDA graphs of 8 and of 1
  // iteration (they touch only this workspace and the operator's own buffers)
  cudaGraphExec_t it8 = nullptr, it1 = nullptr;
  // the same iterations applying another operator (the reduced-precision one of a relaxed
  // solve) to this workspace's vectors; recorded for the operator whose serial is lo_serial
  cudaGraphExec_t lo8 = nullptr, lo1 = nullptr;
  uint64_t lo_serial = 0;
  cudaStream_t cap = nullptr;  // private stream the graphs are captured on
  int ensure(int64_t n, int nseg = 1);
  void drop_graphs();
  CgWork() = default;
  CgWork(const CgWork&) = delete;
  CgWork& operator=(const CgWork&) = delete;
  ~CgWork();
};

// y <- beta y + alpha A x on the operator's stream-ordered passes (normalop.cu)
int normalop_apply_internal(mrsr_normalop* op, const float2* x, float2* y, float2 alpha, float2 beta, cudaStream_t st);

// `code` is the operator's device error word as read back after a synchronisation:
// nonzero (a bounded wait inside an apply kernel gave up) clears the word on `st`
// and returns MRSR_ERR_DEVICE with a message; zero returns MRSR_OK.
int device_error_status(mrsr_normalop* op, int code, cudaStream_t st);

// nseg independent CG solves on the nseg consecutive planes of b and x (a stacked
// operator's right-hand sides); iters and res receive nseg entries
int cg_run(mrsr_normalop* op, CgWork& w, const float2* b, float2* x, int maxiter, double reltol, double abstol,
           cudaStream_t st, int* iters, double* res, int nseg = 1);

// `iters` CG iterations with no tolerance test and no host synchronisation,
// so the sequence can be recorded into a CUDA graph; op->cg must already be
// sized (CgWork::ensure).  cg_fixed_result reads the iteration count and
// residual norm after the stream has finished.
int cg_fixed_enqueue(mrsr_normalop* op, const float2* b, float2* x, int iters, cudaStream_t st);
// the same in two parts: x = 0, r = b (with the iteration limit `iters`), and one iteration;
// iterations after the limit or the tolerance return at once.  apply_op (same size; null =
// op) takes the iteration's product while the CG vectors stay in op's workspace: the relaxed
// schedule's reduced-precision iterations.
int cg_fixed_init_enqueue(mrsr_normalop* op, const float2* b, float2* x, int iters, cudaStream_t st);
int cg_fixed_iter_enqueue(mrsr_normalop* op, float2* x, cudaStream_t st, mrsr_normalop* apply_op = nullptr);
int cg_fixed_result(mrsr_normalop* op, int* iters, double* res);

}  // namespace mrsr
