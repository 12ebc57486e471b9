// Internal state of a subspace Toeplitz normal operator handle.
#pragma once
#include <atomic>
#include <memory>

#include "cg.cuh"
#include "fft.cuh"

namespace mrsr {

// How the per-voxel K x K kernel is stored.
enum LamMode : int {
  LAM_PACKED_REAL = 0,  // P = K(K+1)/2 reals, symmetric (real basis, ext:140-191)
  LAM_PACKED_CPLX = 1,  // P complex, Hermitian upper triangle (ext:89-137)
  LAM_FULL_CPLX = 2,    // K*K complex, column-major (FFTNormalOp, src/FFTNormalOp.jl:331)
  // an operator on stacked right-hand sides (mrsr_normalop_stack): K planes, each
  // transformed by the same scalar kernel of a rank-1 operator (P = 1)
  LAM_DIAG_REAL = 3,
  LAM_DIAG_CPLX = 4
};
__host__ __device__ inline bool lam_is_diag(int mode) { return mode == LAM_DIAG_REAL || mode == LAM_DIAG_CPLX; }
__host__ __device__ inline bool lam_is_real(int mode) { return mode == LAM_PACKED_REAL || mode == LAM_DIAG_REAL; }

struct OpGeom {
  int ndims = 2;
  int64_t n[3] = {1, 1, 1};  // image shape
  int64_t g[3] = {1, 1, 1};  // FFT grid (2n for the NFFT operator, n for the FFT operator)
  int K = 1;
  int ncoils = 1;
  int64_t nimg() const { return n[0] * n[1] * n[2]; }
  int64_t ngrid() const { return g[0] * g[1] * g[2]; }
  // Λ-pass (last axis) tiling
  int64_t inner() const { return ndims == 2 ? g[0] : g[0] * g[1]; }
  int64_t glast() const { return g[ndims - 1]; }
  int64_t nlast() const { return n[ndims - 1]; }
};

// The Toeplitz kernel and its kmask, shared (read-only) by every operator
// made from it with mrsr_normalop_share.
struct LamStore {
  DevBuf kmask;      // int64 nk, 1-based column-major grid indices
  DevBuf lam;        // [tile][chunk][P][FC][TC] of float / float2 (chunked along f_last)
  DevBuf lam_scale;  // fp16: one float per tile
  DevBuf lam_half;   // fp16: the chunked kernel in half precision
  DevBuf lam_max;    // fp16-tc: largest |component| of Λ (float)
  DevBuf lam_tc;     // fp16-tc: Λ rearranged for the tensor-core Λ pass
  DevBuf tc_consts;  // fp16-tc: DFT-64 MMA operand and twiddles
};

}  // namespace mrsr

namespace mrsr {
// Device copies of x and y for host-buffer applies (mrsr_normalop_apply_host), made on first use.
struct HostIo {
  DevBuf x, y;
};
}  // namespace mrsr

struct mrsr_normalop {
  mrsr_normalop() : mrsr_normalop(std::make_shared<mrsr::LamStore>()) {}
  explicit mrsr_normalop(std::shared_ptr<mrsr::LamStore> s)
      : store(std::move(s)), kmask(store->kmask), lam(store->lam), lam_scale(store->lam_scale),
        lam_half(store->lam_half), lam_max(store->lam_max), lam_tc(store->lam_tc), tc_consts(store->tc_consts) {}
  mrsr_normalop(const mrsr_normalop&) = delete;
  mrsr_normalop& operator=(const mrsr_normalop&) = delete;

  int kind = MRSR_KIND_NFFT;
  int precision = MRSR_PREC_FP32;
  mrsr::OpGeom geo;
  int lam_mode = mrsr::LAM_PACKED_CPLX;
  int P = 1;      // kernel entries per voxel in the internal layout
  int64_t nk = 0;
  int TC = 4;     // Λ-pass tile width (columns)
  int FC = 1;     // Λ chunk length along the last dim
  int Cg = 1;     // coils per group
  int launches = 0;
  // process-unique id (never reused, unlike the address): CG workspaces key the graphs they
  // recorded with another operator's apply by it
  uint64_t serial = next_serial();
  static uint64_t next_serial() {
    static std::atomic<uint64_t> n{0};
    return ++n;
  }
  std::shared_ptr<mrsr::LamStore> store;
  mrsr::DevBuf& kmask;
  mrsr::DevBuf& lam;
  mrsr::DevBuf& lam_scale;
  mrsr::DevBuf& lam_half;
  mrsr::DevBuf& lam_max;   // the fp16-tc members are built once per kernel and shared
  mrsr::DevBuf& lam_tc;
  mrsr::DevBuf& tc_consts;
  mrsr::DevBuf cmaps;      // (img..., ncoils) complex; empty = unit coil
  mrsr::DevBuf stack1, stack2;  // intermediates of one coil group
  mrsr::DevBuf scale1, scale2;  // fp16 per-line scales
  mrsr::DevBuf errflag;         // device int
  mrsr::FftPlanHost plan[3];
  mrsr::CgWork cg;              // CG vectors, allocated on first solve
  mrsr::HostIo hio;             // host-buffer applies
  // recorded after every call that enqueues work on the operator; the
  // destructor frees the buffers only after it (stream-ordered, no device sync)
  cudaEvent_t last_use = nullptr;
  ~mrsr_normalop();
};

namespace mrsr {
// Build helpers shared by the constructors (normalop.cu).
// kmax: the largest K accepted (the rank limit of the K x K contraction unless the
// operator is a stacked one, whose planes are independent)
int op_init_geometry(mrsr_normalop* op, int kind, int ndims, const int64_t* img_shape, int K,
                     int ncoils, int precision, int kmax = 8);
int op_set_cmaps(mrsr_normalop* op, const float* cmaps, cudaStream_t st);
int op_finalize(mrsr_normalop* op, cudaStream_t st);
// Λ from the reference's packed (P, nk) layout at 1-based kmask cells.
int op_set_lambda_packed(mrsr_normalop* op, const void* lam_packed, int is_complex, const int64_t* kmask,
                         int64_t nk, cudaStream_t st);
// Λ of an FFT operator from the reference's full (K, K, grid...) complex array; kmask = Λ[1,1,:] .!= 0.
int op_set_lambda_full(mrsr_normalop* op, const float2* lam_full, cudaStream_t st);
// record op->last_use on `st` (the work enqueued so far on st may use op)
int mark_use(const mrsr_normalop* op, cudaStream_t st);
// marks the operator's use when the entry point returns
struct OpUse {
  const mrsr_normalop* op;
  cudaStream_t st;
  ~OpUse() {
    if (op) mark_use(op, st);
  }
};
// Stream compaction: 1-based indices of nonzero flags, sorted.
int compact_nonzero(const uint8_t* flags, int64_t n, DevBuf& out, int64_t* count, cudaStream_t st);
}  // namespace mrsr
