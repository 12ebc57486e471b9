// Kernel arguments of the apply passes and the per-voxel K x K product,
// shared by the generic (Stockham) and the register four-step kernels.
#pragma once
#include "normalop.cuh"

namespace mrsr {

constexpr int KMAX = 8;        // largest subspace rank compiled into the contraction
constexpr int kStackMax = 64;  // most right-hand sides of a stacked operator (mrsr_normalop_stack)

struct RowsFwdArgs {
  FftPlan pl;        // along dim 1, L = g1
  int n1;            // valid input length (image dim 1)
  int64_t nrows;     // rows per plane: n2 * n3
  int rpc;           // rows per CTA
  int K;
  int c0;            // first coil of the group
  int lstride;       // smem line stride (float2)
  const float2* x;   // (n1, nrows, K)
  const float2* cmaps;  // (n1, nrows, ncoils) or null
  float2* out;       // [cl][k][row][L]
};

struct LamPassArgs {
  FftPlan pl;          // along the last dim
  int nin, nout;       // valid input rows / kept output rows (same storage rows: nrow)
  int nrow;            // stored rows of a plane along the last dim
  int64_t inner;       // stored plane width (contiguous)
  int TC, K, P;
  int lam_mode;
  int lstride;         // = L * TC (+ pad)
  const void* lam;     // [tile][chunk][P][FC][TC]
  float2* stack;       // planes [cl][k][row][inner], in place
  int FC, NCH;         // Λ chunk: frequencies per chunk, chunks per tile (L = FC * NCH)
  int ncg = 1;         // coils of the launch (four-step kernel: block = tile * ncg + coil)
  FastDiv fcd;         // division by FC
};

// Element (tile, frequency f, column li, entry p) of the chunked Λ layout;
// consecutive p are FC*TC apart.
__host__ __device__ __forceinline__ int64_t lam_elem(int64_t tile, int f, int li, int p, int TC, int P, int FC, int NCH) {
  const int ch = f / FC, fc = f - ch * FC;
  return (((tile * NCH + ch) * P + p) * (int64_t)FC + fc) * TC + li;
}

struct MidArgs {
  FftPlan pl;        // along dim 2
  int nin, nout;     // valid input rows / kept output rows along dim 2
  int64_t width;     // contiguous extent (g1)
  int64_t n3;        // outer count (image dim 3)
  int TC, NOo;       // columns and outer slices per CTA
  int lstride;
  float sgn;
  const float2* in;  // planes [p][i3][nin][width]
  float2* out;       // planes [p][i3][nout][width]
};

struct RowsInvArgs {
  FftPlan pl;        // along dim 1
  int n1;            // kept output length
  int64_t nrows;
  int rpc;
  int K;
  int c0, ncg;       // coils of this group
  int lstride;
  int first;         // first coil group: apply beta
  float2 alpha;      // alpha / prod(grid)
  float2 beta;
  const float2* stack;  // [cl][k][row][L]
  const float2* cmaps;  // (n1, nrows, ncoils) or null
  float2* y;            // (n1, nrows, K)
};

// Stacked right-hand sides: v <- λ v with the plane-independent scalar kernel entry at idx.
__device__ __forceinline__ float2 lam_diag_entry(int mode, const void* lam, int64_t idx) {
  return mode == LAM_DIAG_REAL ? make_float2(reinterpret_cast<const float*>(lam)[idx], 0.f)
                               : reinterpret_cast<const float2*>(lam)[idx];
}

// Per-voxel K x K product Y = Λ X at one frequency (X, Y in registers).
// lam points at entry p = 0 of this voxel; consecutive entries are pstride apart.
template <int KM>
__device__ __forceinline__ void lam_apply_ptr(int mode, int K, const void* lamv, int64_t lbase, int64_t pstride,
                                              const float2* X, float2* Y) {
#pragma unroll
  for (int j = 0; j < KM; ++j) Y[j] = make_float2(0.f, 0.f);
  if (mode == LAM_PACKED_REAL) {
    const float* lam = reinterpret_cast<const float*>(lamv) + lbase;
    int p = 0;
#pragma unroll
    for (int k2 = 0; k2 < KM; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 <= k2; ++k1) {
        if (k2 < K) {
          const float l = lam[p * pstride];
          Y[k1].x += l * X[k2].x;
          Y[k1].y += l * X[k2].y;
          if (k1 != k2) {
            Y[k2].x += l * X[k1].x;
            Y[k2].y += l * X[k1].y;
          }
        }
        ++p;
      }
    }
  } else if (mode == LAM_PACKED_CPLX) {
    const float2* lam = reinterpret_cast<const float2*>(lamv) + lbase;
    int p = 0;
#pragma unroll
    for (int k2 = 0; k2 < KM; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 <= k2; ++k1) {
        if (k2 < K) {
          const float2 l = lam[p * pstride];
          Y[k1] = cadd(Y[k1], cmul(l, X[k2]));
          if (k1 != k2) Y[k2] = cadd(Y[k2], cmul(cconj(l), X[k1]));
        }
        ++p;
      }
    }
  } else {
    const float2* lam = reinterpret_cast<const float2*>(lamv) + lbase;
#pragma unroll
    for (int k2 = 0; k2 < KM; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 < KM; ++k1) {
        if (k1 < K && k2 < K) {
          const float2 l = lam[(k1 + K * k2) * pstride];
          Y[k1] = cadd(Y[k1], cmul(l, X[k2]));
        }
      }
    }
  }
}

// Y = Λ X at one voxel for the packed real kernel, Λ values already in registers.
template <int K>
__device__ __forceinline__ void lam_real_regs(const float* l, const float2* X, float2* Y) {
#pragma unroll
  for (int k = 0; k < K; ++k) Y[k] = make_float2(0.f, 0.f);
  int p = 0;
#pragma unroll
  for (int k2 = 0; k2 < K; ++k2)
#pragma unroll
    for (int k1 = 0; k1 <= k2; ++k1, ++p) {
      Y[k1].x = fmaf(l[p], X[k2].x, Y[k1].x);
      Y[k1].y = fmaf(l[p], X[k2].y, Y[k1].y);
      if (k1 != k2) {
        Y[k2].x = fmaf(l[p], X[k1].x, Y[k2].x);
        Y[k2].y = fmaf(l[p], X[k1].y, Y[k2].y);
      }
    }
}

template <int KM>
__device__ __forceinline__ void lam_apply(const LamPassArgs& a, int64_t lbase, int64_t pstride, const float2* X,
                                          float2* Y) {
  lam_apply_ptr<KM>(a.lam_mode, a.K, a.lam, lbase, pstride, X, Y);
}

// Four-step fast paths (apply_fast.cu): return MRSR_ERR_UNSUPPORTED when the
// transform length has no compiled split, so the caller uses the generic kernels.
bool fast_length(int L);
int fast_rows_fwd(const RowsFwdArgs& a, int64_t nrows, int ncg, cudaStream_t st);
int fast_lambda(const LamPassArgs& a, int ncg, int planes_total, int* errword, cudaStream_t st);
// three-step Λ pass (apply_lam8.cu): 256- or 512-point lines pruned to half, 4- or 8-column tiles, K <= 6
bool lambda8_supported(const LamPassArgs& a);
int fast_lambda8(const LamPassArgs& a, int ncg, cudaStream_t st);
// three-step inverse row pass (apply_rows8.cu): 256- or 512-point rows of the zero-padded
// half, <= 20 coils per group
bool rows8_inv_supported(const RowsInvArgs& a);
int fast_rows8_inv(const RowsInvArgs& a, cudaStream_t st);
int fast_mid(const MidArgs& a, int nplanes, cudaStream_t st);
int fast_rows_inv(const RowsInvArgs& a, int64_t nrows, cudaStream_t st);

// tensor-core Λ pass (apply_tc.cu): 512-point pruned column transforms on 4-column tiles
bool tc_lambda_supported(int L, int nin, int nout, int inner, int K);
int tc_lambda(const LamPassArgs& a, int ncg, const float* lam_max, const void* consts, int* errword,
              cudaStream_t st);
int tc_build_constants(void* out, cudaStream_t st);  // DFT-64 operand + twiddles, tc_constants_bytes()
size_t tc_constants_bytes();
int tc_lambda_bound(const void* lam, size_t bytes, float* out, cudaStream_t st);
bool tc_rows_supported(int L, int n1, int ncg);
int tc_rows_inv(const RowsInvArgs& a, const void* consts, int* errword, cudaStream_t st);
int tc_lambda_layout(const void* lam, void* out, int64_t inner, int P, int FC, int NCH, int TC, bool real,
                     cudaStream_t st);

// fp16-storage operator (apply_half.cu)
bool half_supported(const mrsr_normalop* op);
int half_lambda_convert(mrsr_normalop* op, cudaStream_t st);
int half_alloc_scales(mrsr_normalop* op);
int apply_half_impl(mrsr_normalop* op, const float2* x, float2* y, float2 alpha, float2 beta, cudaStream_t st,
                    void (*record)(void*), void* rec_ctx);

}  // namespace mrsr
