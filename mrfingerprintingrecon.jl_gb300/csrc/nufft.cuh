// Non-uniform FFT building blocks (exponential-of-semicircle kernel).
//
// Type 1 (adjoint):  F(j) = sum_n v_n exp(+2 pi i j . k_n)
// Type 2 (forward):  y_n  = sum_j f(j) exp(-2 pi i j . k_n)
// with k_n in [-0.5, 0.5]^d (the reference's trajectory units).  The grid is
// oversampled by 2 (M = 2 * modes per dimension); spreading uses the ES
// kernel phi(z) = exp(beta (sqrt(1 - z^2) - 1)) of width w = 8 cells and
// beta = 2.30 w (Barnett, Magland, af Klinteberg, SIAM J. Sci. Comput. 41,
// 2019), with the Fourier-side correction 1 / psi_hat(j) obtained by
// Gauss-Legendre quadrature.
#pragma once
#include "fftnd.cuh"

namespace mrsr {

constexpr int kEsWidth = 8;
constexpr float kEsBeta = 2.30f * kEsWidth;

// Samples of a (trajectory, mask) pair in the order trj[:, sample_mask] takes them.
struct SampleSet {
  const float* trj = nullptr;    // (d, ns_pf, nt) column-major
  int d = 2;
  int64_t ns_pf = 0, nt = 0;
  const int64_t* list = nullptr; // 1-based linear (s + ns_pf t) indices of kept samples, or null = all
  int64_t n = 0;                 // kept samples
};

// Owner of a compacted sample list.
struct SampleList {
  DevBuf list;
  SampleSet set;
  int init(int d, const float* trj, int64_t ns_pf, int64_t nt, const uint8_t* mask, cudaStream_t st);
};

// Tap weights of one sample: lane i < w*d computes the weight of tap (i % w)
// of dimension i / w; the first tap index per dimension is l0[d].
// u = k M (float32 k, integer M < 2^24) is carried exactly as uh + ul with
// ul = fma(k, M, -uh), so the first tap l = ceil(u - w/2) is exact and the
// kernel argument z = (l + t - u) / (w/2) is rounded once, all in float32
// arithmetic (float64 is a small fraction of float32 throughput on this GPU):
// with f = floor(uh) and r = (uh - f) + ul, u = f + r, r in (-1, 1), so
// l = f - w/2 + [r > 0] and z = ([r > 0] - w/2 + t - r) / (w/2).
__device__ __forceinline__ void es_lane_weight(const float* kd, const int64_t* M, int d, int lane, float* wt_out,
                                               int64_t* l0) {
  const int hw = kEsWidth / 2;
  float wt = 0.f;
#pragma unroll
  for (int dd = 0; dd < 3; ++dd) {
    if (dd < d) {
      const float m = (float)M[dd];
      const float uh = kd[dd] * m;
      const float ul = fmaf(kd[dd], m, -uh);
      const float f = floorf(uh);
      const float r = (uh - f) + ul;
      const int c = r > 0.f ? 1 : 0;
      l0[dd] = (int64_t)f - hw + c;
      if (lane / kEsWidth == dd) {
        const int t = lane % kEsWidth;
        const float z = ((float)(c - hw + t) - r) * (1.f / hw);
        wt = (fabsf(z) < 1.f) ? expf(kEsBeta * (sqrtf(1.f - z * z) - 1.f)) : 0.f;
      }
    }
  }
  *wt_out = wt;
}

// Deconvolution factors 1/psi_hat(j) for j = jmin .. jmin + count - 1 on an upsampled grid of size M.
int es_inv_psi_table(int64_t M, int64_t jmin, int64_t count, DevBuf& out);

// grid[ch][cell] += sum over samples of value(ch, n) * phi taps, cells column-major on dims M.
// value(ch, n): Λ precompute channels (pairs of basis columns) or data channels.
struct SpreadLambdaArgs {
  SampleSet S;
  int64_t M[3], cells;
  const void* U;      // (nt, K) real or complex
  int u_complex, K;
  int P;              // channels: packed pairs k1 <= k2
  int p0, np;         // spread only channels p0 .. p0+np-1
  float2* grid;       // [np][cells]
};
int spread_lambda(const SpreadLambdaArgs& a, cudaStream_t st);

struct SpreadDataArgs {
  SampleSet S;
  int64_t M[3], cells;
  const float2* data;   // (ns_pf, nt, ncoils)
  int c0, nc;           // coil range
  const void* U;        // (nt, K) or null (identity)
  int u_complex, K;
  int dcf_kind;
  const float* dcf;     // per kept sample (dcf_kind == array)
  float2* grid;         // [(c - c0) * K + k][cells]
};
int spread_data(const SpreadDataArgs& a, cudaStream_t st);

}  // namespace mrsr
