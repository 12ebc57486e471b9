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
      const float uh = __fmul_rn(kd[dd], m);   // intrinsics: no contraction, so every kernel
      const float ul = fmaf(kd[dd], m, -uh);   // that locates a sample's first tap agrees
      const float f = floorf(uh);
      const float r = __fadd_rn(__fsub_rn(uh, f), ul);
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

// Deconvolution factors 1/psi_hat(j) for j = jmin .. jmin + count - 1 on an upsampled grid
// of size M: a device table of the current device, cached for the life of the process.
int es_inv_psi_table(int64_t M, int64_t jmin, int64_t count, const float** out);

// Fixed-point accumulation of the spread grids.  Each tap's term (a float32 product of
// the sample value and the kernel weights) is scaled by 2^e, rounded to an integer and
// added to a 64-bit grid with integer atomics.  Integer addition is associative, so every
// cell holds the exact sum of its rounded terms whatever order the samples land in: the
// grids are bitwise reproducible run to run, and the sum carries no accumulation error (a
// float32 atomic sum of n terms drifts by ~sqrt(n) float32 roundings of the running total,
// a float64 one by ~n float64 roundings).  e = min(62 - ceil(log2(n_terms max|term|)),
// 40 - ceil(log2(max|term|))) from a device-side bound: no cell sum can leave 63 bits, no
// term reaches 2^40 (a resolution of 2^-40 of the largest term, far below float32's).
//
// A term is never converted with __float2ll_rn, whose rate on this GPU is that of its
// narrow float64 pipe (~0.4 T/s measured; it bounded the spreading kernels).  With a = term
// * 2^-21 (|a| < 2^19) it is split as round(a) * 2^21 + round((a - round(a)) * 2^21), both
// parts rounded by adding 1.5 * 2^23 in float32 (the sum's low mantissa bits are then the
// rounded integer), which takes two float adds, one fma and two integer subtractions.
constexpr int kFxLoBits = 21;
constexpr int kFxTermBits = 40;

struct FixedScale {
  float scale;   // 2^(e - kFxLoBits): value * scale = a
  float inv;     // 2^-e
};

__device__ __forceinline__ void fx_split(float a, int& hi, int& lo) {
  constexpr float kMagic = 12582912.f;  // 1.5 * 2^23
  constexpr int kMagicBits = 0x4B400000;
  const float s1 = __fadd_rn(a, kMagic);
  hi = __float_as_int(s1) - kMagicBits;                    // round(a), |a| < 2^22
  const float d = __fsub_rn(a, __fsub_rn(s1, kMagic));     // a - round(a), exact, |d| <= 1/2
  lo = __float_as_int(__fmaf_rn(d, (float)(1 << kFxLoBits), kMagic)) - kMagicBits;  // |lo| <= 2^20
}

// fx_split of the product a = x * y, the first rounding fused into the product
__device__ __forceinline__ void fx_split_prod(float x, float y, int& hi, int& lo) {
  constexpr float kMagic = 12582912.f;
  constexpr int kMagicBits = 0x4B400000;
  const float s1 = __fmaf_rn(x, y, kMagic);
  hi = __float_as_int(s1) - kMagicBits;                          // round(x y)
  const float d = __fmaf_rn(x, y, -__fsub_rn(s1, kMagic));       // x y - round(x y), |d| <= 1/2
  lo = __float_as_int(__fmaf_rn(d, (float)(1 << kFxLoBits), kMagic)) - kMagicBits;
}

__device__ __forceinline__ long long fx_term(float a) {
  int hi, lo;
  fx_split(a, hi, lo);
  return (long long)hi * (1ll << kFxLoBits) + lo;
}

// grid[ch][part][cell] (part: re, and im for complex grids) += value(ch, n) * phi taps,
// cells column-major on dims M, in units of 2^-e.
// value(ch, n): Λ precompute channels (pairs of basis columns) or data channels.
struct SpreadLambdaArgs {
  SampleSet S;
  int64_t M[3], cells;
  const void* U;      // (nt, K) real or complex
  int u_complex, K;
  int P;              // channels: packed pairs k1 <= k2
  int p0, np;         // spread only channels p0 .. p0+np-1
  int nq;             // parts per cell: 1 (real basis: the spread values are real) or 2
  long long* q;       // [np][nq][cells]
  const FixedScale* fs;
};
// Samples of a 2D set counting-sorted by the 12 x 12 tile of the grid M0 x M1 that holds
// their first tap, in chunks of at most 1024 samples (the work items of the tile-sorted
// spreading kernels).  Built once per sample set and grid, shared by every spread of it.
// build3: for a 3D set, `order` and work items by 8 x 8 x 8 tiles (the global kernels take
// samples in that order, so the warps in flight touch neighbouring grid lines in L2; the
// 3D tile-sorted kernel takes the items).
// prep: the per-sample tap records the 2D tile-sorted kernels read (weights with the
// density compensation folded in, first tap, sample index and frame), after build.
// prep3: the same records for the 3D tile-sorted kernels, after build3.
struct TileSort {
  DevBuf counts, offset, choff, cursor, tile_of, order, items, nitems, next, rec;
  int ntx = 0, nty = 0, ntiles = 0, m0 = 0, m1 = 0, m2 = 0;
  bool rec3 = false;
  int build(const SampleSet& S, int64_t M0, int64_t M1, cudaStream_t st);
  int build3(const SampleSet& S, const int64_t* M, cudaStream_t st);
  int prep(const SampleSet& S, int dcf_kind, const float* dcf, cudaStream_t st);
  int prep3(const SampleSet& S, int dcf_kind, const float* dcf, cudaStream_t st);
};

// ts: tile sort of a.S on a.M.  2D: the tile-sorted kernel; 3D (ts from build3, or null):
// the global kernel (one warp per sample, every term a global atomic).
int spread_lambda(const SpreadLambdaArgs& a, const TileSort* ts, cudaStream_t st);

struct SpreadDataArgs {
  SampleSet S;
  int64_t M[3], cells;
  const float2* data;   // (ns_pf, nt, ncoils)
  int c0, nc;           // coil range
  const void* U;        // (nt, K) or null (identity)
  int u_complex, K;
  int dcf_kind;
  const float* dcf;     // per kept sample (dcf_kind == array)
  long long* q;         // [(c - c0) * K + k][2][cells]
  const FixedScale* fs;
};
int spread_data(const SpreadDataArgs& a, const TileSort* ts, cudaStream_t st);

// Scale of a fixed-point grid: every term's components are bounded by `mult` times the
// product of the largest absolute entries of the nf (<= 3) factor arrays f[i] (n[i]
// floats each), and a cell sums at most `nterms` terms.
int fixed_scale(const float* const* f, const int64_t* n, int nf, double mult, double nterms, FixedScale* out,
                cudaStream_t st);

// out[ch][cell] = complex(q[ch][0][cell], q[ch][1][cell] or 0) * 2^-e, for nch channels.
int fixed_to_grid(const long long* q, int nq, int64_t cells, int64_t nch, const FixedScale* fs, float2* out,
                  cudaStream_t st);

}  // namespace mrsr
