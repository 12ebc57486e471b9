// Register four-step versions of the apply passes (see fft4.cuh).
//
// Same data flow as the generic kernels in normalop.cu; each line transform
// is two register DFT steps with one shared-memory exchange, and the Λ pass
// keeps its spectrum in the exchange buffer for the K x K product.
#include "fft4.cuh"
#include "fft4_launch.cuh"
#include "passes.cuh"

#include <algorithm>
#include <cstdlib>

namespace mrsr {

// ---------------------------------------------------------- kernels ---

// PR: the NFFT operator's zero-padded half (inputs n < L/2 only; outputs kept
// for n < L/2 after inverse transforms).  A compile-time flag, so the register
// DFTs fold the known zeros and drop the unused outputs.
template <class SP, bool PR>
__global__ void __launch_bounds__(512) k4_rows_fwd(RowsFwdArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles_a<SP>(tw, a.pl);
  const int cl = blockIdx.y;
  const int c = a.c0 + cl;
  const int64_t row0 = (int64_t)blockIdx.x * a.rpc;
  const int nr = (int)min((int64_t)a.rpc, a.nrows - row0);
  const int NO = a.rpc * a.K;
  constexpr int nload = PR ? R1 / 2 : R1;
  __syncthreads();
  auto ld = [&](int lo, int, int n) -> float2 {
    const int rl = lo / a.K, k = lo - rl * a.K;
    if (rl >= nr || (!PR && n >= a.n1)) return make_float2(0.f, 0.f);
    const int64_t r = row0 + rl;
    float2 v = a.x[n + (int64_t)a.n1 * (r + a.nrows * k)];
    if (a.cmaps) v = cmul(a.cmaps[n + (int64_t)a.n1 * (r + a.nrows * c)], v);
    return v;
  };
  if constexpr (PR)
    step_a_pf<SP, -1, nload, true>(sm, sl, NO, tw, ld);  // the zero-padded half leaves registers for the prefetch
  else
    step_a<SP, -1, true>(sm, sl, NO, tw, nload, ld);
  __syncthreads();
  step_b<SP, -1>(sm, sl, NO, R2, [&](int lo, int, int f1, int f2, float2 v) {
    const int rl = lo / a.K, k = lo - rl * a.K;
    if (rl < nr) a.out[(((int64_t)cl * a.K + k) * a.nrows + row0 + rl) * L + f1 + R1 * f2] = v;
  });
}

template <class SP, bool PR>
__global__ void __launch_bounds__(512) k4_rows_inv(RowsInvArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles_a<SP>(tw, a.pl);
  const int k = blockIdx.y;
  const int64_t row0 = (int64_t)blockIdx.x * a.rpc;
  const int nr = (int)min((int64_t)a.rpc, a.nrows - row0);
  const int NO = a.rpc * a.ncg;
  constexpr int nkeep = PR ? R2 / 2 : R2;
  __syncthreads();
  step_a_pf<SP, +1, R1, true>(sm, sl, NO, tw, [&](int lo, int, int m) -> float2 {
    const int rl = lo / a.ncg, cl = lo - rl * a.ncg;
    if (rl >= nr) return make_float2(0.f, 0.f);
    return a.stack[(((int64_t)cl * a.K + k) * a.nrows + row0 + rl) * L + m];
  });
  __syncthreads();
  step_b<SP, +1>(sm, sl, NO, nkeep, [&](int lo, int li, int f1, int f2, float2 v) { sm[sl.at(lo, f1, f2, li, R1)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < nr * a.n1; e += blockDim.x) {
    const int rl = e / a.n1, i1 = e - rl * a.n1;
    const int f1 = i1 % R1, f2 = i1 / R1;
    const int64_t r = row0 + rl;
    float2 acc = make_float2(0.f, 0.f);
    for (int cl = 0; cl < a.ncg; ++cl) {
      const float2 v = sm[sl.at(rl * a.ncg + cl, f1, f2, 0, R1)];
      if (a.cmaps)
        acc = cadd(acc, cmulc(v, a.cmaps[i1 + (int64_t)a.n1 * (r + a.nrows * (a.c0 + cl))]));
      else
        acc = cadd(acc, v);
    }
    const int64_t yi = i1 + (int64_t)a.n1 * (r + a.nrows * k);
    float2 yv;
    if (a.first)
      yv = (a.beta.x == 0.f && a.beta.y == 0.f) ? make_float2(0.f, 0.f) : cmul(a.beta, a.y[yi]);
    else
      yv = a.y[yi];
    a.y[yi] = cadd(yv, cmul(a.alpha, acc));
  }
}

// S = -1: forward, input rows n < nin (PR: nin = L/2), all L outputs kept;
// S = +1: inverse, all L inputs, outputs kept for n < nout (PR: nout = L/2).
template <class SP, int S, bool PR>
__global__ void __launch_bounds__(512) k4_mid(MidArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles_a<SP>(tw, a.pl);
  const int64_t col0 = (int64_t)blockIdx.x * a.TC;
  const int64_t o0 = (int64_t)blockIdx.y * a.NOo;
  const int no = (int)min((int64_t)a.NOo, a.n3 - o0);
  const int64_t p = blockIdx.z;
  const float2* ib = a.in + (p * a.n3 + o0) * a.nin * a.width + col0;
  float2* ob = a.out + (p * a.n3 + o0) * a.nout * a.width + col0;
  constexpr int nload = (PR && S < 0) ? R1 / 2 : R1;
  constexpr int nkeep = (PR && S > 0) ? R2 / 2 : R2;
  __syncthreads();
  step_a<SP, S, true>(sm, sl, a.NOo, tw, nload, [&](int o, int li, int n) -> float2 {
    return (o < no && ((PR && S < 0) || n < a.nin)) ? ib[((int64_t)o * a.nin + n) * a.width + li]
                                                    : make_float2(0.f, 0.f);
  });
  __syncthreads();
  step_b<SP, S>(sm, sl, a.NOo, nkeep, [&](int o, int li, int f1, int f2, float2 v) {
    const int n = f1 + R1 * f2;
    if (o < no && ((PR && S > 0) || n < a.nout)) ob[((int64_t)o * a.nout + n) * a.width + li] = v;
  });
}


bool fast_length(int L) { return L == 64 || L == 128 || L == 256 || L == 384 || L == 512 || L == 768 || L == 1024; }

static int round_threads(int tasks) {
  int t = ((tasks + 31) / 32) * 32;
  return t < 128 ? 128 : (t > 512 ? 512 : t);
}

// threads of a row-pass CTA: its step-B tasks, capped at 256 (a thread then runs
// several tasks) so that two CTAs fit next to the register-heavy DFTs.  Measured
// on 256^2, 20 coils: rows inverse 0.079 -> 0.063 ms (320 -> 256 threads).
static int row_threads(int tasks) { return std::min(round_threads(tasks), 256); }

int fast_rows_fwd(const RowsFwdArgs& a, int64_t nrows, int ncg, cudaStream_t st) {
  return with_split(a.pl.L, [&](auto sp) -> int {
    using SP = decltype(sp);
    const Slots sl = make_slots(SP::R2, 1);
    const int NO = a.rpc * a.K;
    const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)NO * SP::R1 * sl.W);
    dim3 grid((unsigned)cdiv(nrows, a.rpc), ncg);
    if (a.n1 * 2 == SP::L) return launch(k4_rows_fwd<SP, true>, grid, row_threads(NO * SP::R1), smem, st, a, sl);
    return launch(k4_rows_fwd<SP, false>, grid, row_threads(NO * SP::R1), smem, st, a, sl);
  });
}

int fast_rows_inv(const RowsInvArgs& a, int64_t nrows, cudaStream_t st) {
  return with_split(a.pl.L, [&](auto sp) -> int {
    using SP = decltype(sp);
    const Slots sl = make_slots(SP::R2, 1);
    const int NO = a.rpc * a.ncg;
    const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)NO * SP::R1 * sl.W);
    dim3 grid((unsigned)cdiv(nrows, a.rpc), a.K);
    if (a.n1 * 2 == SP::L) return launch(k4_rows_inv<SP, true>, grid, row_threads(NO * SP::R1), smem, st, a, sl);
    return launch(k4_rows_inv<SP, false>, grid, row_threads(NO * SP::R1), smem, st, a, sl);
  });
}

int fast_mid(const MidArgs& a, int nplanes, cudaStream_t st) {
  return with_split(a.pl.L, [&](auto sp) -> int {
    using SP = decltype(sp);
    const Slots sl = make_slots(SP::R2, a.TC);
    const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)a.NOo * SP::R1 * sl.W);
    dim3 grid((unsigned)(a.width / a.TC), (unsigned)cdiv(a.n3, a.NOo), (unsigned)nplanes);
    const int thr = round_threads(a.NOo * a.TC * SP::R1);
    const bool pr = a.sgn < 0 ? a.nin * 2 == SP::L : a.nout * 2 == SP::L;
    if (a.sgn < 0) return pr ? launch(k4_mid<SP, -1, true>, grid, thr, smem, st, a, sl)
                             : launch(k4_mid<SP, -1, false>, grid, thr, smem, st, a, sl);
    return pr ? launch(k4_mid<SP, +1, true>, grid, thr, smem, st, a, sl)
              : launch(k4_mid<SP, +1, false>, grid, thr, smem, st, a, sl);
  });
}

}  // namespace mrsr
