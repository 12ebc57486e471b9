// Register four-step versions of the apply passes (see fft4.cuh).
//
// Same data flow as the generic kernels in normalop.cu; each line transform
// is two register DFT steps with one shared-memory exchange, and the Λ pass
// keeps its spectrum in the exchange buffer for the K x K product.
#include "fft4.cuh"
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
  load_twiddles(tw, a.pl);
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
    step_a_pf<SP, -1, nload>(sm, sl, NO, tw, ld);  // the zero-padded half leaves registers for the prefetch
  else
    step_a<SP, -1>(sm, sl, NO, tw, nload, ld);
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
  load_twiddles(tw, a.pl);
  const int k = blockIdx.y;
  const int64_t row0 = (int64_t)blockIdx.x * a.rpc;
  const int nr = (int)min((int64_t)a.rpc, a.nrows - row0);
  const int NO = a.rpc * a.ncg;
  constexpr int nkeep = PR ? R2 / 2 : R2;
  __syncthreads();
  step_a_pf<SP, +1, R1>(sm, sl, NO, tw, [&](int lo, int, int m) -> float2 {
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

// stacked right-hand sides: every plane times the same scalar kernel entry, at every
// frequency f of the tile (any number of planes)
template <class SP>
__device__ __forceinline__ void lam_voxels_diag(const LamPassArgs& a, float2* sm, const Slots& sl, int64_t tile) {
  constexpr int R1 = SP::R1, L = SP::L;
  const int T = L << sl.tcs;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int li = t & (a.TC - 1);
    const int f = t >> sl.tcs;
    const int f1 = f % R1, f2 = f / R1;
    const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
    const float2 l = lam_diag_entry(a.lam_mode, a.lam, ((tile * a.NCH + ch) * (int64_t)a.FC + fc) * a.TC + li);
    for (int k = 0; k < a.K; ++k) {
      float2* v = &sm[sl.at(k, f1, f2, li, R1)];
      *v = cmul(l, *v);
    }
  }
}

// per-voxel K x K product at every frequency f of the tile, rank KK known at compile time
template <class SP, int KK>
__device__ __forceinline__ void lam_voxels(const LamPassArgs& a, float2* sm, const Slots& sl, int64_t tile) {
  constexpr int R1 = SP::R1, L = SP::L;
  const int64_t pstride = (int64_t)a.FC * a.TC;
  const int T = L << sl.tcs;
  if (a.lam_mode == LAM_PACKED_REAL) {
    // packed real kernel: the next voxel's entries load while this one is multiplied
    constexpr int P = KK * (KK + 1) / 2;
    const float* lam = reinterpret_cast<const float*>(a.lam);
    auto lbase_of = [&](int tt) -> int64_t {
      const int f = tt >> sl.tcs;
      const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
      return (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * a.TC + (tt & (a.TC - 1));
    };
    float lc[P];
    int t = threadIdx.x;
    if (t < T) {
      const int64_t lb = lbase_of(t);
#pragma unroll
      for (int p = 0; p < P; ++p) lc[p] = lam[lb + p * pstride];
    }
    for (; t < T; t += blockDim.x) {
      const int tn = t + (int)blockDim.x;
      float ln[P];
      if (tn < T) {
        const int64_t lb = lbase_of(tn);
#pragma unroll
        for (int p = 0; p < P; ++p) ln[p] = lam[lb + p * pstride];
      }
      const int li = t & (a.TC - 1);
      const int f = t >> sl.tcs;
      const int f1 = f % R1, f2 = f / R1;
      float2 X[KK], Y[KK];
#pragma unroll
      for (int k = 0; k < KK; ++k) X[k] = sm[sl.at(k, f1, f2, li, R1)];
      lam_real_regs<KK>(lc, X, Y);
#pragma unroll
      for (int k = 0; k < KK; ++k) sm[sl.at(k, f1, f2, li, R1)] = Y[k];
      if (tn < T) {
#pragma unroll
        for (int p = 0; p < P; ++p) lc[p] = ln[p];
      }
    }
    return;
  }
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int li = t & (a.TC - 1);
    const int f = t >> sl.tcs;          // f = f1 + R1 f2
    const int f1 = f % R1, f2 = f / R1;
    float2 X[KK], Y[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) X[k] = sm[sl.at(k, f1, f2, li, R1)];
    const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
    const int64_t lbase = (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * a.TC + li;
    lam_apply_ptr<KK>(a.lam_mode, KK, a.lam, lbase, pstride, X, Y);
#pragma unroll
    for (int k = 0; k < KK; ++k) sm[sl.at(k, f1, f2, li, R1)] = Y[k];
  }
}

template <class SP, bool PR>
__global__ void __launch_bounds__(256, 2) k4_lambda(LamPassArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles(tw, a.pl);
  // coil fastest: the CTAs of one column tile run together and share its Λ tile in L2
  const int cl = (int)(blockIdx.x % (unsigned)a.ncg);
  const int64_t tile = blockIdx.x / (unsigned)a.ncg;
  const int64_t plane = (int64_t)a.nrow * a.inner;
  float2* base = a.stack + (int64_t)cl * a.K * plane + tile * a.TC;
  constexpr int nload = PR ? R1 / 2 : R1;
  constexpr int nkeep = PR ? R1 / 2 : R1;
  __syncthreads();
  step_a<SP, -1>(sm, sl, a.K, tw, nload, [&](int k, int li, int n) -> float2 {
    return (PR || n < a.nin) ? base[k * plane + (int64_t)n * a.inner + li] : make_float2(0.f, 0.f);
  });
  __syncthreads();
  step_b<SP, -1>(sm, sl, a.K, R2, [&](int lo, int li, int f1, int f2, float2 v) { sm[sl.at(lo, f1, f2, li, R1)] = v; });
  __syncthreads();
  if (lam_is_diag(a.lam_mode)) {
    lam_voxels_diag<SP>(a, sm, sl, tile);
  } else switch (a.K) {
    case 1: lam_voxels<SP, 1>(a, sm, sl, tile); break;
    case 2: lam_voxels<SP, 2>(a, sm, sl, tile); break;
    case 3: lam_voxels<SP, 3>(a, sm, sl, tile); break;
    case 4: lam_voxels<SP, 4>(a, sm, sl, tile); break;
    case 5: lam_voxels<SP, 5>(a, sm, sl, tile); break;
    case 6: lam_voxels<SP, 6>(a, sm, sl, tile); break;
    case 7: lam_voxels<SP, 7>(a, sm, sl, tile); break;
    default: lam_voxels<SP, 8>(a, sm, sl, tile); break;
  }
  __syncthreads();
  inv_step_a_slots<SP>(sm, sl, a.K, tw);
  __syncthreads();
  inv_step_b_slots<SP>(sm, sl, a.K, nkeep, [&](int k, int li, int n, float2 v) {
    if (PR || n < a.nout) base[k * plane + (int64_t)n * a.inner + li] = v;
  });
}

// S = -1: forward, input rows n < nin (PR: nin = L/2), all L outputs kept;
// S = +1: inverse, all L inputs, outputs kept for n < nout (PR: nout = L/2).
template <class SP, int S, bool PR>
__global__ void __launch_bounds__(512) k4_mid(MidArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles(tw, a.pl);
  const int64_t col0 = (int64_t)blockIdx.x * a.TC;
  const int64_t o0 = (int64_t)blockIdx.y * a.NOo;
  const int no = (int)min((int64_t)a.NOo, a.n3 - o0);
  const int64_t p = blockIdx.z;
  const float2* ib = a.in + (p * a.n3 + o0) * a.nin * a.width + col0;
  float2* ob = a.out + (p * a.n3 + o0) * a.nout * a.width + col0;
  constexpr int nload = (PR && S < 0) ? R1 / 2 : R1;
  constexpr int nkeep = (PR && S > 0) ? R2 / 2 : R2;
  __syncthreads();
  step_a<SP, S>(sm, sl, a.NOo, tw, nload, [&](int o, int li, int n) -> float2 {
    return (o < no && ((PR && S < 0) || n < a.nin)) ? ib[((int64_t)o * a.nin + n) * a.width + li]
                                                    : make_float2(0.f, 0.f);
  });
  __syncthreads();
  step_b<SP, S>(sm, sl, a.NOo, nkeep, [&](int o, int li, int f1, int f2, float2 v) {
    const int n = f1 + R1 * f2;
    if (o < no && ((PR && S > 0) || n < a.nout)) ob[((int64_t)o * a.nout + n) * a.width + li] = v;
  });
}


// -------------------------------------------------------- dispatch ---

template <class F>
static int with_split(int L, F f) {
  switch (L) {
    case 64: return f(Split<8, 8>());
    case 128: return f(Split<8, 16>());
    case 256: return f(Split<16, 16>());
    case 384: return f(Split<12, 32>());
    case 512: return f(Split<16, 32>());
    case 768: return f(Split<24, 32>());
    case 1024: return f(Split<32, 32>());
    default: return MRSR_ERR_UNSUPPORTED;
  }
}

bool fast_length(int L) { return L == 64 || L == 128 || L == 256 || L == 384 || L == 512 || L == 768 || L == 1024; }

static Slots make_slots(int R2, int TC) {
  Slots s;
  s.TC = TC;
  s.tcs = 0;
  while ((1 << s.tcs) < TC) ++s.tcs;
  s.W = slots_width(R2, TC);
  return s;
}

template <class K, class A>
static int launch(K k, dim3 grid, int threads, size_t smem, cudaStream_t st, const A& a, const Slots& sl) {
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  if (smem > 48 * 1024) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
  k<<<grid, threads, smem, st>>>(a, sl);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

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

int fast_lambda(const LamPassArgs& a, int ncg, int planes_total, int* errword, cudaStream_t st) {
  return with_split(a.pl.L, [&](auto sp) -> int {
    using SP = decltype(sp);
    const Slots sl = make_slots(SP::R2, a.TC);
    const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)a.K * SP::R1 * sl.W);
    LamPassArgs b = a;
    b.ncg = ncg;
    b.fcd = FastDiv((uint32_t)a.FC);
    dim3 grid((unsigned)((a.inner / a.TC) * ncg));
    if (a.nin * 2 == SP::L && a.nout * 2 == SP::L) return launch(k4_lambda<SP, true>, grid, 256, smem, st, b, sl);
    return launch(k4_lambda<SP, false>, grid, 256, smem, st, b, sl);
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
