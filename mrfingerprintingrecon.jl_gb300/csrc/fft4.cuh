// Register-resident DFTs and the two-step ("four-step") line transform.
//
// A line of length L = R1 * R2 is transformed as
//   X[f1 + R1 f2] = sum_{n2} W_R2^{n2 f2} W_L^{n2 f1} sum_{n1} x[R2 n1 + n2] W_R1^{n1 f1}
// (Bailey's four-step decomposition).  Step A: one task per (line, n2) holds
// the R1 inputs x[R2 n1 + n2] in registers, runs an R1-point DFT and applies
// the twiddle W_L^{n2 f1}.  Step B: one task per (line, f1) holds R2 values
// and runs an R2-point DFT.  The only shared-memory traffic is the exchange
// between the two steps.  The R-point DFTs are unrolled Cooley-Tukey
// compositions of radix 2/3/4/5/8 kernels with twiddles from __constant__
// tables, so every index is a compile-time constant and stays in registers.
//
// Shared-memory slot layout (TC interleaved columns, lo outer lines):
//   slot(lo, li, a, c) = (lo * R1 + a) * W + c * TC + li,  W = R2*TC + pad
// with pad chosen so that W = TC (mod 16): tasks whose li varies fastest and
// then a (= f1) touch 16 distinct 8-byte banks per half warp.
#pragma once
#include "fft.cuh"
#include "twiddles.cuh"

namespace mrsr {

// ---------------------------------------------- compile-time factoring ---
__host__ __device__ constexpr int rdft_first_factor(int R) {
  return (R % 8 == 0 && R != 8) ? 8 : (R % 4 == 0 && R != 4) ? 4 : (R % 2 == 0 && R != 2) ? 2
       : (R % 3 == 0 && R != 3) ? 3 : (R % 5 == 0 && R != 5) ? 5 : R;
}
__host__ __device__ constexpr int rdft_table_base(int R) {
  return (32 % R == 0) ? 32 : (24 % R == 0) ? 24 : (20 % R == 0) ? 20 : (30 % R == 0) ? 30 : 0;
}

// exp(S 2 pi i m / R) from the __constant__ tables (S = -1 forward, +1 inverse)
template <int R, int S>
__device__ __forceinline__ float2 rtw(int m) {
  constexpr int B = rdft_table_base(R);
  static_assert(B != 0, "no twiddle table for this register DFT length");
  const float2* t = (B == 32) ? c_tw32 : (B == 24) ? c_tw24 : (B == 20) ? c_tw20 : c_tw30;
  const float2 w = t[(m % R) * (B / R)];
  return make_float2(w.x, S * w.y);
}

template <int R, int S>
struct RDft {
  static constexpr int A = rdft_first_factor(R);
  static constexpr int B = R / A;
  static __device__ __forceinline__ void run(float2* x) {
    float2 u[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float2 t[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) t[n1] = x[B * n1 + n2];
      RDft<A, S>::run(t);
#pragma unroll
      for (int f1 = 0; f1 < A; ++f1) u[n2 * A + f1] = (n2 * f1 == 0) ? t[f1] : cmul(t[f1], rtw<R, S>(n2 * f1));
    }
#pragma unroll
    for (int f1 = 0; f1 < A; ++f1) {
      float2 t[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) t[n2] = u[n2 * A + f1];
      RDft<B, S>::run(t);
#pragma unroll
      for (int f2 = 0; f2 < B; ++f2) x[f1 + A * f2] = t[f2];
    }
  }
};
template <int S> struct RDft<1, S> { static __device__ __forceinline__ void run(float2*) {} };
template <int S> struct RDft<2, S> { static __device__ __forceinline__ void run(float2* x) { Dft<2>::run(x, (float)S); } };
template <int S> struct RDft<3, S> { static __device__ __forceinline__ void run(float2* x) { Dft<3>::run(x, (float)S); } };
template <int S> struct RDft<4, S> { static __device__ __forceinline__ void run(float2* x) { Dft<4>::run(x, (float)S); } };
template <int S> struct RDft<5, S> { static __device__ __forceinline__ void run(float2* x) { Dft<5>::run(x, (float)S); } };
template <int S> struct RDft<8, S> { static __device__ __forceinline__ void run(float2* x) { Dft<8>::run(x, (float)S); } };

// ------------------------------------------------------ line geometry ---
__host__ __device__ constexpr int slot_pad(int R2, int TC) {
  return TC >= 16 ? 0 : (((TC - (R2 * TC) % 16) % 16) + 16) % 16;
}

template <int R1_, int R2_>
struct Split {
  static constexpr int R1 = R1_;
  static constexpr int R2 = R2_;
  static constexpr int L = R1 * R2;
};

struct Slots {
  int TC, tcs, W;  // columns, log2(TC), row width in float2
  __device__ __forceinline__ int at(int lo, int a, int c, int li, int R1) const { return (lo * R1 + a) * W + c * TC + li; }
};

__host__ __device__ inline int slots_width(int R2, int TC) { return R2 * TC + slot_pad(R2, TC); }

// Twiddle W_L^{S m} from the shared-memory table tw[p] = exp(-2 pi i p / L).
template <int S>
__device__ __forceinline__ float2 twl(const float2* tw, int m, int) {
  float2 w = tw[m];  // m < L for every caller
  if (S > 0) w.y = -w.y;
  return w;
}

// Step-A twiddles in the order step A's lanes read them: tw[f1 * R2 + n2] = W_L^{n2 f1}
// (the lanes of a warp vary n2, so a read is consecutive entries, bank-conflict free; the
// table indexed n2 f1 puts the lanes of an even f1 on shared banks, gcd(f1, 16)-way).
template <class SP>
__device__ __forceinline__ void load_twiddles_a(float2* tw_s, const FftPlan& pl) {
  for (int i = threadIdx.x; i < SP::L; i += blockDim.x) {
    const int f1 = i / SP::R2, n2 = i - f1 * SP::R2;
    tw_s[i] = pl.tw[n2 * f1];  // n2 f1 < R1 R2 = L
  }
}

// Step A of a forward or inverse transform.  Task (lo, li, n2) loads
// x[R2 n1 + n2] (n1 < nload) through ld(lo, li, n), applies the R1-point DFT
// and the twiddle, and writes slot(lo, li, f1, n2).  nload = R1 or R1/2
// (lower-half input, zero-padded embedding).  LT: tw is load_twiddles_a's table, else
// load_twiddles' (tw[p] = W_L^p).
template <class SP, int S, bool LT = false, class SL, class LD>
__device__ __forceinline__ void step_a(float2* sm, const SL& sl, int NO, const float2* tw, int nload, LD ld) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  const int ntask = (NO * R2) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int n2 = r % R2;
    const int lo = r / R2;
    float2 v[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) v[n1] = (n1 < nload) ? ld(lo, li, R2 * n1 + n2) : make_float2(0.f, 0.f);
    RDft<R1, S>::run(v);
#pragma unroll
    for (int f1 = 0; f1 < R1; ++f1) {
      const float2 w = (f1 == 0) ? make_float2(1.f, 0.f) : twl<S>(tw, LT ? f1 * R2 + n2 : n2 * f1, L);
      sm[sl.at(lo, f1, n2, li, R1)] = (f1 == 0) ? v[0] : cmul(v[f1], w);
    }
  }
}

// Step A with the task loop software-pipelined: the inputs of the thread's next task are
// loaded before the current task's DFT, so their latency overlaps it.  NLOAD inputs per
// task are read (the rest are zero), which costs NLOAD extra registers.
template <class SP, int S, int NLOAD, bool LT = false, class SL, class LD>
__device__ __forceinline__ void step_a_pf(float2* sm, const SL& sl, int NO, const float2* tw, LD ld) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  const int ntask = (NO * R2) << sl.tcs;
  auto load = [&](int t, float2* v) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int n2 = r % R2;
    const int lo = r / R2;
#pragma unroll
    for (int n1 = 0; n1 < NLOAD; ++n1) v[n1] = ld(lo, li, R2 * n1 + n2);
  };
  float2 nxt[NLOAD];
  if ((int)threadIdx.x < ntask) load(threadIdx.x, nxt);
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int n2 = r % R2;
    const int lo = r / R2;
    float2 v[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) v[n1] = n1 < NLOAD ? nxt[n1] : make_float2(0.f, 0.f);
    if (t + (int)blockDim.x < ntask) load(t + blockDim.x, nxt);
    RDft<R1, S>::run(v);
#pragma unroll
    for (int f1 = 0; f1 < R1; ++f1) {
      const float2 w = (f1 == 0) ? make_float2(1.f, 0.f) : twl<S>(tw, LT ? f1 * R2 + n2 : n2 * f1, L);
      sm[sl.at(lo, f1, n2, li, R1)] = (f1 == 0) ? v[0] : cmul(v[f1], w);
    }
  }
}

// Step B.  Task (lo, li, f1) reads slot(lo, li, f1, n2) for all n2, applies
// the R2-point DFT and hands X[f1 + R1 f2] for f2 < nkeep to st(lo, li, f1, f2, v).
template <class SP, int S, class SL, class ST>
__device__ __forceinline__ void step_b(float2* sm, const SL& sl, int NO, int nkeep, ST st) {
  constexpr int R1 = SP::R1, R2 = SP::R2;
  const int ntask = (NO * R1) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int f1 = r % R1;
    const int lo = r / R1;
    float2 v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) v[n2] = sm[sl.at(lo, f1, n2, li, R1)];
    RDft<R2, S>::run(v);
#pragma unroll
    for (int f2 = 0; f2 < R2; ++f2)
      if (f2 < nkeep) st(lo, li, f1, f2, v[f2]);
  }
}

// Inverse transform of a spectrum held in the slot layout with frequency
// f = f1 + R1 f2 at slot(lo, li, f1, f2).  Step A': task (lo, li, f1) runs
// the R2-point inverse DFT over f2 (-> g1), twiddle W_L^{+f1 g1}, in place.
template <class SP, class SL>
__device__ __forceinline__ void inv_step_a_slots(float2* sm, const SL& sl, int NO, const float2* tw) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  const int ntask = (NO * R1) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int f1 = r % R1;
    const int lo = r / R1;
    float2 v[R2];
#pragma unroll
    for (int f2 = 0; f2 < R2; ++f2) v[f2] = sm[sl.at(lo, f1, f2, li, R1)];
    RDft<R2, +1>::run(v);
#pragma unroll
    for (int g1 = 0; g1 < R2; ++g1)
      sm[sl.at(lo, f1, g1, li, R1)] = (f1 * g1 == 0) ? v[g1] : cmul(v[g1], twl<+1>(tw, f1 * g1, L));
  }
}

// Step B': task (lo, li, g1) runs the R1-point inverse DFT over f1 (-> g2)
// and hands y[g1 + R2 g2] for g2 < nkeep to st(lo, li, n, v).
template <class SP, class SL, class ST>
__device__ __forceinline__ void inv_step_b_slots(float2* sm, const SL& sl, int NO, int nkeep, ST st) {
  constexpr int R1 = SP::R1, R2 = SP::R2;
  const int ntask = (NO * R2) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int g1 = r % R2;
    const int lo = r / R2;
    float2 v[R1];
#pragma unroll
    for (int f1 = 0; f1 < R1; ++f1) v[f1] = sm[sl.at(lo, f1, g1, li, R1)];
    RDft<R1, +1>::run(v);
#pragma unroll
    for (int g2 = 0; g2 < R1; ++g2)
      if (g2 < nkeep) st(lo, li, g1 + R2 * g2, v[g2]);
  }
}

}  // namespace mrsr
