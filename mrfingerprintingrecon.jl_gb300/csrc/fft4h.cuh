// fp16 register DFTs on pairs of lines.
//
// A value of type hc2 holds one complex sample of each of two lines: the real
// parts in one __half2, the imaginary parts in another.  Every butterfly is a
// packed half2 instruction (HADD2 / HFMA2), so one instruction advances two
// lines; the same Cooley-Tukey compositions as the float32 register DFTs
// (fft4.cuh) are used, with twiddles from broadcast half2 tables.  The two
// lanes are independent lines, so they may carry different scale factors.
#pragma once
#include <cuda_fp16.h>

#include "fft4.cuh"

namespace mrsr {

struct hc2 {
  __half2 re, im;
};

__device__ __forceinline__ __half2 h2u(unsigned int u) { return *reinterpret_cast<const __half2*>(&u); }
__device__ __forceinline__ unsigned int u2h(__half2 h) { return *reinterpret_cast<const unsigned int*>(&h); }

__device__ __forceinline__ hc2 operator+(hc2 a, hc2 b) { return {__hadd2(a.re, b.re), __hadd2(a.im, b.im)}; }
__device__ __forceinline__ hc2 operator-(hc2 a, hc2 b) { return {__hsub2(a.re, b.re), __hsub2(a.im, b.im)}; }
__device__ __forceinline__ hc2 hscale(hc2 a, __half2 c) { return {__hmul2(a.re, c), __hmul2(a.im, c)}; }
// (S i) a
template <int S>
__device__ __forceinline__ hc2 hmul_i(hc2 a) {
  return S < 0 ? hc2{a.im, __hneg2(a.re)} : hc2{__hneg2(a.im), a.re};
}
// a (wr + i wi)
__device__ __forceinline__ hc2 hcmul(hc2 a, __half2 wr, __half2 wi) {
  return {__hfma2(a.re, wr, __hneg2(__hmul2(a.im, wi))), __hfma2(a.re, wi, __hmul2(a.im, wr))};
}
__device__ __forceinline__ hc2 hzero() { return {h2u(0u), h2u(0u)}; }

// pair <-> two half2 complex values (re, im) of lines a and b
__device__ __forceinline__ hc2 hpack(__half2 a, __half2 b) { return {__lows2half2(a, b), __highs2half2(a, b)}; }
__device__ __forceinline__ __half2 hlane_a(hc2 v) { return __lows2half2(v.re, v.im); }
__device__ __forceinline__ __half2 hlane_b(hc2 v) { return __highs2half2(v.re, v.im); }

// fp16 constants (broadcast half2 bit patterns)
constexpr unsigned int kH_SQRT1_2 = 0x39a839a8u;  // 0.70710678
constexpr unsigned int kH_M1_2 = 0xb800b800u;     // -0.5
constexpr unsigned int kH_S3 = 0x3aee3aeeu;       // 0.86602540 = sin(2 pi / 3)
constexpr unsigned int kH_C1 = 0x34f234f2u;       // 0.30901699 = cos(2 pi / 5)
constexpr unsigned int kH_C2 = 0xba79ba79u;       // -0.80901699 = cos(4 pi / 5)
constexpr unsigned int kH_S1 = 0x3b9c3b9cu;       // 0.95105652 = sin(2 pi / 5)
constexpr unsigned int kH_S2 = 0x38b438b4u;       // 0.58778525 = sin(4 pi / 5)

template <int R, int S> struct DftH;
template <int S> struct DftH<1, S> { static __device__ __forceinline__ void run(hc2*) {} };
template <int S> struct DftH<2, S> {
  static __device__ __forceinline__ void run(hc2* v) {
    const hc2 a = v[0], b = v[1];
    v[0] = a + b;
    v[1] = a - b;
  }
};
template <int S> struct DftH<4, S> {
  static __device__ __forceinline__ void run(hc2* v) {
    const hc2 s02 = v[0] + v[2], d02 = v[0] - v[2];
    const hc2 s13 = v[1] + v[3], d13 = hmul_i<S>(v[1] - v[3]);
    v[0] = s02 + s13;
    v[2] = s02 - s13;
    v[1] = d02 + d13;
    v[3] = d02 - d13;
  }
};
template <int S> struct DftH<8, S> {
  static __device__ __forceinline__ void run(hc2* v) {
    hc2 e[4] = {v[0], v[2], v[4], v[6]};
    hc2 o[4] = {v[1], v[3], v[5], v[7]};
    DftH<4, S>::run(e);
    DftH<4, S>::run(o);
    const __half2 h = h2u(kH_SQRT1_2);
    // w8^1 = h (1 + S i), w8^2 = S i, w8^3 = h (-1 + S i)
    const hc2 o1 = S < 0 ? hc2{__hmul2(__hadd2(o[1].re, o[1].im), h), __hmul2(__hsub2(o[1].im, o[1].re), h)}
                         : hc2{__hmul2(__hsub2(o[1].re, o[1].im), h), __hmul2(__hadd2(o[1].im, o[1].re), h)};
    const hc2 o2 = hmul_i<S>(o[2]);
    const hc2 o3 = S < 0 ? hc2{__hmul2(__hsub2(o[3].im, o[3].re), h), __hmul2(__hneg2(__hadd2(o[3].im, o[3].re)), h)}
                         : hc2{__hmul2(__hneg2(__hadd2(o[3].re, o[3].im)), h), __hmul2(__hsub2(o[3].re, o[3].im), h)};
    v[0] = e[0] + o[0];
    v[4] = e[0] - o[0];
    v[1] = e[1] + o1;
    v[5] = e[1] - o1;
    v[2] = e[2] + o2;
    v[6] = e[2] - o2;
    v[3] = e[3] + o3;
    v[7] = e[3] - o3;
  }
};
template <int S> struct DftH<3, S> {
  static __device__ __forceinline__ void run(hc2* v) {
    const __half2 c = h2u(kH_M1_2), s = h2u(kH_S3);
    const hc2 t = v[1] + v[2];
    const hc2 d = hscale(hmul_i<S>(v[1] - v[2]), s);
    const hc2 m = {__hfma2(t.re, c, v[0].re), __hfma2(t.im, c, v[0].im)};
    v[0] = v[0] + t;
    v[1] = m + d;
    v[2] = m - d;
  }
};
template <int S> struct DftH<5, S> {
  static __device__ __forceinline__ void run(hc2* v) {
    const __half2 c1 = h2u(kH_C1), c2 = h2u(kH_C2), s1 = h2u(kH_S1), s2 = h2u(kH_S2);
    const hc2 t1 = v[1] + v[4], t2 = v[2] + v[3];
    const hc2 d1 = v[1] - v[4], d2 = v[2] - v[3];
    const hc2 a1 = {__hfma2(c2, t2.re, __hfma2(c1, t1.re, v[0].re)), __hfma2(c2, t2.im, __hfma2(c1, t1.im, v[0].im))};
    const hc2 a2 = {__hfma2(c1, t2.re, __hfma2(c2, t1.re, v[0].re)), __hfma2(c1, t2.im, __hfma2(c2, t1.im, v[0].im))};
    const hc2 b1 = hmul_i<S>(hc2{__hfma2(s2, d2.re, __hmul2(s1, d1.re)), __hfma2(s2, d2.im, __hmul2(s1, d1.im))});
    const hc2 b2 = hmul_i<S>(hc2{__hfma2(__hneg2(s1), d2.re, __hmul2(s2, d1.re)),
                                 __hfma2(__hneg2(s1), d2.im, __hmul2(s2, d1.im))});
    v[0] = v[0] + (t1 + t2);
    v[1] = a1 + b1;
    v[4] = a1 - b1;
    v[2] = a2 + b2;
    v[3] = a2 - b2;
  }
};

// exp(S 2 pi i m / R) as broadcast half2 (compile-time table index after unrolling)
template <int R, int S>
__device__ __forceinline__ void rtwh(int m, __half2& wr, __half2& wi) {
  constexpr int B = rdft_table_base(R);
  static_assert(B != 0, "no twiddle table for this register DFT length");
  const unsigned int(*t)[2] = (B == 32) ? c_tw32_h2 : (B == 24) ? c_tw24_h2 : (B == 20) ? c_tw20_h2 : c_tw30_h2;
  const int i = (m % R) * (B / R);
  wr = h2u(t[i][0]);
  wi = S < 0 ? __hneg2(h2u(t[i][1])) : h2u(t[i][1]);
}

template <int R, int S>
struct RDftH {
  static constexpr int A = rdft_first_factor(R);
  static constexpr int B = R / A;
  static __device__ __forceinline__ void run(hc2* x) {
    hc2 u[R];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      hc2 t[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) t[n1] = x[B * n1 + n2];
      RDftH<A, S>::run(t);
#pragma unroll
      for (int f1 = 0; f1 < A; ++f1) {
        if (n2 * f1 == 0) {
          u[n2 * A + f1] = t[f1];
        } else {
          __half2 wr, wi;
          rtwh<R, S>(n2 * f1, wr, wi);
          u[n2 * A + f1] = hcmul(t[f1], wr, wi);
        }
      }
    }
#pragma unroll
    for (int f1 = 0; f1 < A; ++f1) {
      hc2 t[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) t[n2] = u[n2 * A + f1];
      RDftH<B, S>::run(t);
#pragma unroll
      for (int f2 = 0; f2 < B; ++f2) x[f1 + A * f2] = t[f2];
    }
  }
};
template <int S> struct RDftH<1, S> { static __device__ __forceinline__ void run(hc2*) {} };
template <int S> struct RDftH<2, S> { static __device__ __forceinline__ void run(hc2* x) { DftH<2, S>::run(x); } };
template <int S> struct RDftH<3, S> { static __device__ __forceinline__ void run(hc2* x) { DftH<3, S>::run(x); } };
template <int S> struct RDftH<4, S> { static __device__ __forceinline__ void run(hc2* x) { DftH<4, S>::run(x); } };
template <int S> struct RDftH<5, S> { static __device__ __forceinline__ void run(hc2* x) { DftH<5, S>::run(x); } };
template <int S> struct RDftH<8, S> { static __device__ __forceinline__ void run(hc2* x) { DftH<8, S>::run(x); } };

// Shared-memory four-step twiddles W_L^m = exp(-2 pi i m / L) as broadcast half2 (re, im).
__device__ __forceinline__ void load_twiddles_h(hc2* tw_s, const FftPlan& pl) {
  for (int i = threadIdx.x; i < pl.L; i += blockDim.x) {
    const float2 w = pl.tw[i];
    tw_s[i] = hc2{__float2half2_rn(w.x), __float2half2_rn(w.y)};
  }
}
template <int S>
__device__ __forceinline__ hc2 twmul_h(hc2 v, const hc2* tw, int m) {
  const hc2 w = tw[m];  // m < L for every caller
  return hcmul(v, w.re, S > 0 ? __hneg2(w.im) : w.im);
}

// The four-step steps of fft4.cuh on pairs; same slot layout (8-byte elements).
template <class SP, int S, class LD>
__device__ __forceinline__ void step_a_h(hc2* sm, const Slots& sl, int NO, const hc2* tw, int nload, LD ld) {
  constexpr int R1 = SP::R1, R2 = SP::R2;
  const int ntask = (NO * R2) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int n2 = r % R2;
    const int lo = r / R2;
    hc2 v[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) v[n1] = (n1 < nload) ? ld(lo, li, R2 * n1 + n2) : hzero();
    RDftH<R1, S>::run(v);
#pragma unroll
    for (int f1 = 0; f1 < R1; ++f1) sm[sl.at(lo, f1, n2, li, R1)] = (f1 == 0) ? v[0] : twmul_h<S>(v[f1], tw, n2 * f1);
  }
}

template <class SP, int S, class ST>
__device__ __forceinline__ void step_b_h(hc2* sm, const Slots& sl, int NO, int nkeep, ST st) {
  constexpr int R1 = SP::R1, R2 = SP::R2;
  const int ntask = (NO * R1) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int f1 = r % R1;
    const int lo = r / R1;
    hc2 v[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) v[n2] = sm[sl.at(lo, f1, n2, li, R1)];
    RDftH<R2, S>::run(v);
#pragma unroll
    for (int f2 = 0; f2 < R2; ++f2)
      if (f2 < nkeep) st(lo, li, f1, f2, v[f2]);
  }
}

// (values are multiplied by `pre` as they are read)
template <class SP>
__device__ __forceinline__ void inv_step_a_slots_h(hc2* sm, const Slots& sl, int NO, const hc2* tw, __half2 pre) {
  constexpr int R1 = SP::R1, R2 = SP::R2;
  const int ntask = (NO * R1) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int f1 = r % R1;
    const int lo = r / R1;
    hc2 v[R2];
#pragma unroll
    for (int f2 = 0; f2 < R2; ++f2) v[f2] = hscale(sm[sl.at(lo, f1, f2, li, R1)], pre);
    RDftH<R2, +1>::run(v);
#pragma unroll
    for (int g1 = 0; g1 < R2; ++g1)
      sm[sl.at(lo, f1, g1, li, R1)] = (f1 * g1 == 0) ? v[g1] : twmul_h<+1>(v[g1], tw, f1 * g1);
  }
}

template <class SP, class ST>
__device__ __forceinline__ void inv_step_b_slots_h(hc2* sm, const Slots& sl, int NO, int nkeep, ST st) {
  constexpr int R1 = SP::R1, R2 = SP::R2;
  const int ntask = (NO * R2) << sl.tcs;
  for (int t = threadIdx.x; t < ntask; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int r = t >> sl.tcs;
    const int g1 = r % R2;
    const int lo = r / R2;
    hc2 v[R1];
#pragma unroll
    for (int f1 = 0; f1 < R1; ++f1) v[f1] = sm[sl.at(lo, f1, g1, li, R1)];
    RDftH<R1, +1>::run(v);
#pragma unroll
    for (int g2 = 0; g2 < R1; ++g2)
      if (g2 < nkeep) st(lo, li, g1 + R2 * g2, v[g2]);
  }
}

}  // namespace mrsr
