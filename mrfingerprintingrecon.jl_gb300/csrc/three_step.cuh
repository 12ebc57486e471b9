// Three-step line transforms of the float32 operator's passes (apply_lam8.cu: the Λ pass,
// apply_rows8.cu: the inverse row pass) for L = R1 x 8 x 8 with R1 = 8 (512 points) or 4 (256):
//   n = 64 n1 + 8 n2 + n3,  f = f1 + R1 f2 + 8 R1 f3,
//   X[f] = sum_n3 w8^(n3 f3) w64^(n3 f2) sum_n2 w8^(n2 f2) [wL^((8 n2 + n3) f1) sum_n1 wR1^(n1 f1) x[n]]
// on lines zero-padded to twice their length (input n1 < R1 / 2) whose inverse keeps the
// first half (output n1 < R1 / 2).  A CTA transforms G groups of TC lines; every task holds
// at most eight values (one DFT-8), so the kernels fit in 64 registers and run 512-thread
// CTAs two per SM.
//
// Shared layout of group g, line li (TC = 4 or 8 lines per group): position (a, b, c) of
// the three digits at g * SP + a * SA + b * SB + c * TC + li (float2 units).  Every step's
// warp varies li and one of a, b, c (the rest fixed); SA and SB are TC (mod 16), so the 16
// lanes of a half-warp (16 / TC values of the running digit) touch 16 distinct 8-byte bank
// pairs for any of the three, and a task's running digit is a compile-time loop index, so
// its addresses are one register plus immediate offsets.  A task reads and writes the same
// positions (one digit running), so every step works in place.  After the forward steps
// X[f] sits at (f1, f2, f3); the inverse steps start from there.
#pragma once
#include "fft4.cuh"
#include "passes.cuh"

namespace mrsr {
namespace l8 {

constexpr int kL8Threads = 512;
constexpr size_t kL8MaxSmem = 227 * 1024;

template <int R1_, int TC_>
struct L8 {
  static constexpr int R1 = R1_, TC = TC_, L = 64 * R1;
  static constexpr int LT = TC == 4 ? 2 : 3;  // log2 TC
  static constexpr int LR = R1 == 4 ? 2 : 3;  // log2 R1
  static constexpr int SB = 8 * TC + TC, SA = 8 * SB + TC, SP = R1 * SA;  // digit b, digit a, plane
  static constexpr int T1 = R1 * 64, T2 = 64, T3 = 64, TW = T1 + T2 + T3;  // twiddle tables
  static constexpr int NT1 = TC * 64;      // tasks per plane of the steps running n1 / f1
  static constexpr int NT2 = TC * 8 * R1;  // tasks per plane of the other steps
  static_assert((TC == 4 || TC == 8) && (R1 == 4 || R1 == 8), "tile of 4 or 8 columns, L = 256 or 512");
  static_assert(SB % 16 == TC && SA % 16 == TC, "a half-warp on 16 distinct bank pairs");
  static constexpr size_t smem(int K) { return sizeof(float2) * ((size_t)TW + (size_t)K * SP); }
  static __device__ __forceinline__ int at(int k, int a, int b, int c, int li) { return k * SP + a * SA + b * SB + c * TC + li; }
};

__device__ __forceinline__ float2 cj(float2 w) { return make_float2(w.x, -w.y); }

// 16-byte global -> shared copy that bypasses L1 (cp.async.cg); both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(float2* dst, const float2* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
// Closes the thread's copies into one group / waits for it (the caller's barrier then makes
// every thread's copies visible to the CTA).
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// DFT-R (R = 4 or 8, sign S) of v[0..R/2-1] followed by R/2 zeros, without the additions of
// the zeros (x + 0 is not folded away by the compiler, as -0 + 0 = +0):
//   R = 4: X[q] = v0 + (S i)^q v1;  R = 8: the even / odd halves of Dft<8> from two such DFT-4s.
template <int R, int S>
__device__ __forceinline__ void dft_half_in(float2* v) {
  const float sg = (float)S;
  if constexpr (R == 4) {
    const float2 a = v[0], b = v[1], ib = cmul_i(b, sg);
    v[0] = cadd(a, b);
    v[1] = cadd(a, ib);
    v[2] = csub(a, b);
    v[3] = csub(a, ib);
  } else {
    static_assert(R == 8, "R = 4 or 8");
    const float h = 0.70710678118654752440f;
    float2 e[4] = {v[0], v[2]}, o[4] = {v[1], v[3]};
    dft_half_in<4, S>(e);
    dft_half_in<4, S>(o);
    // w8^1 = h(1 + S i), w8^2 = S i, w8^3 = h(-1 + S i)
    const float2 o1 = make_float2(h * (o[1].x - sg * o[1].y), h * (o[1].y + sg * o[1].x));
    const float2 o2 = cmul_i(o[2], sg);
    const float2 o3 = make_float2(h * (-o[3].x - sg * o[3].y), h * (-o[3].y + sg * o[3].x));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
}

// Twiddle tables in the order the steps' lanes read them (a warp's lanes vary n3 or f2 with
// the loop digit fixed, so each table read is consecutive entries, bank-conflict free; a
// table indexed (m * f) mod L would put the lanes of an even f on the same banks):
//   t1[f1 * 64 + m] = wL^(m f1), m = 8 n2 + n3     (F1, I2 conjugated)
//   t2[f2 * 8 + n3] = w64^(n3 f2)                  (F2)
//   t3[n3 * 8 + f2] = w64^(-n3 f2)                 (I1)
template <class C>
__device__ __forceinline__ void build_tables(float2* t, const FftPlan& pl) {
  const float2* w = pl.tw;  // wL^p
  for (int i = threadIdx.x; i < C::TW; i += blockDim.x) {
    int p;
    bool conj = false;
    if (i < C::T1) {
      p = (i & 63) * (i >> 6);
    } else if (i < C::T1 + C::T2) {
      const int j = i - C::T1;
      p = C::R1 * (j & 7) * (j >> 3);
    } else {
      const int j = i - C::T1 - C::T2;
      p = C::R1 * (j >> 3) * (j & 7);
      conj = true;
    }
    const float2 v = w[p & (C::L - 1)];
    t[i] = conj ? cj(v) : v;
  }
}

// Every step runs a fixed set of tasks per thread: task t = tid + 512 i, and since the tasks
// of one plane (or, for the voxel step, the frequencies of two Λ chunks) number a divisor of
// 512, the digits a thread owns are the same in every round i and only the plane (or f3)
// moves, by a compile-time step.  So each thread forms its addresses and loads its twiddles
// once per step, and the rounds are unrolled with immediate offsets.
template <int N, class F>
__device__ __forceinline__ void rounds(F&& body) {
  constexpr int IT = (N + kL8Threads - 1) / kL8Threads;
#pragma unroll
  for (int i = 0; i < IT; ++i) {
    if (N % kL8Threads != 0 && (int)threadIdx.x + i * kL8Threads >= N) break;
    body(i);
  }
}

// Thread-owned digits of the two kinds of step (tid = threadIdx.x):
//   n1 / f1 steps (F1, I3): (li, n3, n2), group g = k1 + round * 512 / NT1
//   the other steps:        (li, d1 = n3 or f2, f1), group g = k2 + round * 512 / NT2
template <class C>
struct Own {
  int li, d1, e2, k1, f1o, k2;
  __device__ __forceinline__ Own() {
    const int tid = threadIdx.x;
    li = tid & (C::TC - 1);
    d1 = (tid >> C::LT) & 7;
    e2 = (tid >> (C::LT + 3)) & 7;
    k1 = tid >> (C::LT + 6);
    f1o = (tid >> (C::LT + 3)) & (C::R1 - 1);
    k2 = tid >> (C::LT + 3 + C::LR);
  }
};

// F1: DFT-R1 over n1 of the input staged at the upper slots a = R1/2 + n1 -> f1, twiddle
// wL^((8 n2 + n3) f1); position (f1, n2, n3)
template <class C, int G>
__device__ __forceinline__ void step_f1(float2* sm, const float2* t1, const Own<C>& o) {
  constexpr int R1 = C::R1, H = R1 / 2, SA = C::SA, DK = kL8Threads / C::NT1 * C::SP;
  const int n3 = o.d1, n2 = o.e2, m = 8 * n2 + n3;
  float2 w[R1];
#pragma unroll
  for (int f1 = 1; f1 < R1; ++f1) w[f1] = t1[f1 * 64 + m];
  const int p0 = C::at(o.k1, 0, n2, n3, o.li);
  rounds<G * C::NT1>([&](int i) {
    const int p = p0 + i * DK;
    float2 v[R1];
#pragma unroll
    for (int n1 = 0; n1 < H; ++n1) v[n1] = sm[p + (H + n1) * SA];
    dft_half_in<R1, -1>(v);
    sm[p] = v[0];
#pragma unroll
    for (int f1 = 1; f1 < R1; ++f1) sm[p + f1 * SA] = cmul(v[f1], w[f1]);
  });
}

// F2: DFT-8 over n2 -> f2, twiddle w64^(n3 f2); position (f1, f2, n3)
template <class C, int G>
__device__ __forceinline__ void step_f2(float2* sm, const float2* t2, const Own<C>& o) {
  constexpr int SB = C::SB, DK = kL8Threads / C::NT2 * C::SP;
  const int n3 = o.d1;
  float2 w[8];
#pragma unroll
  for (int f2 = 1; f2 < 8; ++f2) w[f2] = t2[f2 * 8 + n3];
  const int p0 = C::at(o.k2, o.f1o, 0, n3, o.li);
  rounds<G * C::NT2>([&](int i) {
    const int p = p0 + i * DK;
    float2 v[8];
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) v[n2] = sm[p + n2 * SB];
    RDft<8, -1>::run(v);
    sm[p] = v[0];
#pragma unroll
    for (int f2 = 1; f2 < 8; ++f2) sm[p + f2 * SB] = cmul(v[f2], w[f2]);
  });
}

// F3: DFT-8 over n3 -> f3; X[f1 + R1 f2 + 8 R1 f3] at position (f1, f2, f3)
template <class C, int G>
__device__ __forceinline__ void step_f3(float2* sm, const Own<C>& o) {
  constexpr int TC = C::TC, DK = kL8Threads / C::NT2 * C::SP;
  const int p0 = C::at(o.k2, o.f1o, o.d1, 0, o.li);
  rounds<G * C::NT2>([&](int i) {
    const int p = p0 + i * DK;
    float2 v[8];
#pragma unroll
    for (int n3 = 0; n3 < 8; ++n3) v[n3] = sm[p + n3 * TC];
    RDft<8, -1>::run(v);
#pragma unroll
    for (int f3 = 0; f3 < 8; ++f3) sm[p + f3 * TC] = v[f3];
  });
}

// I1: inverse DFT-8 over f3 -> n3, twiddle w64^(-n3 f2); position (f1, f2, n3)
template <class C, int G>
__device__ __forceinline__ void step_i1(float2* sm, const float2* t3, const Own<C>& o) {
  constexpr int TC = C::TC, DK = kL8Threads / C::NT2 * C::SP;
  const int f2 = o.d1;
  float2 w[8];
#pragma unroll
  for (int n3 = 1; n3 < 8; ++n3) w[n3] = t3[n3 * 8 + f2];
  const int p0 = C::at(o.k2, o.f1o, f2, 0, o.li);
  rounds<G * C::NT2>([&](int i) {
    const int p = p0 + i * DK;
    float2 v[8];
#pragma unroll
    for (int f3 = 0; f3 < 8; ++f3) v[f3] = sm[p + f3 * TC];
    RDft<8, +1>::run(v);
    sm[p] = v[0];
#pragma unroll
    for (int n3 = 1; n3 < 8; ++n3) sm[p + n3 * TC] = cmul(v[n3], w[n3]);
  });
}

// I2: inverse DFT-8 over f2 -> n2, twiddle wL^(-(8 n2 + n3) f1); position (f1, n2, n3)
// (row f1 = 0 of the table is exactly 1, so that row's products are exact)
template <class C, int G>
__device__ __forceinline__ void step_i2(float2* sm, const float2* t1, const Own<C>& o) {
  constexpr int SB = C::SB, DK = kL8Threads / C::NT2 * C::SP;
  const int n3 = o.d1;
  float2 w[8];
#pragma unroll
  for (int n2 = 0; n2 < 8; ++n2) w[n2] = cj(t1[o.f1o * 64 + 8 * n2 + n3]);
  const int p0 = C::at(o.k2, o.f1o, 0, n3, o.li);
  rounds<G * C::NT2>([&](int i) {
    const int p = p0 + i * DK;
    float2 v[8];
#pragma unroll
    for (int f2 = 0; f2 < 8; ++f2) v[f2] = sm[p + f2 * SB];
    RDft<8, +1>::run(v);
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) sm[p + n2 * SB] = cmul(v[n2], w[n2]);
  });
}

// I3: inverse DFT-R1 over f1 -> n1; out(i, v) receives the kept half v[n1 < R1/2] of the
// thread's round i (line li of group k1 + i * 512 / NT1, positions n = 64 n1 + 8 n2 + n3).
template <class C, int G, class Out>
__device__ __forceinline__ void step_i3(const float2* sm, const Own<C>& o, Out&& out) {
  constexpr int R1 = C::R1, SA = C::SA, DK = kL8Threads / C::NT1 * C::SP;
  const int p0 = C::at(o.k1, 0, o.e2, o.d1, o.li);
  rounds<G * C::NT1>([&](int i) {
    const int p = p0 + i * DK;
    float2 v[R1];
#pragma unroll
    for (int f1 = 0; f1 < R1; ++f1) v[f1] = sm[p + f1 * SA];
    RDft<R1, +1>::run(v);
    out(i, v);
  });
}

}  // namespace l8
}  // namespace mrsr
