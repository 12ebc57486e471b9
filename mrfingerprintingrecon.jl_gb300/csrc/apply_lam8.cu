// Λ pass of the float32 operator as three DFT steps each way for the two line lengths the
// operators mostly use, L = R1 x 8 x 8: R1 = 8 (512-point lines, the 256^2 images' columns)
// and R1 = 4 (256-point lines, the 128^3 volumes'):
//   n = 64 n1 + 8 n2 + n3,  f = f1 + R1 f2 + 8 R1 f3,
//   X[f] = sum_n3 w8^(n3 f3) w64^(n3 f2) sum_n2 w8^(n2 f2) [wL^((8 n2 + n3) f1) sum_n1 wR1^(n1 f1) x[n]]
// with the input pruned to n1 < R1 / 2 (the zero-padded half) and the inverse's output to
// n1 < R1 / 2 (the kept half).  Every task holds at most eight values (one DFT-8), so the
// kernel fits in 64 registers and runs 512-thread CTAs two per SM: 32 warps per SM against 16
// for the two-step kernels (apply_lam.cu), which are bound by latency, not by arithmetic.
// The price is one more shared-memory exchange each way.
// src/NFFTNormalOp.jl:227-267 / ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218.
//
// Shared layout of plane k, column li (TC = 4 or 8 columns per tile): position (a, b, c) of
// the three digits at k * SP + a * SA + b * SB + c * TC + li (float2 units).  Every step's warp
// varies li and one of a, b, c (the rest fixed); SA and SB are TC (mod 16), so the 16 lanes of
// a half-warp (16 / TC values of the running digit) touch 16 distinct 8-byte bank pairs for
// any of the three, and a task's running digit is a compile-time loop index, so its addresses
// are one register plus immediate offsets.  A task reads and writes the same positions (one
// digit running), so every step works in place.
#include "fft4.cuh"
#include "passes.cuh"

namespace mrsr {

namespace {

constexpr int kL8Threads = 512;
constexpr int kL8MaxK = 6;
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

template <class C, int KK>
__device__ __forceinline__ void lam8_voxels(const LamPassArgs& a, float2* sm, int64_t tile) {
  constexpr int T = C::L * C::TC;
  // two Λ chunks (FC * TC = 256 entries each) per round: entry p of the chunk is 256 apart
  constexpr int PS = 256, DF = kL8Threads / C::TC;  // frequencies per round
  constexpr int DPOS = DF / (8 * C::R1) * C::TC;      // f3 += DF / (8 R1)
  const int tid = threadIdx.x, li = tid & (C::TC - 1), f = tid >> C::LT;
  const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
  const float* lam0 = nullptr;
  const int64_t lb0 = (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * C::TC + li;
  // X[f] of column li sits at (f1, f2, f3) = (f mod R1, (f / R1) mod 8, f / (8 R1))
  const int p0 = C::at(0, f & (C::R1 - 1), (f >> C::LR) & 7, f >> (C::LR + 3), li);
  if (a.lam_mode == LAM_PACKED_REAL) {
    constexpr int P = KK * (KK + 1) / 2;
    lam0 = reinterpret_cast<const float*>(a.lam) + lb0;
    rounds<T>([&](int i) {
      const float* lam = lam0 + (int64_t)i * (2 * PS * P);
      float lc[P];
#pragma unroll
      for (int p = 0; p < P; ++p) lc[p] = lam[p * PS];
      const int q = p0 + i * DPOS;
      float2 X[KK], Y[KK];
#pragma unroll
      for (int k = 0; k < KK; ++k) X[k] = sm[q + k * C::SP];
      lam_real_regs<KK>(lc, X, Y);
#pragma unroll
      for (int k = 0; k < KK; ++k) sm[q + k * C::SP] = Y[k];
    });
    return;
  }
  rounds<T>([&](int i) {
    const int q = p0 + i * DPOS;
    float2 X[KK], Y[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) X[k] = sm[q + k * C::SP];
    lam_apply_ptr<KK>(a.lam_mode, KK, a.lam, lb0 + (int64_t)i * (2 * PS * a.P), PS, X, Y);
#pragma unroll
    for (int k = 0; k < KK; ++k) sm[q + k * C::SP] = Y[k];
  });
}

template <class C, int KK>
__global__ void __launch_bounds__(kL8Threads, 2) k8_lambda(LamPassArgs a) {
  constexpr int R1 = C::R1, TC = C::TC, LT = C::LT, LR = C::LR, H = R1 / 2;
  constexpr int N1 = KK * C::NT1, N2 = KK * C::NT2;
  constexpr int DK1 = kL8Threads / C::NT1 * C::SP, DK2 = kL8Threads / C::NT2 * C::SP;  // plane step per round
  constexpr int SA = C::SA, SB = C::SB;
  extern __shared__ float2 smem[];
  float2* t1 = smem;                 // twiddle tables
  const float2* t2 = smem + C::T1;
  const float2* t3 = smem + C::T1 + C::T2;
  float2* sm = smem + C::TW;         // positions C::at(k, a, b, c, li)
  const int tid = threadIdx.x;
  const int cl = (int)(blockIdx.x % (unsigned)a.ncg);
  const int64_t tile = blockIdx.x / (unsigned)a.ncg;
  const int64_t plane = (int64_t)a.nrow * a.inner;
  float2* base = a.stack + (int64_t)cl * KK * plane + tile * TC;
  // Stage the tile's input (rows n1 < R1/2) into the upper digit slots a = R1/2 + n1 with
  // 16-byte asynchronous copies, all issued before anything waits on them, so the loads of
  // a CTA are in flight together; F1 reads them back and, in place, overwrites them.
  {
    constexpr int NC = KK * H * 64 * (TC / 2);  // 16-byte chunks: two columns each
    for (int c = tid; c < NC; c += kL8Threads) {
      const int j = c & (TC / 2 - 1), r = c >> (LT - 1);
      const int n3 = r & 7, n2 = (r >> 3) & 7, n1 = (r >> 6) % H, k = (r >> 6) / H;
      cp_async16(sm + C::at(k, H + n1, n2, n3, 2 * j), base + k * plane + (int64_t)(64 * n1 + 8 * n2 + n3) * a.inner + 2 * j);
    }
    cp_async_commit();
  }
  build_tables<C>(t1, a.pl);
  cp_async_wait_all();
  __syncthreads();
  // rounds of the steps running n1 / f1: the thread owns (li, n3, n2)
  const int li = tid & (TC - 1), d1 = (tid >> LT) & 7;
  const int e2 = (tid >> (LT + 3)) & 7, k1 = tid >> (LT + 6);
  // rounds of the other steps: the thread owns (li, d1, f1) with d1 = n3 or f2
  const int f1o = (tid >> (LT + 3)) & (R1 - 1), k2 = tid >> (LT + 3 + LR);
  // F1: DFT-R1 over n1 (n1 < R1/2 nonzero) -> f1, twiddle wL^((8 n2 + n3) f1); position (f1, n2, n3)
  {
    const int n3 = d1, n2 = e2, m = 8 * n2 + n3;
    float2 w[R1];
#pragma unroll
    for (int f1 = 1; f1 < R1; ++f1) w[f1] = t1[f1 * 64 + m];
    const int p0 = C::at(k1, 0, n2, n3, li);
    rounds<N1>([&](int i) {
      const int p = p0 + i * DK1;
      float2 v[R1];
#pragma unroll
      for (int n1 = 0; n1 < H; ++n1) v[n1] = sm[p + (H + n1) * SA];
      dft_half_in<R1, -1>(v);
      sm[p] = v[0];
#pragma unroll
      for (int f1 = 1; f1 < R1; ++f1) sm[p + f1 * SA] = cmul(v[f1], w[f1]);
    });
  }
  __syncthreads();
  // F2: DFT-8 over n2 -> f2, twiddle w64^(n3 f2); position (f1, f2, n3)
  {
    const int n3 = d1;
    float2 w[8];
#pragma unroll
    for (int f2 = 1; f2 < 8; ++f2) w[f2] = t2[f2 * 8 + n3];
    const int p0 = C::at(k2, f1o, 0, n3, li);
    rounds<N2>([&](int i) {
      const int p = p0 + i * DK2;
      float2 v[8];
#pragma unroll
      for (int n2 = 0; n2 < 8; ++n2) v[n2] = sm[p + n2 * SB];
      RDft<8, -1>::run(v);
      sm[p] = v[0];
#pragma unroll
      for (int f2 = 1; f2 < 8; ++f2) sm[p + f2 * SB] = cmul(v[f2], w[f2]);
    });
  }
  __syncthreads();
  // F3: DFT-8 over n3 -> f3; X[f1 + R1 f2 + 8 R1 f3] at position (f1, f2, f3)
  {
    const int f2 = d1;
    const int p0 = C::at(k2, f1o, f2, 0, li);
    rounds<N2>([&](int i) {
      const int p = p0 + i * DK2;
      float2 v[8];
#pragma unroll
      for (int n3 = 0; n3 < 8; ++n3) v[n3] = sm[p + n3 * TC];
      RDft<8, -1>::run(v);
#pragma unroll
      for (int f3 = 0; f3 < 8; ++f3) sm[p + f3 * TC] = v[f3];
    });
  }
  __syncthreads();
  lam8_voxels<C, KK>(a, sm, tile);
  __syncthreads();
  // I1: inverse DFT-8 over f3 -> n3, twiddle w64^(-n3 f2); position (f1, f2, n3)
  {
    const int f2 = d1;
    float2 w[8];
#pragma unroll
    for (int n3 = 1; n3 < 8; ++n3) w[n3] = t3[n3 * 8 + f2];
    const int p0 = C::at(k2, f1o, f2, 0, li);
    rounds<N2>([&](int i) {
      const int p = p0 + i * DK2;
      float2 v[8];
#pragma unroll
      for (int f3 = 0; f3 < 8; ++f3) v[f3] = sm[p + f3 * TC];
      RDft<8, +1>::run(v);
      sm[p] = v[0];
#pragma unroll
      for (int n3 = 1; n3 < 8; ++n3) sm[p + n3 * TC] = cmul(v[n3], w[n3]);
    });
  }
  __syncthreads();
  // I2: inverse DFT-8 over f2 -> n2, twiddle wL^(-(8 n2 + n3) f1); position (f1, n2, n3)
  // (row f1 = 0 of the table is exactly 1, so that row's products are exact)
  {
    const int n3 = d1;
    float2 w[8];
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) w[n2] = cj(t1[f1o * 64 + 8 * n2 + n3]);
    const int p0 = C::at(k2, f1o, 0, n3, li);
    rounds<N2>([&](int i) {
      const int p = p0 + i * DK2;
      float2 v[8];
#pragma unroll
      for (int f2 = 0; f2 < 8; ++f2) v[f2] = sm[p + f2 * SB];
      RDft<8, +1>::run(v);
#pragma unroll
      for (int n2 = 0; n2 < 8; ++n2) sm[p + n2 * SB] = cmul(v[n2], w[n2]);
    });
  }
  __syncthreads();
  // I3: inverse DFT-R1 over f1 -> n1, the kept half n1 < R1/2 written back
  {
    const int n3 = d1, n2 = e2;
    const int p0 = C::at(k1, 0, n2, n3, li);
    const int64_t g64 = 64 * a.inner;
    float2* g0 = base + k1 * plane + (int64_t)(8 * n2 + n3) * a.inner + li;
    rounds<N1>([&](int i) {
      const int p = p0 + i * DK1;
      float2 v[R1];
#pragma unroll
      for (int f1 = 0; f1 < R1; ++f1) v[f1] = sm[p + f1 * SA];
      RDft<R1, +1>::run(v);
      float2* g = g0 + (int64_t)i * (kL8Threads / C::NT1) * plane;
#pragma unroll
      for (int n1 = 0; n1 < H; ++n1) g[n1 * g64] = v[n1];
    });
  }
}

template <class C, int KK>
int launch8(const LamPassArgs& a, dim3 grid, cudaStream_t st) {
  if constexpr (C::smem(KK) > kL8MaxSmem) {
    return MRSR_ERR_UNSUPPORTED;
  } else {
    constexpr size_t smem = C::smem(KK);
    MRSR_CHECK_CUDA(cudaFuncSetAttribute(k8_lambda<C, KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k8_lambda<C, KK><<<grid, kL8Threads, smem, st>>>(a);
    MRSR_LAUNCH_CHECK();
    return MRSR_OK;
  }
}

template <class C>
int dispatch8(const LamPassArgs& a, dim3 grid, cudaStream_t st) {
  static_assert(kL8MaxK == 6, "one case per K");
  switch (a.K) {
    case 1: return launch8<C, 1>(a, grid, st);
    case 2: return launch8<C, 2>(a, grid, st);
    case 3: return launch8<C, 3>(a, grid, st);
    case 4: return launch8<C, 4>(a, grid, st);
    case 5: return launch8<C, 5>(a, grid, st);
    default: return launch8<C, 6>(a, grid, st);
  }
}

size_t smem8(int L, int TC, int K) {
  if (L == 512) return TC == 4 ? L8<8, 4>::smem(K) : L8<8, 8>::smem(K);
  return TC == 4 ? L8<4, 4>::smem(K) : L8<4, 8>::smem(K);
}

}  // namespace

bool lambda8_supported(const LamPassArgs& a) {
  const bool shape = (a.pl.L == 512 || a.pl.L == 256) && (a.TC == 4 || a.TC == 8);
  // the voxel step's rounds take two Λ chunks of 256 entries (FC * TC = 256) each
  return shape && a.nin == a.pl.L / 2 && a.nout == a.pl.L / 2 && !lam_is_diag(a.lam_mode) && a.K >= 1 &&
         a.FC * a.TC == 256 && a.NCH * a.FC == a.pl.L &&
         a.K <= kL8MaxK && smem8(a.pl.L, a.TC, a.K) <= kL8MaxSmem && a.inner % a.TC == 0 &&
         (reinterpret_cast<uintptr_t>(a.stack) & 15) == 0;  // 16-byte staging copies
}

int fast_lambda8(const LamPassArgs& a, int ncg, cudaStream_t st) {
  MRSR_REQUIRE(lambda8_supported(a), MRSR_ERR_UNSUPPORTED, "three-step Λ pass: 256- or 512-point pruned lines only");
  LamPassArgs b = a;
  b.ncg = ncg;
  b.fcd = FastDiv((uint32_t)a.FC);
  const dim3 grid((unsigned)((a.inner / a.TC) * ncg));
  if (a.pl.L == 512) return a.TC == 4 ? dispatch8<L8<8, 4>>(b, grid, st) : dispatch8<L8<8, 8>>(b, grid, st);
  return a.TC == 4 ? dispatch8<L8<4, 4>>(b, grid, st) : dispatch8<L8<4, 8>>(b, grid, st);
}

}  // namespace mrsr
