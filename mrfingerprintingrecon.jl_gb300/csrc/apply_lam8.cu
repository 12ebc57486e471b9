// Λ pass of the float32 operator for 512-point lines (the 256^2 NFFT operator's columns) as
// three radix-8 steps each way: 512 = 8 x 8 x 8,
//   n = 64 n1 + 8 n2 + n3,  f = f1 + 8 f2 + 64 f3,
//   X[f] = sum_n3 w8^(n3 f3) w64^(n3 f2) sum_n2 w8^(n2 f2) [w512^((8 n2 + n3) f1) sum_n1 w8^(n1 f1) x[n]]
// with the input pruned to n1 < 4 (the zero-padded half) and the inverse's output to n1 < 4
// (the kept half).  Every task holds eight values (one DFT-8), so the kernel fits in 64
// registers and runs 512-thread CTAs two per SM: 32 warps per SM against 16 for the
// two-step radix-16 x 32 kernel (apply_lam.cu), which is bound by latency, not by its
// arithmetic.  The price is one more shared-memory exchange each way.
// src/NFFTNormalOp.jl:227-267 / ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218.
//
// Shared layout of plane k, column li (TC = 4 columns per tile): position (a, b, c) of three
// octal digits at k * 2336 + a * 292 + b * 36 + c * 4 + li (float2 units).  Every step's warp
// varies li and one of a, b, c (the rest fixed); the strides are 4 (mod 16), so the 16 lanes
// of a half-warp touch 16 distinct 8-byte bank pairs for any of the three, and a task's
// running digit is a compile-time loop index, so its eight addresses are one register plus
// immediate offsets.  A task reads and writes the same eight positions (one digit running),
// so every step works in place.
#include "fft4.cuh"
#include "passes.cuh"

namespace mrsr {

namespace {

constexpr int kL8 = 512, kTC8 = 4, kL8Threads = 512;

constexpr int kSB8 = 36, kSA8 = 292, kSP8 = 2336;  // digit b, digit a and plane strides
static_assert(kSB8 >= 8 * 4 && kSA8 >= 8 * kSB8 && kSP8 >= 8 * kSA8, "8 x 8 x 8 positions x 4 columns");
static_assert(kSB8 % 16 == 4 && kSA8 % 16 == 4, "a half-warp on 16 distinct bank pairs");

__device__ __forceinline__ int p8(int k, int a, int b, int c, int li) { return k * kSP8 + a * kSA8 + b * kSB8 + c * 4 + li; }

__device__ __forceinline__ float2 cj(float2 w) { return make_float2(w.x, -w.y); }

// Twiddle tables in the order the steps' lanes read them (a warp's lanes vary n3 or f2 with
// the loop digit fixed, so each table read is 8 consecutive entries, bank-conflict free; a
// table indexed (m * f) & 511 would put the lanes of an even f on the same banks):
//   t1[f1 * 64 + m] = w512^(m f1), m = 8 n2 + n3     (F1, I2 conjugated)
//   t2[f2 * 8 + n3] = w64^(n3 f2)                    (F2)
//   t3[n3 * 8 + f2] = w64^(-n3 f2)                   (I1)
constexpr int kT1 = 512, kT2 = 64, kT3 = 64, kTwTables = kT1 + kT2 + kT3;

__device__ __forceinline__ void build_tables(float2* t, const FftPlan& pl) {
  const float2* w = pl.tw;  // w512^p
  for (int i = threadIdx.x; i < kTwTables; i += blockDim.x) {
    int p;
    bool conj = false;
    if (i < kT1) {
      p = (i & 63) * (i >> 6);
    } else if (i < kT1 + kT2) {
      const int j = i - kT1;
      p = 8 * (j & 7) * (j >> 3);
    } else {
      const int j = i - kT1 - kT2;
      p = 8 * (j >> 3) * (j & 7);
      conj = true;
    }
    const float2 v = w[p & (kL8 - 1)];
    t[i] = conj ? cj(v) : v;
  }
}

template <int KK>
__device__ __forceinline__ void lam8_voxels(const LamPassArgs& a, float2* sm, int64_t tile) {
  const int64_t pstride = (int64_t)a.FC * kTC8;
  constexpr int T = kL8 * kTC8;
  auto lbase_of = [&](int t) -> int64_t {
    const int f = t >> 2;
    const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
    return (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * kTC8 + (t & 3);
  };
  if (a.lam_mode == LAM_PACKED_REAL) {
    constexpr int P = KK * (KK + 1) / 2;
    const float* lam = reinterpret_cast<const float*>(a.lam);
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
      const int64_t lb = lbase_of(t);
      float lc[P];
#pragma unroll
      for (int p = 0; p < P; ++p) lc[p] = lam[lb + p * pstride];
      const int li = t & 3, f = t >> 2;
      const int f1 = f & 7, f2 = (f >> 3) & 7, f3 = f >> 6;
      float2 X[KK], Y[KK];
#pragma unroll
      for (int k = 0; k < KK; ++k) X[k] = sm[p8(k, f1, f2, f3, li)];
      lam_real_regs<KK>(lc, X, Y);
#pragma unroll
      for (int k = 0; k < KK; ++k) sm[p8(k, f1, f2, f3, li)] = Y[k];
    }
    return;
  }
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int li = t & 3, f = t >> 2;
    const int f1 = f & 7, f2 = (f >> 3) & 7, f3 = f >> 6;
    float2 X[KK], Y[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) X[k] = sm[p8(k, f1, f2, f3, li)];
    lam_apply_ptr<KK>(a.lam_mode, KK, a.lam, lbase_of(t), pstride, X, Y);
#pragma unroll
    for (int k = 0; k < KK; ++k) sm[p8(k, f1, f2, f3, li)] = Y[k];
  }
}

template <int KK>
__global__ void __launch_bounds__(kL8Threads, 2) k8_lambda(LamPassArgs a) {
  extern __shared__ float2 smem[];
  float2* t1 = smem;                 // twiddle tables
  const float2* t2 = smem + kT1;
  const float2* t3 = smem + kT1 + kT2;
  float2* sm = smem + kTwTables;     // positions p8(k, a, b, c, li)
  build_tables(t1, a.pl);
  const int cl = (int)(blockIdx.x % (unsigned)a.ncg);
  const int64_t tile = blockIdx.x / (unsigned)a.ncg;
  const int64_t plane = (int64_t)a.nrow * a.inner;
  float2* base = a.stack + (int64_t)cl * KK * plane + tile * kTC8;
  constexpr int NT = KK * 256;  // tasks per step: k, two octal digits, li
  __syncthreads();
  // F1: DFT-8 over n1 (n1 < 4 nonzero) -> f1, twiddle w512^((8 n2 + n3) f1); position (f1, n2, n3)
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int li = t & 3, n3 = (t >> 2) & 7, n2 = (t >> 5) & 7, k = t >> 8;
    float2 v[8];
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) v[n1] = base[k * plane + (int64_t)(64 * n1 + 8 * n2 + n3) * a.inner + li];
#pragma unroll
    for (int n1 = 4; n1 < 8; ++n1) v[n1] = make_float2(0.f, 0.f);
    RDft<8, -1>::run(v);
    const int m = 8 * n2 + n3;
#pragma unroll
    for (int f1 = 0; f1 < 8; ++f1) sm[p8(k, f1, n2, n3, li)] = f1 == 0 ? v[0] : cmul(v[f1], t1[f1 * 64 + m]);
  }
  __syncthreads();
  // F2: DFT-8 over n2 -> f2, twiddle w64^(n3 f2) = w512^(8 n3 f2); position (f1, f2, n3)
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int li = t & 3, n3 = (t >> 2) & 7, f1 = (t >> 5) & 7, k = t >> 8;
    float2 v[8];
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2) v[n2] = sm[p8(k, f1, n2, n3, li)];
    RDft<8, -1>::run(v);
#pragma unroll
    for (int f2 = 0; f2 < 8; ++f2) sm[p8(k, f1, f2, n3, li)] = f2 == 0 ? v[0] : cmul(v[f2], t2[f2 * 8 + n3]);
  }
  __syncthreads();
  // F3: DFT-8 over n3 -> f3; X[f1 + 8 f2 + 64 f3] at position (f1, f2, f3)
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int li = t & 3, f2 = (t >> 2) & 7, f1 = (t >> 5) & 7, k = t >> 8;
    float2 v[8];
#pragma unroll
    for (int n3 = 0; n3 < 8; ++n3) v[n3] = sm[p8(k, f1, f2, n3, li)];
    RDft<8, -1>::run(v);
#pragma unroll
    for (int f3 = 0; f3 < 8; ++f3) sm[p8(k, f1, f2, f3, li)] = v[f3];
  }
  __syncthreads();
  lam8_voxels<KK>(a, sm, tile);
  __syncthreads();
  // I1: inverse DFT-8 over f3 -> n3, twiddle w64^(-n3 f2); position (f1, f2, n3)
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int li = t & 3, f2 = (t >> 2) & 7, f1 = (t >> 5) & 7, k = t >> 8;
    float2 v[8];
#pragma unroll
    for (int f3 = 0; f3 < 8; ++f3) v[f3] = sm[p8(k, f1, f2, f3, li)];
    RDft<8, +1>::run(v);
#pragma unroll
    for (int n3 = 0; n3 < 8; ++n3) sm[p8(k, f1, f2, n3, li)] = n3 == 0 ? v[0] : cmul(v[n3], t3[n3 * 8 + f2]);
  }
  __syncthreads();
  // I2: inverse DFT-8 over f2 -> n2, twiddle w512^(-(8 n2 + n3) f1); position (f1, n2, n3)
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int li = t & 3, n3 = (t >> 2) & 7, f1 = (t >> 5) & 7, k = t >> 8;
    float2 v[8];
#pragma unroll
    for (int f2 = 0; f2 < 8; ++f2) v[f2] = sm[p8(k, f1, f2, n3, li)];
    RDft<8, +1>::run(v);
#pragma unroll
    for (int n2 = 0; n2 < 8; ++n2)
      sm[p8(k, f1, n2, n3, li)] = f1 == 0 ? v[n2] : cmul(v[n2], cj(t1[f1 * 64 + 8 * n2 + n3]));
  }
  __syncthreads();
  // I3: inverse DFT-8 over f1 -> n1, the kept half n1 < 4 written back
  for (int t = threadIdx.x; t < NT; t += blockDim.x) {
    const int li = t & 3, n3 = (t >> 2) & 7, n2 = (t >> 5) & 7, k = t >> 8;
    float2 v[8];
#pragma unroll
    for (int f1 = 0; f1 < 8; ++f1) v[f1] = sm[p8(k, f1, n2, n3, li)];
    RDft<8, +1>::run(v);
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) base[k * plane + (int64_t)(64 * n1 + 8 * n2 + n3) * a.inner + li] = v[n1];
  }
}

template <int KK>
int launch8(const LamPassArgs& a, dim3 grid, cudaStream_t st) {
  const size_t smem = sizeof(float2) * ((size_t)kTwTables + (size_t)KK * kSP8);
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k8_lambda<KK>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k8_lambda<KK><<<grid, kL8Threads, smem, st>>>(a);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

}  // namespace

bool lambda8_supported(const LamPassArgs& a) {
  return a.pl.L == kL8 && a.TC == kTC8 && a.nin == kL8 / 2 && a.nout == kL8 / 2 && !lam_is_diag(a.lam_mode) &&
         a.K >= 1 && a.K <= 8 && a.inner % kTC8 == 0;
}

int fast_lambda8(const LamPassArgs& a, int ncg, cudaStream_t st) {
  MRSR_REQUIRE(lambda8_supported(a), MRSR_ERR_UNSUPPORTED, "radix-8 Λ pass: 512-point pruned lines only");
  LamPassArgs b = a;
  b.ncg = ncg;
  b.fcd = FastDiv((uint32_t)a.FC);
  const dim3 grid((unsigned)((a.inner / kTC8) * ncg));
  switch (a.K) {
    case 1: return launch8<1>(b, grid, st);
    case 2: return launch8<2>(b, grid, st);
    case 3: return launch8<3>(b, grid, st);
    case 4: return launch8<4>(b, grid, st);
    case 5: return launch8<5>(b, grid, st);
    case 6: return launch8<6>(b, grid, st);
    case 7: return launch8<7>(b, grid, st);
    default: return launch8<8>(b, grid, st);
  }
}

}  // namespace mrsr
