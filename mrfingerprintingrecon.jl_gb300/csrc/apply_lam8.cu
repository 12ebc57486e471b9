// Λ pass of the float32 operator for 256- and 512-point lines (the 128^3 volumes' and the
// 256^2 images' last axes) as the three-step transforms of three_step.cuh: stage the tile's
// zero-padded columns, three forward steps, the K x K kernel at every cell of the line, three
// inverse steps with the kept half written back.  Every task holds at most eight values, so
// the kernel runs 512-thread CTAs two per SM: 32 warps per SM against 16 for the two-step
// kernels (apply_lam.cu), which are bound by latency, not by arithmetic; the price is one
// more shared-memory exchange each way.
// src/NFFTNormalOp.jl:227-267 / ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218.
#include "three_step.cuh"

namespace mrsr {

namespace {

using namespace l8;

constexpr int kL8MaxK = 6;

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
  constexpr int TC = C::TC, LT = C::LT, H = C::R1 / 2;
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
  const Own<C> o;
  step_f1<C, KK>(sm, t1, o);
  __syncthreads();
  step_f2<C, KK>(sm, t2, o);
  __syncthreads();
  step_f3<C, KK>(sm, o);
  __syncthreads();
  lam8_voxels<C, KK>(a, sm, tile);
  __syncthreads();
  step_i1<C, KK>(sm, t3, o);
  __syncthreads();
  step_i2<C, KK>(sm, t1, o);
  __syncthreads();
  // I3: the kept half n1 < R1/2 written back to the columns
  const int64_t g64 = 64 * a.inner;
  float2* g0 = base + o.k1 * plane + (int64_t)(8 * o.e2 + o.d1) * a.inner + o.li;
  step_i3<C, KK>(sm, o, [&](int i, const float2* v) {
    float2* g = g0 + (int64_t)i * (kL8Threads / C::NT1) * plane;
#pragma unroll
    for (int n1 = 0; n1 < H; ++n1) g[n1 * g64] = v[n1];
  });
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
