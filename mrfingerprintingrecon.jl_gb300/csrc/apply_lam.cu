// Λ pass of the float32 operator with register four-step transforms (see fft4.cuh):
// forward FFT along the last axis of K planes of a column tile (the pruned input half
// zero), the per-voxel K x K kernel product on the spectrum held in the exchange buffer,
// and the inverse FFT keeping the image half, in place, one (tile, coil) per CTA.
// src/NFFTNormalOp.jl:227-267 / ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218.
//
// (A variant with the slot geometry fixed at compile time, so that every exchange-buffer
// index folds into an immediate offset, measured 0.1664 against 0.168 ms on 256^2 with
// 20 coils and K = 5 and was not kept: the pass is not bound by its index arithmetic.)
#include "fft4.cuh"
#include "fft4_launch.cuh"
#include "passes.cuh"

namespace mrsr {

// stacked right-hand sides: every plane times the same scalar kernel entry, at every
// frequency f of the tile (any number of planes)
template <class SP, class SL>
__device__ __forceinline__ void lam_voxels_diag(const LamPassArgs& a, float2* sm, const SL& sl, int64_t tile) {
  constexpr int R1 = SP::R1, L = SP::L;
  const int T = L << sl.tcs;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    const int li = t & (sl.TC - 1);
    const int f = t >> sl.tcs;
    const int f1 = f % R1, f2 = f / R1;
    const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
    const float2 l = lam_diag_entry(a.lam_mode, a.lam, ((tile * a.NCH + ch) * (int64_t)a.FC + fc) * sl.TC + li);
    for (int k = 0; k < a.K; ++k) {
      float2* v = &sm[sl.at(k, f1, f2, li, R1)];
      *v = cmul(l, *v);
    }
  }
}

// per-voxel K x K product at every frequency f of the tile, rank KK known at compile time
template <class SP, int KK, class SL>
__device__ __forceinline__ void lam_voxels(const LamPassArgs& a, float2* sm, const SL& sl, int64_t tile) {
  constexpr int R1 = SP::R1, L = SP::L;
  const int64_t pstride = (int64_t)a.FC * sl.TC;
  const int T = L << sl.tcs;
  if (a.lam_mode == LAM_PACKED_REAL) {
    // packed real kernel: the next voxel's entries load while this one is multiplied
    constexpr int P = KK * (KK + 1) / 2;
    const float* lam = reinterpret_cast<const float*>(a.lam);
    auto lbase_of = [&](int tt) -> int64_t {
      const int f = tt >> sl.tcs;
      const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
      return (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * sl.TC + (tt & (sl.TC - 1));
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
      const int li = t & (sl.TC - 1);
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
    const int li = t & (sl.TC - 1);
    const int f = t >> sl.tcs;          // f = f1 + R1 f2
    const int f1 = f % R1, f2 = f / R1;
    float2 X[KK], Y[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) X[k] = sm[sl.at(k, f1, f2, li, R1)];
    const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
    const int64_t lbase = (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * sl.TC + li;
    lam_apply_ptr<KK>(a.lam_mode, KK, a.lam, lbase, pstride, X, Y);
#pragma unroll
    for (int k = 0; k < KK; ++k) sm[sl.at(k, f1, f2, li, R1)] = Y[k];
  }
}

template <class SP, bool PR, class SL>
__global__ void __launch_bounds__(256, 2) k4_lambda(LamPassArgs a, SL sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles(tw, a.pl);
  // coil fastest: the CTAs of one column tile run together and share its Λ tile in L2
  const int cl = (int)(blockIdx.x % (unsigned)a.ncg);
  const int64_t tile = blockIdx.x / (unsigned)a.ncg;
  const int64_t plane = (int64_t)a.nrow * a.inner;
  float2* base = a.stack + (int64_t)cl * a.K * plane + tile * sl.TC;
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

int fast_lambda(const LamPassArgs& a, int ncg, int planes_total, int* errword, cudaStream_t st) {
  return with_split(a.pl.L, [&](auto sp) -> int {
    using SP = decltype(sp);
    const Slots sl = make_slots(SP::R2, a.TC);
    const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)a.K * SP::R1 * sl.W);
    LamPassArgs b = a;
    b.ncg = ncg;
    b.fcd = FastDiv((uint32_t)a.FC);
    dim3 grid((unsigned)((a.inner / a.TC) * ncg));
    if (a.nin * 2 == SP::L && a.nout * 2 == SP::L) return launch(k4_lambda<SP, true, Slots>, grid, 256, smem, st, b, sl);
    return launch(k4_lambda<SP, false, Slots>, grid, 256, smem, st, b, sl);
  });
}

}  // namespace mrsr
