// Launch helpers of the register four-step kernels (apply_fast.cu, apply_lam.cu).
#pragma once
#include "fft4.cuh"
#include "passes.cuh"

namespace mrsr {

// -------------------------------------------------------- dispatch ---

template <class F>
inline int with_split(int L, F f) {
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

inline Slots make_slots(int R2, int TC) {
  Slots s;
  s.TC = TC;
  s.tcs = 0;
  while ((1 << s.tcs) < TC) ++s.tcs;
  s.W = slots_width(R2, TC);
  return s;
}

template <class K, class A, class SL>
int launch(K k, dim3 grid, int threads, size_t smem, cudaStream_t st, const A& a, const SL& sl) {
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  if (smem > 48 * 1024) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
  k<<<grid, threads, smem, st>>>(a, sl);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

}  // namespace mrsr
