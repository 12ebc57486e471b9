// Shared pieces of the fp16-storage operator (apply_half.cu):
// tile geometry of the per-tile scale arrays and launch helpers.
#pragma once
#include <algorithm>

#include "fft4.cuh"
#include "normalop.cuh"

namespace mrsr {

__device__ __forceinline__ float amax2(float2 v) { return fmaxf(fabsf(v.x), fabsf(v.y)); }

// block-wide max of per-thread maxima; every thread of the block calls it.
// Non-negative floats order like their bit patterns read as unsigned.
__device__ __forceinline__ void block_max_commit(float* m, float local) {
  const unsigned u = __reduce_max_sync(0xffffffffu, __float_as_uint(local));
  if ((threadIdx.x & 31) == 0) atomicMax(reinterpret_cast<unsigned*>(m), u);
}

struct HalfTiles {
  int rpc;           // rows per CTA of the row passes
  int64_t nrowblk;   // row blocks per plane group
  int TCm, NOo;      // dim-2 pass tiling (3D)
  int64_t nslab, nmtile;
  float* s_rows;     // [coil][row block]
  float* s_mid;      // [plane][slab][column tile]
  float* s_lam;      // [coil][tile]
  float* s_mid2;     // [plane][slab][column tile]
};

template <class F>
inline int with_split_h(int L, F f) {
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

inline Slots slots_for(int R2, int TC) {
  Slots s;
  s.TC = TC;
  s.tcs = 0;
  while ((1 << s.tcs) < TC) ++s.tcs;
  s.W = slots_width(R2, TC);
  return s;
}

inline int rthreads(int tasks) {
  int t = ((tasks + 31) / 32) * 32;
  return t < 128 ? 128 : (t > 512 ? 512 : t);
}

// scale-array sizes of the fp16 tiles (same formulas as the launches below)
inline HalfTiles tiles_of(const mrsr_normalop* op) {
  const OpGeom& g = op->geo;
  HalfTiles t{};
  const int L1 = (int)g.g[0];
  const int64_t nrows = g.n[1] * g.n[2];
  t.rpc = (int)std::max<int64_t>(1, std::min<int64_t>(4096 / ((int64_t)std::max(g.K, op->Cg) * L1), nrows));
  t.nrowblk = cdiv(nrows, t.rpc);
  t.TCm = 8;
  while (t.TCm > 1 && g.g[0] % t.TCm) t.TCm >>= 1;
  t.NOo = (int)std::max<int64_t>(1, std::min<int64_t>(4096 / ((int64_t)t.TCm * g.g[1]), g.n[2]));
  t.nslab = cdiv(g.n[2], t.NOo);
  t.nmtile = g.g[0] / t.TCm;
  return t;
}

}  // namespace mrsr
