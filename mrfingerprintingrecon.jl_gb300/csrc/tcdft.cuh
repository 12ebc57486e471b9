// Shared pieces of the tensor-core passes (apply_tc.cu, apply_tc_rows.cu): the real
// 64-point DFT matrix as an fp16 K-major MMA operand, the 512-point twiddles, radix-4
// butterflies, power-of-two operand scales and the TMEM loads.
#pragma once
#include "umma.cuh"

#include <cuda_fp16.h>

namespace mrsr {
namespace tcdft {

constexpr int kL = 512;        // transform length: 8 x 64
constexpr int kAbytes = 128 * 128 * 2;

constexpr int kConstBytes = kAbytes + kL * 8;  // the DFT-64 operand, then the twiddles

// Copy of the constants built once per operator (build_constants): 16-byte vector loads.
__device__ __forceinline__ void load_constants(unsigned char* sA, float2* tw, const unsigned char* g, int tid,
                                               int nthreads) {
  const uint4* src = reinterpret_cast<const uint4*>(g);
  for (int i = tid; i < kAbytes / 16; i += nthreads) reinterpret_cast<uint4*>(sA)[i] = src[i];
  for (int i = tid; i < kL * 8 / 16; i += nthreads) reinterpret_cast<uint4*>(tw)[i] = src[kAbytes / 16 + i];
}

// A[m][kk], m = 2 f2 + {re, im}, kk = 2 n2 + {re, im}: the real form of w64^(n2 f2),
// written in the K-major core-matrix layout with LBO = 128, SBO = 2048; tw[p] = w512^p.
__device__ __forceinline__ void setup_constants(unsigned char* sA, float2* tw, int tid, int nthreads) {
  for (int e = tid; e < 128 * 128; e += nthreads) {
    const int m = e >> 7, kk = e & 127;
    const int f2 = m >> 1, n2 = kk >> 1;
    float s, c;
    sincospif((float)((f2 * n2) & 63) / 32.f, &s, &c);  // w64^(n2 f2) = c - i s
    float v;
    if ((m & 1) == 0)
      v = (kk & 1) == 0 ? c : s;   // Re: c * xr - (-s) * xi
    else
      v = (kk & 1) == 0 ? -s : c;  // Im: (-s) * xr + c * xi
    *reinterpret_cast<__half*>(sA + umma::kmajor_off16(m, kk, 128)) = __float2half_rn(v);
  }
  for (int p = tid; p < kL; p += nthreads) {
    float s, c;
    sincospif((float)p / 256.f, &s, &c);
    tw[p] = make_float2(c, -s);
  }
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 cmulcf(float2 a, float2 b) {  // a * conj(b)
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ float2 caddf(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csubf(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 mul_mi(float2 a) { return make_float2(a.y, -a.x); }  // -i a
__device__ __forceinline__ float2 mul_pi(float2 a) { return make_float2(-a.y, a.x); }  // +i a

// 4-point DFT, sign S = -1 forward (w = -i), +1 inverse (w = +i)
template <int S>
__device__ __forceinline__ void dft4(float2 a, float2 b, float2 c, float2 d, float2* o) {
  const float2 s0 = caddf(a, c), s1 = csubf(a, c), s2 = caddf(b, d), s3 = csubf(b, d);
  const float2 r3 = S < 0 ? mul_mi(s3) : mul_pi(s3);
  o[0] = caddf(s0, s2);
  o[1] = caddf(s1, r3);
  o[2] = csubf(s0, s2);
  o[3] = csubf(s1, r3);
}

template <int NTHREADS>
__device__ __forceinline__ float block_max(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float m = red[0];
#pragma unroll
  for (int w = 1; w < NTHREADS / 32; ++w) m = fmaxf(m, red[w]);
  __syncthreads();
  return m;
}

// power-of-two scale that maps a bound `m` below 2^14 (fp16's largest finite is 65504)
__device__ __forceinline__ int scale_exp(float m) { return m > 0.f ? 13 - ilogbf(m) : 0; }

__device__ __forceinline__ void st_half2(unsigned char* base, uint32_t off, float re, float im) {
  *reinterpret_cast<__half2*>(base + off) = __floats2half2_rn(re, im);
}

// Two adjacent TMEM columns (this lane's row) of each of the K planes, one wait for all.
template <int K>
__device__ __forceinline__ void tmem_ld2_planes(uint32_t taddr, float (*v)[2]) {
  uint32_t r[16];
  // columns k * 32 (k < K; k >= K repeats the last plane)
  const uint32_t a0 = taddr, a1 = taddr + 32 * (1 < K), a2 = taddr + 32 * (2 < K ? 2 : K - 1),
                 a3 = taddr + 32 * (3 < K ? 3 : K - 1), a4 = taddr + 32 * (4 < K ? 4 : K - 1),
                 a5 = taddr + 32 * (5 < K ? 5 : K - 1), a6 = taddr + 32 * (6 < K ? 6 : K - 1),
                 a7 = taddr + 32 * (7 < K ? 7 : K - 1);
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%16];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%2,%3}, [%17];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%4,%5}, [%18];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%6,%7}, [%19];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%8,%9}, [%20];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%10,%11}, [%21];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%12,%13}, [%22];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x2.b32 {%14,%15}, [%23];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(a4), "r"(a5), "r"(a6), "r"(a7)
      : "memory");
#pragma unroll
  for (int k = 0; k < K; ++k) {
    v[k][0] = __uint_as_float(r[2 * k]);
    v[k][1] = __uint_as_float(r[2 * k + 1]);
  }
}

// 32 consecutive TMEM columns of this lane's row.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}


// 8 consecutive TMEM columns of this lane's row.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tcdft
}  // namespace mrsr
