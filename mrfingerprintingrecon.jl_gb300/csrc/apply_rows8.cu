// Inverse row pass of the float32 operator for 256- and 512-point rows (the first axis of the
// 128^3 volumes and 256^2 images, twice oversampled) as the three-step inverse transform of
// three_step.cuh: transform back, keep the first half, combine the coils with conj(cmaps),
// y = alpha * sum + beta * y.  A CTA takes one row of one plane and all coils of the group
// (G = ceil(Nc / 4) groups of 4 lines, Nc <= 20); its first step reads the lines from global
// memory and its last sums the coils from registers: across the four lines of a group by
// warp shuffles, across the groups in registers and, for the two thread halves, through
// shared memory.  512-thread CTAs two per SM: 32 warps per SM against 16 for the two-step
// kernel (apply_fast.cu), whose radix-32 register DFTs need 109 registers.  (The forward row
// pass stays two-step: it writes twice what it reads and has one exchange instead of two, and
// a three-step form measured 0.045 against 0.039 ms on 256^2 with 20 coils.)
// src/NFFTNormalOp.jl:227-267 / ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218
// (the ifft! of the oversampled coil images and the sum over coils).
#include "three_step.cuh"

namespace mrsr {

namespace {

using namespace l8;

constexpr int kRowsTC = 4;     // lines per group
constexpr int kRowsMaxG = 5;   // inverse: coil groups per CTA (20 coils)

template <class C, int G>
__global__ void __launch_bounds__(kL8Threads, 2) k8_rows_inv(RowsInvArgs a) {
  constexpr int R1 = C::R1, L = C::L, H = R1 / 2, LR = C::LR, TC = C::TC;
  static_assert(TC == kRowsTC && C::NT1 * 2 == kL8Threads, "four coils per group, two thread halves");
  extern __shared__ float2 smem[];
  float2* t1 = smem;
  const float2* t3 = smem + C::T1 + C::T2;
  float2* sm = smem + C::TW;
  const int tid = threadIdx.x;
  const int64_t r = blockIdx.x;
  const int k = blockIdx.y;
  const int n1len = L / 2;
  // ask L2 for the CTA's lines and coil map rows first (128-byte lines), so that the loads of
  // the first and the last step find them there
  {
    constexpr int LPL = L * 8 / 128;        // 128-byte lines per stack line
    constexpr int LPC = (L / 2) * 8 / 128;  // per coil map row
    const int nst = a.ncg * LPL, ncm = a.cmaps ? a.ncg * LPC : 0;
    for (int j = tid; j < nst + ncm; j += kL8Threads) {
      const float2* q;
      if (j < nst) {
        const int cl = j / LPL;
        q = a.stack + (((int64_t)cl * a.K + k) * a.nrows + r) * L + (j - cl * LPL) * 16;
      } else {
        const int jc = j - nst, cl = jc / LPC;
        q = a.cmaps + (int64_t)n1len * (r + a.nrows * (a.c0 + cl)) + (jc - cl * LPC) * 16;
      }
      asm volatile("prefetch.global.L2 [%0];" ::"l"(q));
    }
  }
  build_tables<C>(t1, a.pl);
  __syncthreads();
  const Own<C> o;
  // I1 straight from global memory: the thread owns (li, f1, f2) of the coil groups g0,
  // g0 + 512 / NT2, ...; its inputs are X[f1 + R1 f2 + 8 R1 f3] of coil 4 g + li, lanes vary
  // li and f1 (four coils x eight consecutive frequencies), and the writes at (f1, f2, n3) are
  // conflict-free
  {
    const int li = tid & (TC - 1), f1 = (tid >> 2) & (R1 - 1), f2 = (tid >> (2 + LR)) & 7, g0 = tid >> (2 + LR + 3);
    float2 w[8];
#pragma unroll
    for (int n3 = 1; n3 < 8; ++n3) w[n3] = t3[n3 * 8 + f2];
    const int p0 = C::at(g0, f1, f2, 0, li);
    constexpr int DG = kL8Threads / C::NT2;
    rounds<G * C::NT2>([&](int i) {
      const int p = p0 + i * DG * C::SP;
      const int cl = TC * (g0 + i * DG) + li;
      float2 v[8];
      if (cl < a.ncg) {
        const float2* q = a.stack + (((int64_t)cl * a.K + k) * a.nrows + r) * L + f1 + R1 * f2;
#pragma unroll
        for (int f3 = 0; f3 < 8; ++f3) v[f3] = q[8 * R1 * f3];
      } else {
#pragma unroll
        for (int f3 = 0; f3 < 8; ++f3) v[f3] = make_float2(0.f, 0.f);
      }
      RDft<8, +1>::run(v);
      sm[p] = v[0];
#pragma unroll
      for (int n3 = 1; n3 < 8; ++n3) sm[p + n3 * TC] = cmul(v[n3], w[n3]);
    });
  }
  __syncthreads();
  step_i2<C, G>(sm, t1, o);
  __syncthreads();
  // I3 with the coil sum: the thread's outputs are n = 64 n1 + 8 n2 + n3 (n1 < R1/2) of line
  // li in the groups k1, k1 + 2, ...
  const int nb = 8 * o.e2 + o.d1;
  float2 acc[H];
#pragma unroll
  for (int n1 = 0; n1 < H; ++n1) acc[n1] = make_float2(0.f, 0.f);
  step_i3<C, G>(sm, o, [&](int i, const float2* v) {
    const int cl = TC * (o.k1 + 2 * i) + o.li;
    if (cl >= a.ncg) return;
    if (a.cmaps) {
      const float2* cm = a.cmaps + nb + (int64_t)n1len * (r + a.nrows * (a.c0 + cl));
#pragma unroll
      for (int n1 = 0; n1 < H; ++n1) acc[n1] = cadd(acc[n1], cmulc(v[n1], cm[64 * n1]));
    } else {
#pragma unroll
      for (int n1 = 0; n1 < H; ++n1) acc[n1] = cadd(acc[n1], v[n1]);
    }
  });
  // the four lines of a group are adjacent lanes
#pragma unroll
  for (int n1 = 0; n1 < H; ++n1) {
#pragma unroll
    for (int s = 1; s < TC; s <<= 1) {
      acc[n1].x += __shfl_xor_sync(0xffffffffu, acc[n1].x, s);
      acc[n1].y += __shfl_xor_sync(0xffffffffu, acc[n1].y, s);
    }
  }
  // lane li keeps output n1 = li; the upper thread half hands its sums to the lower through
  // the first twiddle table, which the last step no longer reads
  float2 mine = acc[0];
#pragma unroll
  for (int n1 = 1; n1 < H; ++n1)
    if (o.li == n1) mine = acc[n1];
  float2* red = t1;
  if (o.k1 == 1 && o.li < H) red[64 * o.li + nb] = mine;
  __syncthreads();
  if (o.k1 == 0 && o.li < H) {
    const int n = 64 * o.li + nb;
    const float2 s = cadd(mine, red[n]);
    const int64_t yi = n + (int64_t)n1len * (r + a.nrows * k);
    float2 yv;
    if (a.first)
      yv = (a.beta.x == 0.f && a.beta.y == 0.f) ? make_float2(0.f, 0.f) : cmul(a.beta, a.y[yi]);
    else
      yv = a.y[yi];
    a.y[yi] = cadd(yv, cmul(a.alpha, s));
  }
}

template <class K, class A>
int launch_rows(K kern, dim3 grid, size_t smem, cudaStream_t st, const A& a) {
  MRSR_REQUIRE(smem <= kL8MaxSmem, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, kL8Threads, smem, st>>>(a);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

template <class C>
int inv8(const RowsInvArgs& a, cudaStream_t st) {
  const int G = (int)cdiv(a.ncg, kRowsTC);
  const dim3 grid((unsigned)a.nrows, (unsigned)a.K);
  const size_t smem = C::smem(G);
  switch (G) {
    case 1: return launch_rows(k8_rows_inv<C, 1>, grid, smem, st, a);
    case 2: return launch_rows(k8_rows_inv<C, 2>, grid, smem, st, a);
    case 3: return launch_rows(k8_rows_inv<C, 3>, grid, smem, st, a);
    case 4: return launch_rows(k8_rows_inv<C, 4>, grid, smem, st, a);
    default: return launch_rows(k8_rows_inv<C, 5>, grid, smem, st, a);
  }
}

}  // namespace

bool rows8_inv_supported(const RowsInvArgs& a) {
  return (a.pl.L == 512 || a.pl.L == 256) && a.n1 * 2 == a.pl.L && a.ncg >= 1 && a.ncg <= kRowsTC * kRowsMaxG &&
         a.nrows <= 0x7fffffff && a.K <= 65535;
}

int fast_rows8_inv(const RowsInvArgs& a, cudaStream_t st) {
  MRSR_REQUIRE(rows8_inv_supported(a), MRSR_ERR_UNSUPPORTED, "three-step row pass: 256- or 512-point rows, <= 20 coils");
  return a.pl.L == 512 ? inv8<L8<8, kRowsTC>>(a, st) : inv8<L8<4, kRowsTC>>(a, st);
}

}  // namespace mrsr
