// Λ pass with the column DFTs on the tensor cores (tcgen05), for the operator
// precision MRSR_PREC_FP16_TC: fp16 operands with per-tile power-of-two scales,
// float32 accumulation in TMEM; the row passes and the stack stay float32.
//
// A column of the NFFT operator's 2x grid has L = 512 = 8 x 64 points, of which
// the first 256 are nonzero on input and kept on output.  Four-step split:
//   n = 64 n1 + n2, f = f1 + 8 f2 (n1, f1 < 8; n2, f2 < 64)
//   X[f1 + 8 f2] = sum_n2 w64^(n2 f2) [ w512^(n2 f1) sum_{n1<4} x[64 n1 + n2] w8^(n1 f1) ]
// The bracket (a pruned DFT-8 and a twiddle) runs on the CUDA cores; the DFT-64
// is one MMA, D = A B with A the real form of the 64-point DFT matrix
// (rows 2 f2 + {re, im}, columns 2 n2 + {re, im}; M = K = 128) and B the
// bracket values of every (k, column, f1) vector (N = 32 K).  Each TMEM lane then
// holds one frequency row f2 (re or im) for all vectors, so the per-voxel K x K
// product needs only the re/im exchange between neighbouring lanes.  The inverse
// uses the same matrix on conjugated data, IDFT(Y) = conj(DFT(conj Y)), followed
// by the twiddle and an output-pruned inverse DFT-8 on the CUDA cores.
#include "passes.cuh"
#include "tma.cuh"
#include "umma.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace mrsr {

namespace {

constexpr int kTcL = 512, kTcTC = 4;  // L = 8 x 64; four columns per tile
constexpr int kTcThreads = 256;
constexpr uint32_t kTcTmemCols = 256;
constexpr uint32_t kTcWaitLimit = 1u << 26;  // mbarrier polls before the kernel reports a timeout
constexpr int kTcAbytes = 128 * 128 * 2;     // fp16 DFT-64 matrix, K-major core matrices

struct TcArgs {
  LamPassArgs a;
  int64_t nitems;        // column tiles x coils of the group
  int* err;
  const float* lam_max;  // device: largest |component| of any Λ entry
};

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

__device__ __forceinline__ float block_max(float v, float* red) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float m = red[0];
#pragma unroll
  for (int w = 1; w < kTcThreads / 32; ++w) m = fmaxf(m, red[w]);
  __syncthreads();
  return m;
}

// power-of-two scale that maps a bound `m` below 2^14 (fp16's largest finite is 65504)
__device__ __forceinline__ int scale_exp(float m) { return m > 0.f ? 13 - ilogbf(m) : 0; }

__device__ __forceinline__ void st_half2(unsigned char* base, uint32_t off, float re, float im) {
  *reinterpret_cast<__half2*>(base + off) = __floats2half2_rn(re, im);
}

// Λ entries of one (tile, p, j) block: 2 column pairs x 64 rows f2 x 2 (entries p are
// 8 such blocks apart)
constexpr int64_t kTcLamPstride = 8 * 256;

// Operand B: row r = k * 32 + f1 * 4 + li (a thread's two columns of one voxel are
// adjacent in TMEM), K index kk = 2 n2 + {re, im}; core matrices along K 192 bytes
// apart (128 + 64 of padding, so the half2 stores of a warp spread over all banks),
// 8-row groups 16 * 192 bytes apart.
constexpr uint32_t kTcLbo = 192, kTcSbo = 16 * kTcLbo;
__device__ __forceinline__ uint32_t boff(int r, int kk) {
  return (uint32_t)((r >> 3) * kTcSbo + (kk >> 3) * kTcLbo + (r & 7) * 16 + (kk & 7) * 2);
}
__host__ __device__ constexpr size_t tc_bbytes(int K) { return (size_t)K * 4 * kTcSbo; }
constexpr int kTcStg = kTcTC + 1;  // staging row stride (float2), padded against bank conflicts

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

// Y = Λ X at one voxel for the packed real kernel, Λ values already in registers.
template <int K>
__device__ __forceinline__ void lam_real_regs(const float* l, const float2* X, float2* Y) {
#pragma unroll
  for (int k = 0; k < K; ++k) Y[k] = make_float2(0.f, 0.f);
  int p = 0;
#pragma unroll
  for (int k2 = 0; k2 < K; ++k2)
#pragma unroll
    for (int k1 = 0; k1 <= k2; ++k1, ++p) {
      Y[k1].x = fmaf(l[p], X[k2].x, Y[k1].x);
      Y[k1].y = fmaf(l[p], X[k2].y, Y[k1].y);
      if (k1 != k2) {
        Y[k2].x = fmaf(l[p], X[k1].x, Y[k2].x);
        Y[k2].y = fmaf(l[p], X[k1].y, Y[k2].y);
      }
    }
}

template <int K>
__global__ void __launch_bounds__(kTcThreads, K <= 5 ? 2 : 1) kt_lambda(TcArgs t) {
  const LamPassArgs& a = t.a;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;                                        // DFT-64 matrix (fp16)
  unsigned char* sB = smem + kTcAbytes;                            // operand B, then the output staging
  float2* tw = reinterpret_cast<float2*>(sB + tc_bbytes(K));       // w512^p, p < 512
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ float red[kTcThreads / 32];
  __shared__ int abort_flag;
  constexpr int N = K * 32, P = K * (K + 1) / 2;
  constexpr uint32_t idesc = umma::idesc_f16(128, N);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // constant operands: the real 64-point DFT matrix and the 512-point twiddles
  for (int e = tid; e < 128 * 128; e += kTcThreads) {
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
  for (int p = tid; p < kTcL; p += kTcThreads) {
    float s, c;
    sincospif((float)p / 256.f, &s, &c);
    tw[p] = make_float2(c, -s);
  }
  if (warp == 0) umma::tmem_alloc(&tmem_base, kTcTmemCols);
  if (tid == 0) {
    umma::mbar_init(&mbar, 1);
    abort_flag = 0;
  }
  umma::fence_proxy_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base;
  const uint32_t aaddr = umma::smem_u32(sA), baddr = umma::smem_u32(sB);
  uint32_t phase = 0;
  // |Λ entries| <= lam_max: |Y| <= K lam_max |X| bounds the inverse operand's scale
  const float kbound = (float)K * *t.lam_max;

  const int64_t plane = (int64_t)a.nrow * a.inner;
  // F1 task of this thread: column li, row n2 (one per k)
  const int li1 = tid & 3, n2 = tid >> 2;
  // epilogue: TMEM lane m = 32 (warp % 4) + lane = 2 f2 + part; column pair h
  const int q = warp & 3, h = warp >> 2;
  const int m = 32 * q + lane, f2 = m >> 1, part = m & 1;
  const int li = 2 * h + part;
  const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);

  auto issue_mma = [&]() {
    if (tid == 0) {
      umma::fence_after_sync();
#pragma unroll
      for (int s = 0; s < 8; ++s)
        umma::mma_f16(tmem, umma::smem_desc(aaddr + 256 * s, 128, 2048),
                      umma::smem_desc(baddr + 2 * kTcLbo * s, kTcLbo, kTcSbo), idesc, s > 0);
      umma::mma_commit(&mbar);
    }
  };
  // warp 0 polls the mbarrier; the other warps wait at the barrier without issuing
  auto wait_mma = [&]() -> bool {
    if (warp == 0) {
      const bool done = umma::mbar_wait(&mbar, phase, kTcWaitLimit);
      if (!done && lane == 0) abort_flag = 1;
    }
    phase ^= 1u;
    __syncthreads();
    umma::fence_after_sync();
    return abort_flag == 0;
  };
  // the lane pair holds re (even lane) and im (odd lane) of columns li = 2h and 2h + 1:
  // the even lane keeps Re of li = 2h and sends Re of 2h + 1, the odd lane the reverse for Im
  auto pair_value = [&](float c0, float c1) -> float2 {
    const float keep = part ? c1 : c0;
    const float send = part ? c0 : c1;
    const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
    return part ? make_float2(recv, keep) : make_float2(keep, recv);
  };
  // Λ in the tensor-core layout [tile][p][j][h][f2][part]: one warp's loads are contiguous
  constexpr int64_t pstride = kTcLamPstride;
  auto lam_base = [&](int64_t tile, int j) -> int64_t {
    return ((tile * a.P * 8 + j) * 2 + h) * 128 + 2 * f2 + part;
  };

  bool ok = true;
  for (int64_t item = blockIdx.x; item < t.nitems && ok; item += gridDim.x) {
    const int cl = (int)(item % a.ncg);
    const int64_t tile = item / a.ncg;
    float2* base = a.stack + (int64_t)cl * K * plane + tile * kTcTC;
    // ---- F1: pruned DFT-8 over n1 and the w512 twiddle, into operand B
    float2 xin[K][4];
    float mx = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int n1 = 0; n1 < 4; ++n1) {
        xin[k][n1] = base[k * plane + (int64_t)(64 * n1 + n2) * a.inner + li1];
        mx = fmaxf(mx, fmaxf(fabsf(xin[k][n1].x), fabsf(xin[k][n1].y)));
      }
    const int e1 = scale_exp(4.f * block_max(mx, red));
    const float s1 = ldexpf(1.f, e1);
    constexpr float r2 = 0.70710678118654752f;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float2 ev[4], od[4];
      dft4<-1>(xin[k][0], xin[k][1], xin[k][2], xin[k][3], ev);
      const float2 x1 = make_float2(r2 * (xin[k][1].x + xin[k][1].y), r2 * (xin[k][1].y - xin[k][1].x));   // * w8
      const float2 x2 = mul_mi(xin[k][2]);                                                                   // * w8^2
      const float2 x3 = make_float2(r2 * (xin[k][3].y - xin[k][3].x), -r2 * (xin[k][3].x + xin[k][3].y));  // * w8^3
      dft4<-1>(xin[k][0], x1, x2, x3, od);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float2 v0 = cmulf(ev[j], tw[n2 * (2 * j)]);
        const float2 v1 = cmulf(od[j], tw[n2 * (2 * j + 1)]);
        st_half2(sB, boff(k * 32 + (2 * j) * 4 + li1, 2 * n2), v0.x * s1, v0.y * s1);
        st_half2(sB, boff(k * 32 + (2 * j + 1) * 4 + li1, 2 * n2), v1.x * s1, v1.y * s1);
      }
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    issue_mma();
    if (!(ok = wait_mma())) break;
    // ---- spectrum, voxel by voxel: exchange, undo the scale, K x K kernel, write conj(Y)
    // scaled into operand B of the inverse.  |D| < 128 * 2^14 = 2^21, so |X| < 2^(21 - e1)
    // and |Y| < K lam_max 2^(21 - e1): a power-of-two scale from that bound keeps every
    // fp16 value finite without waiting for the block's maximum.
    const float is1 = ldexpf(1.f, -e1);
    const int e2 = scale_exp(kbound * ldexpf(1.f, 21 - e1));
    const float s2 = ldexpf(1.f, e2);
    const bool real_lam = a.lam_mode == LAM_PACKED_REAL;
    const float* lamr = reinterpret_cast<const float*>(a.lam);
    float lcur[P];
    if (real_lam) {
      const int64_t lb = lam_base(tile, 0);
#pragma unroll
      for (int p = 0; p < P; ++p) lcur[p] = lamr[lb + p * pstride];
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      float d[K][2];
      tmem_ld2_planes<K>(tl + (uint32_t)(4 * j + 2 * h), d);
      float2 X[K], Y[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const float2 v = pair_value(d[k][0], d[k][1]);
        X[k] = make_float2(v.x * is1, v.y * is1);
      }
      if (real_lam) {
        float lnext[P];
        if (j < 7) {
          const int64_t lb = lam_base(tile, j + 1);
#pragma unroll
          for (int p = 0; p < P; ++p) lnext[p] = lamr[lb + p * pstride];
        }
        lam_real_regs<K>(lcur, X, Y);
        if (j < 7) {
#pragma unroll
          for (int p = 0; p < P; ++p) lcur[p] = lnext[p];
        }
      } else {
        lam_apply_ptr<K>(a.lam_mode, K, a.lam, lam_base(tile, j), pstride, X, Y);
      }
#pragma unroll
      for (int k = 0; k < K; ++k) st_half2(sB, boff(k * 32 + j * 4 + li, 2 * f2), Y[k].x * s2, -Y[k].y * s2);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    issue_mma();
    if (!(ok = wait_mma())) break;
    // ---- inverse, plane by plane: conj, twiddle, output-pruned inverse DFT-8 over f1,
    // staged as float2 in the operand-B region (the MMA that read it has completed)
    const float is2 = ldexpf(1.f, -e2);
    float2* stg = reinterpret_cast<float2*>(sB);  // [k][n < 256][li], rows kTcStg apart
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float Rk[32];
      tmem_ld32(tl + (uint32_t)(k * 32), Rk);
      float2 z[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 v = pair_value(h ? Rk[4 * j + 2] : Rk[4 * j], h ? Rk[4 * j + 3] : Rk[4 * j + 1]);
        z[j] = cmulcf(make_float2(v.x * is2, -v.y * is2), tw[f2 * j]);
      }
      float2 ev[4], od[4];
      dft4<+1>(z[0], z[2], z[4], z[6], ev);
      dft4<+1>(z[1], z[3], z[5], z[7], od);
      // y[m1] = E[m1] + w8^(-m1) O[m1]
      const float2 o1 = make_float2(r2 * (od[1].x - od[1].y), r2 * (od[1].x + od[1].y));
      const float2 o2 = mul_pi(od[2]);
      const float2 o3 = make_float2(-r2 * (od[3].x + od[3].y), r2 * (od[3].x - od[3].y));
      stg[(k * 256 + 0 * 64 + f2) * kTcStg + li] = caddf(ev[0], od[0]);
      stg[(k * 256 + 1 * 64 + f2) * kTcStg + li] = caddf(ev[1], o1);
      stg[(k * 256 + 2 * 64 + f2) * kTcStg + li] = caddf(ev[2], o2);
      stg[(k * 256 + 3 * 64 + f2) * kTcStg + li] = caddf(ev[3], o3);
    }
    umma::fence_before_sync();
    __syncthreads();
    for (int e = tid; e < K * 256 * kTcTC; e += kTcThreads) {
      const int row = e / kTcTC, c = e - row * kTcTC;  // row = k * 256 + n
      const int k = row >> 8, n = row & 255;
      base[k * plane + (int64_t)n * a.inner + c] = stg[row * kTcStg + c];
    }
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicExch(t.err, KERR_MBAR_TIMEOUT);
    umma::mbar_wait(&mbar, phase ^ 1u, kTcWaitLimit);  // let an MMA still in flight finish
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, kTcTmemCols);
  }
}

int num_sms_tc() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

template <int K>
int launch_tc(const TcArgs& t, cudaStream_t st) {
  // at least 80 KB: at most two CTAs per SM, so their 2 x 256 TMEM columns always fit
  // (K >= 6 is held to one CTA by its registers)
  const size_t smem = std::max<size_t>((size_t)kTcAbytes + tc_bbytes(K) + sizeof(float2) * kTcL, 80u << 10);
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(kt_lambda<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = std::min<int64_t>(t.nitems, 2 * (int64_t)num_sms_tc());
  kt_lambda<K><<<(unsigned)grid, kTcThreads, smem, st>>>(t);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

}  // namespace

// out[0] = max |component| over n floats (one CTA; run once per operator)
__global__ void k_tc_absmax(const float* v, int64_t n, float* out) {
  __shared__ float red[32];
  float m = 0.f;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) m = fmaxf(m, fabsf(v[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, red[w]);
    out[0] = r;
  }
}

// Λ of the chunked layout [tile][chunk][p][fc][4] (f = chunk FC + fc) rearranged for the
// tensor-core pass: dst[tile][p][j][h][f2][part] = src(tile, f = j + 8 f2, li = 2 h + part, p).
template <class T>
__global__ void k_tc_lam_layout(const T* src, T* dst, int64_t ntiles, int P, int FC, int NCH) {
  const int64_t total = ntiles * P * kTcL * kTcTC;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int part = (int)(e & 1), f2 = (int)((e >> 1) & 63), h = (int)((e >> 7) & 1), j = (int)((e >> 8) & 7);
    const int64_t tp = e >> 11;  // tile * P + p
    const int p = (int)(tp % P);
    const int64_t tile = tp / P;
    const int f = j + 8 * f2, li = 2 * h + part;
    const int ch = f / FC, fc = f - ch * FC;
    dst[e] = src[(((tile * NCH + ch) * P + p) * (int64_t)FC + fc) * kTcTC + li];
  }
}

int tc_lambda_layout(const void* lam, void* out, int64_t ntiles, int P, int FC, int NCH, bool real, cudaStream_t st) {
  const int64_t total = ntiles * P * kTcL * kTcTC;
  const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 8192);
  if (real)
    k_tc_lam_layout<float><<<grid, 256, 0, st>>>(reinterpret_cast<const float*>(lam), reinterpret_cast<float*>(out),
                                                   ntiles, P, FC, NCH);
  else
    k_tc_lam_layout<float2><<<grid, 256, 0, st>>>(reinterpret_cast<const float2*>(lam), reinterpret_cast<float2*>(out),
                                                    ntiles, P, FC, NCH);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int tc_lambda_bound(const void* lam, size_t bytes, float* out, cudaStream_t st) {
  k_tc_absmax<<<1, 1024, 0, st>>>(reinterpret_cast<const float*>(lam), (int64_t)(bytes / sizeof(float)), out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

bool tc_lambda_supported(int L, int nin, int nout, int TC, int K) {
  return L == kTcL && nin * 2 == L && nout * 2 == L && TC == kTcTC && K >= 1 && K <= KMAX;
}

int tc_lambda(const LamPassArgs& a, int ncg, const float* lam_max, int* errword, cudaStream_t st) {
  MRSR_REQUIRE(tc_lambda_supported(a.pl.L, a.nin, a.nout, a.TC, a.K), MRSR_ERR_UNSUPPORTED,
               "tensor-core Λ pass: needs a 512-point pruned column transform, 4-column tiles and K <= 8");
  MRSR_REQUIRE(lam_max, MRSR_ERR_STATE, "tensor-core Λ pass: the kernel bound was not computed");
  TcArgs t{a, (int64_t)(a.inner / kTcTC) * ncg, errword, lam_max};
  t.a.ncg = ncg;
  t.a.fcd = FastDiv((uint32_t)a.FC);
  switch (a.K) {
    case 1: return launch_tc<1>(t, st);
    case 2: return launch_tc<2>(t, st);
    case 3: return launch_tc<3>(t, st);
    case 4: return launch_tc<4>(t, st);
    case 5: return launch_tc<5>(t, st);
    case 6: return launch_tc<6>(t, st);
    case 7: return launch_tc<7>(t, st);
    default: return launch_tc<8>(t, st);
  }
}

}  // namespace mrsr
