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
#include "tcdft.cuh"
#include "umma.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace mrsr {

namespace {

using namespace tcdft;
constexpr int kTcL = 512, kTcTC = 4;  // L = 8 x 64; four columns per tile
constexpr int kTcThreads = 256;
constexpr uint32_t kTcTmemCols = 256;
constexpr uint32_t kTcWaitLimit = 1u << 26;  // mbarrier polls before the kernel reports a timeout
constexpr int kTcAbytes = tcdft::kAbytes;      // fp16 DFT-64 matrix, K-major core matrices

struct TcArgs {
  LamPassArgs a;
  int64_t nitems;        // column tiles x coils of the group
  int* err;
  const float* lam_max;  // device: largest |component| of any Λ entry
  const unsigned char* consts;  // DFT-64 operand and twiddles (tcdft::build_constants)
};

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
  tcdft::load_constants(sA, tw, t.consts, tid, kTcThreads);
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

  // this thread's F1 inputs of an item: rows 64 n1 + n2 (n1 < 4) of column li1, all k
  auto item_base = [&](int64_t it) -> float2* {
    const int c = (int)(it % a.ncg);
    return a.stack + (int64_t)c * K * plane + (it / a.ncg) * kTcTC;
  };
  float2 xin[K][4];
  auto load_inputs = [&](int64_t it) {
    const float2* b = item_base(it);
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int n1 = 0; n1 < 4; ++n1) xin[k][n1] = b[k * plane + (int64_t)(64 * n1 + n2) * a.inner + li1];
  };
  if ((int64_t)blockIdx.x < t.nitems) load_inputs(blockIdx.x);

  bool ok = true;
  for (int64_t item = blockIdx.x; item < t.nitems && ok; item += gridDim.x) {
    const int64_t tile = item / a.ncg;
    float2* base = item_base(item);
    // ---- F1: pruned DFT-8 over n1 and the w512 twiddle, into operand B (the inputs were
    // loaded during the previous item)
    float mx = 0.f;
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
      for (int n1 = 0; n1 < 4; ++n1) mx = fmaxf(mx, fmaxf(fabsf(xin[k][n1].x), fabsf(xin[k][n1].y)));
    const int e1 = scale_exp(4.f * block_max<kTcThreads>(mx, red));
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
    // the first voxel's kernel entries load while the MMA runs
    const bool real_lam = a.lam_mode == LAM_PACKED_REAL;
    const float* lamr = reinterpret_cast<const float*>(a.lam);
    float lcur[P];
    if (real_lam) {
      const int64_t lb = lam_base(tile, 0);
#pragma unroll
      for (int p = 0; p < P; ++p) lcur[p] = lamr[lb + p * pstride];
    }
    if (!(ok = wait_mma())) break;
    // ---- spectrum, voxel by voxel: exchange, undo the scale, K x K kernel, write conj(Y)
    // scaled into operand B of the inverse.  |D| < 128 * 2^14 = 2^21, so |X| < 2^(21 - e1)
    // and |Y| < K lam_max 2^(21 - e1): a power-of-two scale from that bound keeps every
    // fp16 value finite without waiting for the block's maximum.
    const float is1 = ldexpf(1.f, -e1);
    const int e2 = scale_exp(kbound * ldexpf(1.f, 21 - e1));
    const float s2 = ldexpf(1.f, e2);
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
      // inverse operand row k * 32 + 16 h + 2 j + part: this thread's columns of plane k
      // come back as one run of 16 (f1 = j, li = 2 h + part)
#pragma unroll
      for (int k = 0; k < K; ++k)
        st_half2(sB, boff(k * 32 + 16 * h + 2 * j + part, 2 * f2), Y[k].x * s2, -Y[k].y * s2);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    issue_mma();
    // the next item's inputs load while this item's inverse runs
    if (item + gridDim.x < t.nitems) load_inputs(item + gridDim.x);
    if (!(ok = wait_mma())) break;
    // ---- inverse, plane by plane: conj, twiddle, output-pruned inverse DFT-8 over f1,
    // staged as float2 in the operand-B region (the MMA that read it has completed)
    const float is2 = ldexpf(1.f, -e2);
    float2* stg = reinterpret_cast<float2*>(sB);  // [k][n < 256][li], rows kTcStg apart
#pragma unroll
    for (int k = 0; k < K; ++k) {
      float Rk[16];
      umma::tmem_ld16(tl + (uint32_t)(k * 32 + 16 * h), Rk);
      float2 z[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 v = pair_value(Rk[2 * j], Rk[2 * j + 1]);
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

// out[0] = max |component| over n floats (run once per operator; out[0] zeroed first).
// Non-negative floats order like their bit patterns, so the grid combines with atomicMax.
__global__ void k_tc_absmax(const float* v, int64_t n, float* out) {
  __shared__ float red[32];
  float m = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(v[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    float r = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, red[w]);
    atomicMax(reinterpret_cast<int*>(out), __float_as_int(r));
  }
}

int tc_lambda_bound(const void* lam, size_t bytes, float* out, cudaStream_t st) {
  MRSR_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(float), st));
  const int64_t n = (int64_t)(bytes / sizeof(float));
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 1023) / 1024, 2048));
  k_tc_absmax<<<grid, 1024, 0, st>>>(reinterpret_cast<const float*>(lam), n, out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// Λ of the chunked layout [tile][chunk][p][fc][TC] (f = chunk FC + fc, any tile width TC)
// rearranged for the tensor-core pass on 4-column tiles:
// dst[tile4][p][j][h][f2][part] = src(column 4 tile4 + 2 h + part, f = j + 8 f2, p).
template <class T>
__global__ void k_tc_lam_layout(const T* src, T* dst, int64_t ntiles4, int P, int FC, int NCH, int TC) {
  const int64_t total = ntiles4 * P * kTcL * kTcTC;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int part = (int)(e & 1), f2 = (int)((e >> 1) & 63), h = (int)((e >> 7) & 1), j = (int)((e >> 8) & 7);
    const int64_t tp = e >> 11;  // tile4 * P + p
    const int p = (int)(tp % P);
    const int64_t col = (tp / P) * kTcTC + 2 * h + part;
    const int64_t tile = col / TC;
    const int li = (int)(col - tile * TC);
    const int f = j + 8 * f2;
    const int ch = f / FC, fc = f - ch * FC;
    dst[e] = src[(((tile * NCH + ch) * P + p) * (int64_t)FC + fc) * TC + li];
  }
}

int tc_lambda_layout(const void* lam, void* out, int64_t inner, int P, int FC, int NCH, int TC, bool real,
                     cudaStream_t st) {
  const int64_t ntiles4 = inner / kTcTC;
  const int64_t total = ntiles4 * P * kTcL * kTcTC;
  const unsigned grid = (unsigned)std::min<int64_t>((total + 255) / 256, 8192);
  if (real)
    k_tc_lam_layout<float><<<grid, 256, 0, st>>>(reinterpret_cast<const float*>(lam), reinterpret_cast<float*>(out),
                                                   ntiles4, P, FC, NCH, TC);
  else
    k_tc_lam_layout<float2><<<grid, 256, 0, st>>>(reinterpret_cast<const float2*>(lam), reinterpret_cast<float2*>(out),
                                                    ntiles4, P, FC, NCH, TC);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}


__global__ void k_tc_constants(unsigned char* g) {
  tcdft::setup_constants(g, reinterpret_cast<float2*>(g + tcdft::kAbytes), threadIdx.x + blockIdx.x * blockDim.x,
                         blockDim.x * gridDim.x);
}

int tc_build_constants(void* out, cudaStream_t st) {
  k_tc_constants<<<16, 256, 0, st>>>(reinterpret_cast<unsigned char*>(out));
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

size_t tc_constants_bytes() { return tcdft::kConstBytes; }

bool tc_lambda_supported(int L, int nin, int nout, int inner, int K) {
  return L == kTcL && nin * 2 == L && nout * 2 == L && inner % kTcTC == 0 && K >= 1 && K <= KMAX;
}

int tc_lambda(const LamPassArgs& a, int ncg, const float* lam_max, const void* consts, int* errword,
              cudaStream_t st) {
  MRSR_REQUIRE(tc_lambda_supported(a.pl.L, a.nin, a.nout, (int)a.inner, a.K), MRSR_ERR_UNSUPPORTED,
               "tensor-core Λ pass: needs a 512-point pruned column transform, a plane width divisible by 4 "
               "and K <= 8");
  MRSR_REQUIRE(lam_max, MRSR_ERR_STATE, "tensor-core Λ pass: the kernel bound was not computed");
  TcArgs t{a, (int64_t)(a.inner / kTcTC) * ncg, errword, lam_max, reinterpret_cast<const unsigned char*>(consts)};
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
