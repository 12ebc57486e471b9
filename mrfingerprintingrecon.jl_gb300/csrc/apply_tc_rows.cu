// Inverse row pass of the precision MRSR_PREC_FP16_TC operator with the 64-point DFTs
// on the tensor cores (the Λ pass is in apply_tc.cu; the four-step split and the
// operand conventions are the same).  One work item is one image row r and one basis
// index k; the MMA's N vectors are (coil, f1) for every coil of the group.  (The
// forward row pass stays the float32 four-step kernel, which is faster there.)
//
// Inverse (DFT^-1 along dim 1, crop to 256, conj map, coil sum, alpha / beta):
//   y[64 m1 + m2] = sum_c conj(S_c) sum_f1 w8^(-m1 f1) w512^(-m2 f1) conj(sum_f2 w64^(m2 f2) conj(Y_c[f1 + 8 f2]))
// Operand B rows are (coil, f1); the core matrices along K sit 144 bytes apart, so the
// half2 stores of a warp (32 consecutive n2 or f2 of one row) hit 32 different banks.
#include "passes.cuh"
#include "tcdft.cuh"
#include "tma.cuh"
#include "umma.cuh"

#include <cuda_fp16.h>

#include <algorithm>

namespace mrsr {

namespace {

using namespace tcdft;
constexpr int kRThreads = 256;
constexpr uint32_t kRTmemCols = 256;
constexpr uint32_t kRWaitLimit = 1u << 26;
constexpr uint32_t kRLbo = 144, kRSbo = 16 * kRLbo;
constexpr int kRMaxCoils = 32;  // N = 8 x coils <= 256

__device__ __forceinline__ uint32_t roff(int r, int kk) {
  return (uint32_t)((r >> 3) * kRSbo + (kk >> 3) * kRLbo + (r & 7) * 16 + (kk & 7) * 2);
}

struct TcRowsArgs {
  RowsInvArgs i;     // inverse pass arguments
  int ncg;           // coils of the group
  int cb;            // coils per MMA: ncg rounded up to a multiple of 4 (<= 32)
  int64_t nitems;    // rows x K
  int* err;
  const unsigned char* consts;  // DFT-64 operand and twiddles (tcdft::build_constants)
};

__device__ __forceinline__ void issue_dft64(int tid, uint32_t tmem, uint32_t aaddr, uint32_t baddr, uint32_t idesc,
                                            uint64_t* mbar) {
  if (tid == 0) {
    umma::fence_after_sync();
#pragma unroll
    for (int s = 0; s < 8; ++s)
      umma::mma_f16(tmem, umma::smem_desc(aaddr + 256 * s, 128, 2048), umma::smem_desc(baddr + 2 * kRLbo * s, kRLbo, kRSbo),
                    idesc, s > 0);
    umma::mma_commit(mbar);
  }
}

// warp 0 polls; the others wait at the barrier.  Returns false on a timeout.
__device__ __forceinline__ bool wait_dft64(int warp, int lane, uint64_t* mbar, uint32_t& phase, int* abort_flag) {
  if (warp == 0) {
    const bool done = umma::mbar_wait(mbar, phase, kRWaitLimit);
    if (!done && lane == 0) *abort_flag = 1;
  }
  phase ^= 1u;
  __syncthreads();
  umma::fence_after_sync();
  return *abort_flag == 0;
}

__device__ __forceinline__ void finish(bool ok, int tid, int warp, uint64_t* mbar, uint32_t phase, uint32_t tmem, int* err) {
  if (!ok) {
    if (tid == 0) atomicExch(err, KERR_MBAR_TIMEOUT);
    umma::mbar_wait(mbar, phase ^ 1u, kRWaitLimit);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    umma::fence_after_sync();
    umma::tmem_dealloc(tmem, kRTmemCols);
  }
}

template <int CB>
__global__ void __launch_bounds__(kRThreads, 2) kt_rows_inv(TcRowsArgs t) {
  const RowsInvArgs& a = t.i;
  extern __shared__ __align__(1024) unsigned char smem[];
  unsigned char* sA = smem;
  unsigned char* sB = smem + kAbytes;
  float2* tw = reinterpret_cast<float2*>(sB + (size_t)CB * kRSbo);
  float2* part_sum = tw + kL;  // [m1 < 4][lane row < 128]: the h = 1 half's coil sums
  __shared__ uint64_t mbar;
  __shared__ uint32_t tmem_base;
  __shared__ float red[kRThreads / 32];
  __shared__ int abort_flag;
  constexpr int N = 8 * CB, NP = CB / 4;
  constexpr uint32_t idesc = umma::idesc_f16(128, N);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  load_constants(sA, tw, t.consts, tid, kRThreads);
  if (warp == 0) umma::tmem_alloc(&tmem_base, kRTmemCols);
  if (tid == 0) {
    umma::mbar_init(&mbar, 1);
    abort_flag = 0;
  }
  umma::fence_proxy_async();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_base, aaddr = umma::smem_u32(sA), baddr = umma::smem_u32(sB);
  uint32_t phase = 0;
  const int f2l = tid & 63, cq = tid >> 6;  // loads: frequency row f2 = f2l, coil 4 p + cq
  const int q = warp & 3, h = warp >> 2;
  const int m = 32 * q + lane, m2 = m >> 1, part = m & 1;
  const uint32_t tl = tmem + ((uint32_t)(32 * q) << 16);
  float2 twr[8];  // w512^(m2 f1), conjugated on use
#pragma unroll
  for (int f1 = 0; f1 < 8; ++f1) twr[f1] = tw[m2 * f1];
  constexpr float r2 = 0.70710678118654752f;
  const int L = kL;

  bool ok = true;
  for (int64_t item = blockIdx.x; item < t.nitems && ok; item += gridDim.x) {
    const int64_t r = item / a.K;
    const int k = (int)(item - r * a.K);
    // ---- conj(Y) of every (coil, f1) vector along f2, scaled, into operand B
    float2 v[NP][8];
    float mx = 0.f;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int cl = 4 * p + cq;
      if (cl < t.ncg) {
        const float4* src =
            reinterpret_cast<const float4*>(a.stack + (((int64_t)cl * a.K + k) * a.nrows + r) * L + 8 * f2l);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 w4 = src[i];
          v[p][2 * i] = make_float2(w4.x, w4.y);
          v[p][2 * i + 1] = make_float2(w4.z, w4.w);
        }
      } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) v[p][i] = make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int i = 0; i < 8; ++i) mx = fmaxf(mx, fmaxf(fabsf(v[p][i].x), fabsf(v[p][i].y)));
    }
    const int e1 = scale_exp(block_max<kRThreads>(mx, red));
    const float s1 = ldexpf(1.f, e1);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const int cl = 4 * p + cq;
#pragma unroll
      for (int f1 = 0; f1 < 8; ++f1) st_half2(sB, roff(cl * 8 + f1, 2 * f2l), v[p][f1].x * s1, -v[p][f1].y * s1);
    }
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    issue_dft64(tid, tmem, aaddr, baddr, idesc, &mbar);
    // the maps this thread multiplies with, conj(S_c[64 m1 + m2, r]) for its coils
    // c = h CB / 2 + 2 i + part, load while the MMA runs
    float2 smap[CB / 4][4];
#pragma unroll
    for (int i = 0; i < CB / 4; ++i) {
      const int cl = h * (CB / 2) + 2 * i + part;
#pragma unroll
      for (int m1 = 0; m1 < 4; ++m1)
        smap[i][m1] = (a.cmaps && cl < t.ncg) ? a.cmaps[64 * m1 + m2 + (int64_t)a.n1 * (r + a.nrows * (a.c0 + cl))]
                                              : make_float2(1.f, 0.f);
    }
    if (!(ok = wait_dft64(warp, lane, &mbar, phase, &abort_flag))) break;
    // ---- epilogue: coils of half h in pairs; the even lane takes the first coil of a
    // pair, the odd lane the second, each receiving the other part from its partner
    const float is1 = ldexpf(1.f, -e1);
    float2 acc[4] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
    for (int i = 0; i < CB / 4; ++i) {
      const int cp = h * (CB / 2) + 2 * i;
      float da[8], db[8];
      tmem_ld8(tl + (uint32_t)(cp * 8), da);
      tmem_ld8(tl + (uint32_t)((cp + 1) * 8), db);
      const int cl = cp + part;
      float2 z[8];
#pragma unroll
      for (int f1 = 0; f1 < 8; ++f1) {
        const float keep = part ? db[f1] : da[f1];
        const float send = part ? da[f1] : db[f1];
        const float recv = __shfl_xor_sync(0xffffffffu, send, 1);
        // D holds DFT64(conj Y): Z = conj(D) / s1, then the w512^(-m2 f1) twiddle
        const float2 dv = part ? make_float2(recv, keep) : make_float2(keep, recv);
        z[f1] = cmulcf(make_float2(dv.x * is1, -dv.y * is1), twr[f1]);
      }
      float2 ev[4], od[4];
      dft4<+1>(z[0], z[2], z[4], z[6], ev);
      dft4<+1>(z[1], z[3], z[5], z[7], od);
      float2 yv[4];
      yv[0] = caddf(ev[0], od[0]);
      yv[1] = caddf(ev[1], make_float2(r2 * (od[1].x - od[1].y), r2 * (od[1].x + od[1].y)));
      yv[2] = caddf(ev[2], mul_pi(od[2]));
      yv[3] = caddf(ev[3], make_float2(-r2 * (od[3].x + od[3].y), r2 * (od[3].x - od[3].y)));
      if (cl < t.ncg) {
#pragma unroll
        for (int m1 = 0; m1 < 4; ++m1) acc[m1] = caddf(acc[m1], cmulcf(yv[m1], smap[i][m1]));
      }
    }
    // ---- coil sum: lane pair, then the two halves through shared memory
#pragma unroll
    for (int m1 = 0; m1 < 4; ++m1) {
      acc[m1].x += __shfl_xor_sync(0xffffffffu, acc[m1].x, 1);
      acc[m1].y += __shfl_xor_sync(0xffffffffu, acc[m1].y, 1);
    }
    umma::fence_before_sync();
    if (h == 1) {
#pragma unroll
      for (int m1 = 0; m1 < 4; ++m1) part_sum[m1 * 128 + m] = acc[m1];
    }
    __syncthreads();
    if (h == 0) {
      // the even lane writes m1 = 0, 1 and the odd lane m1 = 2, 3
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int m1 = 2 * part + i;
        const float2 own = part ? acc[2 + i] : acc[i];
        const float2 s = caddf(own, part_sum[m1 * 128 + m]);
        const int n = 64 * m1 + m2;
        const int64_t yi = n + (int64_t)a.n1 * (r + a.nrows * k);
        float2 yv;
        if (a.first)
          yv = (a.beta.x == 0.f && a.beta.y == 0.f) ? make_float2(0.f, 0.f) : cmul(a.beta, a.y[yi]);
        else
          yv = a.y[yi];
        a.y[yi] = caddf(yv, cmul(a.alpha, s));
      }
    }
    __syncthreads();
  }
  finish(ok, tid, warp, &mbar, phase, tmem, t.err);
}

int num_sms_rows() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

template <int CB>
int launch_rows(void (*kern)(TcRowsArgs), const TcRowsArgs& t, size_t extra, cudaStream_t st) {
  // at least 80 KB: two CTAs per SM at most, so the 2 x 256 TMEM columns always fit
  const size_t smem = std::max<size_t>((size_t)kAbytes + (size_t)CB * kRSbo + sizeof(float2) * kL + extra, 80u << 10);
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t grid = std::min<int64_t>(t.nitems, 2 * (int64_t)num_sms_rows());
  kern<<<(unsigned)grid, kRThreads, smem, st>>>(t);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

template <int CB>
int dispatch_cb(const TcRowsArgs& t, cudaStream_t st) {
  return launch_rows<CB>(kt_rows_inv<CB>, t, sizeof(float2) * 4 * 128, st);
}

int dispatch(const TcRowsArgs& t, cudaStream_t st) {
  switch (t.cb) {
    case 4: return dispatch_cb<4>(t, st);
    case 8: return dispatch_cb<8>(t, st);
    case 12: return dispatch_cb<12>(t, st);
    case 16: return dispatch_cb<16>(t, st);
    case 20: return dispatch_cb<20>(t, st);
    case 24: return dispatch_cb<24>(t, st);
    case 28: return dispatch_cb<28>(t, st);
    default: return dispatch_cb<32>(t, st);
  }
}

}  // namespace

bool tc_rows_supported(int L, int n1, int ncg) { return L == kL && 2 * n1 == L && ncg >= 1 && ncg <= kRMaxCoils; }

int tc_rows_inv(const RowsInvArgs& a, const void* consts, int* errword, cudaStream_t st) {
  MRSR_REQUIRE(tc_rows_supported(a.pl.L, a.n1, a.ncg), MRSR_ERR_UNSUPPORTED,
               "tensor-core row pass: needs 512-point rows of 256 image samples and <= %d coils per group", kRMaxCoils);
  TcRowsArgs t{};
  t.i = a;
  t.ncg = a.ncg;
  t.cb = (a.ncg + 3) / 4 * 4;
  t.nitems = a.nrows * a.K;
  t.err = errword;
  t.consts = reinterpret_cast<const unsigned char*>(consts);
  return dispatch(t, st);
}

}  // namespace mrsr
