// Mixed-precision apply: the oversampled K-stack and the Toeplitz kernel are
// stored in fp16 with one float32 scale per tile; all arithmetic (FFTs, the
// K x K product, coil sums) is float32.  Same pass structure as the float32
// four-step kernels (apply_fast.cu).  Each producing CTA writes its results to
// shared memory, reduces the largest component magnitude of its tile, and
// stores value / scale as half2 with scale = max / kHalfTarget; the consumer
// multiplies by the producer tile's scale when it loads.
//
// Tiles (producer -> scale array):
//   rows forward  (row block, coil)           -> s_rows[coil][row block]
//   dim-2 forward (column tile, slice block, plane) -> s_mid[plane][slice block][column tile]   (3D)
//   Λ pass        (column tile, coil)         -> s_lam[coil][tile]
//   dim-2 inverse (column tile, slice block, plane) -> s_mid2[...]                             (3D)
#include <algorithm>

#include "fft4.cuh"
#include "half.cuh"
#include "passes.cuh"

namespace mrsr {

constexpr float kHalfTarget = 30000.f;  // largest stored magnitude (< 65504)

__device__ __forceinline__ float2 ld_h(const __half2* p, int64_t i, float s) {
  const float2 v = __half22float2(p[i]);
  return make_float2(v.x * s, v.y * s);
}


__device__ __forceinline__ float scale_of(float mx) { return mx > 0.f ? mx / kHalfTarget : 1.f; }

struct HalfArgs {
  FftPlan pl;
  // geometry
  int d, K, n1;
  int64_t nrows;     // n2 * n3
  int64_t g1, g2, n2, n3;
  int c0, ncg;
  // Λ pass
  int TC, P, lam_mode, FC, NCH;
  int64_t inner, ntiles;
  int nlast, glast;
  const void* lam;   // half / half2 chunked layout
  const float* lam_scale;  // [tile]
  // data
  const float2* x;
  const float2* cmaps;
  float2* y;
  float2 alpha, beta;
  int first;
  __half2* st1;      // rows output / Λ-pass (2D) stack
  __half2* st2;      // 3D dim-2 stack
  HalfTiles t;
  // divisions of the per-element scale lookups (all operands < 2^31)
  FastDiv fd_rpc, fd_noo, fd_tcm, fd_tc, fd_n2, fd_fc;
};

// ------------------------------------------------------------ rows forward ---
template <class SP, bool PR>
__global__ void __launch_bounds__(512) kh_rows_fwd(HalfArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  __shared__ float smax;
  load_twiddles(tw, a.pl);
  if (threadIdx.x == 0) smax = 0.f;
  const int cl = blockIdx.y, c = a.c0 + cl;
  const int64_t rb = blockIdx.x;
  const int64_t row0 = rb * a.t.rpc;
  const int nr = (int)min((int64_t)a.t.rpc, a.nrows - row0);
  const int NO = a.t.rpc * a.K;
  constexpr int nload = PR ? R1 / 2 : R1;
  __syncthreads();
  step_a<SP, -1>(sm, sl, NO, tw, nload, [&](int lo, int, int n) -> float2 {
    const int rl = lo / a.K, k = lo - rl * a.K;
    if (rl >= nr || (!PR && n >= a.n1)) return make_float2(0.f, 0.f);
    const int64_t r = row0 + rl;
    float2 v = a.x[n + (int64_t)a.n1 * (r + a.nrows * k)];
    if (a.cmaps) v = cmul(a.cmaps[n + (int64_t)a.n1 * (r + a.nrows * c)], v);
    return v;
  });
  __syncthreads();
  float lmax = 0.f;
  step_b<SP, -1>(sm, sl, NO, R2, [&](int lo, int li, int f1, int f2, float2 v) {
    sm[sl.at(lo, f1, f2, li, R1)] = v;
    lmax = fmaxf(lmax, amax2(v));
  });
  block_max_commit(&smax, lmax);
  __syncthreads();
  const float s = scale_of(smax), inv = 1.f / s;
  if (threadIdx.x == 0) a.t.s_rows[(int64_t)cl * a.t.nrowblk + rb] = s;
  for (int e = threadIdx.x; e < nr * a.K * L; e += blockDim.x) {
    const int lo = e / L, f = e - lo * L;
    const int rl = lo / a.K, k = lo - rl * a.K;
    const float2 v = sm[sl.at(lo, f % R1, f / R1, 0, R1)];
    a.st1[(((int64_t)cl * a.K + k) * a.nrows + row0 + rl) * L + f] = __floats2half2_rn(v.x * inv, v.y * inv);
  }
}

// ---------------------------------------------------------- dim-2 passes ---
// forward: st1 (g1, n2, n3) -> st2 (g1, g2, n3);  inverse: st2 -> st1
template <class SP, int S, bool PR>
__global__ void __launch_bounds__(512) kh_mid(HalfArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  __shared__ float smax;
  load_twiddles(tw, a.pl);
  if (threadIdx.x == 0) smax = 0.f;
  const int TC = a.t.TCm;
  const int64_t ct = blockIdx.x, ob = blockIdx.y, p = blockIdx.z;  // column tile, slab, plane (cl K + k)
  const int64_t col0 = ct * TC, o0 = ob * a.t.NOo;
  const int no = (int)min((int64_t)a.t.NOo, a.n3 - o0);
  const int cl = (int)(p / a.K), k = (int)(p - (int64_t)cl * a.K);
  const int nin = S < 0 ? (int)a.n2 : L, nout = S < 0 ? L : (int)a.n2;
  const __half2* ib = (S < 0 ? a.st1 : a.st2) + (p * a.n3 + o0) * nin * a.g1 + col0;
  __half2* ob_ = (S < 0 ? a.st2 : a.st1) + (p * a.n3 + o0) * nout * a.g1 + col0;
  constexpr int nload = (PR && S < 0) ? R1 / 2 : R1;
  constexpr int nkeep = (PR && S > 0) ? R2 / 2 : R2;
  __syncthreads();
  step_a<SP, S>(sm, sl, a.t.NOo, tw, nload, [&](int o, int li, int n) -> float2 {
    if (o >= no || (!(PR && S < 0) && n >= nin)) return make_float2(0.f, 0.f);
    float s;
    if (S < 0) {  // producer: rows forward, row r = n + n2 (o0 + o)
      const uint32_t r = (uint32_t)(n + a.n2 * (o0 + o));
      s = a.t.s_rows[(int64_t)cl * a.t.nrowblk + a.fd_rpc.div(r)];
    } else {      // producer: Λ pass, inner = (col0 + li) + g1 * n
      const uint32_t inner = (uint32_t)(col0 + li + a.g1 * n);
      s = a.t.s_lam[(int64_t)cl * a.ntiles + a.fd_tc.div(inner)];
    }
    return ld_h(ib, ((int64_t)o * nin + n) * a.g1 + li, s);
  });
  __syncthreads();
  float lmax = 0.f;
  step_b<SP, S>(sm, sl, a.t.NOo, nkeep, [&](int o, int li, int f1, int f2, float2 v) {
    sm[sl.at(o, f1, f2, li, R1)] = v;
    if (o < no) lmax = fmaxf(lmax, amax2(v));
  });
  block_max_commit(&smax, lmax);
  __syncthreads();
  const float s = scale_of(smax), inv = 1.f / s;
  float* sarr = S < 0 ? a.t.s_mid : a.t.s_mid2;
  if (threadIdx.x == 0) sarr[(p * a.t.nslab + ob) * a.t.nmtile + ct] = s;
  for (int e = threadIdx.x; e < no * nout * TC; e += blockDim.x) {
    const int li = e % TC;
    const int t = e / TC;
    const int n = t % nout, o = t / nout;
    const float2 v = sm[sl.at(o, n % R1, n / R1, li, R1)];
    ob_[((int64_t)o * nout + n) * a.g1 + li] = __floats2half2_rn(v.x * inv, v.y * inv);
  }
  (void)k;
}

// ------------------------------------------------------------- Λ pass ---
template <int KM>
__device__ __forceinline__ void lam_apply_half(int mode, int K, const void* lamv, int64_t lbase, int64_t pstride,
                                               float ls, const float2* X, float2* Y) {
#pragma unroll
  for (int j = 0; j < KM; ++j) Y[j] = make_float2(0.f, 0.f);
  if (mode == LAM_PACKED_REAL) {
    const __half* lam = reinterpret_cast<const __half*>(lamv) + lbase;
    int p = 0;
#pragma unroll
    for (int k2 = 0; k2 < KM; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 <= k2; ++k1) {
        if (k2 < K) {
          const float l = __half2float(lam[p * pstride]) * ls;
          Y[k1].x += l * X[k2].x;
          Y[k1].y += l * X[k2].y;
          if (k1 != k2) {
            Y[k2].x += l * X[k1].x;
            Y[k2].y += l * X[k1].y;
          }
        }
        ++p;
      }
    }
  } else if (mode == LAM_PACKED_CPLX) {
    const __half2* lam = reinterpret_cast<const __half2*>(lamv) + lbase;
    int p = 0;
#pragma unroll
    for (int k2 = 0; k2 < KM; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 <= k2; ++k1) {
        if (k2 < K) {
          const float2 l = cscale(__half22float2(lam[p * pstride]), ls);
          Y[k1] = cadd(Y[k1], cmul(l, X[k2]));
          if (k1 != k2) Y[k2] = cadd(Y[k2], cmul(cconj(l), X[k1]));
        }
        ++p;
      }
    }
  } else {
    const __half2* lam = reinterpret_cast<const __half2*>(lamv) + lbase;
#pragma unroll
    for (int k2 = 0; k2 < KM; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 < KM; ++k1) {
        if (k1 < K && k2 < K) {
          const float2 l = cscale(__half22float2(lam[(k1 + K * k2) * pstride]), ls);
          Y[k1] = cadd(Y[k1], cmul(l, X[k2]));
        }
      }
    }
  }
}

template <class SP, int KK>
__device__ __forceinline__ void lam_voxels_half(const HalfArgs& a, float2* sm, const Slots& sl, int64_t tile, float ls) {
  constexpr int R1 = SP::R1, L = SP::L;
  const int64_t pstride = (int64_t)a.FC * a.TC;
  for (int t = threadIdx.x; t < (L << sl.tcs); t += blockDim.x) {
    const int li = t & (a.TC - 1);
    const int f = t >> sl.tcs;  // f = f1 + R1 f2
    const int f1 = f % R1, f2 = f / R1;
    float2 X[KK], Y[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) X[k] = sm[sl.at(k, f1, f2, li, R1)];
    const int ch = (int)a.fd_fc.div((uint32_t)f), fc = f - ch * a.FC;
    const int64_t lbase = (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * a.TC + li;
    lam_apply_half<KK>(a.lam_mode, KK, a.lam, lbase, pstride, ls, X, Y);
#pragma unroll
    for (int k = 0; k < KK; ++k) sm[sl.at(k, f1, f2, li, R1)] = Y[k];
  }
}

template <class SP, bool PR>
__global__ void __launch_bounds__(256, 2) kh_lambda(HalfArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  __shared__ float smax;
  load_twiddles(tw, a.pl);
  if (threadIdx.x == 0) smax = 0.f;
  const int cl = (int)(blockIdx.x % (unsigned)a.ncg);  // coil fastest (Λ tile shared in L2)
  const int64_t tile = blockIdx.x / (unsigned)a.ncg;
  const int64_t plane = (int64_t)a.nlast * a.inner;
  __half2* stack = a.d == 2 ? a.st1 : a.st2;
  __half2* base = stack + (int64_t)cl * a.K * plane + tile * a.TC;
  constexpr int nload = PR ? R1 / 2 : R1;
  constexpr int nkeep = PR ? R1 / 2 : R1;
  // 3D: the tile's TC columns lie in one dim-2 column tile (TC and TCm are powers of two dividing g1)
  const int mt = a.d == 3 ? (int)(((tile * a.TC) % a.g1) / a.t.TCm) : 0;
  __syncthreads();
  step_a<SP, -1>(sm, sl, a.K, tw, nload, [&](int k, int li, int n) -> float2 {
    if (!PR && n >= a.nlast) return make_float2(0.f, 0.f);
    float s;
    if (a.d == 2) {  // producer: rows forward, row n
      s = a.t.s_rows[(int64_t)cl * a.t.nrowblk + a.fd_rpc.div((uint32_t)n)];
    } else {         // producer: dim-2 forward, plane (cl,k), slab n / NOo, column tile mt
      s = a.t.s_mid[(((int64_t)cl * a.K + k) * a.t.nslab + a.fd_noo.div((uint32_t)n)) * a.t.nmtile + mt];
    }
    return ld_h(base, k * plane + (int64_t)n * a.inner + li, s);
  });
  __syncthreads();
  step_b<SP, -1>(sm, sl, a.K, R2, [&](int lo, int li, int f1, int f2, float2 v) { sm[sl.at(lo, f1, f2, li, R1)] = v; });
  __syncthreads();
  const float ls = a.lam_scale[tile];
  switch (a.K) {
    case 1: lam_voxels_half<SP, 1>(a, sm, sl, tile, ls); break;
    case 2: lam_voxels_half<SP, 2>(a, sm, sl, tile, ls); break;
    case 3: lam_voxels_half<SP, 3>(a, sm, sl, tile, ls); break;
    case 4: lam_voxels_half<SP, 4>(a, sm, sl, tile, ls); break;
    case 5: lam_voxels_half<SP, 5>(a, sm, sl, tile, ls); break;
    case 6: lam_voxels_half<SP, 6>(a, sm, sl, tile, ls); break;
    case 7: lam_voxels_half<SP, 7>(a, sm, sl, tile, ls); break;
    default: lam_voxels_half<SP, 8>(a, sm, sl, tile, ls); break;
  }
  __syncthreads();
  inv_step_a_slots<SP>(sm, sl, a.K, tw);
  __syncthreads();
  float lmax = 0.f;
  inv_step_b_slots<SP>(sm, sl, a.K, nkeep, [&](int k, int li, int n, float2 v) {
    // output n = g1 + R2 g2 goes back into the task's own column g1 (slot row g2): no other task reads it
    sm[sl.at(k, n / R2, n % R2, li, R1)] = v;
    if (PR || n < a.nlast) lmax = fmaxf(lmax, amax2(v));
  });
  block_max_commit(&smax, lmax);
  __syncthreads();
  const float s = scale_of(smax), inv = 1.f / s;
  if (threadIdx.x == 0) a.t.s_lam[(int64_t)cl * a.ntiles + tile] = s;
  for (int e = threadIdx.x; e < a.K * a.nlast * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % a.nlast, k = t / a.nlast;
    const float2 v = sm[sl.at(k, n / R2, n % R2, li, R1)];
    base[k * plane + (int64_t)n * a.inner + li] = __floats2half2_rn(v.x * inv, v.y * inv);
  }
}

// ------------------------------------------------------------ rows inverse ---
template <class SP, bool PR>
__global__ void __launch_bounds__(512) kh_rows_inv(HalfArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles(tw, a.pl);
  const int k = blockIdx.y;
  const int64_t row0 = (int64_t)blockIdx.x * a.t.rpc;
  const int nr = (int)min((int64_t)a.t.rpc, a.nrows - row0);
  const int NO = a.t.rpc * a.ncg;
  constexpr int nkeep = PR ? R2 / 2 : R2;
  __syncthreads();
  step_a<SP, +1>(sm, sl, NO, tw, R1, [&](int lo, int, int m) -> float2 {
    const int rl = lo / a.ncg, cl = lo - rl * a.ncg;
    if (rl >= nr) return make_float2(0.f, 0.f);
    const int64_t r = row0 + rl;
    float s;
    if (a.d == 2) {  // producer: Λ pass, column m
      s = a.t.s_lam[(int64_t)cl * a.ntiles + a.fd_tc.div((uint32_t)m)];
    } else {         // producer: dim-2 inverse, plane (cl,k), slab i3 / NOo, column tile m / TCm
      const uint32_t i3 = a.fd_n2.div((uint32_t)r);
      s = a.t.s_mid2[(((int64_t)cl * a.K + k) * a.t.nslab + a.fd_noo.div(i3)) * a.t.nmtile + a.fd_tcm.div((uint32_t)m)];
    }
    return ld_h(a.st1, (((int64_t)cl * a.K + k) * a.nrows + r) * L + m, s);
  });
  __syncthreads();
  step_b<SP, +1>(sm, sl, NO, nkeep, [&](int lo, int li, int f1, int f2, float2 v) { sm[sl.at(lo, f1, f2, li, R1)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < nr * a.n1; e += blockDim.x) {
    const int rl = e / a.n1, i1 = e - rl * a.n1;
    const int f1 = i1 % R1, f2 = i1 / R1;
    const int64_t r = row0 + rl;
    float2 acc = make_float2(0.f, 0.f);
    for (int cl = 0; cl < a.ncg; ++cl) {
      const float2 v = sm[sl.at(rl * a.ncg + cl, f1, f2, 0, R1)];
      if (a.cmaps)
        acc = cadd(acc, cmulc(v, a.cmaps[i1 + (int64_t)a.n1 * (r + a.nrows * (a.c0 + cl))]));
      else
        acc = cadd(acc, v);
    }
    const int64_t yi = i1 + (int64_t)a.n1 * (r + a.nrows * k);
    float2 yv;
    if (a.first)
      yv = (a.beta.x == 0.f && a.beta.y == 0.f) ? make_float2(0.f, 0.f) : cmul(a.beta, a.y[yi]);
    else
      yv = a.y[yi];
    a.y[yi] = cadd(yv, cmul(a.alpha, acc));
  }
}

// ----------------------------------------------------- Λ to fp16 tiles ---
// max |entry| over each tile of the float32 chunked Λ, then half storage
__global__ void k_lam_tile_max(const float* lamf, int64_t per_tile, int64_t ntiles, float target, float* scale) {
  __shared__ float red[32];
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    float m = 0.f;
    for (int64_t i = threadIdx.x; i < per_tile; i += blockDim.x) m = fmaxf(m, fabsf(lamf[t * per_tile + i]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      float mm = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mm = fmaxf(mm, red[w]);
      scale[t] = mm > 0.f ? mm / target : 1.f;
    }
    __syncthreads();
  }
}

__global__ void k_lam_to_half(const float* lamf, int64_t per_tile, int64_t n, const float* scale, __half* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2half_rn(lamf[i] / scale[i / per_tile]);
}

// ----------------------------------------------------------- dispatch ---
template <class K>
static int launch_h(K k, dim3 grid, int threads, size_t smem, cudaStream_t st, const HalfArgs& a, const Slots& sl) {
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  if (smem > 48 * 1024) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
  k<<<grid, threads, smem, st>>>(a, sl);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

bool half_supported(const mrsr_normalop* op) {
  for (int i = 0; i < op->geo.ndims; ++i)
    if (!fast_length((int)op->geo.g[i])) return false;
  return op->TC >= 1;
}

int half_lambda_convert(mrsr_normalop* op, cudaStream_t st) {
  const int64_t per_tile = (int64_t)op->P * op->geo.glast() * op->TC * (op->lam_mode == LAM_PACKED_REAL ? 1 : 2);
  const int64_t ntiles = op->geo.inner() / op->TC;
  MRSR_TRY(op->lam_scale.alloc(sizeof(float) * ntiles));
  MRSR_TRY(op->lam_half.alloc(sizeof(__half) * per_tile * ntiles));
  const unsigned b = (unsigned)std::min<int64_t>(ntiles, 65535);
  // tile max scaled to 1: the fp16-arithmetic (pair) kernels need |Λ| <= 1, the float32-arithmetic
  // ones take any scale, and operators of both kinds may share this copy
  const float target = 1.f;
  k_lam_tile_max<<<b, 256, 0, st>>>(op->lam.as<float>(), per_tile, ntiles, target, op->lam_scale.as<float>());
  MRSR_LAUNCH_CHECK();
  const int64_t n = per_tile * ntiles;
  k_lam_to_half<<<(unsigned)std::min<int64_t>(cdiv(n, 256), 65535), 256, 0, st>>>(op->lam.as<float>(), per_tile, n,
                                                                                  op->lam_scale.as<float>(),
                                                                                  op->lam_half.as<__half>());
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int half_alloc_scales(mrsr_normalop* op) {
  const HalfTiles t = tiles_of(op);
  const int64_t n_rows = (int64_t)op->Cg * t.nrowblk;
  const int64_t n_mid = op->geo.ndims == 3 ? (int64_t)op->Cg * op->geo.K * t.nslab * t.nmtile : 1;
  const int64_t n_lam = (int64_t)op->Cg * (op->geo.inner() / op->TC);
  MRSR_TRY(op->scale1.alloc(sizeof(float) * (n_rows + n_lam)));
  MRSR_TRY(op->scale2.alloc(sizeof(float) * 2 * n_mid));
  return MRSR_OK;
}

int apply_half_impl(mrsr_normalop* op, const float2* x, float2* y, float2 alpha, float2 beta, cudaStream_t st,
                    void (*record)(void*), void* rec_ctx) {
  const OpGeom& g = op->geo;
  const int K = g.K;
  const float inv = 1.0f / (float)g.ngrid();
  HalfArgs a{};
  a.d = g.ndims;
  a.K = K;
  a.n1 = (int)g.n[0];
  a.nrows = g.n[1] * g.n[2];
  a.g1 = g.g[0];
  a.g2 = g.g[1];
  a.n2 = g.n[1];
  a.n3 = g.n[2];
  a.TC = op->TC;
  a.P = op->P;
  a.lam_mode = op->lam_mode;
  a.FC = op->FC;
  a.NCH = (int)(g.glast() / op->FC);
  a.inner = g.inner();
  a.ntiles = g.inner() / op->TC;
  a.nlast = (int)g.nlast();
  a.glast = (int)g.glast();
  a.lam = op->lam_half.p;
  a.lam_scale = op->lam_scale.as<float>();
  a.x = x;
  a.cmaps = op->cmaps.p ? op->cmaps.as<float2>() : nullptr;
  a.y = y;
  a.alpha = make_float2(alpha.x * inv, alpha.y * inv);
  a.beta = beta;
  a.st1 = op->stack1.as<__half2>();
  a.st2 = op->stack2.as<__half2>();
  a.t = tiles_of(op);
  a.fd_rpc = FastDiv((uint32_t)a.t.rpc);
  a.fd_noo = FastDiv((uint32_t)a.t.NOo);
  a.fd_tcm = FastDiv((uint32_t)a.t.TCm);
  a.fd_tc = FastDiv((uint32_t)op->TC);
  a.fd_n2 = FastDiv((uint32_t)g.n[1]);
  a.fd_fc = FastDiv((uint32_t)op->FC);
  a.t.s_rows = op->scale1.as<float>();
  a.t.s_lam = op->scale1.as<float>() + (int64_t)op->Cg * a.t.nrowblk;
  const int64_t n_mid = g.ndims == 3 ? (int64_t)op->Cg * K * a.t.nslab * a.t.nmtile : 1;
  a.t.s_mid = op->scale2.as<float>();
  a.t.s_mid2 = op->scale2.as<float>() + n_mid;
  const int ngroups = (int)cdiv(g.ncoils, op->Cg);
  for (int grp = 0; grp < ngroups; ++grp) {
    a.c0 = grp * op->Cg;
    a.ncg = std::min(op->Cg, g.ncoils - a.c0);
    a.first = grp == 0 ? 1 : 0;
    // rows forward
    a.pl = op->plan[0].plan;
    MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
      using SP = decltype(sp);
      const Slots sl = slots_for(SP::R2, 1);
      const int NO = a.t.rpc * K;
      const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)NO * SP::R1 * sl.W);
      const dim3 grid((unsigned)a.t.nrowblk, a.ncg);
      const int thr = std::min(256, rthreads(NO * SP::R1));
      return a.n1 * 2 == SP::L ? launch_h(kh_rows_fwd<SP, true>, grid, thr, smem, st, a, sl)
                               : launch_h(kh_rows_fwd<SP, false>, grid, thr, smem, st, a, sl);
    }));
    if (record) record(rec_ctx);
    if (g.ndims == 3) {
      a.pl = op->plan[1].plan;
      MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
        using SP = decltype(sp);
        const Slots sl = slots_for(SP::R2, a.t.TCm);
        const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)a.t.NOo * SP::R1 * sl.W);
        dim3 grid((unsigned)a.t.nmtile, (unsigned)a.t.nslab, (unsigned)(a.ncg * K));
        const int thr = rthreads(a.t.NOo * a.t.TCm * SP::R1);
        return a.n2 * 2 == SP::L ? launch_h(kh_mid<SP, -1, true>, grid, thr, smem, st, a, sl)
                                 : launch_h(kh_mid<SP, -1, false>, grid, thr, smem, st, a, sl);
      }));
      if (record) record(rec_ctx);
    }
    a.pl = op->plan[g.ndims - 1].plan;
    MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
      using SP = decltype(sp);
      const Slots sl = slots_for(SP::R2, a.TC);
      const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)K * SP::R1 * sl.W);
      const dim3 grid((unsigned)(a.ntiles * a.ncg));
      return a.nlast * 2 == SP::L ? launch_h(kh_lambda<SP, true>, grid, 256, smem, st, a, sl)
                                  : launch_h(kh_lambda<SP, false>, grid, 256, smem, st, a, sl);
    }));
    if (record) record(rec_ctx);
    if (g.ndims == 3) {
      a.pl = op->plan[1].plan;
      MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
        using SP = decltype(sp);
        const Slots sl = slots_for(SP::R2, a.t.TCm);
        const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)a.t.NOo * SP::R1 * sl.W);
        dim3 grid((unsigned)a.t.nmtile, (unsigned)a.t.nslab, (unsigned)(a.ncg * K));
        const int thr = rthreads(a.t.NOo * a.t.TCm * SP::R1);
        return a.n2 * 2 == SP::L ? launch_h(kh_mid<SP, +1, true>, grid, thr, smem, st, a, sl)
                                 : launch_h(kh_mid<SP, +1, false>, grid, thr, smem, st, a, sl);
      }));
      if (record) record(rec_ctx);
    }
    a.pl = op->plan[0].plan;
    MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
      using SP = decltype(sp);
      const Slots sl = slots_for(SP::R2, 1);
      const int NO = a.t.rpc * a.ncg;
      const size_t smem = sizeof(float2) * ((size_t)SP::L + (size_t)NO * SP::R1 * sl.W);
      const dim3 grid((unsigned)a.t.nrowblk, K);
      const int thr = std::min(256, rthreads(NO * SP::R1));
      return a.n1 * 2 == SP::L ? launch_h(kh_rows_inv<SP, true>, grid, thr, smem, st, a, sl)
                               : launch_h(kh_rows_inv<SP, false>, grid, thr, smem, st, a, sl);
    }));
    if (record) record(rec_ctx);
  }
  return MRSR_OK;
}

}  // namespace mrsr
