// fp16-arithmetic apply for 2D operators: the same three passes as the
// float32 four-step kernels (rows forward, Λ pass, rows inverse), with every
// FFT butterfly and the K x K product in packed half2 arithmetic on pairs of
// lines (fft4h.cuh).  The coil sums and the output update are float32.
//
// Scaling.  fp16 holds 11 significant bits and magnitudes below 65504, so every
// value entering a transform is normalised to at most 1 and the transform's
// growth (at most its length) stays in range:
//   * rows forward: x S_c / (max|x| max|S_c|), max|x| reduced on the device per
//     apply and max|S_c| per coil when the maps are set;
//   * stored tiles: value * 2^e with 2^e the largest power of two keeping the
//     tile's largest magnitude <= kPairStore; the float32 scale of the tile
//     (true = stored * scale) goes to a scale array;
//   * a consumer rescales every loaded value to a common scale of its line
//     (pairs have one scale per lane) before transforming;
//   * the Λ pass renormalises after the K x K product by a power of two.
// Powers of two multiply exactly in fp16, so rescaling adds no rounding.
#include <algorithm>
#include <cmath>

#include "fft4h.cuh"
#include "half.cuh"
#include "passes.cuh"

namespace mrsr {

constexpr float kPairStore = 256.f;  // largest stored magnitude of the pair path's stacks

struct PairArgs {
  FftPlan pl;
  int K, n1;
  int64_t nrows;        // rows of the image (n2)
  int c0, ncg;
  int rpf, rpi;         // rows per CTA of rows forward / rows inverse
  int64_t nrbf;         // row blocks of rows forward
  // Λ pass
  int TC, tcs, P, lam_mode, FC, NCH;  // tcs = log2(TC)
  int64_t inner, ntiles;
  int nlast;
  FastDiv fcd;
  const void* lam;          // fp16 kernel, chunked layout, tile max scaled to 1
  const float* lam_scale;   // [tile]
  // data
  const float2* x;
  const float2* cmaps;
  const float* cmax;        // [coil] max |S_c| (NULL: unit coil)
  const float* xmax;        // max |x| of this apply
  float2* y;
  float2 alpha, beta;
  int first;
  __half2* st;              // stack [cl][k][row][L] of half2 (re, im)
  float* s_rows;            // [cl][row block]
  float* s_lam;             // [cl][tile]
  float* s_coil;            // [cl] max over tiles of s_lam
};

__device__ __forceinline__ __half2 habsmax(hc2 v) { return __hmax2(__habs2(v.re), __habs2(v.im)); }
__device__ __forceinline__ float hmax_f(__half2 m) { return fmaxf(__low2float(m), __high2float(m)); }
// largest power of two p with m * p <= target (m > 0)
// (at most 2^15, so that the factor itself is an fp16 number)
__device__ __forceinline__ float pow2_fit(float m, float target) {
  return m > 0.f ? exp2f(fminf(floorf(log2f(target / m)), 15.f)) : 1.f;
}
__device__ __forceinline__ __half2 h2f(float v) { return __float2half2_rn(v); }

// ------------------------------------------------------------ rows forward ---
template <class SP, bool PR>
__global__ void __launch_bounds__(256) kp_rows_fwd(PairArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ hc2 smh[];
  hc2* tw = smh;
  hc2* sm = smh + L;
  load_twiddles_h(tw, a.pl);
  const int cl = blockIdx.y, c = a.c0 + cl;
  const int64_t rb = blockIdx.x;
  const int64_t row0 = rb * a.rpf;
  const int nr = (int)min((int64_t)a.rpf, a.nrows - row0);
  const int NO = nr * a.K;                 // lines of this CTA
  const int NP = (a.rpf * a.K + 1) / 2;    // line pairs (slots)
  const float xs = a.xmax[0] * (a.cmax ? a.cmax[c] : 1.f);
  const float cin = xs > 0.f ? 1.f / xs : 1.f;
  // inputs <= 1, so outputs <= n1: a fixed power-of-two store factor keeps them <= kPairStore
  const float fac = exp2f(floorf(log2f(kPairStore / (float)a.n1)));
  if (threadIdx.x == 0) a.s_rows[(int64_t)cl * a.nrbf + rb] = 1.f / (fac * cin);
  const float cf = cin * fac;  // folded into the input conversion (the transform is linear)
  constexpr int nload = PR ? R1 / 2 : R1;
  __syncthreads();
  auto line = [&](int lo, int n) -> float2 {
    if (lo >= NO || (!PR && n >= a.n1)) return make_float2(0.f, 0.f);
    const int rl = lo / a.K, k = lo - rl * a.K;
    const int64_t r = row0 + rl;
    float2 v = a.x[n + (int64_t)a.n1 * (r + a.nrows * k)];
    if (a.cmaps) v = cmul(a.cmaps[n + (int64_t)a.n1 * (r + a.nrows * c)], v);
    return v;
  };
  step_a_h<SP, -1>(sm, sl, NP, tw, nload, [&](int p, int, int n) -> hc2 {
    const float2 va = line(2 * p, n), vb = line(2 * p + 1, n);
    return hc2{__floats2half2_rn(va.x * cf, vb.x * cf), __floats2half2_rn(va.y * cf, vb.y * cf)};
  });
  __syncthreads();
  step_b_h<SP, -1>(sm, sl, NP, R2, [&](int p, int, int f1, int f2, hc2 v) {
    const int f = f1 + R1 * f2;
#pragma unroll
    for (int lane = 0; lane < 2; ++lane) {
      const int lo = 2 * p + lane;
      if (lo < NO) {
        const int rl = lo / a.K, k = lo - rl * a.K;
        a.st[(((int64_t)cl * a.K + k) * a.nrows + row0 + rl) * L + f] = lane ? hlane_b(v) : hlane_a(v);
      }
    }
  });
}

// ------------------------------------------------------------- Λ pass ---
// Y[k1] = sum_k2 Λ(k1, k2) X[k2] on a pair of columns; Λ pairs are adjacent in the chunked layout
template <int KK>
__device__ __forceinline__ void lam_pair(int mode, const void* lamv, int64_t lbase, int64_t pstride, const hc2* X,
                                         hc2* Y) {
#pragma unroll
  for (int j = 0; j < KK; ++j) Y[j] = hzero();
  if (mode == LAM_PACKED_REAL) {
    const __half* lam = reinterpret_cast<const __half*>(lamv) + lbase;
    int p = 0;
#pragma unroll
    for (int k2 = 0; k2 < KK; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 <= k2; ++k1) {
        const __half2 l = *reinterpret_cast<const __half2*>(lam + p * pstride);
        Y[k1].re = __hfma2(l, X[k2].re, Y[k1].re);
        Y[k1].im = __hfma2(l, X[k2].im, Y[k1].im);
        if (k1 != k2) {
          Y[k2].re = __hfma2(l, X[k1].re, Y[k2].re);
          Y[k2].im = __hfma2(l, X[k1].im, Y[k2].im);
        }
        ++p;
      }
    }
  } else {
    const __half2* lam = reinterpret_cast<const __half2*>(lamv) + lbase;
    const bool packed = mode == LAM_PACKED_CPLX;
    int p = 0;
#pragma unroll
    for (int k2 = 0; k2 < KK; ++k2) {
#pragma unroll
      for (int k1 = 0; k1 < KK; ++k1) {
        if (packed && k1 > k2) continue;
        const int q = packed ? p++ : k1 + KK * k2;
        const uint2 u = *reinterpret_cast<const uint2*>(lam + q * pstride);  // (re, im) of both columns
        const hc2 l = hpack(h2u(u.x), h2u(u.y));
        Y[k1] = Y[k1] + hcmul(X[k2], l.re, l.im);
        if (packed && k1 != k2) Y[k2] = Y[k2] + hcmul(X[k1], l.re, __hneg2(l.im));
      }
    }
  }
}

template <class SP, int KK>
__device__ __forceinline__ __half2 lam_voxels_pair(const PairArgs& a, hc2* sm, const Slots& sl, int64_t tile) {
  constexpr int R1 = SP::R1, L = SP::L;
  const int64_t pstride = (int64_t)a.FC * a.TC;
  __half2 ym = h2u(0u);
  for (int t = threadIdx.x; t < (L << sl.tcs); t += blockDim.x) {
    const int lp = t & (sl.TC - 1);
    const int f = t >> sl.tcs;
    const int f1 = f % R1, f2 = f / R1;
    hc2 X[KK], Y[KK];
#pragma unroll
    for (int k = 0; k < KK; ++k) X[k] = sm[sl.at(k, f1, f2, lp, R1)];
    const int ch = (int)a.fcd.div((uint32_t)f), fc = f - ch * a.FC;
    const int64_t lbase = (((tile * a.NCH + ch) * a.P) * (int64_t)a.FC + fc) * a.TC + 2 * lp;
    lam_pair<KK>(a.lam_mode, a.lam, lbase, pstride, X, Y);
#pragma unroll
    for (int k = 0; k < KK; ++k) {
      sm[sl.at(k, f1, f2, lp, R1)] = Y[k];
      ym = __hmax2(ym, habsmax(Y[k]));
    }
  }
  return ym;
}

template <class SP, bool PR>
__global__ void __launch_bounds__(256, 2) kp_lambda(PairArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ hc2 smh[];
  hc2* tw = smh;
  __half2* ftab = reinterpret_cast<__half2*>(smh + L);  // per input row: load factor (broadcast)
  hc2* sm = smh + L + (a.nlast + 1) / 2;
  __shared__ float sS, sY;
  load_twiddles_h(tw, a.pl);
  if (threadIdx.x == 0) sS = sY = 0.f;
  const int cl = (int)(blockIdx.x % (unsigned)a.ncg);  // coil fastest (Λ tile shared in L2)
  const int64_t tile = blockIdx.x / (unsigned)a.ncg;
  const int64_t plane = (int64_t)a.nlast * a.inner;
  __half2* base = a.st + (int64_t)cl * a.K * plane + tile * a.TC;
  const float* srow = a.s_rows + (int64_t)cl * a.nrbf;
  __syncthreads();
  // common scale of the input rows, and each row's factor to it
  float m = 0.f;
  for (int64_t i = threadIdx.x; i < a.nrbf; i += blockDim.x) m = fmaxf(m, srow[i]);
  block_max_commit(&sS, m);
  __syncthreads();
  const float S = sS;
  for (int n = threadIdx.x; n < a.nlast; n += blockDim.x) ftab[n] = h2f(srow[n / a.rpf] / (S * kPairStore));
  __syncthreads();
  constexpr int nload = PR ? R1 / 2 : R1;
  constexpr int nkeep = PR ? R1 / 2 : R1;
  step_a_h<SP, -1>(sm, sl, a.K, tw, nload, [&](int k, int lp, int n) -> hc2 {
    if (!PR && n >= a.nlast) return hzero();
    const uint2 u = *reinterpret_cast<const uint2*>(base + k * plane + (int64_t)n * a.inner + 2 * lp);
    return hscale(hpack(h2u(u.x), h2u(u.y)), ftab[n]);
  });
  __syncthreads();
  step_b_h<SP, -1>(sm, sl, a.K, R2, [&](int lo, int li, int f1, int f2, hc2 v) { sm[sl.at(lo, f1, f2, li, R1)] = v; });
  __syncthreads();
  __half2 ym;
  switch (a.K) {
    case 1: ym = lam_voxels_pair<SP, 1>(a, sm, sl, tile); break;
    case 2: ym = lam_voxels_pair<SP, 2>(a, sm, sl, tile); break;
    case 3: ym = lam_voxels_pair<SP, 3>(a, sm, sl, tile); break;
    case 4: ym = lam_voxels_pair<SP, 4>(a, sm, sl, tile); break;
    case 5: ym = lam_voxels_pair<SP, 5>(a, sm, sl, tile); break;
    case 6: ym = lam_voxels_pair<SP, 6>(a, sm, sl, tile); break;
    case 7: ym = lam_voxels_pair<SP, 7>(a, sm, sl, tile); break;
    default: ym = lam_voxels_pair<SP, 8>(a, sm, sl, tile); break;
  }
  block_max_commit(&sY, hmax_f(ym));
  __syncthreads();
  const float p2 = pow2_fit(sY, 1.f);  // inverse transform input <= 1
  inv_step_a_slots_h<SP>(sm, sl, a.K, tw, h2f(p2));
  __syncthreads();
  // inverse input <= 1, so outputs <= L: fixed store factor
  const float fo = exp2f(floorf(log2f(kPairStore / (float)L)));
  if (threadIdx.x == 0) {
    const float s = a.lam_scale[tile] * S * kPairStore / (p2 * fo);
    a.s_lam[(int64_t)cl * a.ntiles + tile] = s;
    atomicMax(reinterpret_cast<unsigned*>(a.s_coil + cl), __float_as_uint(s));
  }
  const __half2 fh = h2f(fo);
  inv_step_b_slots_h<SP>(sm, sl, a.K, nkeep, [&](int k, int lp, int n, hc2 v) {
    if (PR || n < a.nlast) {
      v = hscale(v, fh);
      uint2 u;
      u.x = u2h(hlane_a(v));
      u.y = u2h(hlane_b(v));
      *reinterpret_cast<uint2*>(base + k * plane + (int64_t)n * a.inner + 2 * lp) = u;
    }
  });
}

// ------------------------------------------------------------ rows inverse ---
template <class SP, bool PR>
__global__ void __launch_bounds__(512) kp_rows_inv(PairArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ hc2 smh[];
  hc2* tw = smh;
  float* cs = reinterpret_cast<float*>(smh + L);        // [cl] common scale of the coil's lines
  __half* ftab = reinterpret_cast<__half*>(cs + a.ncg);  // [cl][tile] load factor
  const int ftab_elems = a.ncg * (int)a.ntiles;
  hc2* sm = reinterpret_cast<hc2*>(cs) + (a.ncg * 4 + ftab_elems * 2 + 7) / 8;
  load_twiddles_h(tw, a.pl);
  const int k = blockIdx.y;
  const int64_t row0 = (int64_t)blockIdx.x * a.rpi;
  const int nr = (int)min((int64_t)a.rpi, a.nrows - row0);
  const int NO = nr * a.ncg;
  const int NP = (a.rpi * a.ncg + 1) / 2;
  for (int cl = threadIdx.x; cl < a.ncg; cl += blockDim.x) cs[cl] = a.s_coil[cl];
  __syncthreads();
  for (int i = threadIdx.x; i < ftab_elems; i += blockDim.x) {
    const int cl = i / (int)a.ntiles;
    const float c = cs[cl];
    ftab[i] = __float2half_rn(c > 0.f ? a.s_lam[i] / (c * kPairStore) : 0.f);
  }
  __syncthreads();
  constexpr int nkeep = PR ? R2 / 2 : R2;
  auto ld = [&](int lo, int m, __half& f) -> __half2 {
    if (lo >= NO) {
      f = __float2half_rn(0.f);
      return h2u(0u);
    }
    const int rl = lo / a.ncg, cl = lo - rl * a.ncg;
    f = ftab[cl * (int)a.ntiles + (m >> a.tcs)];
    return a.st[(((int64_t)cl * a.K + k) * a.nrows + row0 + rl) * L + m];
  };
  step_a_h<SP, +1>(sm, sl, NP, tw, R1, [&](int p, int, int m) -> hc2 {
    __half fa, fb;
    const __half2 va = ld(2 * p, m, fa), vb = ld(2 * p + 1, m, fb);
    return hscale(hpack(va, vb), __halves2half2(fa, fb));
  });
  __syncthreads();
  step_b_h<SP, +1>(sm, sl, NP, nkeep, [&](int p, int li, int f1, int f2, hc2 v) { sm[sl.at(p, f1, f2, li, R1)] = v; });
  __syncthreads();
  for (int e = threadIdx.x; e < nr * a.n1; e += blockDim.x) {
    const int rl = e / a.n1, i1 = e - rl * a.n1;
    const int f1 = i1 % R1, f2 = i1 / R1;
    const int64_t r = row0 + rl;
    float2 acc = make_float2(0.f, 0.f);
    for (int cl = 0; cl < a.ncg; ++cl) {
      const int lo = rl * a.ncg + cl;
      const hc2 hv = sm[sl.at(lo >> 1, f1, f2, 0, R1)];
      float2 v = __half22float2((lo & 1) ? hlane_b(hv) : hlane_a(hv));
      const float s = cs[cl] * kPairStore;
      v = make_float2(v.x * s, v.y * s);
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

// ---------------------------------------------------------- reductions ---
__global__ void k_absmax_c(const float2* v, int64_t n, float* out) {
  __shared__ float bm;
  if (threadIdx.x == 0) bm = 0.f;
  __syncthreads();
  float m = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, amax2(v[i]));
  block_max_commit(&bm, m);
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(reinterpret_cast<unsigned*>(out), __float_as_uint(bm));
}

// per coil max |S_c|: one block per coil
__global__ void k_coil_absmax(const float2* cm, int64_t nimg, float* out) {
  __shared__ float s;
  if (threadIdx.x == 0) s = 0.f;
  __syncthreads();
  float m = 0.f;
  const float2* p = cm + (int64_t)blockIdx.x * nimg;
  for (int64_t i = threadIdx.x; i < nimg; i += blockDim.x) m = fmaxf(m, amax2(p[i]));
  block_max_commit(&s, m);
  __syncthreads();
  if (threadIdx.x == 0) out[blockIdx.x] = s;
}

// ----------------------------------------------------------- dispatch ---
template <class K>
static int launch_p(K k, dim3 grid, int threads, size_t smem, cudaStream_t st, const PairArgs& a, const Slots& sl) {
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  if (smem > 48 * 1024) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
  k<<<grid, threads, smem, st>>>(a, sl);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// rows per CTA: enough line pairs for ~256 step-B tasks
static int pair_rows(int lines_per_row, int R1, int64_t nrows) {
  const int pairs = std::max(1, 128 / R1);
  return (int)std::max<int64_t>(1, std::min<int64_t>((2 * pairs) / lines_per_row, nrows));
}

static int split_r1(int L) {
  int r1 = 0;
  with_split_h(L, [&](auto sp) -> int {
    r1 = decltype(sp)::R1;
    return MRSR_OK;
  });
  return r1;
}

bool pair_supported(const mrsr_normalop* op) {
  const OpGeom& g = op->geo;
  return op->precision == MRSR_PREC_FP16_ARITH && g.ndims == 2 && fast_length((int)g.g[0]) && fast_length((int)g.g[1]) && op->TC >= 2 && op->TC % 2 == 0;
}

struct PairLayout {
  int rpf, rpi;
  int64_t nrbf;
};

static PairLayout pair_layout(const mrsr_normalop* op) {
  const OpGeom& g = op->geo;
  PairLayout p;
  const int r1 = split_r1((int)g.g[0]);
  p.rpf = pair_rows(g.K, r1, g.n[1]);
  p.rpi = pair_rows(op->Cg, r1, g.n[1]);
  p.nrbf = cdiv(g.n[1], p.rpf);
  return p;
}

// scale arrays of the pair path in op->scale1: s_rows | s_lam | s_coil | xmax | cmax[ncoils]
int pair_alloc(mrsr_normalop* op, cudaStream_t st) {
  const PairLayout pl = pair_layout(op);
  const int64_t n = (int64_t)op->Cg * pl.nrbf + (int64_t)op->Cg * (op->geo.inner() / op->TC) + op->Cg + 1 +
                    op->geo.ncoils;
  MRSR_TRY(op->scale1.alloc(sizeof(float) * n));
  float* cmax = op->scale1.as<float>() + (n - op->geo.ncoils);
  if (op->cmaps.p) {
    k_coil_absmax<<<op->geo.ncoils, 256, 0, st>>>(op->cmaps.as<float2>(), op->geo.nimg(), cmax);
    MRSR_LAUNCH_CHECK();
  }
  op->launches = 1 + 3 * (int)cdiv(op->geo.ncoils, op->Cg);
  return MRSR_OK;
}

int apply_pair_impl(mrsr_normalop* op, const float2* x, float2* y, float2 alpha, float2 beta, cudaStream_t st,
                    void (*record)(void*), void* rec_ctx) {
  const OpGeom& g = op->geo;
  const int K = g.K;
  const PairLayout pl = pair_layout(op);
  PairArgs a{};
  a.K = K;
  a.n1 = (int)g.n[0];
  a.nrows = g.n[1];
  a.rpf = pl.rpf;
  a.rpi = pl.rpi;
  a.nrbf = pl.nrbf;
  a.TC = op->TC;
  a.tcs = 0;
  while ((1 << a.tcs) < a.TC) ++a.tcs;
  a.P = op->P;
  a.lam_mode = op->lam_mode;
  a.FC = op->FC;
  a.NCH = (int)(g.glast() / op->FC);
  a.fcd = FastDiv((uint32_t)op->FC);
  a.inner = g.inner();
  a.ntiles = g.inner() / op->TC;
  a.nlast = (int)g.nlast();
  a.lam = op->lam_half.p;
  a.lam_scale = op->lam_scale.as<float>();
  a.x = x;
  a.cmaps = op->cmaps.p ? op->cmaps.as<float2>() : nullptr;
  a.y = y;
  const float inv = 1.0f / (float)g.ngrid();
  a.alpha = make_float2(alpha.x * inv, alpha.y * inv);
  a.beta = beta;
  a.st = op->stack1.as<__half2>();
  float* sc = op->scale1.as<float>();
  a.s_rows = sc;
  a.s_lam = sc + (int64_t)op->Cg * pl.nrbf;
  a.s_coil = a.s_lam + (int64_t)op->Cg * a.ntiles;
  float* xm = a.s_coil + op->Cg;
  a.xmax = xm;
  a.cmax = a.cmaps ? xm + 1 : nullptr;
  const int64_t nx = g.nimg() * K;
  MRSR_CHECK_CUDA(cudaMemsetAsync(xm, 0, sizeof(float), st));
  k_absmax_c<<<(unsigned)std::min<int64_t>(cdiv(nx, 1024), 304), 1024, 0, st>>>(x, nx, xm);
  MRSR_LAUNCH_CHECK();
  if (record) record(rec_ctx);
  const int ngroups = (int)cdiv(g.ncoils, op->Cg);
  for (int grp = 0; grp < ngroups; ++grp) {
    a.c0 = grp * op->Cg;
    a.ncg = std::min(op->Cg, g.ncoils - a.c0);
    a.first = grp == 0 ? 1 : 0;
    MRSR_CHECK_CUDA(cudaMemsetAsync(a.s_coil, 0, sizeof(float) * op->Cg, st));
    const bool pr = g.n[0] * 2 == g.g[0];
    a.pl = op->plan[0].plan;
    MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
      using SP = decltype(sp);
      const Slots sl = slots_for(SP::R2, 1);
      const int NP = (a.rpf * K + 1) / 2;
      const size_t smem = sizeof(hc2) * ((size_t)SP::L + (size_t)NP * SP::R1 * sl.W);
      const dim3 grid((unsigned)a.nrbf, a.ncg);
      const int thr = std::min(256, rthreads(NP * SP::R2));
      return pr ? launch_p(kp_rows_fwd<SP, true>, grid, thr, smem, st, a, sl)
                : launch_p(kp_rows_fwd<SP, false>, grid, thr, smem, st, a, sl);
    }));
    if (record) record(rec_ctx);
    a.pl = op->plan[1].plan;
    MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
      using SP = decltype(sp);
      const Slots sl = slots_for(SP::R2, a.TC / 2);
      const size_t smem =
          sizeof(hc2) * ((size_t)SP::L + (size_t)(a.nlast + 1) / 2 + (size_t)K * SP::R1 * sl.W);
      const dim3 grid((unsigned)(a.ntiles * a.ncg));
      const bool prl = (int64_t)a.nlast * 2 == SP::L;
      return prl ? launch_p(kp_lambda<SP, true>, grid, 256, smem, st, a, sl)
                 : launch_p(kp_lambda<SP, false>, grid, 256, smem, st, a, sl);
    }));
    if (record) record(rec_ctx);
    a.pl = op->plan[0].plan;
    MRSR_TRY(with_split_h(a.pl.L, [&](auto sp) -> int {
      using SP = decltype(sp);
      const Slots sl = slots_for(SP::R2, 1);
      const int NP = (a.rpi * a.ncg + 1) / 2;
      const size_t head = (size_t)a.ncg * 4 + (size_t)a.ncg * a.ntiles * 2;
      const size_t smem = sizeof(hc2) * ((size_t)SP::L + (head + 7) / 8 + (size_t)NP * SP::R1 * sl.W);
      const dim3 grid((unsigned)cdiv(a.nrows, a.rpi), K);
      const int thr = rthreads(NP * SP::R1);
      return pr ? launch_p(kp_rows_inv<SP, true>, grid, thr, smem, st, a, sl)
                : launch_p(kp_rows_inv<SP, false>, grid, thr, smem, st, a, sl);
    }));
    if (record) record(rec_ctx);
  }
  return MRSR_OK;
}

}  // namespace mrsr
