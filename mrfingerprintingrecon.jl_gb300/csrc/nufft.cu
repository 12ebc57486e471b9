// NUFFT kernels and the paths built on them:
//  * calculate_kmask_indcs / calculate_kernel_noncartesian -> NFFTNormalOp(img_shape, trj, U)
//    (src/NFFTNormalOp.jl:106-225, ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:75-191)
//  * calculate_backprojection (src/BackProjection.jl:23-102, ext/.../BackProjection.jl:1-71)
//  * the forward model of the reference tests (test/reconstruct_radial.jl:62-74)
#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "normalop.cuh"
#include "nufft.cuh"

namespace mrsr {

// ------------------------------------------------------------ samples ---

__device__ __forceinline__ int64_t sample_lin(const SampleSet& S, int64_t i) { return S.list ? S.list[i] - 1 : i; }

// frame of linear sample index li (32-bit division when the operands allow)
__device__ __forceinline__ int64_t frame_of(int64_t li, int64_t ns_pf) {
  return (li | ns_pf) < (1ll << 31) ? (int64_t)((unsigned)li / (unsigned)ns_pf) : li / ns_pf;
}

__global__ void k_mask_to_flags(const uint8_t* mask, int64_t n, uint8_t* flags) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    flags[i] = mask[i] ? 1 : 0;
}

int SampleList::init(int d, const float* trj, int64_t ns_pf, int64_t nt, const uint8_t* mask, cudaStream_t st) {
  set.trj = trj;
  set.d = d;
  set.ns_pf = ns_pf;
  set.nt = nt;
  const int64_t n = ns_pf * nt;
  if (!mask) {
    set.list = nullptr;
    set.n = n;
    return MRSR_OK;
  }
  DevBuf flags;
  MRSR_TRY(flags.alloc(std::max<int64_t>(n, 1)));
  k_mask_to_flags<<<(unsigned)std::min<int64_t>(cdiv(n, 256), 65535), 256, 0, st>>>(mask, n, flags.as<uint8_t>());
  MRSR_LAUNCH_CHECK();
  int64_t cnt = 0;
  MRSR_TRY(compact_nonzero(flags.as<uint8_t>(), n, list, &cnt, st));
  set.list = list.as<int64_t>();
  set.n = cnt;
  return MRSR_OK;
}

// ------------------------------------------------------- ES kernel ---

static double es_phi_host(double z) {
  if (std::fabs(z) >= 1.0) return 0.0;
  return std::exp((double)kEsBeta * (std::sqrt(1.0 - z * z) - 1.0));
}

// Gauss-Legendre nodes/weights on [-1, 1] (Newton iteration on P_n from the Chebyshev guess).
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < (n + 1) / 2; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
    double pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        const double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      const double dz = p1 / pp;
      z -= dz;
      if (std::fabs(dz) < 1e-15) break;
    }
    x[i] = -z;
    x[n - 1 - i] = z;
    w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * pp * pp);
  }
}

// psi_hat(j) = (w/2) int_{-1}^{1} phi(z) cos(pi j w z / M) dz.  The tables are cached per
// (device, M, jmin, count) for the life of the process (a few KB each, never freed): one
// costs count x 200 host cosines, and every kernel build, backprojection and forward model
// needs d of them.
int es_inv_psi_table(int64_t M, int64_t jmin, int64_t count, const float** out) {
  static std::mutex mu;
  static std::map<std::array<int64_t, 4>, float*> cache;
  static std::vector<double> gx, gw, gphi;
  int dev = 0;
  MRSR_CHECK_CUDA(cudaGetDevice(&dev));
  const std::array<int64_t, 4> key{dev, M, jmin, count};
  std::lock_guard<std::mutex> lock(mu);
  const auto it = cache.find(key);
  if (it != cache.end()) {
    *out = it->second;
    return MRSR_OK;
  }
  if (gx.empty()) {
    gauss_legendre(200, gx, gw);
    gphi.resize(gx.size());
    for (size_t q = 0; q < gx.size(); ++q) gphi[q] = gw[q] * es_phi_host(gx[q]);
  }
  std::vector<float> h(count);
  const double hw = 0.5 * kEsWidth;
  for (int64_t i = 0; i < count; ++i) {
    const double j = (double)(jmin + i);
    double s = 0.0;
    for (size_t q = 0; q < gx.size(); ++q) s += gphi[q] * std::cos(M_PI * j * kEsWidth * gx[q] / (double)M);
    h[i] = (float)(1.0 / (hw * s));
  }
  float* d = nullptr;
  MRSR_CHECK_CUDA(cudaMalloc(&d, sizeof(float) * std::max<int64_t>(count, 1)));
  const cudaError_t e = cudaMemcpy(d, h.data(), sizeof(float) * count, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    MRSR_CHECK_CUDA(e);
  }
  cache[key] = d;
  *out = d;
  return MRSR_OK;
}

// --------------------------------------------------------- spreading ---

// one fixed-point term: a = value * 2^(e - 21), added as round(a * 2^21)
__device__ __forceinline__ void fx_add(long long* q, float a) {
  atomicAdd(reinterpret_cast<unsigned long long*>(q), (unsigned long long)fx_term(a));
}

__device__ __forceinline__ int wrap32(int l, int M) {
  l %= M;
  return l < 0 ? l + M : l;
}

// l mod M for -M < l < M (no division)
__device__ __forceinline__ int64_t wrap_near(int64_t l, int64_t M) { return l < 0 ? l + M : l; }

// Element e of an array of `planes` planes of (N0, N1, N2) cells -> plane and per-axis
// position.  Below 2^31 elements by magic-number divisions (FastDiv); this GPU divides 64-bit
// integers in software, tens of instructions each.
struct Decomp {
  int d = 0;
  bool fast = false;
  int64_t cells = 1, N[3] = {1, 1, 1};
  FastDiv fcells, fN[2];
  void init(int dims, const int64_t* n, int64_t planes) {
    d = dims;
    cells = 1;
    for (int i = 0; i < 3; ++i) {
      N[i] = i < dims ? n[i] : 1;
      cells *= N[i];
    }
    fast = cells * planes < (1ll << 31);
    if (fast) {
      fcells = FastDiv((uint32_t)cells);
      fN[0] = FastDiv((uint32_t)N[0]);
      fN[1] = FastDiv((uint32_t)N[1]);
    }
  }
  __device__ __forceinline__ int split(int64_t e, int64_t* pos) const {
    if (fast) {
      const uint32_t ue = (uint32_t)e, pl = fcells.div(ue);
      uint32_t r = ue - pl * fcells.d;
      const uint32_t q0 = fN[0].div(r);
      pos[0] = r - q0 * fN[0].d;
      r = q0;
      const uint32_t q1 = fN[1].div(r);
      pos[1] = r - q1 * fN[1].d;
      pos[2] = q1;
      return (int)pl;
    }
    const int pl = (int)(e / cells);
    int64_t r = e - (int64_t)pl * cells;
    pos[0] = r % N[0];
    r /= N[0];
    pos[1] = r % N[1];
    pos[2] = r / N[1];
    return pl;
  }
};

// Taps of one sample owned by a lane of its warp: lane = t1 + 8 * t2a (t1 < 8, t2a < 4), and
// its J = w^d / 32 taps are t2 = t2a + 4 (j & 1), t3 = j >> 1.  Weights (times `sc`) and
// grid cells (< 2^32, checked by the launchers) are formed once per sample, with 32-bit wraps.
template <int J>
__device__ __forceinline__ void lane_taps(const SampleSet& S, const int64_t* M, int64_t li, int lane, float sc,
                                          float* w, unsigned* cell) {
  constexpr int d = J == 2 ? 2 : 3;
  float kd[3] = {0.f, 0.f, 0.f};
  for (int dd = 0; dd < d; ++dd) kd[dd] = S.trj[dd + (int64_t)d * li];
  float wt;
  int64_t l0[3] = {0, 0, 0};
  es_lane_weight(kd, M, d, lane, &wt, l0);
  const int t1 = lane & 7, t2a = lane >> 3;
  const float wx = __shfl_sync(0xffffffffu, wt, t1) * sc;
  const unsigned x = wrap32((int)l0[0] + t1, (int)M[0]);
#pragma unroll
  for (int j = 0; j < J; ++j) {
    const int t2 = t2a + 4 * (j & 1), t3 = j >> 1;
    float wj = wx * __shfl_sync(0xffffffffu, wt, kEsWidth + t2);
    unsigned c = x + (unsigned)M[0] * (unsigned)wrap32((int)l0[1] + t2, (int)M[1]);
    if (d == 3) {
      wj *= __shfl_sync(0xffffffffu, wt, 2 * kEsWidth + t3);
      c += (unsigned)(M[0] * M[1]) * (unsigned)wrap32((int)l0[2] + t3, (int)M[2]);
    }
    w[j] = wj;
    cell[j] = c;
  }
}

// One warp per kept sample (the 3D grids; tile-sorted kernels below do 2D).  A channel's
// value is formed once per sample; its terms go to the grid as 64-bit atomics.
template <int J>
__global__ void __launch_bounds__(256, 2) k_spread_lambda(SpreadLambdaArgs a, const int* order) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const float sc = a.fs->scale;
  const int64_t chs = (int64_t)a.nq * a.cells;
  for (int64_t i = warp; i < a.S.n; i += nwarps) {
    const int64_t n = order ? (int64_t)order[i] : i;
    const int64_t li = sample_lin(a.S, n);
    const int64_t t = frame_of(li, a.S.ns_pf);
    float w[J];
    unsigned cell[J];
    lane_taps<J>(a.S, a.M, li, lane, sc, w, cell);
    for (int ch = 0; ch < a.np; ++ch) {
      const int p = a.p0 + ch;
      int k2 = 0;
      while ((k2 + 1) * (k2 + 2) / 2 <= p) ++k2;
      const int k1 = p - k2 * (k2 + 1) / 2;
      float2 v;  // conj(U[t,k1]) * U[t,k2]
      if (a.u_complex) {
        const float2* u = reinterpret_cast<const float2*>(a.U);
        v = cmulc(u[t + a.S.nt * k2], u[t + a.S.nt * k1]);
      } else {
        const float* u = reinterpret_cast<const float*>(a.U);
        v = make_float2(u[t + a.S.nt * k2] * u[t + a.S.nt * k1], 0.f);
      }
      long long* q = a.q + (int64_t)ch * chs;
#pragma unroll
      for (int j = 0; j < J; ++j) {
        fx_add(q + cell[j], v.x * w[j]);
        if (a.nq == 2) fx_add(q + a.cells + cell[j], v.y * w[j]);
      }
    }
  }
}

template <int J>
__global__ void __launch_bounds__(256, 2) k_spread_data(SpreadDataArgs a, const int* order) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int d = J == 2 ? 2 : 3;
  const float sc = a.fs->scale;
  const int64_t ns_tot = a.S.ns_pf * a.S.nt;
  for (int64_t i = warp; i < a.S.n; i += nwarps) {
    const int64_t n = order ? (int64_t)order[i] : i;
    const int64_t li = sample_lin(a.S, n);
    const int64_t t = frame_of(li, a.S.ns_pf);
    float dcf = 1.f;
    if (a.dcf_kind == MRSR_DCF_RADIAL_3D || a.dcf_kind == MRSR_DCF_RADIAL_2D) {
      float s2 = 0.f;
      for (int dd = 0; dd < d; ++dd) {
        const float k = a.S.trj[dd + (int64_t)d * li];
        s2 = __fadd_rn(s2, __fmul_rn(k, k));
      }
      dcf = a.dcf_kind == MRSR_DCF_RADIAL_3D ? s2 : sqrtf(s2);
    } else if (a.dcf_kind == MRSR_DCF_ARRAY) {
      dcf = a.dcf[n];
    }
    float w[J];
    unsigned cell[J];
    lane_taps<J>(a.S, a.M, li, lane, sc * dcf, w, cell);
    const int kb = a.U ? 0 : (int)t;  // U = I(nt): only coefficient t
    const int ke = a.U ? a.K : (int)t + 1;
    for (int c = 0; c < a.nc; ++c) {
      const float2 y = a.data[li + ns_tot * (a.c0 + c)];
      for (int k = kb; k < ke; ++k) {
        float2 v;
        if (!a.U) {
          v = y;
        } else if (a.u_complex) {
          v = cmulc(y, reinterpret_cast<const float2*>(a.U)[t + a.S.nt * k]);  // y * conj(U)
        } else {
          const float uu = reinterpret_cast<const float*>(a.U)[t + a.S.nt * k];
          v = make_float2(y.x * uu, y.y * uu);
        }
        long long* q = a.q + ((int64_t)c * a.K + k) * 2 * a.cells;
#pragma unroll
        for (int j = 0; j < J; ++j) {
          fx_add(q + cell[j], v.x * w[j]);
          fx_add(q + a.cells + cell[j], v.y * w[j]);
        }
      }
    }
  }
}

// 3D data spreading with a basis into a [cell][part] accumulator (the NP <= 32 parts of a
// coil batch consecutive: re and im of each coil and coefficient).  One warp per sample,
// lanes over the parts: a lane forms its part's value once, then adds its 512 terms, and
// the 32 atomics of one warp instruction land on one cell's consecutive parts (a few
// 32-byte sectors instead of one sector per lane).  Samples in 8^3-tile order.
__global__ void __launch_bounds__(256, 2) k_spread_data_cp(SpreadDataArgs a, const int* order, int NP) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const float sc = a.fs->scale;
  const int64_t ns_tot = a.S.ns_pf * a.S.nt;
  const bool live = lane < NP;
  const int ch = live ? lane >> 1 : 0, qpart = lane & 1;
  const int c = ch / a.K, k = ch - c * a.K;
  const int M0 = (int)a.M[0], M1 = (int)a.M[1], M2 = (int)a.M[2];
  for (int64_t i = warp; i < a.S.n; i += nwarps) {
    const int64_t n = order ? (int64_t)order[i] : i;
    const int64_t li = sample_lin(a.S, n);
    const int64_t t = frame_of(li, a.S.ns_pf);
    const float kd[3] = {a.S.trj[3 * li], a.S.trj[1 + 3 * li], a.S.trj[2 + 3 * li]};
    float dcf = 1.f;
    if (a.dcf_kind == MRSR_DCF_RADIAL_3D || a.dcf_kind == MRSR_DCF_RADIAL_2D) {
      float s2 = 0.f;
      for (int dd = 0; dd < 3; ++dd) s2 = __fadd_rn(s2, __fmul_rn(kd[dd], kd[dd]));
      dcf = a.dcf_kind == MRSR_DCF_RADIAL_3D ? s2 : sqrtf(s2);
    } else if (a.dcf_kind == MRSR_DCF_ARRAY) {
      dcf = a.dcf[n];
    }
    float wt;
    int64_t l0[3] = {0, 0, 0};
    es_lane_weight(kd, a.M, 3, lane, &wt, l0);
    float wx[kEsWidth], wy[kEsWidth], wz[kEsWidth];
#pragma unroll
    for (int j = 0; j < kEsWidth; ++j) {
      wx[j] = __shfl_sync(0xffffffffu, wt, j);
      wy[j] = __shfl_sync(0xffffffffu, wt, kEsWidth + j);
      wz[j] = __shfl_sync(0xffffffffu, wt, 2 * kEsWidth + j);
    }
    if (!live) continue;
    const float2 y = a.data[li + ns_tot * (a.c0 + c)];
    float2 vv;
    if (a.u_complex) {
      vv = cmulc(y, reinterpret_cast<const float2*>(a.U)[t + a.S.nt * k]);  // y * conj(U)
    } else {
      const float uu = reinterpret_cast<const float*>(a.U)[t + a.S.nt * k];
      vv = make_float2(y.x * uu, y.y * uu);
    }
    const float v = (qpart ? vv.y : vv.x) * sc * dcf;
    unsigned ix[kEsWidth];
    const int x0 = wrap32((int)l0[0], M0), y0 = wrap32((int)l0[1], M1), z0 = wrap32((int)l0[2], M2);
#pragma unroll
    for (int j = 0; j < kEsWidth; ++j) ix[j] = (unsigned)((x0 + j) % M0);
#pragma unroll 1
    for (int t3 = 0; t3 < kEsWidth; ++t3) {
      const unsigned zoff = (unsigned)((z0 + t3) % M2) * (unsigned)M1;
      const float v3 = v * wz[t3];
#pragma unroll
      for (int t2 = 0; t2 < kEsWidth; ++t2) {
        const unsigned rowc = (zoff + (unsigned)((y0 + t2) % M1)) * (unsigned)M0;
        const float w23 = v3 * wy[t2];
#pragma unroll
        for (int t1 = 0; t1 < kEsWidth; ++t1) {
          const unsigned cell = rowc + ix[t1];
          atomicAdd(reinterpret_cast<unsigned long long*>(a.q + (int64_t)cell * NP + lane),
                    (unsigned long long)fx_term(w23 * wx[t1]));
        }
      }
    }
  }
}

// [cell][NP] fixed-point accumulator -> [NP / 2][cell] float2 planes: 32 cells per block
// through a shared tile (coalesced on both sides)
__global__ void k_fixed_to_grid_cp(const long long* q, int NP, int64_t cells, const FixedScale* fs, float2* out) {
  __shared__ float tile[32][33];
  const float inv = fs->inv;
  const int64_t cell0 = (int64_t)blockIdx.x * 32;
  const int nc = cells - cell0 < 32 ? (int)(cells - cell0) : 32;
  for (int e = threadIdx.x; e < nc * NP; e += blockDim.x) {
    const int c = e / NP, p = e - c * NP;
    const long long v = q[(cell0 + c) * NP + p];
    const long long hi = (v + (1ll << 31)) >> 32;
    const int lo = (int)(v - hi * 4294967296ll);
    tile[c][p] = __fmaf_rn((float)(int)hi, 4294967296.f, (float)lo) * inv;
  }
  __syncthreads();
  const int nch = NP / 2;
  for (int e = threadIdx.x; e < nch * 32; e += blockDim.x) {
    const int chn = e >> 5, c = e & 31;
    if (c < nc) out[(int64_t)chn * cells + cell0 + c] = make_float2(tile[c][2 * chn], tile[c][2 * chn + 1]);
  }
}

// taps of one sample that can land on the same cell (the w taps wrap around a grid shorter than w)
static double taps_per_cell(int d, const int64_t* M) {
  double t = 1.0;
  for (int i = 0; i < d; ++i) t *= (double)cdiv(kEsWidth, M[i]);
  return t;
}

static unsigned spread_blocks(int64_t n) { return (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(n * 32, 256), 1), 152 * 64); }

// The w tap weights and wrapped tap indices of one sample along one dimension, in the
// arithmetic of es_lane_weight (every tap of one thread).
__device__ __forceinline__ void es_axis(float k, int M, float* w, int* idx) {
  const int hw = kEsWidth / 2;
  const float m = (float)M;
  const float uh = __fmul_rn(k, m);
  const float ul = fmaf(k, m, -uh);
  const float f = floorf(uh);
  const float r = __fadd_rn(__fsub_rn(uh, f), ul);
  const int c = r > 0.f ? 1 : 0;
  int l = ((int)f - hw + c) % M;
  if (l < 0) l += M;
#pragma unroll
  for (int t = 0; t < kEsWidth; ++t) {
    const float z = ((float)(c - hw + t) - r) * (1.f / hw);
    w[t] = (fabsf(z) < 1.f) ? expf(kEsBeta * (sqrtf(1.f - z * z) - 1.f)) : 0.f;
    idx[t] = l;
    l = l + 1 == M ? 0 : l + 1;
  }
}

// ------------------------------------------------- tile-sorted (2D) ---
//
// 2D grids are spread tile by tile.  Samples are counting-sorted by the 12 x 12 tile that
// holds their first tap; a work item is a chunk of up to kChunk samples of one tile and a
// group of P accumulator parts (a part is the real or the imaginary plane of a channel).
// A CTA sums its item into a shared-memory window of (12 + w - 1)^2 cells x P parts, then
// adds every nonzero window cell to the grid with one global 64-bit atomic, the lanes of a
// warp on consecutive cells of a window row (one coalesced flush per window row and part).
//
// Lanes own parts, not taps: a sample's value for each part is formed once, and its 64
// terms are that value times the separable tap weights, each added at a window offset
// fixed at compile time.  The terms are the fixed-point terms of the global kernels
// (|term| < 2^40) and enter the window as their two fx_split limbs, round(a) and the
// 21-bit remainder: 32-bit shared atomics run at ~5x the rate of 64-bit ones, and the
// limb sums of at most kChunk terms cannot overflow (|low sums| <= 2^30, |high sums| <
// 2^30).  The flush rebuilds each window cell's exact 64-bit sum from its limbs, so every
// grid cell is the exact integer sum of its rounded terms, whatever order the samples and
// items land in: the grids are reproducible run to run.
constexpr int kTile = 12;
constexpr int kWin = kTile + kEsWidth - 1;  // 19
constexpr int kWinCells = kWin * kWin;      // 361: odd, so the part stride is bank-conflict free
constexpr int kChunk = 1024;                // samples per work item
constexpr int kTiledThreads = 512;
static_assert(kChunk * (1ll << (kFxLoBits - 1)) < (1ll << 31), "low limb sums must fit in 31 bits");
static_assert(kChunk * (1ll << (kFxTermBits - kFxLoBits)) < (1ll << 31), "high limb sums must fit in 31 bits");

template <int P>
constexpr int tiled_smem_bytes() { return 2 * P * kWinCells * (int)sizeof(int); }

// home tile of every kept sample: the tile holding its first tap (l0 of es_lane_weight)
__global__ void k_tile_home(SampleSet S, int M0, int M1, int ntx, int* tile_of, int* counts) {
  const int hw = kEsWidth / 2;
  const int M[2] = {M0, M1};
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < S.n; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = sample_lin(S, n);
    int l0[2];
    for (int dd = 0; dd < 2; ++dd) {
      const float m = (float)M[dd];
      const float kd = S.trj[dd + 2 * li];
      const float uh = __fmul_rn(kd, m);  // the arithmetic of es_lane_weight, operation for operation
      const float ul = fmaf(kd, m, -uh);
      const float f = floorf(uh);
      const float r = __fadd_rn(__fsub_rn(uh, f), ul);
      int l = ((int)f - hw + (r > 0.f ? 1 : 0)) % M[dd];
      l0[dd] = l < 0 ? l + M[dd] : l;
    }
    const int t = l0[0] / kTile + ntx * (l0[1] / kTile);
    tile_of[n] = t;
    atomicAdd(&counts[t], 1);
  }
}

// one block: offsets of the tiles' sample lists and of their chunks, and the chunk count
__global__ void __launch_bounds__(1024) k_tile_scan(const int* counts, int ntiles, int* offset, int* choff,
                                                    int* nitems) {
  __shared__ int s_n[1024], s_c[1024];
  const int per = (ntiles + blockDim.x - 1) / blockDim.x;
  const int t0 = threadIdx.x * per, t1 = min(ntiles, t0 + per);
  int sn = 0, sc = 0;
  for (int t = t0; t < t1; ++t) {
    sn += counts[t];
    sc += (counts[t] + kChunk - 1) / kChunk;
  }
  s_n[threadIdx.x] = sn;
  s_c[threadIdx.x] = sc;
  __syncthreads();
  for (int o = 1; o < (int)blockDim.x; o <<= 1) {  // inclusive Hillis-Steele scan
    const int an = threadIdx.x >= (unsigned)o ? s_n[threadIdx.x - o] : 0;
    const int ac = threadIdx.x >= (unsigned)o ? s_c[threadIdx.x - o] : 0;
    __syncthreads();
    s_n[threadIdx.x] += an;
    s_c[threadIdx.x] += ac;
    __syncthreads();
  }
  int on = s_n[threadIdx.x] - sn, oc = s_c[threadIdx.x] - sc;
  for (int t = t0; t < t1; ++t) {
    offset[t] = on;
    choff[t] = oc;
    on += counts[t];
    oc += (counts[t] + kChunk - 1) / kChunk;
  }
  if (threadIdx.x == blockDim.x - 1) *nitems = s_c[threadIdx.x];
}

__global__ void k_tile_scatter(int64_t n, const int* tile_of, const int* offset, int* cursor, int* order) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int t = tile_of[i];
    order[offset[t] + atomicAdd(&cursor[t], 1)] = (int)i;
  }
}

__global__ void k_tile_items(const int* counts, const int* offset, const int* choff, int ntiles, int4* items) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x) {
    const int c = counts[t];
    for (int j = 0; j * kChunk < c; ++j)
      items[choff[t] + j] = make_int4(t, offset[t] + j * kChunk, min(kChunk, c - j * kChunk), 0);
  }
}

// Per-sample tap record of the tile-sorted kernels, in sorted order: the separable weights
// (the density compensation folded into wy), the wrapped first tap, the linear sample index
// and its frame.  Formed once per sample set, read by every part group (a broadcast load
// per sample instead of the weights, shuffles and index arithmetic per group).
struct __align__(16) TapRec {
  float wx[kEsWidth], wy[kEsWidth];
  int li, t, lx0, ly0;
};

__global__ void k_tile_prep(SampleSet S, int M0, int M1, const int* order, int dcf_kind, const float* dcf,
                            TapRec* rec) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < S.n; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = order[s];
    const int64_t li = sample_lin(S, n);
    const float k0 = S.trj[2 * li], k1 = S.trj[2 * li + 1];
    TapRec r;
    int ix[kEsWidth], iy[kEsWidth];
    es_axis(k0, M0, r.wx, ix);
    es_axis(k1, M1, r.wy, iy);
    float w = 1.f;
    if (dcf_kind == MRSR_DCF_RADIAL_3D || dcf_kind == MRSR_DCF_RADIAL_2D) {
      const float s2 = __fadd_rn(__fmul_rn(k0, k0), __fmul_rn(k1, k1));
      w = dcf_kind == MRSR_DCF_RADIAL_3D ? s2 : sqrtf(s2);
    } else if (dcf_kind == MRSR_DCF_ARRAY) {
      w = dcf[n];
    }
#pragma unroll
    for (int j = 0; j < kEsWidth; ++j) r.wy[j] *= w;
    r.li = (int)li;
    r.t = (int)frame_of(li, S.ns_pf);
    r.lx0 = ix[0];
    r.ly0 = iy[0];
    rec[s] = r;
  }
}

int TileSort::prep(const SampleSet& S, int dcf_kind, const float* dcf, cudaStream_t st) {
  MRSR_REQUIRE(S.ns_pf * S.nt < (1ll << 31), MRSR_ERR_UNSUPPORTED, "tile records: < 2^31 samples per set");
  MRSR_TRY(rec.alloc(sizeof(TapRec) * std::max<int64_t>(S.n, 1)));
  const unsigned gb = (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(S.n, 256), 1), 152 * 16);
  k_tile_prep<<<gb, 256, 0, st>>>(S, m0, m1, order.as<int>(), dcf_kind, dcf, rec.as<TapRec>());
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int TileSort::build(const SampleSet& S, int64_t M0, int64_t M1, cudaStream_t st) {
  MRSR_REQUIRE(S.d == 2 && S.n < (1ll << 31) && M0 < (1ll << 24) && M1 < (1ll << 24), MRSR_ERR_UNSUPPORTED,
               "tile-sorted spreading: 2D, < 2^31 samples, grid < 2^24 per dimension");
  ntx = (int)cdiv(M0, kTile);
  ntiles = ntx * (int)cdiv(M1, kTile);
  m0 = (int)M0;
  m1 = (int)M1;
  const int64_t maxitems = ntiles + cdiv(S.n, kChunk);
  MRSR_TRY(counts.alloc(sizeof(int) * ntiles));
  MRSR_TRY(offset.alloc(sizeof(int) * ntiles));
  MRSR_TRY(choff.alloc(sizeof(int) * ntiles));
  MRSR_TRY(cursor.alloc(sizeof(int) * ntiles));
  MRSR_TRY(tile_of.alloc(sizeof(int) * std::max<int64_t>(S.n, 1)));
  MRSR_TRY(order.alloc(sizeof(int) * std::max<int64_t>(S.n, 1)));
  MRSR_TRY(items.alloc(sizeof(int4) * maxitems));
  MRSR_TRY(nitems.alloc(sizeof(int)));
  MRSR_TRY(next.alloc(sizeof(int)));
  MRSR_CHECK_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(int) * ntiles, st));
  MRSR_CHECK_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int) * ntiles, st));
  const unsigned gb = (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(S.n, 256), 1), 152 * 16);
  k_tile_home<<<gb, 256, 0, st>>>(S, m0, m1, ntx, tile_of.as<int>(), counts.as<int>());
  MRSR_LAUNCH_CHECK();
  k_tile_scan<<<1, 1024, 0, st>>>(counts.as<int>(), ntiles, offset.as<int>(), choff.as<int>(), nitems.as<int>());
  MRSR_LAUNCH_CHECK();
  k_tile_scatter<<<gb, 256, 0, st>>>(S.n, tile_of.as<int>(), offset.as<int>(), cursor.as<int>(), order.as<int>());
  MRSR_LAUNCH_CHECK();
  const unsigned gt = (unsigned)std::max<int64_t>(cdiv(ntiles, 256), 1);
  k_tile_items<<<gt, 256, 0, st>>>(counts.as<int>(), offset.as<int>(), choff.as<int>(), ntiles, items.as<int4>());
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

constexpr int kTile3 = 8;

// 3D home tile (kTile3^3) of every kept sample's first tap
__global__ void k_tile_home3(SampleSet S, int M0, int M1, int M2, int* tile_of, int* counts) {
  const int hw = kEsWidth / 2;
  const int M[3] = {M0, M1, M2};
  const int ntx = (M0 + kTile3 - 1) / kTile3, nty = (M1 + kTile3 - 1) / kTile3;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < S.n; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = sample_lin(S, n);
    int l0[3];
    for (int dd = 0; dd < 3; ++dd) {
      const float m = (float)M[dd];
      const float kd = S.trj[dd + 3 * li];
      const float uh = __fmul_rn(kd, m);
      const float ul = fmaf(kd, m, -uh);
      const float f = floorf(uh);
      const float r = __fadd_rn(__fsub_rn(uh, f), ul);
      int l = ((int)f - hw + (r > 0.f ? 1 : 0)) % M[dd];
      l0[dd] = l < 0 ? l + M[dd] : l;
    }
    const int t = l0[0] / kTile3 + ntx * (l0[1] / kTile3 + nty * (l0[2] / kTile3));
    tile_of[n] = t;
    atomicAdd(&counts[t], 1);
  }
}

int TileSort::build3(const SampleSet& S, const int64_t* M, cudaStream_t st) {
  MRSR_REQUIRE(S.d == 3 && S.n < (1ll << 31), MRSR_ERR_UNSUPPORTED, "sample order: 3D, < 2^31 samples");
  const int64_t nt3 = cdiv(M[0], kTile3) * cdiv(M[1], kTile3) * cdiv(M[2], kTile3);
  MRSR_REQUIRE(nt3 < (1ll << 31), MRSR_ERR_UNSUPPORTED, "sample order: too many tiles");
  ntiles = (int)nt3;
  MRSR_TRY(counts.alloc(sizeof(int) * ntiles));
  MRSR_TRY(offset.alloc(sizeof(int) * ntiles));
  MRSR_TRY(choff.alloc(sizeof(int) * ntiles));
  MRSR_TRY(cursor.alloc(sizeof(int) * ntiles));
  MRSR_TRY(tile_of.alloc(sizeof(int) * std::max<int64_t>(S.n, 1)));
  MRSR_TRY(order.alloc(sizeof(int) * std::max<int64_t>(S.n, 1)));
  MRSR_TRY(nitems.alloc(sizeof(int)));
  MRSR_CHECK_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(int) * ntiles, st));
  MRSR_CHECK_CUDA(cudaMemsetAsync(cursor.p, 0, sizeof(int) * ntiles, st));
  const unsigned gb = (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(S.n, 256), 1), 152 * 16);
  k_tile_home3<<<gb, 256, 0, st>>>(S, (int)M[0], (int)M[1], (int)M[2], tile_of.as<int>(), counts.as<int>());
  MRSR_LAUNCH_CHECK();
  k_tile_scan<<<1, 1024, 0, st>>>(counts.as<int>(), ntiles, offset.as<int>(), choff.as<int>(), nitems.as<int>());
  MRSR_LAUNCH_CHECK();
  k_tile_scatter<<<gb, 256, 0, st>>>(S.n, tile_of.as<int>(), offset.as<int>(), cursor.as<int>(), order.as<int>());
  MRSR_LAUNCH_CHECK();
  // work items of the 3D tile-sorted kernel: chunks of at most kChunk samples of one tile
  m0 = (int)M[0];
  m1 = (int)M[1];
  m2 = (int)M[2];
  ntx = (int)cdiv(M[0], kTile3);
  nty = (int)cdiv(M[1], kTile3);
  const int64_t maxitems = ntiles + cdiv(S.n, kChunk);
  MRSR_TRY(items.alloc(sizeof(int4) * maxitems));
  MRSR_TRY(next.alloc(sizeof(int)));
  const unsigned gt = (unsigned)std::max<int64_t>(cdiv(ntiles, 256), 1);
  k_tile_items<<<gt, 256, 0, st>>>(counts.as<int>(), offset.as<int>(), choff.as<int>(), ntiles, items.as<int4>());
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// 3D tap record: weights along x, y, z (the density compensation folded into wz), the
// wrapped first tap, the linear sample index and its frame, in sorted order.
struct __align__(16) TapRec3 {
  float wx[kEsWidth], wy[kEsWidth], wz[kEsWidth];
  int li, t, lx0, ly0, lz0, pad0, pad1, pad2;
};
static_assert(sizeof(TapRec3) == 128, "TapRec3 is eight 16-byte loads");

__global__ void k_tile_prep3(SampleSet S, int M0, int M1, int M2, const int* order, int dcf_kind, const float* dcf,
                             TapRec3* rec) {
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < S.n; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = order[s];
    const int64_t li = sample_lin(S, n);
    const float k0 = S.trj[3 * li], k1 = S.trj[3 * li + 1], k2 = S.trj[3 * li + 2];
    TapRec3 r;
    int ix[kEsWidth], iy[kEsWidth], iz[kEsWidth];
    es_axis(k0, M0, r.wx, ix);
    es_axis(k1, M1, r.wy, iy);
    es_axis(k2, M2, r.wz, iz);
    float w = 1.f;
    if (dcf_kind == MRSR_DCF_RADIAL_3D || dcf_kind == MRSR_DCF_RADIAL_2D) {
      const float s2 = __fadd_rn(__fadd_rn(__fmul_rn(k0, k0), __fmul_rn(k1, k1)), __fmul_rn(k2, k2));
      w = dcf_kind == MRSR_DCF_RADIAL_3D ? s2 : sqrtf(s2);
    } else if (dcf_kind == MRSR_DCF_ARRAY) {
      w = dcf[n];
    }
#pragma unroll
    for (int j = 0; j < kEsWidth; ++j) r.wz[j] *= w;
    r.li = (int)li;
    r.t = (int)frame_of(li, S.ns_pf);
    r.lx0 = ix[0];
    r.ly0 = iy[0];
    r.lz0 = iz[0];
    r.pad0 = r.pad1 = r.pad2 = 0;
    rec[s] = r;
  }
}

int TileSort::prep3(const SampleSet& S, int dcf_kind, const float* dcf, cudaStream_t st) {
  MRSR_REQUIRE(S.ns_pf * S.nt < (1ll << 31), MRSR_ERR_UNSUPPORTED, "tile records: < 2^31 samples per set");
  MRSR_TRY(rec.alloc(sizeof(TapRec3) * std::max<int64_t>(S.n, 1)));
  const unsigned gb = (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(S.n, 256), 1), 152 * 16);
  k_tile_prep3<<<gb, 256, 0, st>>>(S, m0, m1, m2, order.as<int>(), dcf_kind, dcf, rec.as<TapRec3>());
  MRSR_LAUNCH_CHECK();
  rec3 = true;
  return MRSR_OK;
}

struct TiledArgs {
  SampleSet S;
  int M0, M1;
  int64_t cells;
  int nparts;              // parts to spread (grid planes)
  long long* q;            // [nparts][cells]
  const FixedScale* fs;
  int ntx;
  const TapRec* rec;       // per-sample tap records in sorted order
  const int4* items;       // (tile, first sorted position, count, -)
  const int* nitems;
  int* next;               // work counter, zeroed before the launch
};

// Part p of the Λ precompute: pair p0 + p / nq (k1 <= k2, packed k2 (k2 + 1) / 2 + k1), plane
// p % nq; value conj(U[t,k1]) U[t,k2] 2^e (k_spread_lambda's value).
struct LamParts {
  const void* U;
  int u_complex, nq, p0;
  int64_t nt, ns_pf;
  struct Lane {
    int k1, k2, q;
  };
  __device__ Lane bind(int part) const {
    const int ch = part / nq, q = part - ch * nq, p = p0 + ch;
    int k2 = 0;
    while ((k2 + 1) * (k2 + 2) / 2 <= p) ++k2;
    return Lane{p - k2 * (k2 + 1) / 2, k2, q};
  }
  __device__ float value(const Lane& L, int64_t, int64_t t) const {
    if (u_complex) {
      const float2* u = reinterpret_cast<const float2*>(U);
      const float2 v = cmulc(u[t + nt * L.k2], u[t + nt * L.k1]);  // conj(U[t,k1]) * U[t,k2]
      return L.q ? v.y : v.x;
    }
    const float* u = reinterpret_cast<const float*>(U);
    return u[t + nt * L.k2] * u[t + nt * L.k1];
  }
};

// Part p of the backprojection: channel p / 2 = (coil c0 + c) K + k, plane p % 2; value
// y_c conj(U[t,k]) dcf (k_spread_data's value).
struct DataParts {
  const float2* data;
  const void* U;
  int u_complex, K, c0, dcf_kind;
  const float* dcf;
  int64_t nt, ns_pf, ns_tot;
  struct Lane {
    int c, k, q;
  };
  __device__ Lane bind(int part) const {
    const int ch = part >> 1, c = ch / K;
    return Lane{c, ch - c * K, part & 1};
  }
  __device__ float value(const Lane& L, int64_t li, int64_t t) const {
    const float2 y = data[li + ns_tot * (c0 + L.c)];
    float2 v;
    if (u_complex) {
      v = cmulc(y, reinterpret_cast<const float2*>(U)[t + nt * L.k]);  // y * conj(U)
    } else {
      const float uu = reinterpret_cast<const float*>(U)[t + nt * L.k];
      v = make_float2(y.x * uu, y.y * uu);
    }
    return L.q ? v.y : v.x;
  }
};


__device__ __noinline__ void spread_direct(long long* g, int M0, int M1, int lx0, int ly0, float v, const float* wx,
                                           const float* wy) {
  for (int t2 = 0; t2 < kEsWidth; ++t2) {
    const int64_t row = (int64_t)M0 * wrap32(ly0 + t2, M1);
    for (int t1 = 0; t1 < kEsWidth; ++t1)
      atomicAdd(reinterpret_cast<unsigned long long*>(g + row + wrap32(lx0 + t1, M0)),
                (unsigned long long)fx_term(v * wy[t2] * wx[t1]));
  }
}

// Items are taken group-major (all tiles of part group 0, then group 1, ...) from a device
// counter, so the CTAs in flight work on neighbouring tiles of one group and their flushes
// share L2 lines.
template <int P, class Parts>
__global__ void __launch_bounds__(kTiledThreads, 2) k_spread_tiled(TiledArgs a, Parts parts) {
  extern __shared__ __align__(16) int win[];  // [2][P][kWinCells]: low limbs, then high limbs
  int* wlo = win;
  int* whi = win + P * kWinCells;
  __shared__ int s_item;
  constexpr int SPW = 32 / P;  // samples per warp step
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int slot = lane / P, part = lane % P;
  const int nitems = *a.nitems;
  const int ngroups = (a.nparts + P - 1) / P;
  const int total = nitems * ngroups;
  const float sc = a.fs->scale;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.next, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= total) break;
    const int grp = it / nitems;
    const int4 item = a.items[it - grp * nitems];
    const int gpart = grp * P + part;
    const bool live_part = gpart < a.nparts;
    const typename Parts::Lane L = parts.bind(live_part ? gpart : 0);
    const int ox = (item.x % a.ntx) * kTile, oy = (item.x / a.ntx) * kTile;
    int4* w4 = reinterpret_cast<int4*>(win);
    for (int i = threadIdx.x; i < P * kWinCells / 2; i += blockDim.x) w4[i] = make_int4(0, 0, 0, 0);
    __syncthreads();
    for (int s0 = warp * SPW; s0 < item.z; s0 += nwarps * SPW) {
      if (s0 + slot >= item.z || !live_part) continue;
      const float4* r4 = reinterpret_cast<const float4*>(a.rec + item.y + s0 + slot);
      float wx[kEsWidth], wy[kEsWidth];
      {
        const float4 q0 = r4[0], q1 = r4[1], q2 = r4[2], q3 = r4[3];
        wx[0] = q0.x; wx[1] = q0.y; wx[2] = q0.z; wx[3] = q0.w;
        wx[4] = q1.x; wx[5] = q1.y; wx[6] = q1.z; wx[7] = q1.w;
        wy[0] = q2.x; wy[1] = q2.y; wy[2] = q2.z; wy[3] = q2.w;
        wy[4] = q3.x; wy[5] = q3.y; wy[6] = q3.z; wy[7] = q3.w;
      }
      const int4 ri = reinterpret_cast<const int4*>(r4)[4];  // li, t, lx0, ly0
      const float v = parts.value(L, ri.x, ri.y) * sc;
      const int lx0 = ri.z, ly0 = ri.w;
      const int lx = lx0 - ox, ly = ly0 - oy;
      if ((unsigned)lx < (unsigned)kTile && (unsigned)ly < (unsigned)kTile) {
        int* pl = wlo + part * kWinCells + ly * kWin + lx;
        int* ph = whi + part * kWinCells + ly * kWin + lx;
#pragma unroll
        for (int t2 = 0; t2 < kEsWidth; ++t2) {
          const float vy = v * wy[t2];
#pragma unroll
          for (int t1 = 0; t1 < kEsWidth; ++t1) {
            int hi, lo;
            fx_split_prod(vy, wx[t1], hi, lo);
            atomicAdd(pl + t2 * kWin + t1, lo);
            atomicAdd(ph + t2 * kWin + t1, hi);
          }
        }
      } else {
        // the sort put the first tap in this tile (the same float arithmetic); a sample
        // outside it would go straight to the grid rather than out of the window
        spread_direct(a.q + (int64_t)gpart * a.cells, a.M0, a.M1, lx0, ly0, v, wx, wy);
      }
    }
    __syncthreads();
    const int gx = wrap32(ox + lane, a.M0);
    for (int task = warp; task < P * kWin; task += nwarps) {
      const int p = task / kWin, row = task - p * kWin;
      const int gp = grp * P + p;
      if (gp >= a.nparts || lane >= kWin) continue;
      const int c = p * kWinCells + row * kWin + lane;
      const long long v = (long long)whi[c] * (1ll << kFxLoBits) + (long long)wlo[c];
      if (v != 0)
        atomicAdd(reinterpret_cast<unsigned long long*>(a.q + (int64_t)gp * a.cells + gx +
                                                        (int64_t)a.M0 * wrap32(oy + row, a.M1)),
                  (unsigned long long)v);
    }
    __syncthreads();
  }
}

template <int P, class Parts>
static int launch_tiled(const TiledArgs& a, const Parts& parts, cudaStream_t st) {
  constexpr int smem = tiled_smem_bytes<P>();
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_spread_tiled<P, Parts>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  MRSR_CHECK_CUDA(cudaMemsetAsync(a.next, 0, sizeof(int), st));
  k_spread_tiled<P, Parts><<<152 * 2, kTiledThreads, smem, st>>>(a, parts);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

template <class Parts>
static int spread_tiled(const SampleSet& S, const int64_t* M, int64_t cells, int nparts, long long* q,
                        const FixedScale* fs, const TileSort& ts, const Parts& parts, cudaStream_t st) {
  MRSR_REQUIRE(ts.m0 == (int)M[0] && ts.m1 == (int)M[1], MRSR_ERR_STATE, "tile sort built for another grid");
  MRSR_REQUIRE(ts.rec.p != nullptr, MRSR_ERR_STATE, "tile sort without tap records");
  const TiledArgs a{S, ts.m0, ts.m1, cells, nparts, q, fs, ts.ntx,
                    ts.rec.as<TapRec>(), ts.items.as<int4>(), ts.nitems.as<int>(), ts.next.as<int>()};
  return nparts <= 16 ? launch_tiled<16>(a, parts, st) : launch_tiled<32>(a, parts, st);
}

// ------------------------------------------------- tile-sorted (3D) ---
//
// The 2D scheme in three dimensions: samples in 8^3 tiles (home tile of the first tap), work
// items of at most kChunk samples of one tile x a group of kP3 = 4 parts, a window of
// (8 + w - 1)^3 = 15^3 cells x 4 parts of 32-bit limbs in shared memory (106 KB: two CTAs
// per SM), and one global 64-bit atomic per nonzero window cell at the flush, a warp on
// consecutive cells.  A warp takes one sample at a time: lane = 8 part + t1 (part < 4, x tap
// t1 < 8), so a warp instruction adds 8 consecutive cells of 4 parts, and the part stride
// (3384 = 24 mod 32 words) puts the four 8-cell runs in disjoint bank ranges: no bank
// conflicts.  With 64-bit global atomics capped near 0.73 T/s on this GPU, every term as a
// global atomic (the one-warp-per-sample kernels) spends ~0.55 s on the 401 G terms of a
// 128^3, 4.9 M-sample, 16-coil backprojection.
constexpr int kWin3 = kTile3 + kEsWidth - 1;           // 15
constexpr int kWin3Cells = kWin3 * kWin3 * kWin3;      // 3375
constexpr int kWin3Stride = 3384;                      // part stride, = 24 (mod 32)
constexpr int kP3 = 4;
constexpr int kTiled3Smem = 2 * kP3 * kWin3Stride * (int)sizeof(int);
static_assert(kWin3Stride >= kWin3Cells && kWin3Stride % 32 == 24 && kWin3Stride % 4 == 0, "3D window stride");

struct TiledArgs3 {
  SampleSet S;
  int M0, M1, M2;
  int64_t cells;
  int nparts;
  long long* q;            // [nparts][cells]
  const FixedScale* fs;
  int ntx, nty;
  const TapRec3* rec;
  const int4* items;
  const int* nitems;
  int* next;
};

template <class Parts>
__global__ void __launch_bounds__(kTiledThreads, 2) k_spread_tiled3(TiledArgs3 a, Parts parts) {
  extern __shared__ __align__(16) int win3[];  // [2][kP3][kWin3Stride]
  int* wlo = win3;
  int* whi = win3 + kP3 * kWin3Stride;
  __shared__ int s_item;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int part = lane >> 3, t1 = lane & 7;
  const int nitems = *a.nitems;
  const int ngroups = (a.nparts + kP3 - 1) / kP3;
  const int total = nitems * ngroups;
  const float sc = a.fs->scale;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.next, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= total) break;
    const int grp = it / nitems;
    const int4 item = a.items[it - grp * nitems];
    const int gpart = grp * kP3 + part;
    const bool live_part = gpart < a.nparts;
    const typename Parts::Lane L = parts.bind(live_part ? gpart : 0);
    const int tx = item.x % a.ntx, tyz = item.x / a.ntx;
    const int ox = tx * kTile3, oy = (tyz % a.nty) * kTile3, oz = (tyz / a.nty) * kTile3;
    int4* w4 = reinterpret_cast<int4*>(win3);
    for (int i = threadIdx.x; i < 2 * kP3 * kWin3Stride / 4; i += blockDim.x) w4[i] = make_int4(0, 0, 0, 0);
    __syncthreads();
    if (live_part) {
      for (int smp = warp; smp < item.z; smp += nwarps) {
        const float4* r4 = reinterpret_cast<const float4*>(a.rec + item.y + smp);
        float wy[kEsWidth], wz[kEsWidth];
        {
          const float4 q2 = r4[2], q3 = r4[3], q4 = r4[4], q5 = r4[5];
          wy[0] = q2.x; wy[1] = q2.y; wy[2] = q2.z; wy[3] = q2.w;
          wy[4] = q3.x; wy[5] = q3.y; wy[6] = q3.z; wy[7] = q3.w;
          wz[0] = q4.x; wz[1] = q4.y; wz[2] = q4.z; wz[3] = q4.w;
          wz[4] = q5.x; wz[5] = q5.y; wz[6] = q5.z; wz[7] = q5.w;
        }
        const float wx1 = reinterpret_cast<const float*>(r4)[t1];
        const int4 ri = reinterpret_cast<const int4*>(r4)[6];  // li, t, lx0, ly0
        const int lz0 = reinterpret_cast<const int*>(r4)[28];
        const float v = parts.value(L, ri.x, ri.y) * sc * wx1;
        const int lx = ri.z - ox, ly = ri.w - oy, lz = lz0 - oz;
        if ((unsigned)lx < (unsigned)kTile3 && (unsigned)ly < (unsigned)kTile3 && (unsigned)lz < (unsigned)kTile3) {
          const int base = part * kWin3Stride + (lz * kWin3 + ly) * kWin3 + lx + t1;
          int* pl = wlo + base;
          int* ph = whi + base;
#pragma unroll
          for (int t3 = 0; t3 < kEsWidth; ++t3) {
            const float v3 = v * wz[t3];
#pragma unroll
            for (int t2 = 0; t2 < kEsWidth; ++t2) {
              int hi, lo;
              fx_split_prod(v3, wy[t2], hi, lo);
              atomicAdd(pl + (t3 * kWin3 + t2) * kWin3, lo);
              atomicAdd(ph + (t3 * kWin3 + t2) * kWin3, hi);
            }
          }
        } else {
          // the sort put the first tap in this tile (the same float arithmetic); a sample
          // outside it goes straight to the grid rather than out of the window
          long long* g = a.q + (int64_t)gpart * a.cells;
          const int64_t x = wrap32(ri.z + t1, a.M0);
          for (int t3 = 0; t3 < kEsWidth; ++t3)
            for (int t2 = 0; t2 < kEsWidth; ++t2) {
              const int64_t row = (int64_t)a.M0 * (wrap32(ri.w + t2, a.M1) + (int64_t)a.M1 * wrap32(lz0 + t3, a.M2));
              atomicAdd(reinterpret_cast<unsigned long long*>(g + row + x),
                        (unsigned long long)fx_term(v * wz[t3] * wy[t2]));
            }
        }
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kP3 * kWin3Cells; e += blockDim.x) {
      const int p = e / kWin3Cells, c = e - p * kWin3Cells;
      const int gp = grp * kP3 + p;
      if (gp >= a.nparts) continue;
      const int w = p * kWin3Stride + c;
      const long long v = (long long)whi[w] * (1ll << kFxLoBits) + (long long)wlo[w];
      if (v == 0) continue;
      const int cx = c % kWin3, cyz = c / kWin3;
      const int cy = cyz % kWin3, cz = cyz / kWin3;
      const int64_t cell = wrap32(ox + cx, a.M0) +
                           (int64_t)a.M0 * (wrap32(oy + cy, a.M1) + (int64_t)a.M1 * wrap32(oz + cz, a.M2));
      atomicAdd(reinterpret_cast<unsigned long long*>(a.q + (int64_t)gp * a.cells + cell), (unsigned long long)v);
    }
    __syncthreads();
  }
}

template <class Parts>
static int spread_tiled3(const SampleSet& S, const int64_t* M, int64_t cells, int nparts, long long* q,
                         const FixedScale* fs, const TileSort& ts, const Parts& parts, cudaStream_t st) {
  MRSR_REQUIRE(ts.rec3 && ts.m0 == (int)M[0] && ts.m1 == (int)M[1] && ts.m2 == (int)M[2], MRSR_ERR_STATE,
               "3D tile sort built for another grid or without tap records");
  const TiledArgs3 a{S, ts.m0, ts.m1, ts.m2, cells, nparts, q, fs, ts.ntx, ts.nty,
                     ts.rec.as<TapRec3>(), ts.items.as<int4>(), ts.nitems.as<int>(), ts.next.as<int>()};
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_spread_tiled3<Parts>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       kTiled3Smem));
  MRSR_CHECK_CUDA(cudaMemsetAsync(a.next, 0, sizeof(int), st));
  k_spread_tiled3<Parts><<<152 * 2, kTiledThreads, kTiled3Smem, st>>>(a, parts);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int spread_lambda(const SpreadLambdaArgs& a, const TileSort* ts, cudaStream_t st) {
  if (a.S.n == 0) return MRSR_OK;
  if (ts && a.S.d == 2) {
    const LamParts parts{a.U, a.u_complex, a.nq, a.p0, a.S.nt, a.S.ns_pf};
    return spread_tiled(a.S, a.M, a.cells, a.np * a.nq, a.q, a.fs, *ts, parts, st);
  }
  if (ts && a.S.d == 3 && ts->rec3) {
    const LamParts parts{a.U, a.u_complex, a.nq, a.p0, a.S.nt, a.S.ns_pf};
    return spread_tiled3(a.S, a.M, a.cells, a.np * a.nq, a.q, a.fs, *ts, parts, st);
  }
  MRSR_REQUIRE(a.cells < (1ll << 32), MRSR_ERR_UNSUPPORTED, "spreading grid of 2^32 cells or more");
  const int* order = ts ? ts->order.as<int>() : nullptr;
  if (a.S.d == 2)
    k_spread_lambda<2><<<spread_blocks(a.S.n), 256, 0, st>>>(a, order);
  else
    k_spread_lambda<16><<<spread_blocks(a.S.n), 256, 0, st>>>(a, order);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int spread_data(const SpreadDataArgs& a, const TileSort* ts, cudaStream_t st) {
  if (a.S.n == 0) return MRSR_OK;
  if (ts && a.U && (a.S.d == 2 || ts->rec3)) {
    const DataParts parts{a.data, a.U, a.u_complex, a.K, a.c0, a.dcf_kind, a.dcf,
                          a.S.nt, a.S.ns_pf, a.S.ns_pf * a.S.nt};
    if (a.S.d == 2) return spread_tiled(a.S, a.M, a.cells, 2 * a.nc * a.K, a.q, a.fs, *ts, parts, st);
    return spread_tiled3(a.S, a.M, a.cells, 2 * a.nc * a.K, a.q, a.fs, *ts, parts, st);
  }
  MRSR_REQUIRE(a.cells < (1ll << 32), MRSR_ERR_UNSUPPORTED, "spreading grid of 2^32 cells or more");
  const int* order = ts && a.S.d == 3 ? ts->order.as<int>() : nullptr;
  if (a.S.d == 3 && a.U && 2 * a.nc * a.K <= 32) {  // [cell][part] accumulator (the 3D backprojection)
    k_spread_data_cp<<<spread_blocks(a.S.n), 256, 0, st>>>(a, order, 2 * a.nc * a.K);
    MRSR_LAUNCH_CHECK();
    return MRSR_OK;
  }
  if (a.S.d == 2)
    k_spread_data<2><<<spread_blocks(a.S.n), 256, 0, st>>>(a, order);
  else
    k_spread_data<16><<<spread_blocks(a.S.n), 256, 0, st>>>(a, order);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// ------------------------------------------------------- fixed point ---

// amax[slot] = max |f[i]| as float bits (non-negative floats order like their bit patterns)
__global__ void k_absmax(const float* f, int64_t n, unsigned* amax) {
  float m = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(f[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(amax, __float_as_uint(m));
}

// e = min(62 - ceil(log2(nterms * bound)), 40 - ceil(log2(bound))), bound = mult * prod
// amax; e clamped so that 2^(e - 21) and 2^-e are normal floats
__global__ void k_fixed_scale(const unsigned* amax, int nf, double mult, double nterms, FixedScale* out) {
  double bound = mult;
  for (int i = 0; i < nf; ++i) bound *= (double)__uint_as_float(amax[i]);
  int e = 0;
  if (bound > 0.0) e = min(62 - (int)ceil(log2(nterms * bound)), kFxTermBits - (int)ceil(log2(bound)));
  e = max(-100, min(120, e));
  out->scale = ldexpf(1.f, e - kFxLoBits);
  out->inv = ldexpf(1.f, -e);
}

int fixed_scale(const float* const* f, const int64_t* n, int nf, double mult, double nterms, FixedScale* out,
                cudaStream_t st) {
  MRSR_REQUIRE(nf >= 0 && nf <= 3, MRSR_ERR_ARG, "fixed_scale: at most 3 factors");
  DevBuf am;
  MRSR_TRY(am.alloc(4 * sizeof(unsigned)));
  MRSR_CHECK_CUDA(cudaMemsetAsync(am.p, 0, 4 * sizeof(unsigned), st));
  for (int i = 0; i < nf; ++i) {
    const unsigned g = (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(n[i], 1024), 1), 152 * 8);
    k_absmax<<<g, 256, 0, st>>>(f[i], n[i], am.as<unsigned>() + i);
    MRSR_LAUNCH_CHECK();
  }
  k_fixed_scale<<<1, 1, 0, st>>>(am.as<unsigned>(), nf, mult, nterms, out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// int64 -> float32 without the float64 pipe: v = hi * 2^32 + lo with lo in [-2^31, 2^31)
// (so a small negative v is lo alone, with no cancellation), each half converted in float32
// and joined by one fma (within ~2 float32 roundings of v), then scaled by 2^-e
__global__ void k_fixed_to_grid(const long long* q, int nq, int64_t cells, int64_t total, const FixedScale* fs,
                                float2* out) {
  const float inv = fs->inv;
  auto cvt = [inv](long long v) {
    const long long hi = (v + (1ll << 31)) >> 32;
    const int lo = (int)(v - hi * 4294967296ll);
    return __fmaf_rn((float)(int)hi, 4294967296.f, (float)lo) * inv;
  };
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ch = e / cells, cell = e - ch * cells;
    const long long* qc = q + ch * nq * cells + cell;
    out[e] = make_float2(cvt(qc[0]), nq == 2 ? cvt(qc[cells]) : 0.f);
  }
}

int fixed_to_grid(const long long* q, int nq, int64_t cells, int64_t nch, const FixedScale* fs, float2* out,
                  cudaStream_t st) {
  const int64_t total = cells * nch;
  const unsigned g = (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(total, 256), 1), 152 * 32);
  k_fixed_to_grid<<<g, 256, 0, st>>>(q, nq, cells, total, fs, out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

// ----------------------------------------------------------- kmask ---

// Gaussian-footprint mask: cells i0-3 .. i0+4 (mod G) per dimension around
// i0 = floor(fl32(-k * G)) for every kept sample (src/NFFTNormalOp.jl:106-118).  The union
// of the boxes is the seed set {i0} dilated by the box: cell j is marked iff some seed lies
// in j-4 .. j+3 along every dimension.  One byte store per sample marks the seeds, then one
// pass per dimension ORs each cell's 8 neighbours along it (separable, exact for boolean
// masks), instead of 8^d scattered byte stores per sample.
__global__ void k_kmask_seed(SampleSet S, int64_t G0, int64_t G1, int64_t G2, uint8_t* seeds) {
  const int d = S.d;
  const int G[3] = {(int)G0, (int)G1, (int)G2};
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < S.n; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = sample_lin(S, n);
    int64_t cell = 0, stride = 1;
    for (int dd = 0; dd < d; ++dd) {
      const float p = __fmul_rn(-S.trj[dd + (int64_t)d * li], (float)G[dd]);
      int l = (int)floorf(p) % G[dd];
      if (l < 0) l += G[dd];
      cell += (int64_t)l * stride;
      stride *= G[dd];
    }
    seeds[cell] = 1;
  }
}

// out[j] = OR of in[j + s], s = -4 .. 3 (mod G) along dimension `axis`
__global__ void k_kmask_dilate(const uint8_t* in, int64_t G0, int64_t G1, int64_t G2, int axis, uint8_t* out) {
  const int64_t total = G0 * G1 * G2;
  const int64_t stride = axis == 0 ? 1 : (axis == 1 ? G0 : G0 * G1);
  const int64_t Ga = axis == 0 ? G0 : (axis == 1 ? G1 : G2);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < total; c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = (c / stride) % Ga;
    const int64_t base = c - j * stride;
    uint8_t v = 0;
#pragma unroll
    for (int s = -4; s <= 3; ++s) {
      int64_t k = (j + s) % Ga;
      if (k < 0) k += Ga;
      v |= in[base + k * stride];
    }
    out[c] = v ? 1 : 0;
  }
}

// ----------------------------------------------------- Λ precompute ---

struct FoldArgs {
  int d;
  int64_t G[3], M[3];
  int64_t gcells, mcells;
  int P;
  int real_u;
  Decomp dc;              // element -> (p, cell position) over (G0, G1, G2) x P
  const float2* g;        // [P][mcells] after the inverse DFT
  const float* ipsi[3];   // 1/psi_hat(j) for j = -G/2 .. G/2
  float2* c;              // [P][gcells]
};

// c~[p] for the Toeplitz kernel: complex basis uses j in [-G/2, G/2) (FFT
// order, src/NFFTNormalOp.jl:142-158); a real basis follows the real-input
// transform + brfft of :197-214: along dim 1 only j1 in [0, G1/2] is used,
// interior terms doubled, and Λ = Re(FFT(c~)).
__global__ void k_lambda_fold(FoldArgs a) {
  const int64_t total = a.gcells * a.P;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t pd[3] = {0, 0, 0};
    const int p = a.dc.split(e, pd);
    float scale = 1.f;
    int64_t l = 0, mul = 1;
    bool zero = false;
    for (int dd = 0; dd < a.d; ++dd) {
      const int64_t Gd = a.G[dd], half = Gd / 2;
      int64_t j;
      if (a.real_u && dd == 0) {
        if (pd[0] > half) {
          zero = true;
          j = 0;
        } else {
          j = pd[0];
          if (j != 0 && j != half) scale *= 2.f;
        }
      } else {
        j = pd[dd] < half ? pd[dd] : pd[dd] - Gd;
      }
      scale *= a.ipsi[dd][j + half];
      l += wrap_near(j, a.M[dd]) * mul;
      mul *= a.M[dd];
    }
    float2 v = zero ? make_float2(0.f, 0.f) : a.g[(int64_t)p * a.mcells + l];
    a.c[e] = make_float2(v.x * scale, v.y * scale);
  }
}

__global__ void k_lambda_gather(const float2* lam, int64_t gcells, int P, const int64_t* kmask, int64_t nk, int real_u,
                                void* packed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = kmask[i] - 1;
    for (int p = 0; p < P; ++p) {
      const float2 v = lam[(int64_t)p * gcells + cell];
      if (real_u)
        reinterpret_cast<float*>(packed)[p + (int64_t)P * i] = v.x;
      else
        reinterpret_cast<float2*>(packed)[p + (int64_t)P * i] = v;
    }
  }
}

static unsigned grid1d(int64_t n) { return (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(n, 256), 1), 65535); }

// kmask + packed Λ (P, nk) for a trajectory and basis
static int compute_lambda(int d, const int64_t* G, const SampleSet& S, const void* U, int u_complex, int K, DevBuf& kmask,
                          int64_t* nk_out, DevBuf& packed, cudaStream_t st) {
  const int64_t gcells = G[0] * G[1] * (d == 3 ? G[2] : 1);
  MRSR_REQUIRE(S.n > 0, MRSR_ERR_ARG, "AssertionError: Mask removes all samples, cannot compute kernel.");
  // kmask
  {
    DevBuf flags, tmp;
    MRSR_TRY(flags.alloc(gcells));
    MRSR_TRY(tmp.alloc(gcells));
    MRSR_CHECK_CUDA(cudaMemsetAsync(flags.p, 0, gcells, st));
    const int64_t G2 = d == 3 ? G[2] : 1;
    k_kmask_seed<<<(unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(S.n, 256), 1), 152 * 64), 256, 0, st>>>(
        S, G[0], G[1], G2, flags.as<uint8_t>());
    MRSR_LAUNCH_CHECK();
    uint8_t* src = flags.as<uint8_t>();
    uint8_t* dst = tmp.as<uint8_t>();
    for (int ax = 0; ax < d; ++ax) {
      k_kmask_dilate<<<grid1d(gcells), 256, 0, st>>>(src, G[0], G[1], G2, ax, dst);
      MRSR_LAUNCH_CHECK();
      std::swap(src, dst);
    }
    MRSR_TRY(compact_nonzero(src, gcells, kmask, nk_out, st));
  }
  const int P = K * (K + 1) / 2;
  int64_t M[3] = {1, 1, 1};
  for (int i = 0; i < d; ++i) M[i] = 2 * G[i];
  const int64_t mcells = M[0] * M[1] * M[2];
  FftNd fM, fG;
  MRSR_TRY(fM.init(d, M));
  MRSR_TRY(fG.init(d, G));
  const float* ipsi[3] = {nullptr, nullptr, nullptr};
  for (int i = 0; i < d; ++i) MRSR_TRY(es_inv_psi_table(M[i], -G[i] / 2, G[i] + 1, &ipsi[i]));
  // channel batches of ~2 GB of upsampled float2 grid; the 3D tile-sorted kernel takes four
  // parts per pass, so a 3D batch holds at least four channels' parts (8-12 GB on 512^3)
  const int nq = u_complex ? 2 : 1;  // a real basis spreads real values
  const int64_t max_bytes = 2ll << 30;
  int pb = (int)std::max<int64_t>(1, std::min<int64_t>(P, max_bytes / (mcells * (int64_t)sizeof(float2))));
  if (d == 3) pb = std::max(pb, std::min(P, kP3 / nq));
  DevBuf grid, qgrid, cgrid, fsb;
  MRSR_TRY(grid.alloc(sizeof(float2) * mcells * pb));
  MRSR_TRY(qgrid.alloc(sizeof(long long) * nq * mcells * pb));
  MRSR_TRY(cgrid.alloc(sizeof(float2) * gcells * P));
  // fixed-point scale: |term| <= (2 if complex) max|U|^2 (the kernel taps are <= 1), and a cell
  // of the upsampled grid gets at most ceil(w / M) taps per sample and dimension
  MRSR_TRY(fsb.alloc(sizeof(FixedScale)));
  {
    const float* uf = reinterpret_cast<const float*>(U);
    const int64_t nu = S.nt * (int64_t)K * (u_complex ? 2 : 1);
    const float* f[2] = {uf, uf};
    const int64_t n[2] = {nu, nu};
    MRSR_TRY(fixed_scale(f, n, 2, u_complex ? 2.0 : 1.0, (double)S.n * taps_per_cell(d, M), fsb.as<FixedScale>(), st));
  }
  TileSort ts;
  const bool tiled = d == 2 && S.ns_pf * S.nt < (1ll << 31);
  const bool ordered = d == 3 && S.n < (1ll << 31);
  if (tiled) {
    MRSR_TRY(ts.build(S, M[0], M[1], st));
    MRSR_TRY(ts.prep(S, MRSR_DCF_NONE, nullptr, st));
  } else if (ordered) {
    MRSR_TRY(ts.build3(S, M, st));
    if (S.ns_pf * S.nt < (1ll << 31)) MRSR_TRY(ts.prep3(S, MRSR_DCF_NONE, nullptr, st));
  }
  const TileSort* tsp = tiled || ordered ? &ts : nullptr;
  MRSR_TRY(packed.alloc((u_complex ? 8 : 4) * (size_t)P * std::max<int64_t>(*nk_out, 1)));
  // channels in batches of pb: spread, inverse DFT on the upsampled grid, deconvolve and fold onto the 2x grid
  for (int p0 = 0; p0 < P; p0 += pb) {
    const int np = std::min(pb, P - p0);
    MRSR_CHECK_CUDA(cudaMemsetAsync(qgrid.p, 0, sizeof(long long) * nq * mcells * np, st));
    SpreadLambdaArgs sa{S, {M[0], M[1], M[2]}, mcells, U, u_complex, K, P, p0, np, nq, qgrid.as<long long>(),
                        fsb.as<FixedScale>()};
    MRSR_TRY(spread_lambda(sa, tsp, st));
    MRSR_TRY(fixed_to_grid(qgrid.as<long long>(), nq, mcells, np, fsb.as<FixedScale>(), grid.as<float2>(), st));
    MRSR_TRY(fM.run(grid.as<float2>(), np, +1, 1.0f, st));
    FoldArgs fa;
    fa.d = d;
    for (int i = 0; i < 3; ++i) {
      fa.G[i] = i < d ? G[i] : 1;
      fa.M[i] = M[i];
      fa.ipsi[i] = ipsi[i];
    }
    fa.gcells = gcells;
    fa.mcells = mcells;
    fa.P = np;
    fa.dc.init(d, G, np);
    fa.real_u = u_complex ? 0 : 1;
    fa.g = grid.as<float2>();
    fa.c = cgrid.as<float2>() + (int64_t)p0 * gcells;
    k_lambda_fold<<<grid1d(gcells * np), 256, 0, st>>>(fa);
    MRSR_LAUNCH_CHECK();
  }
  MRSR_TRY(fG.run(cgrid.as<float2>(), P, -1, 1.0f, st));
  k_lambda_gather<<<grid1d(*nk_out), 256, 0, st>>>(cgrid.as<float2>(), gcells, P, kmask.as<int64_t>(), *nk_out,
                                                   u_complex ? 0 : 1, packed.p);
  MRSR_LAUNCH_CHECK();
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return MRSR_OK;
}


// ------------------------------------------------ backprojection fold ---

struct BpFoldArgs {
  int d;
  int64_t N[3], M[3], nimg, mcells;
  int K, c0, nc, ncoils;
  Decomp dc;              // element -> (k, image position) over img x K
  const float2* g;        // [(c - c0) K + k][mcells]
  const float* ipsi[3];   // 1/psi_hat(j), j = -N/2 ...
  const float2* cmaps;    // (img..., ncoils) or null -> per-coil output
  float2* out;
};

// out[r, k] += sum_c conj(S_c(r)) x_ck(r)  (src/BackProjection.jl:96), or
// out[r, k, c] = x_ck(r) without coil maps (:54); x_ck(r) = g[(r - N/2) mod M] / psi_hat.
__global__ void k_bp_fold(BpFoldArgs a) {
  const int64_t total = a.nimg * a.K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t pos[3];
    const int k = a.dc.split(e, pos);
    const int64_t r = e - (int64_t)k * a.nimg;
    int64_t l = 0, mul = 1;
    float sc = 1.f;
    for (int dd = 0; dd < a.d; ++dd) {
      const int64_t rd = pos[dd];
      const int64_t j = rd - a.N[dd] / 2;
      sc *= a.ipsi[dd][rd];
      l += wrap_near(j, a.M[dd]) * mul;
      mul *= a.M[dd];
    }
    if (a.cmaps) {
      float2 acc = make_float2(0.f, 0.f);
      for (int c = 0; c < a.nc; ++c) {
        const float2 v = a.g[((int64_t)c * a.K + k) * a.mcells + l];
        acc = cadd(acc, cmulc(v, a.cmaps[r + a.nimg * (a.c0 + c)]));
      }
      a.out[e] = cadd(a.out[e], cscale(acc, sc));
    } else {
      for (int c = 0; c < a.nc; ++c) {
        const float2 v = a.g[((int64_t)c * a.K + k) * a.mcells + l];
        a.out[r + a.nimg * (k + (int64_t)a.K * (a.c0 + c))] = cscale(v, sc);
      }
    }
  }
}

// ------------------------------------------------------ forward model ---

struct FwdPlaceArgs {
  int d;
  int64_t N[3], M[3], nimg, mcells;
  int K, c;
  Decomp dc;             // element -> (k, image position) over img x K
  const float2* x;       // (img..., K)
  const float2* cmaps;   // (img..., ncoils) or null
  const float* ipsi[3];
  float2* g;             // [K][mcells], zeroed
};

__global__ void k_fwd_place(FwdPlaceArgs a) {
  const int64_t total = a.nimg * a.K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t pos[3];
    const int k = a.dc.split(e, pos);
    const int64_t r = e - (int64_t)k * a.nimg;
    int64_t l = 0, mul = 1;
    float sc = 1.f;
    for (int dd = 0; dd < a.d; ++dd) {
      const int64_t rd = pos[dd];
      sc *= a.ipsi[dd][rd];
      l += wrap_near(rd - a.N[dd] / 2, a.M[dd]) * mul;
      mul *= a.M[dd];
    }
    float2 v = a.x[e];
    if (a.cmaps) v = cmul(a.cmaps[r + a.nimg * a.c], v);
    a.g[(int64_t)k * a.mcells + l] = cscale(v, sc);
  }
}

struct InterpArgs {
  SampleSet S;
  int64_t M[3], mcells;
  int K, c, u_complex;
  const void* U;
  const float2* g;       // [mcells][K] after the forward DFT: a cell's K planes side by side
  float2* data;          // (ns_pf, nt, ncoils)
};

// [K][mcells] -> [mcells][K]: after the forward DFT the interpolation reads all K planes at
// each tap, so the K values of a cell are put next to each other (one or two 32-byte sectors
// per tap instead of K).
__global__ void k_interleave(const float2* __restrict__ g, float2* __restrict__ gi, int K, int64_t mcells) {
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < mcells; l += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      if (k < K) gi[l * K + k] = g[(int64_t)k * mcells + l];
  }
}

// 2D: one thread per kept sample, the w^2 taps of the K gridded planes summed in the thread
// (no cross-lane reduction); the 32 samples of a warp are consecutive along the trajectory,
// so their taps share cache lines.
__global__ void __launch_bounds__(256) k_interp(InterpArgs a) {
  const int d = a.S.d;
  const int64_t ns_tot = a.S.ns_pf * a.S.nt;
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < a.S.n; n += (int64_t)gridDim.x * blockDim.x) {
    const int64_t li = sample_lin(a.S, n);
    const int64_t t = frame_of(li, a.S.ns_pf);
    float wx[kEsWidth], wy[kEsWidth], wz[kEsWidth];
    int ix[kEsWidth], iy[kEsWidth], iz[kEsWidth];
    es_axis(a.S.trj[(int64_t)d * li], (int)a.M[0], wx, ix);
    es_axis(a.S.trj[1 + (int64_t)d * li], (int)a.M[1], wy, iy);
    if (d == 3) {
      es_axis(a.S.trj[2 + (int64_t)d * li], (int)a.M[2], wz, iz);
    } else {
#pragma unroll
      for (int j = 0; j < kEsWidth; ++j) {
        wz[j] = j == 0 ? 1.f : 0.f;
        iz[j] = 0;
      }
    }
    float2 z[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) z[k] = make_float2(0.f, 0.f);
    const int nz = d == 3 ? kEsWidth : 1;
#pragma unroll 1
    for (int t3 = 0; t3 < nz; ++t3) {
      const int64_t base3 = (int64_t)iz[t3] * a.M[0] * a.M[1];
      const float w3 = wz[t3];
#pragma unroll
      for (int t2 = 0; t2 < kEsWidth; ++t2) {
        const float w23 = wy[t2] * w3;
        const int64_t row = base3 + (int64_t)iy[t2] * a.M[0];
#pragma unroll
        for (int t1 = 0; t1 < kEsWidth; ++t1) {
          const float w = w23 * wx[t1];
          const float2* cell = a.g + (row + ix[t1]) * a.K;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (k < a.K) {
              const float2 gv = __ldg(cell + k);
              z[k].x = fmaf(w, gv.x, z[k].x);
              z[k].y = fmaf(w, gv.y, z[k].y);
            }
        }
      }
    }
    float2 y = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < a.K) {
        if (a.u_complex)
          y = cadd(y, cmul(reinterpret_cast<const float2*>(a.U)[t + a.S.nt * k], z[k]));
        else
          y = cadd(y, cscale(z[k], reinterpret_cast<const float*>(a.U)[t + a.S.nt * k]));
      }
    }
    a.data[li + ns_tot * a.c] = y;
  }
}

// 2D on the tile sort (the backprojection's 12 x 12 tiles and tap records): a work item,
// up to 1024 samples whose first tap lies in one tile, loads the tile's 19 x 19-cell window of
// the K interleaved planes into shared memory once, and each thread sums one sample's 64 taps
// x K from the window.  Same weights and summation order as k_interp (w = (wy * 1) * wx,
// taps y-major), so the data are bit-identical to it.
struct InterpTiledArgs {
  int M0, M1, K, c, u_complex, ntx;
  int64_t nt, ns_tot;
  const void* U;
  const float2* g;         // [mcells][K]
  float2* data;            // (ns_pf, nt, ncoils)
  const TapRec* rec;       // tap records in sorted order
  const int4* items;       // (tile, first sorted position, count, -)
  const int* nitems;
  int* next;               // work counter, zeroed before the launch
};

__global__ void __launch_bounds__(kTiledThreads, 2) k_interp_tiled(InterpTiledArgs a) {
  extern __shared__ float2 wk[];  // [kWinCells][K]
  __shared__ int s_item;
  const int K = a.K;
  const int nitems = *a.nitems;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.next, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const int4 item = a.items[it];
    const int ox = (item.x % a.ntx) * kTile, oy = (item.x / a.ntx) * kTile;
    for (int cw = threadIdx.x; cw < kWinCells; cw += blockDim.x) {
      const int row = cw / kWin, col = cw - row * kWin;
      const float2* src = a.g + (wrap32(ox + col, a.M0) + (int64_t)a.M0 * wrap32(oy + row, a.M1)) * K;
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < K) wk[cw * K + k] = src[k];
    }
    __syncthreads();
    for (int sidx = threadIdx.x; sidx < item.z; sidx += blockDim.x) {
      const float4* r4 = reinterpret_cast<const float4*>(a.rec + item.y + sidx);
      float wx[kEsWidth], wy[kEsWidth];
      {
        const float4 q0 = r4[0], q1 = r4[1], q2 = r4[2], q3 = r4[3];
        wx[0] = q0.x; wx[1] = q0.y; wx[2] = q0.z; wx[3] = q0.w;
        wx[4] = q1.x; wx[5] = q1.y; wx[6] = q1.z; wx[7] = q1.w;
        wy[0] = q2.x; wy[1] = q2.y; wy[2] = q2.z; wy[3] = q2.w;
        wy[4] = q3.x; wy[5] = q3.y; wy[6] = q3.z; wy[7] = q3.w;
      }
      const int4 ri = reinterpret_cast<const int4*>(r4)[4];  // li, t, lx0, ly0
      const int lx = ri.z - ox, ly = ri.w - oy;
      float2 z[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) z[k] = make_float2(0.f, 0.f);
      const bool in_win = (unsigned)lx < (unsigned)kTile && (unsigned)ly < (unsigned)kTile;
#pragma unroll
      for (int t2 = 0; t2 < kEsWidth; ++t2) {
        const float w23 = wy[t2] * 1.f;
#pragma unroll
        for (int t1 = 0; t1 < kEsWidth; ++t1) {
          const float w = w23 * wx[t1];
          // the sort put the first tap in this tile (the same float arithmetic); a sample
          // outside it would read the grid itself
          const float2* cell = in_win ? wk + ((ly + t2) * kWin + lx + t1) * K
                                      : a.g + (wrap32(ri.z + t1, a.M0) + (int64_t)a.M0 * wrap32(ri.w + t2, a.M1)) * K;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            if (k < K) {
              const float2 gv = cell[k];
              z[k].x = fmaf(w, gv.x, z[k].x);
              z[k].y = fmaf(w, gv.y, z[k].y);
            }
        }
      }
      const int64_t t = ri.y;
      float2 y = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (k < K) {
          if (a.u_complex)
            y = cadd(y, cmul(reinterpret_cast<const float2*>(a.U)[t + a.nt * k], z[k]));
          else
            y = cadd(y, cscale(z[k], reinterpret_cast<const float*>(a.U)[t + a.nt * k]));
        }
      }
      a.data[ri.x + a.ns_tot * a.c] = y;
    }
    __syncthreads();
  }
}

// 3D: one warp per sample, lanes over its 512 taps (16 each, lane_taps), one shuffle
// reduction per plane; for 512 taps per sample this beats a thread per sample (which
// serialises 512 x K gathers in one thread).
__global__ void __launch_bounds__(256) k_interp3(InterpArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t ns_tot = a.S.ns_pf * a.S.nt;
  for (int64_t n = warp; n < a.S.n; n += nwarps) {
    const int64_t li = sample_lin(a.S, n);
    const int64_t t = frame_of(li, a.S.ns_pf);
    float w[16];
    unsigned cell[16];
    lane_taps<16>(a.S, a.M, li, lane, 1.f, w, cell);
    float2 z[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) z[k] = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < a.K) {
          const float2 gv = __ldg(a.g + (int64_t)cell[j] * a.K + k);
          z[k].x = fmaf(w[j], gv.x, z[k].x);
          z[k].y = fmaf(w[j], gv.y, z[k].y);
        }
    }
    float2 y = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (k < a.K) {
        float2 v = z[k];
        for (int o = 16; o > 0; o >>= 1) {
          v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
          v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
        }
        if (a.u_complex)
          y = cadd(y, cmul(reinterpret_cast<const float2*>(a.U)[t + a.S.nt * k], v));
        else
          y = cadd(y, cscale(v, reinterpret_cast<const float*>(a.U)[t + a.S.nt * k]));
      }
    }
    if (lane == 0) a.data[li + ns_tot * a.c] = y;
  }
}

// 3D on the tile sort (the backprojection's 8^3 tiles and tap records): a work item, up to
// 1024 samples whose first tap lies in one tile, loads the tile's 15^3-cell window of the K
// interleaved planes into shared memory once (216 KB for K = 8); a warp per sample, lanes over
// its 512 taps as in k_interp3 (lane = x tap + 8 y tap, 16 taps each), one shuffle reduction
// per plane.
struct InterpTiled3Args {
  int M0, M1, M2, K, c, u_complex, ntx, nty;
  int64_t nt, ns_tot;
  const void* U;
  const float2* g;         // [mcells][K]
  float2* data;            // (ns_pf, nt, ncoils)
  const TapRec3* rec;      // tap records in sorted order
  const int4* items;       // (tile, first sorted position, count, -)
  const int* nitems;
  int* next;               // work counter, zeroed before the launch
};

__global__ void __launch_bounds__(kTiledThreads, 1) k_interp_tiled3(InterpTiled3Args a) {
  extern __shared__ float2 wk[];  // [kWin3Cells][K]
  __shared__ int s_item;
  const int K = a.K;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int t1 = lane & 7, t2a = lane >> 3;
  const int nitems = *a.nitems;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(a.next, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= nitems) break;
    const int4 item = a.items[it];
    const int tx = item.x % a.ntx, ty = (item.x / a.ntx) % a.nty, tz = item.x / (a.ntx * a.nty);
    const int ox = tx * kTile3, oy = ty * kTile3, oz = tz * kTile3;
    for (int cw = threadIdx.x; cw < kWin3Cells; cw += blockDim.x) {
      const int wz = cw / (kWin3 * kWin3), r2 = cw - wz * kWin3 * kWin3, wy = r2 / kWin3, wx = r2 - wy * kWin3;
      const float2* src = a.g + (wrap32(ox + wx, a.M0) +
                                 (int64_t)a.M0 * (wrap32(oy + wy, a.M1) + (int64_t)a.M1 * wrap32(oz + wz, a.M2))) * K;
#pragma unroll
      for (int k = 0; k < 8; ++k)
        if (k < K) wk[cw * K + k] = src[k];
    }
    __syncthreads();
    for (int sidx = warp; sidx < item.z; sidx += nwarps) {
      const TapRec3& r = a.rec[item.y + sidx];
      const int li = r.li, t = r.t, lx0 = r.lx0, ly0 = r.ly0, lz0 = r.lz0;
      const int lx = lx0 - ox, ly = ly0 - oy, lz = lz0 - oz;
      const bool in_win = (unsigned)lx < (unsigned)kTile3 && (unsigned)ly < (unsigned)kTile3 && (unsigned)lz < (unsigned)kTile3;
      const float wxl = r.wx[t1];
      float2 z[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) z[k] = make_float2(0.f, 0.f);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int t2 = t2a + 4 * (j & 1), t3 = j >> 1;
        const float w = (wxl * r.wy[t2]) * r.wz[t3];
        // the sort put the first tap in this tile (the same float arithmetic); a sample
        // outside it would read the grid itself
        const float2* cell =
            in_win ? wk + (((lz + t3) * kWin3 + ly + t2) * kWin3 + lx + t1) * K
                   : a.g + (wrap32(lx0 + t1, a.M0) +
                            (int64_t)a.M0 * (wrap32(ly0 + t2, a.M1) + (int64_t)a.M1 * wrap32(lz0 + t3, a.M2))) * K;
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (k < K) {
            const float2 gv = cell[k];
            z[k].x = fmaf(w, gv.x, z[k].x);
            z[k].y = fmaf(w, gv.y, z[k].y);
          }
      }
      float2 y = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (k < K) {
          float2 v = z[k];
          for (int o = 16; o > 0; o >>= 1) {
            v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
            v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
          }
          if (a.u_complex)
            y = cadd(y, cmul(reinterpret_cast<const float2*>(a.U)[t + a.nt * k], v));
          else
            y = cadd(y, cscale(v, reinterpret_cast<const float*>(a.U)[t + a.nt * k]));
        }
      }
      if (lane == 0) a.data[li + a.ns_tot * a.c] = y;
    }
    __syncthreads();
  }
}

static int check_smooth(int d, const int64_t* G) {
  for (int i = 0; i < d; ++i) {
    int rad[kMaxStages], ns;
    MRSR_REQUIRE(build_radices((int)G[i], rad, &ns), MRSR_ERR_ARG,
                 "AssertionError: img_shape_os has to be composed of the prime factors 2, 3, and 5 (cf. NonuniformFFTs.jl "
                 "documentation).");
  }
  return MRSR_OK;
}

}  // namespace mrsr

using namespace mrsr;

static cudaStream_t nstream(mrsr_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" int mrsr_nfft_normalop_create(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                                         const float* trj, const uint8_t* sample_mask, const void* U, int u_is_complex,
                                         int K, const float* cmaps, int ncoils, int precision, mrsr_stream_t stream,
                                         mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(trj && U, MRSR_ERR_ARG, "trj and U must be device pointers");
  MRSR_REQUIRE(ns_per_frame >= 1 && nt >= 1, MRSR_ERR_ARG, "empty trajectory");
  cudaStream_t st = nstream(stream);
  mrsr_normalop* op = new mrsr_normalop();
  int s = op_init_geometry(op, MRSR_KIND_NFFT, ndims, img_shape, K, cmaps ? ncoils : 1, precision);
  if (s == MRSR_OK) s = op_set_cmaps(op, cmaps, st);
  SampleList sl;
  DevBuf kmask, packed;
  int64_t nk = 0;
  if (s == MRSR_OK) s = check_smooth(ndims, op->geo.g);
  if (s == MRSR_OK) s = sl.init(ndims, trj, ns_per_frame, nt, sample_mask, st);
  if (s == MRSR_OK) s = compute_lambda(ndims, op->geo.g, sl.set, U, u_is_complex, K, kmask, &nk, packed, st);
  if (s == MRSR_OK) s = op_set_lambda_packed(op, packed.p, u_is_complex, kmask.as<int64_t>(), nk, st);
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  *out = op;
  return MRSR_OK;
}

extern "C" int mrsr_backprojection(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt, int ncoils,
                                   const float* data, const float* trj, const uint8_t* sample_mask, const void* U,
                                   int u_is_complex, int K, const float* cmaps, int dcf_kind, const float* dcf_array,
                                   float* out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3");
  MRSR_REQUIRE(img_shape && data && trj && out, MRSR_ERR_ARG, "NULL argument to mrsr_backprojection");
  MRSR_REQUIRE(ncoils >= 1 && ns_per_frame >= 1 && nt >= 1, MRSR_ERR_ARG, "empty data");
  if (!U) K = (int)nt;
  MRSR_REQUIRE(K >= 1, MRSR_ERR_ARG, "K must be >= 1");
  MRSR_REQUIRE(U != nullptr || K <= 1 << 20, MRSR_ERR_ARG, "too many frames for an identity basis");
  MRSR_REQUIRE(dcf_kind >= MRSR_DCF_NONE && dcf_kind <= MRSR_DCF_ARRAY, MRSR_ERR_ARG,
               "`density_compensation` can only be `:radial_3D`, `:radial_2D`, `:none`, or of type `AbstractArray`");
  MRSR_REQUIRE(dcf_kind != MRSR_DCF_ARRAY || dcf_array, MRSR_ERR_ARG, "density compensation array is NULL");
  cudaStream_t st = nstream(stream);
  int64_t N[3] = {1, 1, 1}, M[3] = {1, 1, 1};
  for (int i = 0; i < ndims; ++i) {
    N[i] = img_shape[i];
    M[i] = 2 * N[i];
  }
  MRSR_TRY(check_smooth(ndims, M));
  const int64_t nimg = N[0] * N[1] * N[2], mcells = M[0] * M[1] * M[2];
  SampleList sl;
  MRSR_TRY(sl.init(ndims, trj, ns_per_frame, nt, sample_mask, st));
  MRSR_REQUIRE(sl.set.n > 0, MRSR_ERR_ARG, "AssertionError: Sample mask removes all samples, cannot compute backprojection.");
  FftNd fM;
  MRSR_TRY(fM.init(ndims, M));
  const float* ipsi[3] = {nullptr, nullptr, nullptr};
  for (int i = 0; i < ndims; ++i) MRSR_TRY(es_inv_psi_table(M[i], -(N[i] / 2), N[i], &ipsi[i]));
  // coil batches of ~2 GB of float2 grid
  const int64_t max_bytes = 2ll << 30;
  const int64_t per_coil = (int64_t)K * mcells * (int64_t)sizeof(float2);
  int cc = (int)std::max<int64_t>(1, std::min<int64_t>(ncoils, max_bytes / std::max<int64_t>(per_coil, 1)));
  // 3D with a basis: the batch's parts (2 per coil and coefficient) interleaved per cell, at
  // most 32 (one per lane of k_spread_data_cp)
  const bool tiled3 = ndims == 3 && U != nullptr && sl.set.n < (1ll << 31) && ns_per_frame * nt < (1ll << 31);
  const bool parts_layout = ndims == 3 && U != nullptr && !tiled3 && 2 * K <= 32;
  if (parts_layout) cc = std::min(cc, 16 / K);
  DevBuf grid, qgrid, fsb;
  MRSR_TRY(grid.alloc((size_t)per_coil * cc));
  MRSR_TRY(qgrid.alloc((size_t)per_coil * 2 * cc));  // fixed-point re and im, 8 bytes each
  // fixed-point scale: |term component| <= max|data| max|U| (x2 for complex U) x dcf bound,
  // at most ceil(w / M) taps per sample, cell and dimension
  MRSR_TRY(fsb.alloc(sizeof(FixedScale)));
  // an identity basis gives every sample one channel: the global kernel
  const bool tiled = ndims == 2 && U != nullptr && ns_per_frame * nt < (1ll << 31);
  {
    const float* f[3];
    int64_t n[3];
    int nf = 0;
    double mult = 1.0;
    f[nf] = data;
    n[nf++] = 2 * ns_per_frame * nt * (int64_t)ncoils;
    if (U) {
      f[nf] = reinterpret_cast<const float*>(U);
      n[nf++] = nt * (int64_t)K * (u_is_complex ? 2 : 1);
      if (u_is_complex) mult *= 2.0;
    }
    if (dcf_kind == MRSR_DCF_RADIAL_2D) mult *= 0.5 * std::sqrt((double)ndims);  // |k| <= sqrt(d) / 2
    if (dcf_kind == MRSR_DCF_RADIAL_3D) mult *= 0.25 * ndims;                   // |k|^2 <= d / 4
    if (dcf_kind == MRSR_DCF_ARRAY) {
      f[nf] = dcf_array;
      n[nf++] = sl.set.n;
    }
    MRSR_TRY(fixed_scale(f, n, nf, mult, (double)sl.set.n * taps_per_cell(ndims, M), fsb.as<FixedScale>(), st));
  }
  TileSort ts;
  if (tiled) {
    MRSR_TRY(ts.build(sl.set, M[0], M[1], st));
    MRSR_TRY(ts.prep(sl.set, dcf_kind, dcf_array, st));
  }
  const bool ordered = ndims == 3 && sl.set.n < (1ll << 31);
  if (ordered) MRSR_TRY(ts.build3(sl.set, M, st));
  if (tiled3) MRSR_TRY(ts.prep3(sl.set, dcf_kind, dcf_array, st));
  const int64_t out_elems = nimg * K * (cmaps ? 1 : ncoils);
  if (cmaps) MRSR_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(float2) * out_elems, st));
  for (int c0 = 0; c0 < ncoils; c0 += cc) {
    const int nc = std::min(cc, ncoils - c0);
    MRSR_CHECK_CUDA(cudaMemsetAsync(qgrid.p, 0, (size_t)per_coil * 2 * nc, st));
    SpreadDataArgs sa{sl.set, {M[0], M[1], M[2]}, mcells, reinterpret_cast<const float2*>(data), c0, nc, U,
                      u_is_complex, K, dcf_kind, dcf_array, qgrid.as<long long>(), fsb.as<FixedScale>()};
    MRSR_TRY(spread_data(sa, tiled || ordered ? &ts : nullptr, st));
    if (parts_layout) {
      k_fixed_to_grid_cp<<<(unsigned)cdiv(mcells, 32), 256, 0, st>>>(qgrid.as<long long>(), 2 * nc * K, mcells,
                                                                    fsb.as<FixedScale>(), grid.as<float2>());
      MRSR_LAUNCH_CHECK();
    } else {
      MRSR_TRY(fixed_to_grid(qgrid.as<long long>(), 2, mcells, (int64_t)nc * K, fsb.as<FixedScale>(),
                             grid.as<float2>(), st));
    }
    MRSR_TRY(fM.run(grid.as<float2>(), (int64_t)nc * K, +1, 1.0f, st));
    BpFoldArgs fa;
    fa.d = ndims;
    for (int i = 0; i < 3; ++i) {
      fa.N[i] = N[i];
      fa.M[i] = M[i];
      fa.ipsi[i] = ipsi[i];
    }
    fa.nimg = nimg;
    fa.mcells = mcells;
    fa.K = K;
    fa.dc.init(ndims, N, K);
    fa.c0 = c0;
    fa.nc = nc;
    fa.ncoils = ncoils;
    fa.g = grid.as<float2>();
    fa.cmaps = reinterpret_cast<const float2*>(cmaps);
    fa.out = reinterpret_cast<float2*>(out);
    k_bp_fold<<<grid1d(nimg * K), 256, 0, st>>>(fa);
    MRSR_LAUNCH_CHECK();
  }
  return MRSR_OK;  // asynchronous on `st`; the temporaries are freed in stream order
}

extern "C" int mrsr_forward_model(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt, int ncoils,
                                  const float* x, const float* trj, const void* U, int u_is_complex, int K,
                                  const float* cmaps, float* data_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3");
  MRSR_REQUIRE(img_shape && x && trj && U && data_out, MRSR_ERR_ARG, "NULL argument to mrsr_forward_model");
  MRSR_REQUIRE(K >= 1 && K <= 8, MRSR_ERR_UNSUPPORTED, "forward model supports 1 <= K <= 8");
  MRSR_REQUIRE(ncoils >= 1, MRSR_ERR_ARG, "ncoils must be >= 1");
  MRSR_REQUIRE(cmaps || ncoils == 1, MRSR_ERR_ARG, "cmaps == NULL requires ncoils == 1");
  cudaStream_t st = nstream(stream);
  int64_t N[3] = {1, 1, 1}, M[3] = {1, 1, 1};
  for (int i = 0; i < ndims; ++i) {
    N[i] = img_shape[i];
    M[i] = 2 * N[i];
  }
  MRSR_TRY(check_smooth(ndims, M));
  const int64_t nimg = N[0] * N[1] * N[2], mcells = M[0] * M[1] * M[2];
  SampleList sl;
  MRSR_TRY(sl.init(ndims, trj, ns_per_frame, nt, nullptr, st));
  FftNd fM;
  MRSR_TRY(fM.init(ndims, M));
  const float* ipsi[3] = {nullptr, nullptr, nullptr};
  for (int i = 0; i < ndims; ++i) MRSR_TRY(es_inv_psi_table(M[i], -(N[i] / 2), N[i], &ipsi[i]));
  DevBuf grid, gridi;
  MRSR_TRY(grid.alloc(sizeof(float2) * K * mcells));
  MRSR_TRY(gridi.alloc(sizeof(float2) * K * mcells));
  // the interpolation runs on the tile sort of the samples (built once for all coils)
  TileSort ts;
  const bool small = sl.set.n < (1ll << 31) && ns_per_frame * nt < (1ll << 31);
  const bool tiled = ndims == 2 && small && M[0] < (1ll << 24) && M[1] < (1ll << 24);
  const int64_t ntiles3 = cdiv(M[0], kTile3) * cdiv(M[1], kTile3) * cdiv(M[2], kTile3);
  const bool tiled3 = ndims == 3 && small && ntiles3 < (1ll << 31) && mcells < (1ll << 32);
  if (tiled) {
    MRSR_TRY(ts.build(sl.set, M[0], M[1], st));
    MRSR_TRY(ts.prep(sl.set, MRSR_DCF_NONE, nullptr, st));
  } else if (tiled3) {
    MRSR_TRY(ts.build3(sl.set, M, st));
    MRSR_TRY(ts.prep3(sl.set, MRSR_DCF_NONE, nullptr, st));
  }
  const size_t win_bytes = sizeof(float2) * kWinCells * (size_t)K;
  const size_t win3_bytes = sizeof(float2) * kWin3Cells * (size_t)K;
  if (tiled) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_interp_tiled, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)win_bytes));
  if (tiled3)
    MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_interp_tiled3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)win3_bytes));
  for (int c = 0; c < ncoils; ++c) {
    MRSR_CHECK_CUDA(cudaMemsetAsync(grid.p, 0, sizeof(float2) * K * mcells, st));
    FwdPlaceArgs pa;
    pa.d = ndims;
    for (int i = 0; i < 3; ++i) {
      pa.N[i] = N[i];
      pa.M[i] = M[i];
      pa.ipsi[i] = ipsi[i];
    }
    pa.nimg = nimg;
    pa.mcells = mcells;
    pa.K = K;
    pa.dc.init(ndims, N, K);
    pa.c = c;
    pa.x = reinterpret_cast<const float2*>(x);
    pa.cmaps = reinterpret_cast<const float2*>(cmaps);
    pa.g = grid.as<float2>();
    k_fwd_place<<<grid1d(nimg * K), 256, 0, st>>>(pa);
    MRSR_LAUNCH_CHECK();
    MRSR_TRY(fM.run(grid.as<float2>(), K, -1, 1.0f, st));
    k_interleave<<<grid1d(mcells), 256, 0, st>>>(grid.as<float2>(), gridi.as<float2>(), K, mcells);
    MRSR_LAUNCH_CHECK();
    InterpArgs ia{sl.set, {M[0], M[1], M[2]}, mcells, K, c, u_is_complex, U, gridi.as<float2>(),
                  reinterpret_cast<float2*>(data_out)};
    if (tiled3) {
      InterpTiled3Args ta;
      ta.M0 = (int)M[0];
      ta.M1 = (int)M[1];
      ta.M2 = (int)M[2];
      ta.K = K;
      ta.c = c;
      ta.u_complex = u_is_complex;
      ta.ntx = ts.ntx;
      ta.nty = ts.nty;
      ta.nt = nt;
      ta.ns_tot = ns_per_frame * nt;
      ta.U = U;
      ta.g = gridi.as<float2>();
      ta.data = reinterpret_cast<float2*>(data_out);
      ta.rec = ts.rec.as<TapRec3>();
      ta.items = ts.items.as<int4>();
      ta.nitems = ts.nitems.as<int>();
      ta.next = ts.next.as<int>();
      MRSR_CHECK_CUDA(cudaMemsetAsync(ts.next.p, 0, sizeof(int), st));
      k_interp_tiled3<<<152, kTiledThreads, win3_bytes, st>>>(ta);
    } else if (ndims == 3) {
      MRSR_REQUIRE(mcells < (1ll << 32), MRSR_ERR_UNSUPPORTED, "forward model grid of 2^32 cells or more");
      k_interp3<<<spread_blocks(sl.set.n), 256, 0, st>>>(ia);
    } else if (tiled) {
      InterpTiledArgs ta;
      ta.M0 = (int)M[0];
      ta.M1 = (int)M[1];
      ta.K = K;
      ta.c = c;
      ta.u_complex = u_is_complex;
      ta.ntx = ts.ntx;
      ta.nt = nt;
      ta.ns_tot = ns_per_frame * nt;
      ta.U = U;
      ta.g = gridi.as<float2>();
      ta.data = reinterpret_cast<float2*>(data_out);
      ta.rec = ts.rec.as<TapRec>();
      ta.items = ts.items.as<int4>();
      ta.nitems = ts.nitems.as<int>();
      ta.next = ts.next.as<int>();
      MRSR_CHECK_CUDA(cudaMemsetAsync(ts.next.p, 0, sizeof(int), st));
      k_interp_tiled<<<152 * 2, kTiledThreads, win_bytes, st>>>(ta);
    } else {
      k_interp<<<(unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(sl.set.n, 256), 1), 152 * 64), 256, 0, st>>>(ia);
    }
    MRSR_LAUNCH_CHECK();
  }
  return MRSR_OK;  // asynchronous on `st`
}
