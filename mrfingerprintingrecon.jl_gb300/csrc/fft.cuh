// Batched mixed-radix FFT on shared memory (radix 2, 3, 4, 5, 8).
//
// Each CTA transforms a set of lines held in shared memory.  Line l = lo*TC + li
// (lo < NO "outer" lines, li < TC interleaved lines) stores element n at
//   s[lo * lstride + n * TC + li]
// so TC adjacent columns of a strided array can be loaded with coalesced
// TC-wide rows and transformed together.
//
// Algorithm: Stockham autosort formulation (Govindaraju et al., "High
// performance discrete Fourier transforms on graphics processors", SC'08).
// Stage with radix R after Ns = product of the previous radices:
//   for butterfly j < L/R:  v[q] = in[j + q L/R] * W_{Ns R}^{q (j mod Ns)},
//   v = DFT_R(v),  out[(j/Ns) Ns R + (j mod Ns) + q Ns] = v[q].
// Stages alternate between two shared-memory buffers (one butterfly per
// thread in flight keeps register use low); one barrier per stage.
//
// Pruning.  With the first radix even and only the lower half of the input
// non-zero (zero-padded Toeplitz embedding), the first stage reads q < R/2
// only; with the last radix even and only the lower half of the output
// wanted (crop), the last stage writes q < R/2 only.
#pragma once
#include "common.cuh"

namespace mrsr {

constexpr int kMaxStages = 16;

struct FftPlan {
  int L = 0;
  int nstages = 0;
  int radix[kMaxStages] = {0};
  const float2* tw = nullptr;  // device table: tw[p] = exp(-2 pi i p / L), p < L
  bool first_even() const { return nstages > 0 && (radix[0] % 2 == 0); }
  bool last_even() const { return nstages > 0 && (radix[nstages - 1] % 2 == 0); }
};

// Host: factor L into radices {8,4,2,3,5}; even radices are placed at both
// ends when there are at least two of them so that pruning applies.
bool build_radices(int L, int* radix, int* nstages);

// ------------------------------------------------------------- DFT_R ---
// sgn = -1: forward (exp(-2 pi i qm/R)), sgn = +1: inverse.
template <int R> struct Dft;

template <> struct Dft<2> {
  static __device__ __forceinline__ void run(float2* v, float) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};
template <> struct Dft<4> {
  static __device__ __forceinline__ void run(float2* v, float sgn) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = cmul_i(csub(v[1], v[3]), sgn);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
  }
};
template <> struct Dft<8> {
  static __device__ __forceinline__ void run(float2* v, float sgn) {
    const float h = 0.70710678118654752440f;
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4>::run(e, sgn);
    Dft<4>::run(o, sgn);
    // w8^1 = h(1 + sgn i), w8^2 = sgn i, w8^3 = h(-1 + sgn i)
    float2 o1 = make_float2(h * (o[1].x - sgn * o[1].y), h * (o[1].y + sgn * o[1].x));
    float2 o2 = cmul_i(o[2], sgn);
    float2 o3 = make_float2(h * (-o[3].x - sgn * o[3].y), h * (-o[3].y + sgn * o[3].x));
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[5] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[6] = csub(e[2], o2);
    v[3] = cadd(e[3], o3);
    v[7] = csub(e[3], o3);
  }
};
template <> struct Dft<3> {
  static __device__ __forceinline__ void run(float2* v, float sgn) {
    const float c = -0.5f, s = 0.86602540378443864676f;
    float2 t = cadd(v[1], v[2]);
    float2 d = cmul_i(csub(v[1], v[2]), sgn * s);
    float2 m = make_float2(v[0].x + c * t.x, v[0].y + c * t.y);
    v[0] = cadd(v[0], t);
    v[1] = cadd(m, d);
    v[2] = csub(m, d);
  }
};
template <> struct Dft<5> {
  static __device__ __forceinline__ void run(float2* v, float sgn) {
    const float c1 = 0.30901699437494742410f, c2 = -0.80901699437494742410f;
    const float s1 = 0.95105651629515357212f, s2 = 0.58778525229247312917f;
    float2 t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    float2 d1 = csub(v[1], v[4]), d2 = csub(v[2], v[3]);
    float2 a1 = make_float2(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    float2 a2 = make_float2(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    float2 b1 = cmul_i(make_float2(s1 * d1.x + s2 * d2.x, s1 * d1.y + s2 * d2.y), sgn);
    float2 b2 = cmul_i(make_float2(s2 * d1.x - s1 * d2.x, s2 * d1.y - s1 * d2.y), sgn);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a1, b1);
    v[4] = csub(a1, b1);
    v[2] = cadd(a2, b2);
    v[3] = csub(a2, b2);
  }
};

// ---------------------------------------------------------- one stage ---
struct LineLayout {
  int NO;       // outer lines
  int TC;       // interleaved lines (columns), a power of two
  int lstride;  // float2 between outer lines
};

// One Stockham stage from src to dst (two shared-memory buffers).
// prune_in: read only q < R/2 (first stage, lower-half input).
// prune_out: write only q < R/2 (last stage, lower-half output).
template <int R>
__device__ __forceinline__ void fft_stage(const float2* __restrict__ src, float2* __restrict__ dst, int L, int Ns,
                                          const LineLayout& ly, int tcshift, float sgn,
                                          const float2* __restrict__ tw, bool prune_in, bool prune_out) {
  const int Lr = L / R;
  const int nbf = (ly.NO * Lr) << tcshift;
  const int twstep = L / (Ns * R);
  const int tcmask = ly.TC - 1;
  for (int bf = threadIdx.x; bf < nbf; bf += blockDim.x) {
    const int li = bf & tcmask;
    const int t = bf >> tcshift;
    const int j = t % Lr;
    const int lo = t / Lr;
    const float2* sb = src + lo * ly.lstride + li;
    float2* db = dst + lo * ly.lstride + li;
    float2 v[R];
#pragma unroll
    for (int q = 0; q < R; ++q) {
      if (!prune_in || q < R / 2)
        v[q] = sb[(j + q * Lr) << tcshift];
      else
        v[q] = make_float2(0.f, 0.f);
    }
    const int kk = j % Ns;
    if (kk != 0) {
#pragma unroll
      for (int q = 1; q < R; ++q) {
        float2 w = tw[q * kk * twstep];
        w.y *= -sgn;  // table holds exp(-i..); the inverse uses the conjugate
        v[q] = cmul(v[q], w);
      }
    }
    Dft<R>::run(v, sgn);
    const int m0 = (j - kk) * R + kk;  // (j / Ns) * Ns * R + j % Ns
#pragma unroll
    for (int q = 0; q < R; ++q)
      if (!prune_out || q < R / 2) db[(m0 + q * Ns) << tcshift] = v[q];
  }
  __syncthreads();
}

__device__ __forceinline__ int ilog2_pow2(int x) { return 31 - __clz(x); }

// Full transform of all lines.  Input in buf0; the stages alternate between
// buf0 and buf1; returns the buffer that holds the result.  The caller has
// synchronised after filling buf0.
// sgn = -1 forward (unnormalised), +1 inverse (unnormalised).
__device__ __forceinline__ float2* fft_lines(float2* __restrict__ buf0, float2* __restrict__ buf1, const FftPlan& pl,
                                          const LineLayout& ly, float sgn, const float2* __restrict__ tw_s,
                                          bool prune_in, bool prune_out) {
  int Ns = 1;
  float2* src = buf0;
  float2* dst = buf1;
  const int tcs = ilog2_pow2(ly.TC);
  for (int st = 0; st < pl.nstages; ++st) {
    const int R = pl.radix[st];
    const bool pin = prune_in && st == 0 && (R % 2 == 0);
    const bool pout = prune_out && st == pl.nstages - 1 && (R % 2 == 0);
    switch (R) {
      case 8: fft_stage<8>(src, dst, pl.L, Ns, ly, tcs, sgn, tw_s, pin, pout); break;
      case 4: fft_stage<4>(src, dst, pl.L, Ns, ly, tcs, sgn, tw_s, pin, pout); break;
      case 2: fft_stage<2>(src, dst, pl.L, Ns, ly, tcs, sgn, tw_s, pin, pout); break;
      case 3: fft_stage<3>(src, dst, pl.L, Ns, ly, tcs, sgn, tw_s, pin, pout); break;
      case 5: fft_stage<5>(src, dst, pl.L, Ns, ly, tcs, sgn, tw_s, pin, pout); break;
      default: break;
    }
    Ns *= R;
    float2* t = src;
    src = dst;
    dst = t;
  }
  return src;
}

// Copy the twiddle table of a plan into shared memory (caller syncs).
__device__ __forceinline__ void load_twiddles(float2* tw_s, const FftPlan& pl) {
  for (int i = threadIdx.x; i < pl.L; i += blockDim.x) tw_s[i] = pl.tw[i];
}

// Whether the stage-0 read / last-stage write pruning applies for a plan.
__host__ __device__ __forceinline__ bool can_prune_in(const FftPlan& p, int nvalid) {
  return nvalid * 2 == p.L && p.nstages > 0 && p.radix[0] % 2 == 0;
}
__host__ __device__ __forceinline__ bool can_prune_out(const FftPlan& p, int nkeep) {
  return nkeep * 2 == p.L && p.nstages > 0 && p.radix[p.nstages - 1] % 2 == 0;
}

// Host-side owner of a plan and its twiddle table.
struct FftPlanHost {
  FftPlan plan;
  DevBuf tw;
  int init(int L);  // builds radices and uploads twiddles (synchronous)
};

}  // namespace mrsr
