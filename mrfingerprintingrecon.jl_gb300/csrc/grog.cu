// GROG self-calibration and gridding (src/GROG.jl).
//
// grog_calib (src/GROG.jl:14-51), per spoke of Nr samples and Nc coils:
//   G = (D1 \ D2)^T with D1 = rows 1..Nr-1, D2 = rows 2..Nr,   v = log(G),
// then lnG[:, i, j] = nm \ v[:, i, j] over all spokes, nm = Nr * (k_2 - k_1).
// The least squares run in float64 through the normal equations (Gram
// matrices accumulated in float64, Gauss-Jordan with partial pivoting); the
// principal matrix logarithm runs in float32, the precision the reference
// computes log(G) in, by inverse scaling and squaring: Denman-Beavers square
// roots until ||Y - I||_F <= 1/4, then log(I + X) by the m-point Gauss-Legendre
// quadrature of int_0^1 X (I + t X)^{-1} dt (the diagonal Pade approximant),
// times 2^s (Higham, Functions of Matrices, SIAM 2008, ch. 11).
//
// grog_gridding! (src/GROG.jl:73-102): per sample and dimension the grid index
// follows the reference's float32/float64 promotion bit for bit, and
// data <- exp(shift lnG_d) data is applied as exp(s_j lnG_d) exp((shift - s_j) lnG_d)
// on the Nc x Nrep block: the first factor from a per-call table over a grid of
// s_j, the second as a Horner-evaluated Taylor series of its action (the
// reference forms the Higham-2005 Pade exponential of each float32 matrix and
// multiplies).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "common.cuh"

namespace mrsr {

constexpr int kGrogMaxCoils = 32;
constexpr int kLogGL = 12;  // Gauss-Legendre nodes of the log quadrature

// ------------------------------------------------------- spoke Grams ---
// A = D1^H D1, B = D1^H D2 for spoke `blockIdx.x`; one thread per (i, j).  The sums run on
// the float32 cores in float-float form: each product is split exactly into p + e (one
// FMA) and added to a (hi, lo) pair by Knuth's TwoSum, the compensated dot product of
// Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26, 2005): the result is as accurate as a
// float64 sum up to a relative n^2 u^2 of sum |d_i d_j| (u = 2^-24), which float64
// itself only meets to n u_64.  The rounded intrinsics keep the compiler from fusing the
// product into the following addition, which would lose the exact split.
struct FF {
  float hi = 0.f, lo = 0.f;
};
__device__ __forceinline__ void ff_madd(FF& s, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = fmaf(a, b, -p);  // a b = p + e exactly
  const float t = __fadd_rn(s.hi, p);
  const float z = __fsub_rn(t, s.hi);
  const float err = __fadd_rn(__fsub_rn(s.hi, __fsub_rn(t, z)), __fsub_rn(p, z));  // s.hi + p = t + err
  s.hi = t;
  s.lo = __fadd_rn(s.lo, __fadd_rn(err, e));
}
__device__ __forceinline__ double ff_value(const FF& s) { return (double)s.hi + (double)s.lo; }

constexpr int kGramRows = 128;  // samples of a spoke staged in shared memory at a time

struct GramArgs {
  const float2* data;   // (ns_pf, nt, nc, nrep)
  int64_t ns_pf, nt;
  int nc, nrep, nr, spf;  // spokes per frame
  double2* AB;          // [spoke][2][nc][nc] (column-major i + nc j)
};

__global__ void __launch_bounds__(1024, 2) k_grog_gram(GramArgs a) {
  extern __shared__ float2 sd[];  // [row][coil], row stride nc + 1 (conflict-free staging)
  const int n = a.nc, ld = n + 1;
  const int64_t ip = blockIdx.x;
  const int64_t rep = ip / ((int64_t)a.spf * a.nt);
  const int64_t rem = ip - rep * a.spf * a.nt;
  const int64_t t = rem / a.spf;
  const int64_t sif = rem - t * a.spf;
  const int64_t ns_tot = a.ns_pf * a.nt;
  const float2* src = a.data + sif * a.nr + a.ns_pf * t + ns_tot * a.nc * rep;  // coil stride ns_tot
  const int i = threadIdx.x % kGrogMaxCoils, j = threadIdx.x / kGrogMaxCoils;
  const bool act = i < n && j < n;
  FF are, aim, bre, bim;
  for (int r0 = 0; r0 + 1 < a.nr; r0 += kGramRows) {
    const int rows = min(kGramRows + 1, a.nr - r0);  // one extra row: B reads sample r + 1
    __syncthreads();
    for (int e = threadIdx.x; e < rows * n; e += blockDim.x) {
      const int r = e % rows, c = e / rows;
      sd[r * ld + c] = src[r0 + r + ns_tot * c];
    }
    __syncthreads();
    if (act) {
      const int last = min(kGramRows, a.nr - 1 - r0);
      for (int r = 0; r < last; ++r) {
        const float2 di = sd[r * ld + i], dj = sd[r * ld + j], dk = sd[(r + 1) * ld + j];
        // conj(di) dj and conj(di) dk
        ff_madd(are, di.x, dj.x);
        ff_madd(are, di.y, dj.y);
        ff_madd(aim, di.x, dj.y);
        ff_madd(aim, -di.y, dj.x);
        ff_madd(bre, di.x, dk.x);
        ff_madd(bre, di.y, dk.y);
        ff_madd(bim, di.x, dk.y);
        ff_madd(bim, -di.y, dk.x);
      }
    }
  }
  if (act) {
    double2* out = a.AB + ip * 2 * a.nc * a.nc;
    out[i + a.nc * j] = make_double2(ff_value(are), ff_value(aim));
    out[a.nc * a.nc + i + a.nc * j] = make_double2(ff_value(bre), ff_value(bim));
  }
}

// ------------------------------------------ small dense linear algebra ---
// All routines: one CTA, n <= 32, column-major n x n complex matrices in shared
// memory, templated on the complex type (double2 for the least squares solve,
// float2 for the logarithm).

template <class C> struct Cx;
template <> struct Cx<double2> {
  using R = double;
  static constexpr double kTiny = 1e-280;  // |pivot|^2 below this: the column is singular
  static __device__ __forceinline__ double2 mk(double x, double y) { return make_double2(x, y); }
};
template <> struct Cx<float2> {
  using R = float;
  static constexpr float kTiny = 1e-36f;
  static __device__ __forceinline__ float2 mk(float x, float y) { return make_float2(x, y); }
};
template <class C> __device__ __forceinline__ C cx_zero() { return Cx<C>::mk(0, 0); }
template <class C> __device__ __forceinline__ C cx_sub(C a, C b) { return Cx<C>::mk(a.x - b.x, a.y - b.y); }
template <class C> __device__ __forceinline__ C cx_mul(C a, C b) {
  return Cx<C>::mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class C> __device__ __forceinline__ typename Cx<C>::R cx_abs2(C a) { return a.x * a.x + a.y * a.y; }
template <class C> __device__ __forceinline__ C cx_shfl(C v, int src) {
  return Cx<C>::mk(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src));
}

// Pivot bookkeeping of one Gauss-Jordan step, double-buffered by step parity.
template <class C> struct GjStep {
  C f[2][kGrogMaxCoils];  // column k after the row swap: the elimination multipliers
  C rinv[2];              // 1 / pivot
  int p[2];               // pivot row
  int sing[2];            // |pivot|^2 < kTiny: basic solution with x_k = 0
};

// Warp-wide pivot choice for column k, lane r holding row r: the first row r >= k of
// largest modulus (partial pivoting); writes the step record `b`.
template <class C>
__device__ __forceinline__ void gj_pivot(C v, int k, int n, GjStep<C>& st, int b) {
  using R = typename Cx<C>::R;
  const int lane = threadIdx.x & 31;
  R best = (lane >= k && lane < n) ? cx_abs2(v) : R(-1);
  int idx = lane;
  for (int o = 16; o > 0; o >>= 1) {
    const R ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ob > best || (ob == best && oi < idx)) {
      best = ob;
      idx = oi;
    }
  }
  int p = __shfl_sync(0xffffffffu, idx, 0);
  if (p < k || p >= n) p = k;  // non-finite column: keep the row order (indices stay in range)
  const C vk = cx_shfl(v, k), vp = cx_shfl(v, p);
  if (lane < n) st.f[b][lane] = lane == p ? vk : v;
  if (lane == 0) {
    const R d = cx_abs2(vp);
    const bool s = !(d >= Cx<C>::kTiny);
    st.p[b] = p;
    st.sing[b] = s;
    st.rinv[b] = s ? cx_zero<C>() : Cx<C>::mk(vp.x / d, -vp.y / d);
  }
}

// Solve M X = R in place (R <- X, M destroyed), partial pivoting.  One warp per column of
// [M | R], lane r holding row r.  At step k only the columns of M right of k and all of R
// are updated (M's columns <= k are never read again), and the warp that updates column
// k+1 of M also picks the pivot of step k+1, so a step costs one barrier.
template <class C>
__device__ void gj_solve(C* M, C* R, int n, GjStep<C>& st) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (warp == 0) gj_pivot(lane < n ? M[lane] : cx_zero<C>(), 0, n, st, 0);
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const int b = k & 1;
    const int p = st.p[b];
    const bool sing = st.sing[b] != 0;
    const C rinv = st.rinv[b];
    const C f = lane < n ? st.f[b][lane] : cx_zero<C>();
    // new value of row `lane` of column c from its old value vr
    auto update = [&](int c, C vr) -> C {
      const C vk = cx_shfl(vr, k), vp = cx_shfl(vr, p);
      const C own = lane == p ? vk : vr;  // row `lane` after the swap of rows k and p
      if (sing) return lane == k ? (c < n ? vp : cx_zero<C>()) : own;
      const C rk = cx_mul(vp, rinv);
      return lane == k ? rk : cx_sub(own, cx_mul(f, rk));
    };
    auto column = [&](int c) -> C* { return c < n ? M + n * c : R + n * (c - n); };
    int c = k + 1 + warp;
    // two columns at a time, so the loads and shuffles of one overlap those of the other;
    // the warp's first column is k + 1 only in the first pair (warp 0)
    for (; c + nw < 2 * n; c += 2 * nw) {
      C* col0 = column(c);
      C* col1 = column(c + nw);
      const C v0 = lane < n ? col0[lane] : cx_zero<C>();
      const C v1 = lane < n ? col1[lane] : cx_zero<C>();
      const C n0 = update(c, v0), n1 = update(c + nw, v1);
      if (lane < n) {
        col0[lane] = n0;
        col1[lane] = n1;
      }
      if (c == k + 1 && c < n) gj_pivot(n0, k + 1, n, st, b ^ 1);
    }
    if (c < 2 * n) {
      C* col = column(c);
      const C nv = update(c, lane < n ? col[lane] : cx_zero<C>());
      if (lane < n) col[lane] = nv;
      if (c == k + 1 && c < n) gj_pivot(nv, k + 1, n, st, b ^ 1);
    }
    __syncthreads();
  }
}

// dst = src^{-1}; src is preserved (copied to scratch first).
template <class C>
__device__ void mat_inv(C* dst, const C* src, C* scratch, int n, GjStep<C>& st) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    scratch[e] = src[e];
    dst[e] = Cx<C>::mk((e % n) == (e / n) ? 1 : 0, 0);
  }
  __syncthreads();
  gj_solve(scratch, dst, n, st);
}

// Block sum of a per-thread value (all threads receive it).
template <class R>
__device__ __forceinline__ R block_sum(R acc, R* red) {
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  R s = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

// || Y - I ||_F^2
template <class C>
__device__ typename Cx<C>::R dist_eye2(const C* Y, int n, typename Cx<C>::R* red) {
  typename Cx<C>::R acc = 0;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    C v = Y[e];
    if ((e % n) == (e / n)) v.x -= 1;
    acc += cx_abs2(v);
  }
  return block_sum(acc, red);
}

struct LogArgs {
  const double2* AB;    // [spoke][2][nc][nc]
  int nc;
  double2* vth;         // [spoke][nc][nc] = log(G)
  const double* gl_t;   // Gauss-Legendre nodes on [0, 1]
  const double* gl_w;
  int* err;
};

// One spoke: X = A^{-1} B in float64 (A is a Gram matrix: its condition number is the
// square of the data's), G = X^T, v = log(G) in float32 (the reference works in the data's
// float32 throughout).  Shared memory: the float64 pair (A, B) occupies the first 2 n^2
// double2 slots, and the six float32 matrices alias them; G is written to the float slot
// that overlaps A, which is dead once the solve ends.
__global__ void __launch_bounds__(1024) k_grog_solve_log(LogArgs a) {
  extern __shared__ __align__(16) unsigned char sraw[];
  const int n = a.nc, nn = n * n;
  __shared__ GjStep<double2> std_;
  __shared__ GjStep<float2> stf;
  __shared__ float red[32];
  {
    double2* Ad = reinterpret_cast<double2*>(sraw);
    double2* Bd = Ad + nn;
    const double2* AB = a.AB + (int64_t)blockIdx.x * 2 * nn;
    for (int e = threadIdx.x; e < 2 * nn; e += blockDim.x) Ad[e] = AB[e];
    __syncthreads();
    gj_solve(Ad, Bd, n, std_);  // Bd = A^{-1} B = X
    float2* Yf = reinterpret_cast<float2*>(sraw) + nn;  // second half of Ad
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      const int i = e % n, j = e / n;
      const double2 x = Bd[j + n * i];  // G = X^T
      Yf[e] = make_float2((float)x.x, (float)x.y);
    }
    __syncthreads();
  }
  float2* M = reinterpret_cast<float2*>(sraw);  // scratch
  float2* Y = M + nn;                           // root iterate
  float2* Z = M + 2 * nn;
  float2* T1 = M + 3 * nn;
  float2* T2 = M + 4 * nn;
  float2* L = M + 5 * nn;                       // log accumulator
  // inverse scaling: square roots until ||Y - I||_F <= 0.25, each by the product form of
  // the Denman-Beavers iteration (Cheng, Higham, Kenney and Laub, SIAM J. Matrix Anal.
  // Appl. 22, 2001): M0 = Y0 = A, Y <- Y (I + M^{-1}) / 2, M <- I/2 + (M + M^{-1}) / 4;
  // Y -> A^{1/2} and M -> I quadratically.  With Y = A^{1/2} (I + E), M = (I + E)^2 and the
  // step maps E to E^2 / 2: once ||M - I||_F^2 <= 1e-8 n, one more step brings E to the
  // float32 rounding level.
  int s = 0;
  while (s < 40 && dist_eye2(Y, n, red) > 0.0625f) {
    for (int e = threadIdx.x; e < nn; e += blockDim.x) Z[e] = Y[e];  // M
    __syncthreads();
    bool last = false;
    for (int it = 0; it < 40; ++it) {
      mat_inv(T1, Z, M, n, stf);  // M^{-1}
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {  // T2 = Y (I + M^{-1})
        const int i = e % n, j = e / n;
        float2 acc = Y[i + n * j];
        for (int l = 0; l < n; ++l) {
          const float2 u = Y[i + n * l], v = T1[l + n * j];
          acc.x = fmaf(u.x, v.x, fmaf(-u.y, v.y, acc.x));
          acc.y = fmaf(u.x, v.y, fmaf(u.y, v.x, acc.y));
        }
        T2[e] = acc;
      }
      __syncthreads();
      float dacc = 0.f;
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        const bool diag = (e % n) == (e / n);
        Y[e] = make_float2(0.5f * T2[e].x, 0.5f * T2[e].y);
        float2 m = make_float2(0.25f * (Z[e].x + T1[e].x) + (diag ? 0.5f : 0.f), 0.25f * (Z[e].y + T1[e].y));
        Z[e] = m;
        if (diag) m.x -= 1.f;
        dacc += m.x * m.x + m.y * m.y;
      }
      const float tot = block_sum(dacc, red);
      if (last) break;
      last = tot <= 1e-8f * n;
    }
    ++s;
  }
  if (s >= 40 && threadIdx.x == 0) atomicExch(a.err, 2);
  // log(I + X), X = Y - I:  sum_j w_j X (I + t_j X)^{-1}
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    float2 v = Y[e];
    if ((e % n) == (e / n)) v.x -= 1.f;
    Z[e] = v;  // X
    L[e] = make_float2(0.f, 0.f);
  }
  __syncthreads();
  for (int q = 0; q < kLogGL; ++q) {
    const float tq = (float)a.gl_t[q], wq = (float)a.gl_w[q];
    // solve (I + t X) W = X  ->  W = (I + t X)^{-1} X = X (I + t X)^{-1} (they commute)
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      float2 v = make_float2(tq * Z[e].x, tq * Z[e].y);
      if ((e % n) == (e / n)) v.x += 1.f;
      M[e] = v;
      T1[e] = Z[e];
    }
    __syncthreads();
    gj_solve(M, T1, n, stf);
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      L[e].x = fmaf(wq, T1[e].x, L[e].x);
      L[e].y = fmaf(wq, T1[e].y, L[e].y);
    }
    __syncthreads();
  }
  const double sc = ldexp(1.0, s);
  double2* out = a.vth + (int64_t)blockIdx.x * nn;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) out[e] = make_double2(sc * L[e].x, sc * L[e].y);
}
// nm (nspk x d) and the d x d pseudo-inverse factor P = (nm^T nm)^{-1}; single CTA.
struct NmArgs {
  const float* trj;   // (d, ns_pf, nt)
  int d, nr, spf;
  int64_t ns_pf, nt, nspk0;  // spokes of one repetition
  double* nm;         // [nspk0][d]
  double* Pinv;       // [d][d]
  int nrep;
};

__global__ void k_grog_nm(NmArgs a) {
  __shared__ double red[9][32];
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int64_t ip = threadIdx.x; ip < a.nspk0; ip += blockDim.x) {
    const int64_t t = ip / a.spf, sif = ip - t * a.spf;
    const int64_t s0 = sif * a.nr;
    double v[3];
    for (int dd = 0; dd < a.d; ++dd) {
      const float k0 = a.trj[dd + (int64_t)a.d * (s0 + a.ns_pf * t)];
      const float k1 = a.trj[dd + (int64_t)a.d * (s0 + 1 + a.ns_pf * t)];
      const float df = __fsub_rn(k1, k0);
      v[dd] = (double)__fmul_rn(df, (float)a.nr);  // Float32 diff times Int Nr -> Float32
      a.nm[ip * a.d + dd] = v[dd];
    }
    for (int p = 0; p < a.d; ++p)
      for (int q = 0; q < a.d; ++q) acc[p * 3 + q] += v[p] * v[q];
  }
  for (int e = 0; e < 9; ++e) {
    double x = acc[e];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) red[e][threadIdx.x >> 5] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double m[9];
    for (int e = 0; e < 9; ++e) {
      double s = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[e][w];
      m[e] = s * a.nrep;  // the nm rows repeat once per repetition
    }
    if (a.d == 2) {
      const double det = m[0] * m[4] - m[1] * m[3];
      a.Pinv[0] = m[4] / det;
      a.Pinv[1] = -m[1] / det;
      a.Pinv[2] = -m[3] / det;
      a.Pinv[3] = m[0] / det;
    } else {
      const double A = m[0], B = m[1], C = m[2], D = m[3], E = m[4], F = m[5], G = m[6], H = m[7], I = m[8];
      const double c00 = E * I - F * H, c01 = -(D * I - F * G), c02 = D * H - E * G;
      const double det = A * c00 + B * c01 + C * c02;
      double inv[9] = {c00, -(B * I - C * H), B * F - C * E, c01, A * I - C * G, -(A * F - C * D), c02,
                       -(A * H - B * G), A * E - B * D};
      for (int e = 0; e < 9; ++e) {
        const int r = e / 3, c = e % 3;
        a.Pinv[r * 3 + c] = inv[r * 3 + c] / det;
      }
    }
  }
}

// lnG[d, i, j] = sum_p (P nm^T)[d, p] v[p, i, j] over all spokes (all repetitions).
__global__ void k_grog_lng(const double* nm, const double* Pinv, const double2* vth, int d, int nc, int64_t nspk0,
                           int nrep, float2* lnG) {
  const int nn = nc * nc;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += gridDim.x * blockDim.x) {
    double2 acc[3] = {make_double2(0, 0), make_double2(0, 0), make_double2(0, 0)};
    for (int rep = 0; rep < nrep; ++rep)
      for (int64_t ip = 0; ip < nspk0; ++ip) {
        const double2 v = vth[(rep * nspk0 + ip) * nn + e];
        for (int dd = 0; dd < d; ++dd) {
          double c = 0.0;
          for (int q = 0; q < d; ++q) c += Pinv[dd * d + q] * nm[ip * d + q];
          acc[dd].x += c * v.x;
          acc[dd].y += c * v.y;
        }
      }
    for (int dd = 0; dd < d; ++dd) lnG[dd + (int64_t)d * e] = make_float2((float)acc[dd].x, (float)acc[dd].y);
  }
}

// ----------------------------------------------------------- gridding ---
// exp(shift L_d) v for every sample, factored as exp(s_j L_d) exp((shift - s_j) L_d) v with
// s_j = j h the table point nearest the shift: the table exp(s_j L_d), j = -J..J, is built
// once per call, and the remaining factor, ||(shift - s_j) L_d||_1 <= h ||L_d||_1 / 2 <= 1/2,
// needs a Taylor polynomial of degree <= 8 instead of a scaled degree-24 series.
constexpr int kGridTabMax = 8;       // J <= 8: 17 tables of n x n in shared memory
constexpr int kExpTaylor = 12;       // table entries: ||.||_1 <= 1 after scaling, 1/13! < 2^-32
constexpr float kGridTol = 7.4505806e-9f;  // 2^-27: Taylor truncation bound of the remainder

// Table of exp(s_j L) for s_j = (blockIdx.x - J) h, one CTA per entry: scaling to
// ||s_j L / 2^q||_1 <= 1, degree-12 Taylor polynomial by Horner, q squarings (float32,
// the precision the reference forms its exponentials in).
struct TabArgs {
  const float2* lnG;  // (d, nc, nc)
  int d, dd, n, J;
  float h, lnorm;     // table spacing, ||L_dd||_1
  float2* tab;        // [2J + 1][nc][nc]
};

__global__ void __launch_bounds__(1024) k_grog_exp_table(TabArgs a) {
  __shared__ float2 Y[kGrogMaxCoils * kGrogMaxCoils], E[kGrogMaxCoils * kGrogMaxCoils],
      T[kGrogMaxCoils * kGrogMaxCoils];
  const int n = a.n, nn = n * n;
  const float s = (float)((int)blockIdx.x - a.J) * a.h;
  const float nrm = fabsf(s) * a.lnorm;
  int q = 0;
  while (nrm > ldexpf(1.f, q) && q < 60) ++q;
  const float sc = ldexpf(s, -q);
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    const float2 l = a.lnG[a.dd + (int64_t)a.d * e];
    Y[e] = make_float2(sc * l.x, sc * l.y);
    E[e] = make_float2((e % n) == (e / n) ? 1.f : 0.f, 0.f);
  }
  __syncthreads();
  auto matmul = [&](const float2* A, const float2* B) {  // T = A B
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      const int i = e % n, c = e / n;
      float2 acc = make_float2(0.f, 0.f);
      for (int l = 0; l < n; ++l) acc = cadd(acc, cmul(A[i + n * l], B[l + n * c]));
      T[e] = acc;
    }
    __syncthreads();
  };
  for (int k = kExpTaylor; k >= 1; --k) {  // E <- I + (Y / k) E
    matmul(Y, E);
    const float rk = 1.f / (float)k;
    for (int e = threadIdx.x; e < nn; e += blockDim.x)
      E[e] = make_float2(((e % n) == (e / n) ? 1.f : 0.f) + rk * T[e].x, rk * T[e].y);
    __syncthreads();
  }
  for (int r = 0; r < q; ++r) {
    matmul(E, E);
    for (int e = threadIdx.x; e < nn; e += blockDim.x) E[e] = T[e];
    __syncthreads();
  }
  float2* out = a.tab + (int64_t)blockIdx.x * nn;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) out[e] = E[e];
}

struct GridArgs {
  float2* data;           // (ns_pf, nt, nc, nrep), in place
  const float* trj;       // (d, ns_pf, nt)
  const float2* lnG;      // (d, nc, nc)
  const float2* tab;      // [2J + 1][nc][nc] for dimension dd
  int32_t* trj_cart;      // (d, ns_pf, nt)
  int d, dd, nc, nrep, J;
  int64_t ns_pf, nt, Nd, nr;
  float h, lnorm;         // table spacing, ||lnG_dd||_1 (max column sum)
};

// One pass per dimension, in the reference's order.  One warp per (sample, frame); lane i
// owns coil i of every repetition.  The matrices sit in shared memory column-major:
// L at [0, n^2), table j at [(j + 1) n^2, (j + 2) n^2).
__global__ void __launch_bounds__(1024, 1) k_grog_grid(GridArgs a) {
  extern __shared__ float2 Ls[];
  const int n = a.nc, nn = n * n, ntab = 2 * a.J + 1;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) Ls[e] = a.lnG[a.dd + (int64_t)a.d * e];
  for (int e = threadIdx.x; e < ntab * nn; e += blockDim.x) Ls[nn + e] = a.tab[e];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t total = a.ns_pf * a.nt;
  // y = M w for the n x n matrix M at `Mat` (lane i gets row i)
  auto matvec = [&](const float2* Mat, float2 w) {
    float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
    for (int j = 0; j < n; j += 2) {
      const float2 w0 = make_float2(__shfl_sync(0xffffffffu, w.x, j), __shfl_sync(0xffffffffu, w.y, j));
      const float2 w1 = make_float2(__shfl_sync(0xffffffffu, w.x, j + 1), __shfl_sync(0xffffffffu, w.y, j + 1));
      if (lane < n) {
        acc0 = cadd(acc0, cmul(Mat[lane + n * j], w0));
        if (j + 1 < n) acc1 = cadd(acc1, cmul(Mat[lane + n * (j + 1)], w1));
      }
    }
    return cadd(acc0, acc1);
  };
  for (int64_t li = warp; li < total; li += nwarps) {
    const float p = __fmul_rn(a.trj[a.dd + (int64_t)a.d * li], (float)a.Nd);  // Float32 * Int -> Float32
    const double t = __dadd_rn((double)p, 0.5);                                // + 1/2 -> Float64
    const double k = rint(t);                                                  // round: ties to even
    const double shift = __ddiv_rn(__dmul_rn(__dsub_rn(k, t), (double)a.nr), (double)a.Nd);
    if (lane == 0) a.trj_cart[a.dd + (int64_t)a.d * li] = (int32_t)((int64_t)k + a.Nd / 2);
    const float s = (float)shift;
    const int j = max(-a.J, min(a.J, (int)rintf(s / a.h)));
    const float del = s - (float)j * a.h;
    const float nrm = fabsf(del) * a.lnorm;
    int q = 0;  // normally 0: the remainder is within half a table step
    while (nrm > ldexpf(1.f, q) && q < 20) ++q;
    const float x = ldexpf(nrm, -q), sq = ldexpf(del, -q);
    int m = 0;  // smallest degree with x^(m+1) / (m+1)! <= 2^-27
    for (float tm = x; tm > kGridTol && m < 30;) {
      ++m;
      tm *= x / (float)(m + 1);
    }
    const float2* Ej = Ls + (int64_t)(j + a.J + 1) * nn;
    for (int rep = 0; rep < a.nrep; ++rep) {
      float2 v = make_float2(0.f, 0.f);
      const int64_t base = li + total * ((int64_t)a.nc * rep);
      if (lane < n) v = a.data[base + total * lane];
      for (int rr = 0; rr < (1 << q); ++rr) {
        float2 w = v;  // Horner: w = v + (sq/m) L (v + (sq/(m-1)) L (... ))
        for (int mm = m; mm >= 1; --mm) {
          const float2 lw = matvec(Ls, w);
          const float c = sq / (float)mm;
          w = make_float2(v.x + c * lw.x, v.y + c * lw.y);
        }
        v = w;
      }
      v = matvec(Ej, v);
      if (lane < n) a.data[base + total * lane] = v;
    }
  }
}

static int grog_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 1;
  }();
  return n;
}

// Threads of the per-spoke logarithm CTA.
constexpr unsigned kGrogLogThreads = 256;

static void gauss_legendre01(int n, std::vector<double>& t, std::vector<double>& w) {
  t.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), pp = 0.0;
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
    t[i] = 0.5 * (1.0 - z);
    w[i] = 1.0 / ((1.0 - z * z) * pp * pp);  // (2 / ((1-z^2) pp^2)) / 2 on [0, 1]
  }
}

}  // namespace mrsr

using namespace mrsr;

extern "C" int mrsr_grog_calib(int ndims, int64_t nr, int64_t ns_per_frame, int64_t nt, int ncoils, int nrep,
                               const float* data, const float* trj, float* lnG_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3");
  MRSR_REQUIRE(data && trj && lnG_out, MRSR_ERR_ARG, "NULL argument to mrsr_grog_calib");
  MRSR_REQUIRE(nr >= 2 && ns_per_frame % nr == 0, MRSR_ERR_ARG, "samples per frame must be a multiple of Nr >= 2");
  MRSR_REQUIRE(ncoils >= 1 && ncoils <= kGrogMaxCoils, MRSR_ERR_UNSUPPORTED, "GROG supports 1..%d coils",
               kGrogMaxCoils);
  MRSR_REQUIRE(nrep >= 1, MRSR_ERR_ARG, "nrep must be >= 1");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int spf = (int)(ns_per_frame / nr);
  const int64_t nspk0 = (int64_t)spf * nt, nspk = nspk0 * nrep;
  const int nn = ncoils * ncoils;
  DevBuf AB, vth, nm, Pinv, glt, glw, err;
  MRSR_TRY(AB.alloc(sizeof(double2) * 2 * nn * nspk));
  MRSR_TRY(vth.alloc(sizeof(double2) * nn * nspk));
  MRSR_TRY(nm.alloc(sizeof(double) * ndims * nspk0));
  MRSR_TRY(Pinv.alloc(sizeof(double) * 9));
  std::vector<double> t, w;
  gauss_legendre01(kLogGL, t, w);
  MRSR_TRY(glt.alloc(sizeof(double) * kLogGL));
  MRSR_TRY(glw.alloc(sizeof(double) * kLogGL));
  MRSR_TRY(copy_h2d(glt.p, t.data(), sizeof(double) * kLogGL));
  MRSR_TRY(copy_h2d(glw.p, w.data(), sizeof(double) * kLogGL));
  MRSR_TRY(err.alloc(sizeof(int)));
  MRSR_CHECK_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  const size_t smem_g = sizeof(float2) * (kGramRows + 1) * (ncoils + 1);
  GramArgs ga{reinterpret_cast<const float2*>(data), ns_per_frame, nt, ncoils, nrep, (int)nr, spf, AB.as<double2>()};
  k_grog_gram<<<(unsigned)nspk, 1024, smem_g, st>>>(ga);
  MRSR_LAUNCH_CHECK();
  const size_t smem_l = std::max(sizeof(double2) * 2, sizeof(float2) * 6) * nn;
  // opt in whatever the size: the dynamic part plus the kernel's static pivot records can pass 48 KB
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_grog_solve_log, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_l));
  LogArgs la{AB.as<double2>(), ncoils, vth.as<double2>(), glt.as<double>(), glw.as<double>(), err.as<int>()};
  k_grog_solve_log<<<(unsigned)nspk, kGrogLogThreads, smem_l, st>>>(la);
  MRSR_LAUNCH_CHECK();
  NmArgs na{trj, ndims, (int)nr, spf, ns_per_frame, nt, nspk0, nm.as<double>(), Pinv.as<double>(), nrep};
  k_grog_nm<<<1, 1024, 0, st>>>(na);
  MRSR_LAUNCH_CHECK();
  k_grog_lng<<<(unsigned)cdiv(nn, 128), 128, 0, st>>>(nm.as<double>(), Pinv.as<double>(), vth.as<double2>(), ndims,
                                                     ncoils, nspk0, nrep, reinterpret_cast<float2*>(lnG_out));
  MRSR_LAUNCH_CHECK();
  int herr = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  MRSR_REQUIRE(herr == 0, MRSR_ERR_ARG, "matrix logarithm did not converge (a spoke operator has eigenvalues near 0)");
  return MRSR_OK;
}

extern "C" int mrsr_grog_gridding(int ndims, const int64_t* img_shape, int64_t nr, int64_t ns_per_frame, int64_t nt,
                                  int ncoils, int nrep, float* data, const float* trj, const float* lnG,
                                  int32_t* trj_cart_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3");
  MRSR_REQUIRE(img_shape && data && trj && lnG && trj_cart_out, MRSR_ERR_ARG, "NULL argument to mrsr_grog_gridding");
  MRSR_REQUIRE(ncoils >= 1 && ncoils <= kGrogMaxCoils, MRSR_ERR_UNSUPPORTED, "GROG supports 1..%d coils",
               kGrogMaxCoils);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  // ||lnG_d||_1 on the host (tiny)
  std::vector<float2> h((size_t)ndims * ncoils * ncoils);
  MRSR_CHECK_CUDA(cudaMemcpyAsync(h.data(), lnG, sizeof(float2) * h.size(), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  const int nn = ncoils * ncoils;
  DevBuf tab;
  MRSR_TRY(tab.alloc(sizeof(float2) * (2 * kGridTabMax + 1) * nn * ndims));
  const int64_t total = ns_per_frame * nt;
  for (int dd = 0; dd < ndims; ++dd) {
    float lnorm = 0.f;
    for (int j = 0; j < ncoils; ++j) {
      float s = 0.f;
      for (int i = 0; i < ncoils; ++i) {
        const float2 v = h[dd + (size_t)ndims * (i + (size_t)ncoils * j)];
        s += std::sqrt(v.x * v.x + v.y * v.y);
      }
      lnorm = std::max(lnorm, s);
    }
    // |shift| <= Nr / (2 N_d); spacing h with h ||L||_1 <= 1 unless that needs more than 2 kGridTabMax + 1 tables
    const double smax = 0.5 * (double)nr / (double)img_shape[dd];
    int J = 0;
    float hs = 1.f;
    if (lnorm > 0.f) {
      J = (int)std::min<double>(kGridTabMax, std::ceil(smax * lnorm));
      hs = J > 0 ? (float)std::max(1.0 / lnorm, smax / J) : 1.f;
    }
    float2* tabd = tab.as<float2>() + (size_t)dd * (2 * kGridTabMax + 1) * nn;
    TabArgs ta{reinterpret_cast<const float2*>(lnG), ndims, dd, ncoils, J, hs, lnorm, tabd};
    k_grog_exp_table<<<(unsigned)(2 * J + 1), 1024, 0, st>>>(ta);
    MRSR_LAUNCH_CHECK();
    GridArgs g{};
    g.data = reinterpret_cast<float2*>(data);
    g.trj = trj;
    g.lnG = reinterpret_cast<const float2*>(lnG);
    g.tab = tabd;
    g.trj_cart = trj_cart_out;
    g.d = ndims;
    g.dd = dd;
    g.nc = ncoils;
    g.nrep = nrep;
    g.J = J;
    g.ns_pf = ns_per_frame;
    g.nt = nt;
    g.Nd = img_shape[dd];
    g.nr = nr;
    g.h = hs;
    g.lnorm = lnorm;
    const size_t smem = sizeof(float2) * (size_t)(2 * J + 2) * nn;
    MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_grog_grid, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(cdiv(total, 32), grog_sms()));
    k_grog_grid<<<blocks, 1024, smem, st>>>(g);
    MRSR_LAUNCH_CHECK();
  }
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return MRSR_OK;
}
