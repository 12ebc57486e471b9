// GROG self-calibration and gridding (src/GROG.jl).
//
// grog_calib (src/GROG.jl:14-51), per spoke of Nr samples and Nc coils:
//   G = (D1 \ D2)^T with D1 = rows 1..Nr-1, D2 = rows 2..Nr,   v = log(G),
// then lnG[:, i, j] = nm \ v[:, i, j] over all spokes, nm = Nr * (k_2 - k_1).
// The least squares run in float64 through the normal equations (Gram
// matrices accumulated in float64, Gauss-Jordan with partial pivoting); the
// principal matrix logarithm uses inverse scaling and squaring: Denman-Beavers
// square roots until ||Y - I||_F <= 1/4, then log(I + X) by the m-point
// Gauss-Legendre quadrature of int_0^1 X (I + t X)^{-1} dt (the diagonal Pade
// approximant), times 2^s (Higham, Functions of Matrices, SIAM 2008, ch. 11).
//
// grog_gridding! (src/GROG.jl:73-102): per sample and dimension the grid index
// follows the reference's float32/float64 promotion bit for bit, and
// data <- exp(shift lnG_d) data is applied as a Horner-evaluated Taylor series
// of the action on the Nc x Nrep block (the reference forms the Higham-2005
// Pade exponential of the float32 matrix and multiplies).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace mrsr {

constexpr int kGrogMaxCoils = 32;
constexpr int kLogGL = 12;  // Gauss-Legendre nodes of the log quadrature

__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 zmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zconjmul(double2 a, double2 b) {  // conj(a) * b
  return make_double2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double2 zdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return make_double2((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}
__device__ __forceinline__ double zabs2(double2 a) { return a.x * a.x + a.y * a.y; }

// ------------------------------------------------------- spoke Grams ---
// A = D1^H D1, B = D1^H D2 for spoke `blockIdx.x`; one thread per (i, j).
struct GramArgs {
  const float2* data;   // (ns_pf, nt, nc, nrep)
  int64_t ns_pf, nt;
  int nc, nrep, nr, spf;  // spokes per frame
  double2* AB;          // [spoke][2][nc][nc] (column-major i + nc j)
};

__global__ void __launch_bounds__(1024) k_grog_gram(GramArgs a) {
  extern __shared__ float2 sd[];  // [c][r] spoke samples
  const int64_t ip = blockIdx.x;
  const int64_t rep = ip / ((int64_t)a.spf * a.nt);
  const int64_t rem = ip - rep * a.spf * a.nt;
  const int64_t t = rem / a.spf;
  const int64_t sif = rem - t * a.spf;
  const int64_t ns_tot = a.ns_pf * a.nt;
  for (int e = threadIdx.x; e < a.nr * a.nc; e += blockDim.x) {
    const int r = e % a.nr, c = e / a.nr;
    sd[c * a.nr + r] = a.data[(sif * a.nr + r) + a.ns_pf * t + ns_tot * (c + (int64_t)a.nc * rep)];
  }
  __syncthreads();
  const int i = threadIdx.x % kGrogMaxCoils, j = threadIdx.x / kGrogMaxCoils;
  if (i < a.nc && j < a.nc) {
    double2 s1 = make_double2(0, 0), s2 = make_double2(0, 0);
    for (int r = 0; r + 1 < a.nr; ++r) {
      const float2 di = sd[i * a.nr + r];
      const float2 dj = sd[j * a.nr + r];
      const float2 dj1 = sd[j * a.nr + r + 1];
      const double2 ci = make_double2(di.x, di.y);
      s1 = zadd(s1, zconjmul(ci, make_double2(dj.x, dj.y)));
      s2 = zadd(s2, zconjmul(ci, make_double2(dj1.x, dj1.y)));
    }
    double2* out = a.AB + ip * 2 * a.nc * a.nc;
    out[i + a.nc * j] = s1;
    out[a.nc * a.nc + i + a.nc * j] = s2;
  }
}

// ------------------------------------------ small dense linear algebra ---
// All routines: one CTA of 1024 threads, n <= 32, column-major n x n in shared memory.

// Solve M X = R in place (M destroyed, R <- X), partial pivoting; M, R n x n.
__device__ void gj_solve(double2* M, double2* R, int n, int* piv_s) {
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = zabs2(M[k + n * k]);
      for (int r = k + 1; r < n; ++r) {
        const double v = zabs2(M[r + n * k]);
        if (v > best) {
          best = v;
          p = r;
        }
      }
      *piv_s = p;
    }
    __syncthreads();
    const int p = *piv_s;
    if (p != k) {
      for (int c = threadIdx.x; c < 2 * n; c += blockDim.x) {
        double2* col = c < n ? M + n * c : R + n * (c - n);
        const double2 tmp = col[k];
        col[k] = col[p];
        col[p] = tmp;
      }
      __syncthreads();
    }
    const double2 pivot = M[k + n * k];
    __syncthreads();
    if (zabs2(pivot) < 1e-280) {  // exactly singular column: basic solution with x_k = 0
      for (int c = threadIdx.x; c < n; c += blockDim.x) R[k + n * c] = make_double2(0.0, 0.0);
      __syncthreads();
      continue;
    }
    // row k scaled
    for (int c = threadIdx.x; c < 2 * n; c += blockDim.x) {
      double2* col = c < n ? M + n * c : R + n * (c - n);
      col[k] = zdiv(col[k], pivot);
    }
    __syncthreads();
    // eliminate column k from the other rows
    for (int e = threadIdx.x; e < n * 2 * n; e += blockDim.x) {
      const int r = e % n, c = e / n;
      if (r == k) continue;
      double2* col = c < n ? M + n * c : R + n * (c - n);
      const double2 f = M[r + n * k];
      if (c == k) continue;
      col[r] = zsub(col[r], zmul(f, col[k]));
    }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x)
      if (r != k) M[r + n * k] = make_double2(0.0, 0.0);
    __syncthreads();
  }
}

__device__ void mat_copy(double2* dst, const double2* src, int n) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) dst[e] = src[e];
  __syncthreads();
}
__device__ void mat_eye(double2* dst, int n) {
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) dst[e] = make_double2((e % n) == (e / n) ? 1.0 : 0.0, 0.0);
  __syncthreads();
}
// dst = inverse(src) (src preserved through a scratch copy)
__device__ void mat_inv(double2* dst, const double2* src, double2* scratch, int n, int* piv_s) {
  mat_copy(scratch, src, n);
  mat_eye(dst, n);
  gj_solve(scratch, dst, n, piv_s);
}

// || Y - I ||_F^2 into *out (thread 0 reduces)
__device__ double dist_eye2(const double2* Y, int n, double* red) {
  double acc = 0.0;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    double2 v = Y[e];
    if ((e % n) == (e / n)) v.x -= 1.0;
    acc += zabs2(v);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
  __syncthreads();
  return s;
}

struct LogArgs {
  const double2* AB;    // [spoke][2][nc][nc]
  int nc;
  double2* vth;         // [spoke][nc][nc] = log(G)
  const double* gl_t;   // Gauss-Legendre nodes on [0, 1]
  const double* gl_w;
  int* err;
};

// One spoke: X = A^{-1} B, G = X^T, v = log(G).
__global__ void __launch_bounds__(1024) k_grog_solve_log(LogArgs a) {
  extern __shared__ double2 sm[];
  const int n = a.nc, nn = n * n;
  double2* M = sm;            // scratch / A
  double2* Y = sm + nn;       // root iterate
  double2* Z = sm + 2 * nn;
  double2* T1 = sm + 3 * nn;
  double2* T2 = sm + 4 * nn;
  double2* L = sm + 5 * nn;   // log accumulator
  __shared__ int piv;
  __shared__ double red[32];
  const double2* AB = a.AB + (int64_t)blockIdx.x * 2 * nn;
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    M[e] = AB[e];
    T1[e] = AB[nn + e];
  }
  __syncthreads();
  gj_solve(M, T1, n, &piv);  // T1 = A^{-1} B = X
  // G = X^T
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    const int i = e % n, j = e / n;
    Y[e] = T1[j + n * i];
  }
  __syncthreads();
  // inverse scaling: square roots until ||Y - I||_F <= 0.25, each by the product form of
  // the Denman-Beavers iteration (Cheng, Higham, Kenney and Laub, SIAM J. Matrix Anal.
  // Appl. 22, 2001): M0 = Y0 = A, Y <- Y (I + M^{-1}) / 2, M <- I/2 + (M + M^{-1}) / 4;
  // Y -> A^{1/2} and M -> I quadratically.  One inversion per step, and the stopping
  // test ||M - I||_F^2 <= 1e-26 n is scale free (M tends to I whatever the size of A).
  int s = 0;
  while (s < 40 && dist_eye2(Y, n, red) > 0.0625) {
    mat_copy(Z, Y, n);  // M
    for (int it = 0; it < 60; ++it) {
      mat_inv(T1, Z, M, n, &piv);  // M^{-1}
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {  // T2 = Y (I + M^{-1})
        const int i = e % n, j = e / n;
        double2 acc = Y[i + n * j];
        for (int l = 0; l < n; ++l) {
          const double2 u = Y[i + n * l], v = T1[l + n * j];
          acc.x += u.x * v.x - u.y * v.y;
          acc.y += u.x * v.y + u.y * v.x;
        }
        T2[e] = acc;
      }
      __syncthreads();
      double dacc = 0.0;
      for (int e = threadIdx.x; e < nn; e += blockDim.x) {
        const bool diag = (e % n) == (e / n);
        Y[e] = make_double2(0.5 * T2[e].x, 0.5 * T2[e].y);
        double2 m = make_double2(0.25 * (Z[e].x + T1[e].x) + (diag ? 0.5 : 0.0), 0.25 * (Z[e].y + T1[e].y));
        Z[e] = m;
        if (diag) m.x -= 1.0;
        dacc += zabs2(m);
      }
      for (int o = 16; o > 0; o >>= 1) dacc += __shfl_down_sync(0xffffffffu, dacc, o);
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = dacc;
      __syncthreads();
      double tot = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += red[w];
      __syncthreads();
      if (tot < 1e-26 * n) break;
    }
    ++s;
  }
  if (s >= 40 && threadIdx.x == 0) atomicExch(a.err, 2);
  // log(I + X), X = Y - I:  sum_j w_j X (I + t_j X)^{-1}
  for (int e = threadIdx.x; e < nn; e += blockDim.x) {
    double2 v = Y[e];
    if ((e % n) == (e / n)) v.x -= 1.0;
    Z[e] = v;  // X
    L[e] = make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int q = 0; q < kLogGL; ++q) {
    const double tq = a.gl_t[q], wq = a.gl_w[q];
    // solve (I + t X) W = X  ->  W = (I + t X)^{-1} X = X (I + t X)^{-1} (they commute)
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      double2 v = make_double2(tq * Z[e].x, tq * Z[e].y);
      if ((e % n) == (e / n)) v.x += 1.0;
      M[e] = v;
      T1[e] = Z[e];
    }
    __syncthreads();
    gj_solve(M, T1, n, &piv);
    for (int e = threadIdx.x; e < nn; e += blockDim.x) {
      L[e].x += wq * T1[e].x;
      L[e].y += wq * T1[e].y;
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
struct GridArgs {
  float2* data;           // (ns_pf, nt, nc, nrep), in place
  const float* trj;       // (d, ns_pf, nt)
  const float2* lnG;      // (d, nc, nc)
  int32_t* trj_cart;      // (d, ns_pf, nt)
  int d, nc, nrep;
  int64_t ns_pf, nt, N[3], nr;
  float lnorm[3];         // ||lnG_d||_1 (max column sum)
};

// One warp per (sample, frame); lane i owns coil i of every repetition.
__global__ void __launch_bounds__(256) k_grog_grid(GridArgs a) {
  __shared__ float2 Ls[3][kGrogMaxCoils * kGrogMaxCoils];
  const int n = a.nc;
  for (int e = threadIdx.x; e < a.d * n * n; e += blockDim.x) {
    const int dd = e / (n * n), ij = e - dd * n * n;
    Ls[dd][ij] = a.lnG[dd + (int64_t)a.d * ij];  // Ls[d][i + n j] = lnG[d][i, j]
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t total = a.ns_pf * a.nt;
  for (int64_t li = warp; li < total; li += nwarps) {
    double shift[3];
    for (int dd = 0; dd < a.d; ++dd) {
      const int64_t Nd = a.N[dd];
      const float p = __fmul_rn(a.trj[dd + (int64_t)a.d * li], (float)Nd);   // Float32 * Int -> Float32
      const double t = __dadd_rn((double)p, 0.5);                             // + 1/2 -> Float64
      const double k = rint(t);                                              // round: ties to even
      shift[dd] = __ddiv_rn(__dmul_rn(__dsub_rn(k, t), (double)a.nr), (double)Nd);
      if (lane == 0) a.trj_cart[dd + (int64_t)a.d * li] = (int32_t)((int64_t)k + Nd / 2);
    }
    for (int rep = 0; rep < a.nrep; ++rep) {
      float2 v = make_float2(0.f, 0.f);
      const int64_t base = li + total * ((int64_t)a.nc * rep);
      if (lane < n) v = a.data[base + total * lane];
      for (int dd = 0; dd < a.d; ++dd) {
        const float s = (float)shift[dd];
        const float nrm = fabsf(s) * a.lnorm[dd];
        int q = 0;  // scaling: exp(A) = exp(A / 2^q)^(2^q) with ||A / 2^q|| <= 2
        while (nrm > 2.0f * (float)(1 << q) && q < 20) ++q;
        const float sq = ldexpf(s, -q);
        for (int rr = 0; rr < (1 << q); ++rr) {
          // Horner: w = v + (s/M) L (v + (s/(M-1)) L (... ))
          float2 w = v;
          for (int m = 24; m >= 1; --m) {
            float2 lw = make_float2(0.f, 0.f);
            for (int j = 0; j < n; ++j) {
              const float2 wj = make_float2(__shfl_sync(0xffffffffu, w.x, j), __shfl_sync(0xffffffffu, w.y, j));
              if (lane < n) lw = cadd(lw, cmul(Ls[dd][lane + n * j], wj));
            }
            const float c = sq / (float)m;
            w = make_float2(v.x + c * lw.x, v.y + c * lw.y);
          }
          v = w;
        }
      }
      if (lane < n) a.data[base + total * lane] = v;
    }
  }
}

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
  MRSR_REQUIRE((size_t)nr * ncoils * sizeof(float2) <= 200 * 1024, MRSR_ERR_UNSUPPORTED, "spoke too long for GROG");
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
  const size_t smem_g = sizeof(float2) * nr * ncoils;
  if (smem_g > 48 * 1024)
    MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_grog_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_g));
  GramArgs ga{reinterpret_cast<const float2*>(data), ns_per_frame, nt, ncoils, nrep, (int)nr, spf, AB.as<double2>()};
  k_grog_gram<<<(unsigned)nspk, 1024, smem_g, st>>>(ga);
  MRSR_LAUNCH_CHECK();
  const size_t smem_l = sizeof(double2) * 6 * nn;
  if (smem_l > 48 * 1024)
    MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_grog_solve_log, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_l));
  LogArgs la{AB.as<double2>(), ncoils, vth.as<double2>(), glt.as<double>(), glw.as<double>(), err.as<int>()};
  k_grog_solve_log<<<(unsigned)nspk, 1024, smem_l, st>>>(la);
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
  GridArgs g{};
  g.data = reinterpret_cast<float2*>(data);
  g.trj = trj;
  g.lnG = reinterpret_cast<const float2*>(lnG);
  g.trj_cart = trj_cart_out;
  g.d = ndims;
  g.nc = ncoils;
  g.nrep = nrep;
  g.ns_pf = ns_per_frame;
  g.nt = nt;
  g.nr = nr;
  for (int i = 0; i < 3; ++i) g.N[i] = i < ndims ? img_shape[i] : 1;
  // ||lnG_d||_1 on the host (tiny)
  std::vector<float2> h((size_t)ndims * ncoils * ncoils);
  MRSR_CHECK_CUDA(cudaMemcpyAsync(h.data(), lnG, sizeof(float2) * h.size(), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  for (int dd = 0; dd < ndims; ++dd) {
    float best = 0.f;
    for (int j = 0; j < ncoils; ++j) {
      float s = 0.f;
      for (int i = 0; i < ncoils; ++i) {
        const float2 v = h[dd + (size_t)ndims * (i + (size_t)ncoils * j)];
        s += std::sqrt(v.x * v.x + v.y * v.y);
      }
      best = std::max(best, s);
    }
    g.lnorm[dd] = best;
  }
  const int64_t total = ns_per_frame * nt;
  const unsigned blocks = (unsigned)std::min<int64_t>(cdiv(total * 32, 256), 152 * 32);
  k_grog_grid<<<blocks, 256, 0, st>>>(g);
  MRSR_LAUNCH_CHECK();
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return MRSR_OK;
}
