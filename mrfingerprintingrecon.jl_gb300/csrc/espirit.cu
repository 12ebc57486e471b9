// ESPIRiT coil-sensitivity estimation on the device: the last step of
// calculate_coil_maps (src/CoilMaps.jl:55-57, :89-91), which the reference hands to
// MRICoilSensitivities.jl's `espirit` on the host even in its GPU extension
// (ext/MRISubspaceReconCUDAExt/CoilMaps.jl:29-31: `espirit(Array(kbp), ...)`).
//
// The algorithm is the published one (Uecker, Lai, Murphy, Virtue, Elad, Pauly,
// Vasanawala, Lustig, Magn. Reson. Med. 71, 2014):
//  1. calibration matrix: one row per position p of a k^d kernel inside the centred
//     calibration k-space kbp (calib..., Nc); here its transpose B (n = k^d Nc rows,
//     one column per position, column p = the patch of position p, kernel offsets
//     kappa column-major, coil outermost);
//  2. its signal subspace: B's left singular vectors with sigma >= eigThresh_1 sigma_max,
//     by a one-sided (Hestenes) Jacobi SVD on B's columns -- the columns converge to
//     sigma_i w_i with w_i the left singular vectors, which span the patches;
//  3. the patch-space projector P = sum w_i w_i^H and its kernel-offset sums
//     Q_cc'(delta) = sum_kappa P[(kappa, c), (kappa + delta, c')];
//  4. the image-space operator at every pixel r of the N^d image (centre N/2):
//     W(r)_cc' = (1/k^d) sum_delta Q_cc'(delta) exp(-2 pi i delta.(r - N/2)/N), one
//     forward FFT per coil pair of Q placed on the image grid (the shift by N/2 is the
//     phase exp(2 pi i delta.(N/2)/N) on Q, a sign (-1)^(sum delta) for even N);
//  5. per pixel, the leading eigenvector(s) of the Hermitian Nc x Nc W(r) by power
//     iteration (one warp per pixel, lane c holding row c; the second map after
//     deflation), zero where the eigenvalue is below eigThresh_2, rotated so that the
//     coil-1 entry is real and non-negative.
#include <algorithm>
#include <cmath>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "fftnd.cuh"

namespace mrsr {

namespace cg = cooperative_groups;

namespace {

constexpr int kEspMaxCoils = 32;   // one lane per coil in the per-pixel eigensolver
constexpr int kEspMaxMaps = 2;
constexpr int kJacThreads = 128;
constexpr int kEspIters = 120;     // power-iteration matrix products per map
constexpr int kMaxSweeps = 40;
constexpr float kJacTol = 1e-5f;   // |b_i^H b_j| <= tol |b_i| |b_j| counts as orthogonal (float32 dots)

struct EspGeom {
  int64_t calib[3], k[3], np[3], img[3];
  int64_t ncal, npos, M, n, nimg;
  int Nc, nq;
};

__global__ void k_esp_patches(const float2* kbp, EspGeom g, float2* B) {
  const int64_t total = g.n * g.npos;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = e % g.n, p = e / g.n;
    const int64_t c = a / g.M, kap = a - c * g.M;
    const int64_t k0 = kap % g.k[0], k1 = (kap / g.k[0]) % g.k[1], k2 = kap / (g.k[0] * g.k[1]);
    const int64_t p0 = p % g.np[0], p1 = (p / g.np[0]) % g.np[1], p2 = p / (g.np[0] * g.np[1]);
    const int64_t idx = (p0 + k0) + g.calib[0] * ((p1 + k1) + g.calib[1] * (p2 + k2));
    B[e] = kbp[idx + g.ncal * c];
  }
}

__global__ void k_esp_fro2(const float2* B, int64_t total, double* out) {
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = B[e];
    s += (double)v.x * v.x + (double)v.y * v.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(out, t);
  }
}

// One round of the round-robin ("circle") schedule over m2 = m + (m & 1) columns: the
// block's pair is (t, m2 - 1) for block 0, ((t + k) % (m2 - 1), (t - k) mod (m2 - 1)) for
// block k; pairs touching the padding column (index m) are skipped.  Columns whose energy
// is below 1e-10 of the matrix's are left alone (null directions would keep exchanging
// rounding noise).  A rotation that makes the pair orthogonal is applied when
// |b_i^H b_j| > tol |b_i| |b_j| and |b_i^H b_j| > 1e-10 |B|_F^2, and counted: the second
// bound stops pairs of weak columns (far below the eigThresh_1 cut) from chasing the
// float32 rounding that rotations of strong columns leave in them.
__device__ __forceinline__ void esp_jacobi_pair(float2* B, int64_t n, int m, int m2, int t, const double* fro2,
                                                float tol, int* nrot) {
  const int k = blockIdx.x;
  int i, j;
  if (k == 0) {
    i = t;
    j = m2 - 1;
  } else {
    i = (t + k) % (m2 - 1);
    j = (t - k + (m2 - 1)) % (m2 - 1);
  }
  if (i >= m || j >= m) return;
  float2* bi = B + (int64_t)i * n;
  float2* bj = B + (int64_t)j * n;
  float a = 0.f, b = 0.f, gr = 0.f, gi = 0.f;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const float2 u = bi[e], v = bj[e];
    a = fmaf(u.x, u.x, fmaf(u.y, u.y, a));
    b = fmaf(v.x, v.x, fmaf(v.y, v.y, b));
    gr = fmaf(u.x, v.x, fmaf(u.y, v.y, gr));   // Re(conj(u) v)
    gi = fmaf(u.x, v.y, fmaf(-u.y, v.x, gi));  // Im(conj(u) v)
  }
  __shared__ double red[4][kJacThreads / 32];
  double s[4] = {a, b, gr, gi};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = s[q];
  }
  __syncthreads();
  double A = 0.0, Bn = 0.0, Gr = 0.0, Gi = 0.0;
  for (int w = 0; w < kJacThreads / 32; ++w) {
    A += red[0][w];
    Bn += red[1][w];
    Gr += red[2][w];
    Gi += red[3][w];
  }
  const double g = sqrt(Gr * Gr + Gi * Gi);
  const double floor2 = 1e-10 * *fro2;
  if (fmax(A, Bn) <= floor2 || !(g > (double)tol * sqrt(A * Bn)) || !(g > floor2)) return;
  // real Jacobi rotation in the plane of b_i and e^{-i phi} b_j (b_i^H b_j = g e^{i phi}):
  // tan(theta) = t solves t^2 + 2 zeta t - 1 = 0, zeta = (|b_j|^2 - |b_i|^2) / (2 g), smaller root
  const double zeta = (Bn - A) / (2.0 * g);
  const double tt = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
  const double cs = 1.0 / sqrt(1.0 + tt * tt);
  const float c = (float)cs, sn = (float)(cs * tt);
  const float ph_r = (float)(Gr / g), ph_i = (float)(Gi / g);
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const float2 u = bi[e], v = bj[e];
    const float2 ev = make_float2(v.x * ph_r + v.y * ph_i, v.y * ph_r - v.x * ph_i);  // e^{-i phi} v
    const float2 eu = make_float2(u.x * ph_r - u.y * ph_i, u.y * ph_r + u.x * ph_i);  // e^{+i phi} u
    bi[e] = make_float2(c * u.x - sn * ev.x, c * u.y - sn * ev.y);
    bj[e] = make_float2(sn * eu.x + c * v.x, sn * eu.y + c * v.y);
  }
  if (threadIdx.x == 0) atomicAdd(nrot, 1);
}

// one round per launch
__global__ void __launch_bounds__(kJacThreads) k_esp_jacobi(float2* B, int64_t n, int m, int m2, int t,
                                                           const double* fro2, float tol, int* nrot) {
  esp_jacobi_pair(B, n, m, m2, t, fro2, tol, nrot);
}

// A whole sweep (the m2 - 1 rounds) in one cooperative launch: every CTA takes its pair of
// the round, then the grid synchronises before the next round.  The launch is cooperative,
// so all m2 / 2 CTAs are resident and the grid barrier always completes; 361 round launches
// of ~14 us each (launch and latency bound) become one.
__global__ void __launch_bounds__(kJacThreads) k_esp_jacobi_sweep(float2* B, int64_t n, int m, int m2,
                                                                 const double* fro2, float tol, int* nrot) {
  cg::grid_group grid = cg::this_grid();
  for (int t = 0; t < m2 - 1; ++t) {
    esp_jacobi_pair(B, n, m, m2, t, fro2, tol, nrot);
    grid.sync();
  }
}

// sig2[p] = |column p|^2 and the largest of them (float bits, non-negative: atomicMax)
__global__ void k_esp_colnorm(const float2* B, int64_t n, int m, float* sig2, unsigned* maxbits) {
  const int p = blockIdx.x;
  if (p >= m) return;
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const float2 v = B[(int64_t)p * n + e];
    s += (double)v.x * v.x + (double)v.y * v.y;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    sig2[p] = (float)t;
    atomicMax(maxbits, __float_as_uint((float)t));
  }
}

// wgt[p] = 1 / sigma_p^2 for the kept columns (sigma_p >= thr sigma_max), else 0
__global__ void k_esp_weights(const float* sig2, int m, const unsigned* maxbits, float thr, float* wgt) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < m; p += gridDim.x * blockDim.x) {
    const float smax2 = __uint_as_float(*maxbits);
    const bool keep = smax2 > 0.f && sig2[p] >= thr * thr * smax2 && sig2[p] > 0.f;
    wgt[p] = keep ? 1.f / sig2[p] : 0.f;
  }
}

// P[a, b] = sum_p wgt[p] B[a, p] conj(B[b, p])   (n x n, column-major), 16 x 16 tiles
__global__ void k_esp_proj(const float2* B, const float* wgt, int64_t n, int m, float2* P) {
  __shared__ float2 sa[16][17], sb[16][17];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int64_t a = (int64_t)blockIdx.y * 16 + ty, bb = (int64_t)blockIdx.x * 16 + tx;
  float2 acc = make_float2(0.f, 0.f);
  for (int p0 = 0; p0 < m; p0 += 16) {
    const int pa = p0 + tx;
    const int64_t ra = (int64_t)blockIdx.y * 16 + ty, rb = (int64_t)blockIdx.x * 16 + ty;
    float2 va = make_float2(0.f, 0.f), vb = make_float2(0.f, 0.f);
    if (pa < m) {
      const float w = wgt[pa];
      if (ra < n) {
        va = B[(int64_t)pa * n + ra];
        va = make_float2(va.x * w, va.y * w);
      }
      if (rb < n) vb = B[(int64_t)pa * n + rb];
    }
    sa[ty][tx] = va;  // row ra, position p0 + tx
    sb[ty][tx] = vb;  // row rb, position p0 + tx
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float2 u = sa[ty][q], v = sb[tx][q];
      acc.x = fmaf(u.x, v.x, fmaf(u.y, v.y, acc.x));   // u conj(v)
      acc.y = fmaf(u.y, v.x, fmaf(-u.x, v.y, acc.y));
    }
    __syncthreads();
  }
  if (a < n && bb < n) P[a + n * bb] = acc;
}

__host__ __device__ inline int pair_index(int a, int b, int Nc) { return a * Nc - a * (a - 1) / 2 + (b - a); }

// plane[pair(c, c')][delta mod N] = exp(2 pi i delta.(N/2)/N) / M sum_kappa P[(kappa, c), (kappa + delta, c')]
// for c <= c' and every offset delta in (-k, k)^d (planes zeroed before); the phase moves
// the image centre to N/2 (a sign (-1)^(sum delta) for even N)
__global__ void k_esp_qplanes(const float2* P, EspGeom g, float2* planes) {
  const int64_t nd0 = 2 * g.k[0] - 1, nd1 = 2 * g.k[1] - 1, nd2 = 2 * g.k[2] - 1;
  const int64_t ndel = nd0 * nd1 * nd2;
  const int64_t total = ndel * g.nq;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t di = e % ndel, q = e / ndel;
    // pair q -> (c, c') with c <= c'
    int c = 0;
    while (c + 1 < g.Nc && pair_index(c + 1, c + 1, g.Nc) <= q) ++c;
    const int cp = c + (int)(q - pair_index(c, c, g.Nc));
    const int64_t d0 = di % nd0 - (g.k[0] - 1), d1 = (di / nd0) % nd1 - (g.k[1] - 1), d2 = di / (nd0 * nd1) - (g.k[2] - 1);
    float2 s = make_float2(0.f, 0.f);
    for (int64_t k2 = 0; k2 < g.k[2]; ++k2) {
      const int64_t l2 = k2 + d2;
      if (l2 < 0 || l2 >= g.k[2]) continue;
      for (int64_t k1 = 0; k1 < g.k[1]; ++k1) {
        const int64_t l1 = k1 + d1;
        if (l1 < 0 || l1 >= g.k[1]) continue;
        for (int64_t k0 = 0; k0 < g.k[0]; ++k0) {
          const int64_t l0 = k0 + d0;
          if (l0 < 0 || l0 >= g.k[0]) continue;
          const int64_t ka = k0 + g.k[0] * (k1 + g.k[1] * k2), kb = l0 + g.k[0] * (l1 + g.k[1] * l2);
          const float2 v = P[(ka + g.M * c) + g.n * (kb + g.M * cp)];
          s.x += v.x;
          s.y += v.y;
        }
      }
    }
    const int64_t r0 = (d0 + g.img[0]) % g.img[0], r1 = (d1 + g.img[1]) % g.img[1], r2 = (d2 + g.img[2]) % g.img[2];
    // fraction of a turn: sum_i (delta_i (N_i / 2) mod N_i) / N_i
    const double fr = (double)((r0 * (g.img[0] / 2)) % g.img[0]) / (double)g.img[0] +
                      (double)((r1 * (g.img[1] / 2)) % g.img[1]) / (double)g.img[1] +
                      (double)((r2 * (g.img[2] / 2)) % g.img[2]) / (double)g.img[2];
    double sn, cs;
    sincospi(2.0 * fr, &sn, &cs);
    const float ph_r = (float)(cs / (double)g.M), ph_i = (float)(sn / (double)g.M);
    planes[q * g.nimg + r0 + g.img[0] * (r1 + g.img[1] * r2)] =
        make_float2(s.x * ph_r - s.y * ph_i, s.x * ph_i + s.y * ph_r);
  }
}

__device__ __forceinline__ float2 cmacc(float2 acc, float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x)), fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y)));
}

// y_lane = sum_c' W[lane][c'] v_c' (v_c' from lane c')
__device__ __forceinline__ float2 esp_matvec(const float2* w, float2 v, int Nc) {
  float2 y = make_float2(0.f, 0.f);
#pragma unroll
  for (int cc = 0; cc < kEspMaxCoils; ++cc) {
    if (cc < Nc) {
      const float2 vc = make_float2(__shfl_sync(0xffffffffu, v.x, cc), __shfl_sync(0xffffffffu, v.y, cc));
      y = cmacc(y, w[cc], vc);
    }
  }
  return y;
}

__device__ __forceinline__ float warp_sum(float s) {
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// One warp per pixel: the leading eigenvector(s) of W(r), thresholded and phase-normalised.
__global__ void __launch_bounds__(256) k_esp_eig(const float2* planes, EspGeom g, int nmaps, float thr2, float2* maps,
                                                 float* eigs) {
  const int lane = threadIdx.x & 31;
  const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  if (r >= g.nimg) return;  // uniform per warp
  const int Nc = g.Nc;
  const bool act = lane < Nc;
  float2 w[kEspMaxCoils];
#pragma unroll
  for (int cc = 0; cc < kEspMaxCoils; ++cc) {
    w[cc] = make_float2(0.f, 0.f);
    if (act && cc < Nc) {
      if (lane <= cc) {
        w[cc] = planes[(int64_t)pair_index(lane, cc, Nc) * g.nimg + r];
      } else {
        const float2 t = planes[(int64_t)pair_index(cc, lane, Nc) * g.nimg + r];
        w[cc] = make_float2(t.x, -t.y);
      }
    }
  }
  for (int mi = 0; mi < nmaps; ++mi) {
    // start from the column with the largest diagonal entry
    float dg = -1.f;
#pragma unroll
    for (int cc = 0; cc < kEspMaxCoils; ++cc)
      if (cc == lane) dg = act ? w[cc].x : -1.f;
    int best = lane;
    for (int o = 16; o > 0; o >>= 1) {
      const float od = __shfl_xor_sync(0xffffffffu, dg, o);
      const int ob = __shfl_xor_sync(0xffffffffu, best, o);
      if (od > dg || (od == dg && ob < best)) {
        dg = od;
        best = ob;
      }
    }
    float2 v = make_float2(0.f, 0.f);
#pragma unroll
    for (int cc = 0; cc < kEspMaxCoils; ++cc)
      if (cc == best && act) v = w[cc];
    float nv = warp_sum(v.x * v.x + v.y * v.y);
    if (nv <= 0.f) {
      v = make_float2(lane == 0 ? 1.f : 0.f, 0.f);
      nv = 1.f;
    }
    float inv = rsqrtf(nv);
    v = make_float2(v.x * inv, v.y * inv);
    for (int it = 0; it < kEspIters; ++it) {
      const float2 y = esp_matvec(w, v, Nc);
      const float ny = warp_sum(act ? y.x * y.x + y.y * y.y : 0.f);
      if (!(ny > 0.f)) break;
      inv = rsqrtf(ny);
      v = act ? make_float2(y.x * inv, y.y * inv) : make_float2(0.f, 0.f);
    }
    const float2 y = esp_matvec(w, v, Nc);
    const float lam = warp_sum(act ? v.x * y.x + v.y * y.y : 0.f);  // Re(v^H W v), |v| = 1
    // phase: coil 1 real and non-negative
    const float v0x = __shfl_sync(0xffffffffu, v.x, 0), v0y = __shfl_sync(0xffffffffu, v.y, 0);
    const float m0 = sqrtf(v0x * v0x + v0y * v0y);
    float2 out = v;
    if (m0 > 0.f) {
      const float rx = v0x / m0, ry = -v0y / m0;
      out = make_float2(v.x * rx - v.y * ry, v.x * ry + v.y * rx);
    }
    if (!(lam >= thr2)) out = make_float2(0.f, 0.f);
    if (act) maps[r + g.nimg * (lane + (int64_t)Nc * mi)] = out;
    if (eigs && lane == 0) eigs[r + g.nimg * mi] = lam;
    // deflate: W <- W - lam v v^H (row lane: w[c'] -= lam v_lane conj(v_c'))
    if (mi + 1 < nmaps) {
#pragma unroll
      for (int cc = 0; cc < kEspMaxCoils; ++cc) {
        if (cc < Nc) {
          const float vcx = __shfl_sync(0xffffffffu, v.x, cc), vcy = __shfl_sync(0xffffffffu, v.y, cc);
          const float px = v.x * vcx + v.y * vcy, py = v.y * vcx - v.x * vcy;  // v_lane conj(v_cc)
          if (act) w[cc] = make_float2(w[cc].x - lam * px, w[cc].y - lam * py);
        }
      }
    }
  }
}

unsigned blocks_for(int64_t n, int threads, int64_t cap) {
  return (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(n, threads), 1), cap);
}

}  // namespace
}  // namespace mrsr

using namespace mrsr;

extern "C" int mrsr_espirit(int ndims, const int64_t* img_shape, const int64_t* calib_shape, int ncoils,
                            const float* kbp, const int64_t* kernel_size, double eig_thresh_1, double eig_thresh_2,
                            int nmaps, float* maps_out, float* eig_out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(img_shape && calib_shape && kernel_size && kbp && maps_out, MRSR_ERR_ARG, "NULL argument to mrsr_espirit");
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3");
  MRSR_REQUIRE(ndims == 2, MRSR_ERR_UNSUPPORTED,
               "mrsr_espirit: 3D calibration (k^3 Nc columns) is not built; 2D only");
  MRSR_REQUIRE(ncoils >= 1 && ncoils <= kEspMaxCoils, MRSR_ERR_UNSUPPORTED, "mrsr_espirit supports 1..%d coils (got %d)",
               kEspMaxCoils, ncoils);
  MRSR_REQUIRE(nmaps >= 1 && nmaps <= kEspMaxMaps, MRSR_ERR_UNSUPPORTED, "mrsr_espirit supports nmaps 1..%d",
               kEspMaxMaps);
  MRSR_REQUIRE(eig_thresh_1 >= 0.0 && eig_thresh_1 <= 1.0, MRSR_ERR_ARG, "eigThresh_1 must be in [0, 1]");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  EspGeom g{};
  g.Nc = ncoils;
  g.ncal = g.M = g.npos = g.nimg = 1;
  for (int i = 0; i < 3; ++i) {
    g.calib[i] = i < ndims ? calib_shape[i] : 1;
    g.k[i] = i < ndims ? kernel_size[i] : 1;
    g.img[i] = i < ndims ? img_shape[i] : 1;
    MRSR_REQUIRE(g.k[i] >= 1 && g.calib[i] >= g.k[i], MRSR_ERR_ARG,
                 "kernel_size must be >= 1 and no larger than the calibration region (dimension %d)", i + 1);
    MRSR_REQUIRE(g.img[i] >= 2 * g.k[i] - 1, MRSR_ERR_ARG, "image smaller than the kernel's offset range (dimension %d)",
                 i + 1);
    g.np[i] = g.calib[i] - g.k[i] + 1;
    g.ncal *= g.calib[i];
    g.M *= g.k[i];
    g.npos *= g.np[i];
    g.nimg *= g.img[i];
  }
  g.n = g.M * g.Nc;
  g.nq = g.Nc * (g.Nc + 1) / 2;
  MRSR_REQUIRE(g.npos <= (1 << 20) && g.n <= (1 << 20), MRSR_ERR_UNSUPPORTED, "calibration matrix too large");
  FftNd fft;
  MRSR_TRY(fft.init(ndims, g.img));
  const int m = (int)g.npos, m2 = m + (m & 1);
  DevBuf B, fro, nrot, sig2, maxb, wgt, P, planes;
  MRSR_TRY(B.alloc(sizeof(float2) * g.n * g.npos));
  MRSR_TRY(fro.alloc(sizeof(double)));
  MRSR_TRY(nrot.alloc(sizeof(int)));
  MRSR_TRY(sig2.alloc(sizeof(float) * m));
  MRSR_TRY(maxb.alloc(sizeof(unsigned)));
  MRSR_TRY(wgt.alloc(sizeof(float) * m));
  MRSR_TRY(P.alloc(sizeof(float2) * g.n * g.n));
  MRSR_TRY(planes.alloc(sizeof(float2) * g.nq * g.nimg));
  k_esp_patches<<<blocks_for(g.n * g.npos, 256, 152 * 16), 256, 0, st>>>(reinterpret_cast<const float2*>(kbp), g,
                                                                       B.as<float2>());
  MRSR_LAUNCH_CHECK();
  MRSR_CHECK_CUDA(cudaMemsetAsync(fro.p, 0, sizeof(double), st));
  k_esp_fro2<<<blocks_for(g.n * g.npos, 256, 152 * 4), 256, 0, st>>>(B.as<float2>(), g.n * g.npos, fro.as<double>());
  MRSR_LAUNCH_CHECK();
  // one-sided Jacobi sweeps until a sweep applies no rotation; a sweep is one cooperative
  // launch when its m2 / 2 CTAs fit on the device at once, else one launch per round
  int dev = 0, nsm = 0, per_sm = 0, coop = 0;
  MRSR_CHECK_CUDA(cudaGetDevice(&dev));
  MRSR_CHECK_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  MRSR_CHECK_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  MRSR_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_esp_jacobi_sweep, kJacThreads, 0));
  const bool one_launch = coop && (int64_t)per_sm * nsm >= m2 / 2;
  int last = -1;
  for (int sweep = 0; sweep < kMaxSweeps; ++sweep) {
    MRSR_CHECK_CUDA(cudaMemsetAsync(nrot.p, 0, sizeof(int), st));
    if (one_launch) {
      float2* Bp = B.as<float2>();
      int64_t nn = g.n;
      int mm = m, mm2 = m2;
      const double* fp = fro.as<double>();
      float tol = kJacTol;
      int* np_ = nrot.as<int>();
      void* args[] = {&Bp, &nn, &mm, &mm2, &fp, &tol, &np_};
      MRSR_CHECK_CUDA(cudaLaunchCooperativeKernel((const void*)k_esp_jacobi_sweep, dim3(m2 / 2), dim3(kJacThreads), args,
                                                  0, st));
    } else {
      for (int t = 0; t < m2 - 1; ++t) {
        k_esp_jacobi<<<m2 / 2, kJacThreads, 0, st>>>(B.as<float2>(), g.n, m, m2, t, fro.as<double>(), kJacTol,
                                                     nrot.as<int>());
        MRSR_LAUNCH_CHECK();
      }
    }
    MRSR_CHECK_CUDA(cudaMemcpyAsync(&last, nrot.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
    if (last == 0) break;
  }
  MRSR_REQUIRE(last == 0, MRSR_ERR_DEVICE, "mrsr_espirit: the calibration SVD did not converge in %d sweeps", kMaxSweeps);
  MRSR_CHECK_CUDA(cudaMemsetAsync(maxb.p, 0, sizeof(unsigned), st));
  k_esp_colnorm<<<m, 128, 0, st>>>(B.as<float2>(), g.n, m, sig2.as<float>(), maxb.as<unsigned>());
  MRSR_LAUNCH_CHECK();
  k_esp_weights<<<blocks_for(m, 256, 64), 256, 0, st>>>(sig2.as<float>(), m, maxb.as<unsigned>(), (float)eig_thresh_1,
                                                       wgt.as<float>());
  MRSR_LAUNCH_CHECK();
  const dim3 pg((unsigned)cdiv(g.n, 16), (unsigned)cdiv(g.n, 16));
  k_esp_proj<<<pg, dim3(16, 16), 0, st>>>(B.as<float2>(), wgt.as<float>(), g.n, m, P.as<float2>());
  MRSR_LAUNCH_CHECK();
  MRSR_CHECK_CUDA(cudaMemsetAsync(planes.p, 0, sizeof(float2) * g.nq * g.nimg, st));
  const int64_t ndel = (2 * g.k[0] - 1) * (2 * g.k[1] - 1) * (2 * g.k[2] - 1);
  k_esp_qplanes<<<blocks_for(ndel * g.nq, 256, 152 * 16), 256, 0, st>>>(P.as<float2>(), g, planes.as<float2>());
  MRSR_LAUNCH_CHECK();
  MRSR_TRY(fft.run(planes.as<float2>(), g.nq, -1, 1.0f, st));
  k_esp_eig<<<blocks_for(g.nimg * 32, 256, INT32_MAX), 256, 0, st>>>(planes.as<float2>(), g, nmaps,
                                                                      (float)eig_thresh_2,
                                                                      reinterpret_cast<float2*>(maps_out), eig_out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;  // asynchronous on `st` from here; the temporaries are freed in stream order
}
