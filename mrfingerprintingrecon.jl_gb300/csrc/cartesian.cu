// Cartesian paths: FFTNormalOp constructors and the integer-trajectory backprojection.
//  * calculate_kernel_cartesian(img_shape, trj, U; sample_mask)  src/FFTNormalOp.jl:81-97
//  * calculate_kernel_cartesian(M, U)                            src/FFTNormalOp.jl:99-109
//  * FFTNormalOp(...) -> operator                                src/FFTNormalOp.jl:28-64
//  * calculate_backprojection with integer trj                   src/BackProjection.jl:104-156
// Grid index of a sample: mod1(trj - N ÷ 2, N) per dimension (the ifftshift of :88).
#include <algorithm>

#include "fftnd.cuh"
#include "normalop.cuh"

namespace mrsr {

__device__ __forceinline__ int64_t cart_cell(const int32_t* trj, int d, int64_t li, const int64_t* N) {
  int64_t cell = 0, mul = 1;
  for (int dd = 0; dd < d; ++dd) {
    int64_t v = (int64_t)trj[dd + (int64_t)d * li] - N[dd] / 2 - 1;
    v %= N[dd];
    if (v < 0) v += N[dd];
    cell += v * mul;
    mul *= N[dd];
  }
  return cell;
}

__device__ __forceinline__ float2 u_at(const void* U, int cplx, int64_t nt, int K, int64_t t, int k, int rep) {
  const int64_t i = t + nt * (k + (int64_t)K * rep);
  if (cplx) return reinterpret_cast<const float2*>(U)[i];
  return make_float2(reinterpret_cast<const float*>(U)[i], 0.f);
}

struct CartLamArgs {
  const int32_t* trj;
  const uint8_t* mask;
  int d;
  int64_t N[3];
  int64_t ns, nt;
  const void* U;
  int ucplx, K, nrep, P;
  double2* acc;  // [cell][P]
};

// Λ[k1,k2,cell] += sum_rep conj(U[t,k1,rep]) U[t,k2,rep] for every kept sample (float64 accumulation)
__global__ void k_cart_lambda(CartLamArgs a) {
  const int64_t n = a.ns * a.nt;
  for (int64_t li = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; li < n; li += (int64_t)gridDim.x * blockDim.x) {
    if (a.mask && !a.mask[li]) continue;
    const int64_t t = li / a.ns;
    const int64_t cell = cart_cell(a.trj, a.d, li, a.N);
    int p = 0;
    for (int k2 = 0; k2 < a.K; ++k2)
      for (int k1 = 0; k1 <= k2; ++k1, ++p) {
        double re = 0.0, im = 0.0;
        for (int r = 0; r < a.nrep; ++r) {
          const float2 u1 = u_at(a.U, a.ucplx, a.nt, a.K, t, k1, r), u2 = u_at(a.U, a.ucplx, a.nt, a.K, t, k2, r);
          re += (double)u1.x * u2.x + (double)u1.y * u2.y;
          im += (double)u1.x * u2.y - (double)u1.y * u2.x;
        }
        atomicAdd(&a.acc[cell * a.P + p].x, re);
        atomicAdd(&a.acc[cell * a.P + p].y, im);
      }
  }
}

// Λ[:,:,cell] = U' (M[ifftshift(cell), :] .* U)
__global__ void k_cart_lambda_mask(const uint8_t* M, int d, int64_t N0, int64_t N1, int64_t N2, int64_t nt, const void* U,
                                   int ucplx, int K, int P, double2* acc) {
  const int64_t ncell = N0 * N1 * N2;
  const int64_t N[3] = {N0, N1, N2};
  for (int64_t cell = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; cell < ncell;
       cell += (int64_t)gridDim.x * blockDim.x) {
    int64_t rem = cell, q = 0, mul = 1;
    for (int dd = 0; dd < 3; ++dd) {
      const int64_t pd = rem % N[dd];
      rem /= N[dd];
      q += ((pd + N[dd] / 2) % N[dd]) * mul;
      mul *= N[dd];
    }
    int p = 0;
    for (int k2 = 0; k2 < K; ++k2)
      for (int k1 = 0; k1 <= k2; ++k1, ++p) {
        double re = 0.0, im = 0.0;
        for (int64_t t = 0; t < nt; ++t) {
          if (!M[q + ncell * t]) continue;
          const float2 u1 = u_at(U, ucplx, nt, K, t, k1, 0), u2 = u_at(U, ucplx, nt, K, t, k2, 0);
          re += (double)u1.x * u2.x + (double)u1.y * u2.y;
          im += (double)u1.x * u2.y - (double)u1.y * u2.x;
        }
        acc[cell * P + p] = make_double2(re, im);
      }
  }
}

__global__ void k_cart_flags(const double2* acc, int64_t ncell, int P, uint8_t* flags) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell; c += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = acc[c * P];
    const float2 f = make_float2((float)v.x, (float)v.y);
    flags[c] = (f.x != 0.f || f.y != 0.f) ? 1 : 0;
  }
}

__global__ void k_cart_pack(const double2* acc, int P, const int64_t* kmask, int64_t nk, int real, void* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = kmask[i] - 1;
    for (int p = 0; p < P; ++p) {
      const double2 v = acc[cell * P + p];
      if (real)
        reinterpret_cast<float*>(out)[p + (int64_t)P * i] = (float)v.x;
      else
        reinterpret_cast<float2*>(out)[p + (int64_t)P * i] = make_float2((float)v.x, (float)v.y);
    }
  }
}

static unsigned g1d(int64_t n) { return (unsigned)std::min<int64_t>(std::max<int64_t>(cdiv(n, 256), 1), 65535); }

// dense float64 Λ -> kmask + packed kernel on the operator
static int finish_cartesian(mrsr_normalop* op, DevBuf& acc, int real, cudaStream_t st) {
  const int64_t ncell = op->geo.ngrid();
  const int K = op->geo.K;
  const int P = K * (K + 1) / 2;
  DevBuf flags, km, packed;
  MRSR_TRY(flags.alloc(ncell));
  k_cart_flags<<<g1d(ncell), 256, 0, st>>>(acc.as<double2>(), ncell, P, flags.as<uint8_t>());
  MRSR_LAUNCH_CHECK();
  int64_t nk = 0;
  MRSR_TRY(compact_nonzero(flags.as<uint8_t>(), ncell, km, &nk, st));
  MRSR_REQUIRE(nk >= 1, MRSR_ERR_ARG, "AssertionError: the sampling pattern selects no k-space location");
  MRSR_TRY(packed.alloc((real ? 4 : 8) * (size_t)P * nk));
  k_cart_pack<<<g1d(nk), 256, 0, st>>>(acc.as<double2>(), P, km.as<int64_t>(), nk, real, packed.p);
  MRSR_LAUNCH_CHECK();
  return op_set_lambda_packed(op, packed.p, real ? 0 : 1, km.as<int64_t>(), nk, st);
}

// ---------------------------------------------------- backprojection ---

struct CartBpArgs {
  const int32_t* trj;
  const uint8_t* mask;
  int d;
  int64_t N[3], ncell;
  int64_t ns, nt;
  int c0, nc, nrep, ncoils;
  const float2* data;   // (ns, nt, ncoils, nrep)
  const void* U;        // (nt, K, nrep) or null = I(nt)
  int ucplx, K;
  float2* grid;         // [(c - c0) K + k][ncell]
};

__global__ void k_cart_bin(CartBpArgs a) {
  const int64_t n = a.ns * a.nt;
  for (int64_t li = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; li < n; li += (int64_t)gridDim.x * blockDim.x) {
    if (a.mask && !a.mask[li]) continue;
    const int64_t t = li / a.ns;
    const int64_t cell = cart_cell(a.trj, a.d, li, a.N);
    for (int c = 0; c < a.nc; ++c) {
      const int kb = a.U ? 0 : (int)t, ke = a.U ? a.K : (int)t + 1;
      for (int k = kb; k < ke; ++k) {
        float2 acc = make_float2(0.f, 0.f);
        for (int r = 0; r < a.nrep; ++r) {
          const float2 y = a.data[li + n * ((a.c0 + c) + (int64_t)a.ncoils * r)];
          if (a.U)
            acc = cadd(acc, cmulc(y, u_at(a.U, a.ucplx, a.nt, a.K, t, k, r)));
          else
            acc = cadd(acc, y);
        }
        atomicAdd(&a.grid[((int64_t)c * a.K + k) * a.ncell + cell], acc);
      }
    }
  }
}

// out[r, k] += conj(S_c(r)) * fftshift(grid)[r]  (or per coil without maps)
__global__ void k_cart_fold(CartBpArgs a, const float2* cmaps, float2* out) {
  const int64_t total = a.ncell * a.K;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(e / a.ncell);
    const int64_t r = e - (int64_t)k * a.ncell;
    int64_t rem = r, q = 0, mul = 1;
    for (int dd = 0; dd < 3; ++dd) {
      const int64_t pd = rem % a.N[dd];
      rem /= a.N[dd];
      int64_t s = (pd - a.N[dd] / 2) % a.N[dd];
      if (s < 0) s += a.N[dd];
      q += s * mul;
      mul *= a.N[dd];
    }
    if (cmaps) {
      float2 acc = make_float2(0.f, 0.f);
      for (int c = 0; c < a.nc; ++c)
        acc = cadd(acc, cmulc(a.grid[((int64_t)c * a.K + k) * a.ncell + q], cmaps[r + a.ncell * (a.c0 + c)]));
      out[e] = cadd(out[e], acc);
    } else {
      for (int c = 0; c < a.nc; ++c)
        out[r + a.ncell * (k + (int64_t)a.K * (a.c0 + c))] = a.grid[((int64_t)c * a.K + k) * a.ncell + q];
    }
  }
}

}  // namespace mrsr

using namespace mrsr;

static cudaStream_t cstream(mrsr_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" int mrsr_fft_normalop_create(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                                        const int32_t* trj, const uint8_t* sample_mask, const void* U, int u_is_complex,
                                        int K, int nrep, const float* cmaps, int ncoils, int precision,
                                        mrsr_stream_t stream, mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(trj && U, MRSR_ERR_ARG, "trj and U must be device pointers");
  MRSR_REQUIRE(nrep >= 1 && ns_per_frame >= 1 && nt >= 1, MRSR_ERR_ARG, "empty trajectory");
  cudaStream_t st = cstream(stream);
  mrsr_normalop* op = new mrsr_normalop();
  int s = op_init_geometry(op, MRSR_KIND_FFT, ndims, img_shape, K, cmaps ? ncoils : 1, precision);
  if (s == MRSR_OK) s = op_set_cmaps(op, cmaps, st);
  DevBuf acc;
  const int P = K * (K + 1) / 2;
  if (s == MRSR_OK) s = acc.alloc(sizeof(double2) * P * op->geo.ngrid());
  if (s == MRSR_OK && cudaMemsetAsync(acc.p, 0, acc.bytes, st) != cudaSuccess) s = MRSR_ERR_CUDA;
  if (s == MRSR_OK) {
    CartLamArgs a{trj, sample_mask, ndims, {op->geo.n[0], op->geo.n[1], op->geo.n[2]}, ns_per_frame, nt, U,
                  u_is_complex, K, nrep, P, acc.as<double2>()};
    k_cart_lambda<<<g1d(ns_per_frame * nt), 256, 0, st>>>(a);
    if (cudaGetLastError() != cudaSuccess) s = MRSR_ERR_CUDA;
  }
  if (s == MRSR_OK) s = finish_cartesian(op, acc, u_is_complex ? 0 : 1, st);
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  *out = op;
  return MRSR_OK;
}

extern "C" int mrsr_fft_normalop_create_from_mask(int ndims, const int64_t* img_shape, int64_t nt, const uint8_t* M,
                                                  const void* U, int u_is_complex, int K, const float* cmaps,
                                                  int ncoils, int precision, mrsr_stream_t stream,
                                                  mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(M && U, MRSR_ERR_ARG, "M and U must be device pointers");
  cudaStream_t st = cstream(stream);
  mrsr_normalop* op = new mrsr_normalop();
  int s = op_init_geometry(op, MRSR_KIND_FFT, ndims, img_shape, K, cmaps ? ncoils : 1, precision);
  if (s == MRSR_OK) s = op_set_cmaps(op, cmaps, st);
  DevBuf acc;
  const int P = K * (K + 1) / 2;
  if (s == MRSR_OK) s = acc.alloc(sizeof(double2) * P * op->geo.ngrid());
  if (s == MRSR_OK) {
    k_cart_lambda_mask<<<g1d(op->geo.ngrid()), 256, 0, st>>>(M, ndims, op->geo.n[0], op->geo.n[1], op->geo.n[2], nt, U,
                                                               u_is_complex, K, P, acc.as<double2>());
    if (cudaGetLastError() != cudaSuccess) s = MRSR_ERR_CUDA;
  }
  if (s == MRSR_OK) s = finish_cartesian(op, acc, u_is_complex ? 0 : 1, st);
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  *out = op;
  return MRSR_OK;
}

extern "C" int mrsr_backprojection_cartesian(int ndims, const int64_t* img_shape, int64_t ns_per_frame, int64_t nt,
                                             int ncoils, int nrep, const float* data, const int32_t* trj,
                                             const uint8_t* sample_mask, const void* U, int u_is_complex, int K,
                                             const float* cmaps, float* out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3");
  MRSR_REQUIRE(img_shape && data && trj && out, MRSR_ERR_ARG, "NULL argument");
  MRSR_REQUIRE(ncoils >= 1 && nrep >= 1, MRSR_ERR_ARG, "empty data");
  if (!U) K = (int)nt;
  cudaStream_t st = cstream(stream);
  int64_t N[3] = {1, 1, 1};
  for (int i = 0; i < ndims; ++i) N[i] = img_shape[i];
  const int64_t ncell = N[0] * N[1] * N[2];
  FftNd f;
  MRSR_TRY(f.init(ndims, N));
  const int64_t per_coil = (int64_t)K * ncell * (int64_t)sizeof(float2);
  const int cc = (int)std::max<int64_t>(1, std::min<int64_t>(ncoils, (2ll << 30) / std::max<int64_t>(per_coil, 1)));
  DevBuf grid;
  MRSR_TRY(grid.alloc((size_t)per_coil * cc));
  if (cmaps) MRSR_CHECK_CUDA(cudaMemsetAsync(out, 0, sizeof(float2) * ncell * K, st));
  for (int c0 = 0; c0 < ncoils; c0 += cc) {
    const int nc = std::min(cc, ncoils - c0);
    MRSR_CHECK_CUDA(cudaMemsetAsync(grid.p, 0, (size_t)per_coil * nc, st));
    CartBpArgs a{trj, sample_mask, ndims, {N[0], N[1], N[2]}, ncell, ns_per_frame, nt, c0, nc, nrep, ncoils,
                 reinterpret_cast<const float2*>(data), U, u_is_complex, K, grid.as<float2>()};
    k_cart_bin<<<g1d(ns_per_frame * nt), 256, 0, st>>>(a);
    MRSR_LAUNCH_CHECK();
    MRSR_TRY(f.run(grid.as<float2>(), (int64_t)nc * K, +1, 1.0f / (float)ncell, st));
    k_cart_fold<<<g1d(ncell * K), 256, 0, st>>>(a, reinterpret_cast<const float2*>(cmaps), reinterpret_cast<float2*>(out));
    MRSR_LAUNCH_CHECK();
  }
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return MRSR_OK;
}
