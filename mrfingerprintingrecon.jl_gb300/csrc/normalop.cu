// Subspace Toeplitz normal operator: fused pruned-FFT passes.
//
// Reference: mul!(x, ::_NFFTNormalOp, b, α, β) in src/NFFTNormalOp.jl:227-267
// (CPU) and ext/MRISubspaceReconCUDAExt/NFFTNormalOp.jl:193-218 (GPU), and
// mul!(x, ::_FFTNormalOp, ...) in src/FFTNormalOp.jl:111-149.
//
//   y <- beta y + alpha sum_c conj(S_c) . crop F^-1 Λ F pad (S_c . x)
//
// The 2D operator runs as three passes per group of coils:
//   P1 rows:   pad + coil multiply + forward FFT along dim 1        -> stack
//   P2 lines:  forward FFT along the last dim, per-voxel K x K Λ,
//              inverse FFT along the last dim (in place)            -> stack
//   P3 rows:   inverse FFT along dim 1 + crop + conj coil + coil sum -> y
// The 3D operator adds a forward and an inverse pass along dim 2 around the
// Λ pass.  Image and kernel layouts are the reference's (column-major,
// image at the low corner of the 2x grid, no shift); F is the unnormalised
// forward FFT and F^-1 carries 1/prod(grid) (folded into alpha).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "passes.cuh"

namespace mrsr {

// ------------------------------------------------------------- kernels ---



__global__ void __launch_bounds__(512) k_rows_fwd(RowsFwdArgs a) {
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + a.pl.L;
  const int L = a.pl.L;
  float2* s1 = s + a.rpc * a.K * a.lstride;
  load_twiddles(tw, a.pl);
  const int cl = blockIdx.y;
  const int c = a.c0 + cl;
  const int64_t row0 = (int64_t)blockIdx.x * a.rpc;
  const int nr = (int)min((int64_t)a.rpc, a.nrows - row0);
  const int NO = a.rpc * a.K;
  const bool pin = can_prune_in(a.pl, a.n1);
  for (int e = threadIdx.x; e < NO * a.n1; e += blockDim.x) {
    const int lo = e / a.n1, i1 = e - lo * a.n1;
    const int rl = lo / a.K, k = lo - rl * a.K;
    float2 v = make_float2(0.f, 0.f);
    if (rl < nr) {
      const int64_t r = row0 + rl;
      v = a.x[i1 + (int64_t)a.n1 * (r + a.nrows * k)];
      if (a.cmaps) v = cmul(a.cmaps[i1 + (int64_t)a.n1 * (r + a.nrows * c)], v);
    }
    s[lo * a.lstride + i1] = v;
  }
  if (!pin && a.n1 < L) {
    const int nz = L - a.n1;
    for (int e = threadIdx.x; e < NO * nz; e += blockDim.x) {
      const int lo = e / nz, i = e - lo * nz;
      s[lo * a.lstride + a.n1 + i] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  LineLayout ly{NO, 1, a.lstride};
  const float2* res = fft_lines(s, s1, a.pl, ly, -1.f, tw, pin, false);
  for (int e = threadIdx.x; e < nr * a.K * L; e += blockDim.x) {
    const int lo = e / L, f = e - lo * L;
    const int rl = lo / a.K, k = lo - rl * a.K;
    const int64_t r = row0 + rl;
    a.out[(((int64_t)cl * a.K + k) * a.nrows + r) * L + f] = res[lo * a.lstride + f];
  }
}





__global__ void __launch_bounds__(512) k_lambda_pass(LamPassArgs a) {
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + a.pl.L;
  float2* s1 = s + a.K * a.lstride;
  load_twiddles(tw, a.pl);
  const int L = a.pl.L;
  const int cl = blockIdx.y;
  const int64_t tile = blockIdx.x;
  const int64_t col0 = tile * a.TC;
  const bool pin = can_prune_in(a.pl, a.nin);
  const bool pout = can_prune_out(a.pl, a.nout);
  const int64_t plane = (int64_t)a.nrow * a.inner;
  float2* base = a.stack + (int64_t)cl * a.K * plane + col0;
  // load: s[k][n][li]
  for (int e = threadIdx.x; e < a.K * a.nin * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % a.nin;
    const int k = t / a.nin;
    s[k * a.lstride + n * a.TC + li] = base[k * plane + (int64_t)n * a.inner + li];
  }
  if (!pin && a.nin < L) {
    const int nz = (L - a.nin) * a.TC;
    for (int e = threadIdx.x; e < a.K * nz; e += blockDim.x) {
      const int k = e / nz, i = e - k * nz;
      s[k * a.lstride + a.nin * a.TC + i] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  LineLayout ly{a.K, a.TC, a.lstride};
  float2* X0 = fft_lines(s, s1, a.pl, ly, -1.f, tw, pin, false);
  float2* X1 = (X0 == s) ? s1 : s;
  // per-voxel contraction (in place in the spectrum buffer)
  if (lam_is_diag(a.lam_mode)) {
    for (int pos = threadIdx.x; pos < a.TC * L; pos += blockDim.x) {
      const float2 l = lam_diag_entry(a.lam_mode, a.lam, lam_elem(tile, pos / a.TC, pos % a.TC, 0, a.TC, 1, a.FC, a.NCH));
      for (int k = 0; k < a.K; ++k) X0[k * a.lstride + pos] = cmul(l, X0[k * a.lstride + pos]);
    }
  }
  for (int pos = threadIdx.x; pos < a.TC * L && !lam_is_diag(a.lam_mode); pos += blockDim.x) {
    const int li = pos % a.TC;
    const int f = pos / a.TC;
    float2 X[KMAX], Y[KMAX];
#pragma unroll
    for (int k = 0; k < KMAX; ++k) X[k] = (k < a.K) ? X0[k * a.lstride + pos] : make_float2(0.f, 0.f);
    const int64_t lbase = lam_elem(tile, f, li, 0, a.TC, a.P, a.FC, a.NCH);
    lam_apply<KMAX>(a, lbase, (int64_t)a.FC * a.TC, X, Y);
#pragma unroll
    for (int k = 0; k < KMAX; ++k)
      if (k < a.K) X0[k * a.lstride + pos] = Y[k];
  }
  __syncthreads();
  const float2* res = fft_lines(X0, X1, a.pl, ly, +1.f, tw, false, pout);
  for (int e = threadIdx.x; e < a.K * a.nout * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % a.nout;
    const int k = t / a.nout;
    base[k * plane + (int64_t)n * a.inner + li] = res[k * a.lstride + n * a.TC + li];
  }
}



__global__ void __launch_bounds__(512) k_mid_fft(MidArgs a) {
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + a.pl.L;
  float2* s1 = s + a.NOo * a.lstride;
  load_twiddles(tw, a.pl);
  const int L = a.pl.L;
  const int64_t col0 = (int64_t)blockIdx.x * a.TC;
  const int64_t o0 = (int64_t)blockIdx.y * a.NOo;
  const int no = (int)min((int64_t)a.NOo, a.n3 - o0);
  const int64_t p = blockIdx.z;
  const bool pin = (a.sgn < 0) && can_prune_in(a.pl, a.nin);
  const bool pout = (a.sgn > 0) && can_prune_out(a.pl, a.nout);
  const float2* ib = a.in + (p * a.n3 + o0) * a.nin * a.width + col0;
  float2* ob = a.out + (p * a.n3 + o0) * a.nout * a.width + col0;
  for (int e = threadIdx.x; e < a.NOo * a.nin * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % a.nin;
    const int o = t / a.nin;
    float2 v = make_float2(0.f, 0.f);
    if (o < no) v = ib[((int64_t)o * a.nin + n) * a.width + li];
    s[o * a.lstride + n * a.TC + li] = v;
  }
  if (!pin && a.nin < L) {
    const int nz = (L - a.nin) * a.TC;
    for (int e = threadIdx.x; e < a.NOo * nz; e += blockDim.x) {
      const int o = e / nz, i = e - o * nz;
      s[o * a.lstride + a.nin * a.TC + i] = make_float2(0.f, 0.f);
    }
  }
  __syncthreads();
  LineLayout ly{a.NOo, a.TC, a.lstride};
  const float2* res = fft_lines(s, s1, a.pl, ly, a.sgn, tw, pin, pout);
  for (int e = threadIdx.x; e < no * a.nout * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % a.nout;
    const int o = t / a.nout;
    ob[((int64_t)o * a.nout + n) * a.width + li] = res[o * a.lstride + n * a.TC + li];
  }
}



__global__ void __launch_bounds__(512) k_rows_inv(RowsInvArgs a) {
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s = smem + a.pl.L;
  float2* s1 = s + a.rpc * a.ncg * a.lstride;
  load_twiddles(tw, a.pl);
  const int L = a.pl.L;
  const int k = blockIdx.y;
  const int64_t row0 = (int64_t)blockIdx.x * a.rpc;
  const int nr = (int)min((int64_t)a.rpc, a.nrows - row0);
  const int NO = a.rpc * a.ncg;
  const bool pout = can_prune_out(a.pl, a.n1);
  for (int e = threadIdx.x; e < NO * L; e += blockDim.x) {
    const int lo = e / L, f = e - lo * L;
    const int rl = lo / a.ncg, cl = lo - rl * a.ncg;
    float2 v = make_float2(0.f, 0.f);
    if (rl < nr) v = a.stack[(((int64_t)cl * a.K + k) * a.nrows + row0 + rl) * L + f];
    s[lo * a.lstride + f] = v;
  }
  __syncthreads();
  LineLayout ly{NO, 1, a.lstride};
  const float2* res = fft_lines(s, s1, a.pl, ly, +1.f, tw, false, pout);
  for (int e = threadIdx.x; e < nr * a.n1; e += blockDim.x) {
    const int rl = e / a.n1, i1 = e - rl * a.n1;
    const int64_t r = row0 + rl;
    float2 acc = make_float2(0.f, 0.f);
    for (int cl = 0; cl < a.ncg; ++cl) {
      const float2 v = res[(rl * a.ncg + cl) * a.lstride + i1];
      if (a.cmaps)
        acc = cadd(acc, cmulc(v, a.cmaps[i1 + (int64_t)a.n1 * (r + a.nrows * (a.c0 + cl))]));
      else
        acc = cadd(acc, v);
    }
    const int64_t yi = i1 + (int64_t)a.n1 * (r + a.nrows * k);
    float2 yv;
    if (a.first) {
      yv = (a.beta.x == 0.f && a.beta.y == 0.f) ? make_float2(0.f, 0.f) : cmul(a.beta, a.y[yi]);
    } else {
      yv = a.y[yi];
    }
    a.y[yi] = cadd(yv, cmul(a.alpha, acc));
  }
}

// ---------------------------------------------------- Λ layout kernels ---

struct LamLayout {
  int64_t inner;   // Λ-pass plane width
  int64_t L;       // last-dim grid length
  int TC, P, FC, NCH;
  int64_t ngrid;
};

__device__ __forceinline__ int64_t lam_int_index(const LamLayout& g, int64_t cell, int p) {
  const int64_t f = cell / g.inner;
  const int64_t in = cell - f * g.inner;
  const int64_t tile = in / g.TC;
  const int64_t li = in - tile * g.TC;
  return lam_elem(tile, (int)f, (int)li, p, g.TC, g.P, g.FC, g.NCH);
}

template <class T>
__global__ void k_lam_from_packed(LamLayout g, const T* packed, const int64_t* kmask, int64_t nk, T* lam,
                                  int* err) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = kmask[i] - 1;
    if (cell < 0 || cell >= g.ngrid) {
      atomicExch(err, 1);
      continue;
    }
    for (int p = 0; p < g.P; ++p) lam[lam_int_index(g, cell, p)] = packed[p + (int64_t)g.P * i];
  }
}

template <class T>
__global__ void k_lam_to_packed(LamLayout g, const T* lam, const int64_t* kmask, int64_t nk, T* packed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = kmask[i] - 1;
    for (int p = 0; p < g.P; ++p) packed[p + (int64_t)g.P * i] = lam[lam_int_index(g, cell, p)];
  }
}

// the same rank-1 kernel in another chunked layout (P = 1 in both), every grid cell
template <class T>
__global__ void k_lam_relayout(LamLayout src, LamLayout dst, const T* a, T* b) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < dst.ngrid; c += (int64_t)gridDim.x * blockDim.x)
    b[lam_int_index(dst, c, 0)] = a[lam_int_index(src, c, 0)];
}

__global__ void k_flags_nonzero_c(const float2* lam_full, int64_t stride, int64_t n, uint8_t* flags) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = lam_full[i * stride];
    flags[i] = (v.x != 0.f || v.y != 0.f) ? 1 : 0;
  }
}

__global__ void k_lam_full_to_packed(const float2* lam_full, int K, const int64_t* kmask, int64_t nk, float2* packed) {
  const int P = K * K;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = kmask[i] - 1;
    for (int p = 0; p < P; ++p) packed[p + (int64_t)P * i] = lam_full[p + (int64_t)P * cell];
  }
}

// ----------------------------------------------------- stream compaction ---
constexpr int kScanBlock = 1024;

__global__ void k_count_blocks(const uint8_t* flags, int64_t n, int64_t* counts) {
  __shared__ int64_t red[32];
  const int64_t i0 = (int64_t)blockIdx.x * kScanBlock * 8;
  int64_t c = 0;
  for (int j = 0; j < 8; ++j) {
    const int64_t i = i0 + (int64_t)j * kScanBlock + threadIdx.x;
    if (i < n && flags[i]) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    c = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if (threadIdx.x == 0) counts[blockIdx.x] = c;
  }
}

// exclusive scan of counts (single CTA), total written to counts[nb]
__global__ void k_scan_counts(int64_t* counts, int64_t nb) {
  __shared__ int64_t carry;
  __shared__ int64_t warp_sums[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < nb; base += blockDim.x) {
    const int64_t i = base + threadIdx.x;
    int64_t v = (i < nb) ? counts[i] : 0;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_sums[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int64_t w = (threadIdx.x < (blockDim.x >> 5)) ? warp_sums[threadIdx.x] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (threadIdx.x >= o) w += y;
      }
      warp_sums[threadIdx.x] = w;
    }
    __syncthreads();
    const int64_t wprefix = (threadIdx.x >= 32) ? warp_sums[(threadIdx.x >> 5) - 1] : 0;
    const int64_t incl = x + wprefix + carry;
    if (i < nb) counts[i] = incl - v;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[nb] = carry;
}

__global__ void k_scatter_blocks(const uint8_t* flags, int64_t n, const int64_t* offsets, int64_t* out) {
  __shared__ int64_t warp_off[33];
  int64_t off = offsets[blockIdx.x];
  const int64_t i0 = (int64_t)blockIdx.x * kScanBlock * 8;
  for (int j = 0; j < 8; ++j) {
    const int64_t i = i0 + (int64_t)j * kScanBlock + threadIdx.x;
    const int f = (i < n && flags[i]) ? 1 : 0;
    const unsigned m = __ballot_sync(0xffffffffu, f);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) warp_off[w] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      int64_t acc = 0;
      for (int q = 0; q < kScanBlock / 32; ++q) {
        int64_t c = warp_off[q];
        warp_off[q] = acc;
        acc += c;
      }
      warp_off[32] = acc;
    }
    __syncthreads();
    if (f) out[off + warp_off[w] + __popc(m & ((1u << lane) - 1u))] = i + 1;
    const int64_t tot = warp_off[32];
    __syncthreads();
    off += tot;
  }
}

int compact_nonzero(const uint8_t* flags, int64_t n, DevBuf& out, int64_t* count, cudaStream_t st) {
  const int64_t nb = cdiv(n, (int64_t)kScanBlock * 8);
  DevBuf counts;
  MRSR_TRY(counts.alloc(sizeof(int64_t) * (nb + 1)));
  k_count_blocks<<<(unsigned)nb, kScanBlock, 0, st>>>(flags, n, counts.as<int64_t>());
  MRSR_LAUNCH_CHECK();
  k_scan_counts<<<1, 1024, 0, st>>>(counts.as<int64_t>(), nb);
  MRSR_LAUNCH_CHECK();
  int64_t total = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&total, counts.as<int64_t>() + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  MRSR_TRY(out.alloc(sizeof(int64_t) * std::max<int64_t>(total, 1)));
  if (total > 0) {
    k_scatter_blocks<<<(unsigned)nb, kScanBlock, 0, st>>>(flags, n, counts.as<int64_t>(), out.as<int64_t>());
    MRSR_LAUNCH_CHECK();
  }
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  *count = total;
  return MRSR_OK;
}

// -------------------------------------------------------- host driver ---

template <class Args>
static int launch_fft_kernel(void (*k)(Args), dim3 grid, int threads, size_t smem, cudaStream_t st, const Args& a) {
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "shared memory request %zu too large", smem);
  if (smem > 48 * 1024) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
  k<<<grid, threads, smem, st>>>(a);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

struct Recorder {
  std::vector<cudaEvent_t>* ev = nullptr;
  cudaStream_t st = nullptr;
  int record() {
    if (!ev) return MRSR_OK;
    cudaEvent_t e;
    MRSR_CHECK_CUDA(cudaEventCreate(&e));
    MRSR_CHECK_CUDA(cudaEventRecord(e, st));
    ev->push_back(e);
    return MRSR_OK;
  }
};

// Launch shapes.  Each CTA holds two ping-pong copies of its lines in shared
// memory plus the twiddle table of the transform length.
constexpr int64_t kRowElems = 4096;  // line elements per CTA of the row passes
constexpr int64_t kMidElems = 4096;

struct RowTiling {
  int threads, rpc, lstride;
  size_t smem;
};


// R1 of the register four-step split of L (apply_fast.cu's table), 0 if none
static int fast_r1(int L) {
  switch (L) {
    case 64: case 128: return 8;
    case 256: case 512: return 16;
    case 384: return 12;
    case 768: return 24;
    case 1024: return 32;
    default: return 0;
  }
}

// Rows per CTA of the four-step forward row pass: the smallest count (up to twice the
// line-element budget) whose step-B tasks rpc * lines * R1 best fill the CTA's threads
// (a multiple of 32, at least 128, at most 256 per round).  For K = 5 lines of 512
// points this is 2 rows (160 tasks, 160 threads) instead of 1 (80 tasks on 128 threads):
// 0.043 -> 0.038 ms on 256^2 with 20 coils.
static int balanced_rpc(int L, int lines, int64_t elems) {
  const int r1 = fast_r1(L);
  const int rmax = (int)std::max<int64_t>(1, 2 * elems / ((int64_t)lines * L));
  int best = (int)std::max<int64_t>(1, elems / ((int64_t)lines * L));
  if (!r1) return best;
  double best_u = 0.0;
  for (int r = 1; r <= rmax; ++r) {
    const int t = r * lines * r1;
    const int thr = std::min(std::max(((t + 31) / 32) * 32, 128), 256);
    const int rounds = (t + thr - 1) / thr;
    const double u = (double)t / ((double)rounds * thr);
    if (u > best_u + 1e-9) {
      best_u = u;
      best = r;
    }
  }
  return best;
}

static RowTiling rows_tiling(int L, int lines_per_row, int64_t nrows, bool balance = false) {
  RowTiling t;
  t.lstride = L;
  const int64_t elems = kRowElems;
  int rpc = (int)std::max<int64_t>(1, elems / ((int64_t)lines_per_row * L));
  if (balance && fast_length(L)) rpc = balanced_rpc(L, lines_per_row, elems);
  rpc = (int)std::min<int64_t>(rpc, nrows);
  t.rpc = rpc;
  t.threads = 256;
  t.smem = sizeof(float2) * ((size_t)L + 2 * (size_t)rpc * lines_per_row * t.lstride);
  return t;
}

static int mid_tc(const mrsr_normalop* op) {
  int TC = 8;
  while (TC > 1 && op->geo.g[0] % TC) TC >>= 1;
  return TC;
}

static void record_cb(void* ctx) { static_cast<Recorder*>(ctx)->record(); }

static int apply_impl(mrsr_normalop* op, const float2* x, float2* y, float2 alpha, float2 beta, cudaStream_t st,
                      Recorder rec) {
  if (op->precision == MRSR_PREC_FP16) {
    return apply_half_impl(op, x, y, alpha, beta, st, rec.ev ? record_cb : nullptr, &rec);
  }
  const OpGeom& g = op->geo;
  const int K = g.K;
  const float inv = 1.0f / (float)g.ngrid();
  const float2 al = make_float2(alpha.x * inv, alpha.y * inv);
  const float2* cm = op->cmaps.p ? op->cmaps.as<float2>() : nullptr;
  const int64_t nrows = g.n[1] * g.n[2];
  const int L1 = (int)g.g[0];
  const int ngroups = (int)cdiv(g.ncoils, op->Cg);
  float2* st1 = op->stack1.as<float2>();
  float2* st2 = op->stack2.as<float2>();
  for (int grp = 0; grp < ngroups; ++grp) {
    const int c0 = grp * op->Cg;
    const int ncg = std::min(op->Cg, g.ncoils - c0);
    // fp16-tc: the inverse row pass runs on the tensor cores too.  The forward row pass stays
    // the float32 four-step kernel: on 256^2 with 20 coils it takes 0.039 ms against 0.042 ms
    // for a tensor-core form, and adds no fp16 rounding.
    const bool tc_rows = op->precision == MRSR_PREC_FP16_TC && tc_rows_supported(L1, (int)g.n[0], ncg);
    // a stacked operator's planes are independent: without coil maps the rows pass sees
    // them as more rows of one plane, and the Λ pass as more coils, so small images still
    // fill the GPU (the stack layout [coil][plane][row][...] is the same either way)
    const bool diag = lam_is_diag(op->lam_mode);
    const bool flat_rows = diag && !cm;
    // P1: rows forward
    {
      const int Kr = flat_rows ? 1 : K;
      const int64_t nr = flat_rows ? nrows * K : nrows;
      RowTiling t = rows_tiling(L1, Kr, nr, true);
      RowsFwdArgs a{op->plan[0].plan, (int)g.n[0], nr, t.rpc, Kr, c0, t.lstride, x, cm, st1};
      dim3 grid((unsigned)cdiv(nr, t.rpc), ncg);
      if (fast_length(L1))
        MRSR_TRY(fast_rows_fwd(a, nr, ncg, st));
      else
        MRSR_TRY(launch_fft_kernel<RowsFwdArgs>(k_rows_fwd, grid, t.threads, t.smem, st, a));
      MRSR_TRY(rec.record());
    }
    float2* lam_stack = st1;
    if (g.ndims == 3) {
      // dim-2 forward: st1 (g1, n2, n3) -> st2 (g1, g2, n3)
      const int L2 = (int)g.g[1];
      const int TC = mid_tc(op);
      int NOo = (int)std::max<int64_t>(1, kMidElems / ((int64_t)TC * L2));
      NOo = (int)std::min<int64_t>(NOo, g.n[2]);
      MidArgs a{op->plan[1].plan, (int)g.n[1], L2, g.g[0], g.n[2], TC, NOo, L2 * TC, -1.f, st1, st2};
      dim3 grid((unsigned)(g.g[0] / TC), (unsigned)cdiv(g.n[2], NOo), (unsigned)(ncg * K));
      const size_t smem = sizeof(float2) * ((size_t)L2 + 2 * (size_t)NOo * a.lstride);
      if (fast_length(L2))
        MRSR_TRY(fast_mid(a, ncg * K, st));
      else
        MRSR_TRY(launch_fft_kernel<MidArgs>(k_mid_fft, grid, 256, smem, st, a));
      MRSR_TRY(rec.record());
      lam_stack = st2;
    }
    // Λ pass along the last dim, in place
    {
      const int Ll = (int)g.glast();
      const int TC = op->TC;
      const int Kl = diag ? 1 : K, ncl = diag ? ncg * K : ncg;
      LamPassArgs a{op->plan[g.ndims - 1].plan, (int)g.nlast(), (int)g.nlast(), (int)g.nlast(), g.inner(), TC, Kl,
                    op->P, op->lam_mode, Ll * TC, op->lam.p, lam_stack, op->FC, (int)(Ll / op->FC)};
      dim3 grid((unsigned)(g.inner() / TC), ncl);
      const size_t smem = sizeof(float2) * ((size_t)Ll + 2 * (size_t)Kl * a.lstride);
      if (op->precision == MRSR_PREC_FP16_TC) {
        a.lam = op->lam_tc.p;
        MRSR_TRY(tc_lambda(a, ncg, op->lam_max.as<float>(), op->tc_consts.p, op->errflag.as<int>(), st));
      } else if (lambda8_supported(a)) {
        MRSR_TRY(fast_lambda8(a, ncl, st));
      } else if (fast_length(Ll))
        MRSR_TRY(fast_lambda(a, ncl, op->Cg * K, op->errflag.as<int>(), st));
      else
        MRSR_TRY(launch_fft_kernel<LamPassArgs>(k_lambda_pass, grid, 512, smem, st, a));
      MRSR_TRY(rec.record());
    }
    if (g.ndims == 3) {
      const int L2 = (int)g.g[1];
      const int TC = mid_tc(op);
      int NOo = (int)std::max<int64_t>(1, kMidElems / ((int64_t)TC * L2));
      NOo = (int)std::min<int64_t>(NOo, g.n[2]);
      MidArgs a{op->plan[1].plan, L2, (int)g.n[1], g.g[0], g.n[2], TC, NOo, L2 * TC, +1.f, st2, st1};
      dim3 grid((unsigned)(g.g[0] / TC), (unsigned)cdiv(g.n[2], NOo), (unsigned)(ncg * K));
      const size_t smem = sizeof(float2) * ((size_t)L2 + 2 * (size_t)NOo * a.lstride);
      if (fast_length(L2))
        MRSR_TRY(fast_mid(a, ncg * K, st));
      else
        MRSR_TRY(launch_fft_kernel<MidArgs>(k_mid_fft, grid, 256, smem, st, a));
      MRSR_TRY(rec.record());
    }
    // P3: rows inverse + crop + coil combine
    {
      RowTiling t = rows_tiling(L1, ncg, nrows);
      RowsInvArgs a{op->plan[0].plan, (int)g.n[0], nrows, t.rpc, K, c0, ncg, t.lstride, grp == 0 ? 1 : 0, al, beta,
                    st1, cm, y};
      dim3 grid((unsigned)cdiv(nrows, t.rpc), K);
      if (tc_rows)
        MRSR_TRY(tc_rows_inv(a, op->tc_consts.p, op->errflag.as<int>(), st));
      else if (rows8_inv_supported(a))
        MRSR_TRY(fast_rows8_inv(a, st));
      else if (fast_length(L1))
        MRSR_TRY(fast_rows_inv(a, nrows, st));
      else
        MRSR_TRY(launch_fft_kernel<RowsInvArgs>(k_rows_inv, grid, t.threads, t.smem, st, a));
      MRSR_TRY(rec.record());
    }
  }
  return MRSR_OK;
}

int device_error_status(mrsr_normalop* op, int code, cudaStream_t st) {
  if (code == 0) return MRSR_OK;
  cudaMemsetAsync(op->errflag.p, 0, sizeof(int), st);
  set_error("a bounded device wait timed out during an apply (code %d): results since the last check are not valid",
            code);
  return MRSR_ERR_DEVICE;
}

int normalop_apply_internal(mrsr_normalop* op, const float2* x, float2* y, float2 alpha, float2 beta, cudaStream_t st) {
  return apply_impl(op, x, y, alpha, beta, st, Recorder{});
}

// ---------------------------------------------------------- builders ---

int op_init_geometry(mrsr_normalop* op, int kind, int ndims, const int64_t* img_shape, int K, int ncoils,
                     int precision, int kmax) {
  MRSR_REQUIRE(ndims == 2 || ndims == 3, MRSR_ERR_ARG, "ndims must be 2 or 3 (got %d)", ndims);
  MRSR_REQUIRE(img_shape != nullptr, MRSR_ERR_ARG, "img_shape is NULL");
  MRSR_REQUIRE(K >= 1 && K <= kmax, MRSR_ERR_UNSUPPORTED, "rank K=%d outside 1..%d", K, kmax);
  MRSR_REQUIRE(ncoils >= 1, MRSR_ERR_ARG, "ncoils must be >= 1");
  MRSR_REQUIRE(precision == MRSR_PREC_FP32 || precision == MRSR_PREC_FP16 || precision == MRSR_PREC_FP16_TC, MRSR_ERR_ARG,
               "unknown precision %d",
               precision);
  op->kind = kind;
  op->precision = precision;
  OpGeom& g = op->geo;
  g.ndims = ndims;
  g.K = K;
  g.ncoils = ncoils;
  for (int i = 0; i < 3; ++i) {
    g.n[i] = i < ndims ? img_shape[i] : 1;
    MRSR_REQUIRE(g.n[i] >= 1, MRSR_ERR_ARG, "image dimension %d must be positive", i + 1);
    g.g[i] = i < ndims ? (kind == MRSR_KIND_NFFT ? 2 * g.n[i] : g.n[i]) : 1;
  }
  for (int i = 0; i < ndims; ++i) {
    int rad[kMaxStages], ns;
    MRSR_REQUIRE(build_radices((int)g.g[i], rad, &ns), MRSR_ERR_ARG,
                 "AssertionError: img_shape_os has to be composed of the prime factors 2, 3, and 5 (dimension %d has %lld)", i + 1,
                 (long long)g.g[i]);
    MRSR_TRY(op->plan[i].init((int)g.g[i]));
  }
  // Λ-pass tile width: up to 8 columns, a divisor of the plane width, <= 16384 elements per CTA
  // generic kernels: two K*TC*L buffers; four-step kernels: one K*TC*L exchange buffer (<= ~110 KB, 2 CTAs/SM)
  int TC = 8;
  const int64_t budget = fast_length((int)g.glast()) ? 13000 : 12288;
  while (TC > 1 && ((int64_t)K * TC * g.glast() > budget || g.inner() % TC != 0)) TC >>= 1;
  op->TC = TC;
  if (precision == MRSR_PREC_FP16_TC) {
    const int nl = (int)g.n[ndims - 1], gl = (int)g.glast();
    MRSR_REQUIRE(kind == MRSR_KIND_NFFT && tc_lambda_supported(gl, nl, nl, (int)g.inner(), K), MRSR_ERR_UNSUPPORTED,
                 "the tensor-core Λ pass needs an NFFT operator whose last grid length is 512 (got %d)", gl);
  }
  MRSR_TRY(op->errflag.alloc(sizeof(int)));
  MRSR_CHECK_CUDA(cudaMemsetAsync(op->errflag.p, 0, sizeof(int), call_stream()));
  return MRSR_OK;
}

int op_set_cmaps(mrsr_normalop* op, const float* cmaps, cudaStream_t st) {
  if (!cmaps) {
    MRSR_REQUIRE(op->geo.ncoils == 1, MRSR_ERR_ARG, "cmaps == NULL requires ncoils == 1");
    op->cmaps.release();
    return MRSR_OK;
  }
  const size_t bytes = sizeof(float2) * op->geo.nimg() * op->geo.ncoils;
  MRSR_TRY(op->cmaps.alloc(bytes));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(op->cmaps.p, cmaps, bytes, cudaMemcpyDeviceToDevice, st));
  return MRSR_OK;
}

int op_finalize(mrsr_normalop* op, cudaStream_t st) {
  const OpGeom& g = op->geo;
  const bool half = op->precision == MRSR_PREC_FP16;
  MRSR_REQUIRE(!half || half_supported(op), MRSR_ERR_UNSUPPORTED,
               "fp16 storage needs grid lengths with a register four-step split (64, 128, 256, 384, 512, 768, 1024)");
  const int64_t esz = half ? 4 : (int64_t)sizeof(float2);
  // coils per group: keep one group's stack within ~112 MB so it stays in the 129 MB L2
  // between the three passes (measured on 256^2, K=5, Nc=20: one group of 20 coils is 5%
  // faster than groups of 7 or 10)
  const int64_t per_coil = (int64_t)g.K * g.g[0] * g.n[1] * g.n[2] * esz;
  int64_t cg;
  if (g.ndims == 2) {
    cg = std::max<int64_t>(1, (112ll << 20) / std::max<int64_t>(per_coil, 1));
  } else {
    // 3D stacks are far larger than L2; group as many coils as a 12 GB stack budget
    // allows, so one Λ pass streams the kernel once for all of them
    const int64_t per_coil3 = per_coil + (int64_t)g.K * g.g[0] * g.g[1] * g.n[2] * esz;
    cg = std::max<int64_t>(1, (12288ll << 20) / std::max<int64_t>(per_coil3, 1));
  }
  // rows inverse holds one row of every coil of the group in shared memory (<= ~200 KB)
  cg = std::min<int64_t>(cg, std::max<int64_t>(1, (200ll << 10) / (9 * g.g[0])));
  cg = std::min<int64_t>(cg, g.ncoils);
  const int64_t ngroups = cdiv(g.ncoils, cg);
  cg = cdiv(g.ncoils, ngroups);
  op->Cg = (int)cg;
  MRSR_TRY(op->stack1.alloc((size_t)(per_coil * cg)));
  if (g.ndims == 3) {
    const int64_t per_coil2 = (int64_t)g.K * g.g[0] * g.g[1] * g.n[2] * esz;
    MRSR_TRY(op->stack2.alloc((size_t)(per_coil2 * cg)));
  }
  op->launches = (int)ngroups * (g.ndims == 2 ? 3 : 5);
  if (half) {
    if (!op->lam_half.p) MRSR_TRY(half_lambda_convert(op, st));  // a shared kernel may already have it
    MRSR_TRY(half_alloc_scales(op));
  }
  if (op->precision == MRSR_PREC_FP16_TC && !op->lam_tc.p) {  // a shared kernel may already have them
    MRSR_TRY(op->tc_consts.alloc(tc_constants_bytes()));
    MRSR_TRY(tc_build_constants(op->tc_consts.p, st));
    MRSR_TRY(op->lam_max.alloc(sizeof(float)));
    MRSR_TRY(tc_lambda_bound(op->lam.p, op->lam.bytes, op->lam_max.as<float>(), st));
    const size_t esz = op->lam_mode == LAM_PACKED_REAL ? sizeof(float) : sizeof(float2);
    MRSR_TRY(op->lam_tc.alloc(esz * (size_t)g.inner() * op->P * g.glast()));
    MRSR_TRY(tc_lambda_layout(op->lam.p, op->lam_tc.p, g.inner(), op->P, op->FC, (int)(g.glast() / op->FC), op->TC,
                              op->lam_mode == LAM_PACKED_REAL, st));
  }
  // the operator's buffers came from the pool on `st`: make them usable on any stream
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return MRSR_OK;
}

static LamLayout lam_layout(const mrsr_normalop* op) {
  LamLayout l;
  l.inner = op->geo.inner();
  l.L = op->geo.glast();
  l.TC = op->TC;
  l.P = op->P;
  l.FC = op->FC;
  l.NCH = (int)(l.L / op->FC);
  l.ngrid = op->geo.ngrid();
  return l;
}

// Λ chunk length: the largest divisor of L with at most 256 positions (FC*TC)
// and at most 16 KB per chunk, so a chunk streams through a small shared ring.
static void choose_fc(mrsr_normalop* op) {
  const int L = (int)op->geo.glast();
  const int esz = lam_is_real(op->lam_mode) ? 4 : 8;
  int best = 1;
  for (int fc = 1; fc <= L; ++fc) {
    if (L % fc) continue;
    if ((int64_t)fc * op->TC > 256) continue;
    if ((int64_t)fc * op->TC * op->P * esz > 16384) continue;
    best = fc;
  }
  op->FC = best;
}

int op_set_lambda_packed(mrsr_normalop* op, const void* lam_packed, int is_complex, const int64_t* kmask, int64_t nk,
                         cudaStream_t st) {
  const int K = op->geo.K;
  MRSR_REQUIRE(lam_packed && kmask, MRSR_ERR_ARG, "Λ and kmask_indcs must be device pointers");
  MRSR_REQUIRE(nk >= 1, MRSR_ERR_ARG, "kmask_indcs is empty");
  op->lam_mode = is_complex ? LAM_PACKED_CPLX : LAM_PACKED_REAL;
  op->P = K * (K + 1) / 2;
  op->nk = nk;
  choose_fc(op);
  const size_t esz = is_complex ? sizeof(float2) : sizeof(float);
  MRSR_TRY(op->lam.alloc(esz * op->P * op->geo.ngrid()));
  MRSR_CHECK_CUDA(cudaMemsetAsync(op->lam.p, 0, op->lam.bytes, st));
  MRSR_TRY(op->kmask.alloc(sizeof(int64_t) * nk));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(op->kmask.p, kmask, sizeof(int64_t) * nk, cudaMemcpyDeviceToDevice, st));
  MRSR_CHECK_CUDA(cudaMemsetAsync(op->errflag.p, 0, sizeof(int), st));
  LamLayout l = lam_layout(op);
  const unsigned blocks = (unsigned)std::min<int64_t>(cdiv(nk, 256), 65535);
  if (is_complex)
    k_lam_from_packed<float2><<<blocks, 256, 0, st>>>(l, (const float2*)lam_packed, op->kmask.as<int64_t>(), nk,
                                                      op->lam.as<float2>(), op->errflag.as<int>());
  else
    k_lam_from_packed<float><<<blocks, 256, 0, st>>>(l, (const float*)lam_packed, op->kmask.as<int64_t>(), nk,
                                                     op->lam.as<float>(), op->errflag.as<int>());
  MRSR_LAUNCH_CHECK();
  int err = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&err, op->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  MRSR_REQUIRE(err == 0, MRSR_ERR_ARG, "AssertionError: kmask_indcs must lie in 1..prod(2 .* img_shape)");
  return MRSR_OK;
}

int op_set_lambda_full(mrsr_normalop* op, const float2* lam_full, cudaStream_t st) {
  const int K = op->geo.K;
  const int64_t ng = op->geo.ngrid();
  DevBuf flags;
  MRSR_TRY(flags.alloc(ng));
  const unsigned blocks = (unsigned)std::min<int64_t>(cdiv(ng, 256), 65535);
  k_flags_nonzero_c<<<blocks, 256, 0, st>>>(lam_full, (int64_t)K * K, ng, flags.as<uint8_t>());
  MRSR_LAUNCH_CHECK();
  int64_t nk = 0;
  DevBuf km;
  MRSR_TRY(compact_nonzero(flags.as<uint8_t>(), ng, km, &nk, st));
  MRSR_REQUIRE(nk >= 1, MRSR_ERR_ARG, "Λ[1,1,:] is zero everywhere");
  op->lam_mode = LAM_FULL_CPLX;
  op->P = K * K;
  op->nk = nk;
  choose_fc(op);
  MRSR_TRY(op->lam.alloc(sizeof(float2) * op->P * ng));
  MRSR_CHECK_CUDA(cudaMemsetAsync(op->lam.p, 0, op->lam.bytes, st));
  DevBuf packed;
  MRSR_TRY(packed.alloc(sizeof(float2) * op->P * nk));
  const unsigned b2 = (unsigned)std::min<int64_t>(cdiv(nk, 256), 65535);
  k_lam_full_to_packed<<<b2, 256, 0, st>>>(lam_full, K, km.as<int64_t>(), nk, packed.as<float2>());
  MRSR_LAUNCH_CHECK();
  LamLayout l = lam_layout(op);
  MRSR_CHECK_CUDA(cudaMemsetAsync(op->errflag.p, 0, sizeof(int), st));
  k_lam_from_packed<float2><<<b2, 256, 0, st>>>(l, packed.as<float2>(), km.as<int64_t>(), nk, op->lam.as<float2>(),
                                                op->errflag.as<int>());
  MRSR_LAUNCH_CHECK();
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  std::swap(op->kmask.p, km.p);
  std::swap(op->kmask.bytes, km.bytes);
  return MRSR_OK;
}

}  // namespace mrsr

using namespace mrsr;

static cudaStream_t as_stream(mrsr_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" int mrsr_nfft_normalop_from_lambda(int ndims, const int64_t* img_shape, int K, const void* lambda_packed,
                                              int lambda_is_complex, const int64_t* kmask_indcs, int64_t nk,
                                              const float* cmaps, int ncoils, int precision, mrsr_stream_t stream,
                                              mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  cudaStream_t st = as_stream(stream);
  mrsr_normalop* op = new mrsr_normalop();
  int s = op_init_geometry(op, MRSR_KIND_NFFT, ndims, img_shape, K, cmaps ? ncoils : 1, precision);
  if (s == MRSR_OK) s = op_set_cmaps(op, cmaps, st);
  if (s == MRSR_OK) s = op_set_lambda_packed(op, lambda_packed, lambda_is_complex, kmask_indcs, nk, st);
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  *out = op;
  return MRSR_OK;
}

extern "C" int mrsr_fft_normalop_from_lambda(int ndims, const int64_t* img_shape, int K, const float* lambda_full,
                                             const float* cmaps, int ncoils, int precision, mrsr_stream_t stream,
                                             mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(lambda_full, MRSR_ERR_ARG, "Λ is NULL");
  cudaStream_t st = as_stream(stream);
  mrsr_normalop* op = new mrsr_normalop();
  int s = op_init_geometry(op, MRSR_KIND_FFT, ndims, img_shape, K, cmaps ? ncoils : 1, precision);
  if (s == MRSR_OK) s = op_set_cmaps(op, cmaps, st);
  if (s == MRSR_OK) s = op_set_lambda_full(op, reinterpret_cast<const float2*>(lambda_full), st);
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  *out = op;
  return MRSR_OK;
}

extern "C" int mrsr_normalop_apply(mrsr_normalop* op, const float* x, float* y, float alpha_re, float alpha_im,
                                   float beta_re, float beta_im, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && x && y, MRSR_ERR_ARG, "NULL argument to mrsr_normalop_apply");
  MRSR_REQUIRE((const void*)x != (const void*)y, MRSR_ERR_ARG, "x and y must not alias");
  OpUse use{op, as_stream(stream)};
  return apply_impl(op, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(y),
                    make_float2(alpha_re, alpha_im), make_float2(beta_re, beta_im), as_stream(stream), Recorder{});
}

// Host -> device copy by the SMs: 16-byte loads over the CPU-GPU link from device-addressable
// host memory, many in flight (n16 16-byte units; both addresses 16-byte aligned).
__global__ void __launch_bounds__(256) k_copy_in(const float4* __restrict__ src, float4* __restrict__ dst, int64_t n16) {
  constexpr int U = 4;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n16; i += U * step) {
    float4 v[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i + u * step < n16) v[u] = src[i + u * step];
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (i + u * step < n16) dst[i + u * step] = v[u];
  }
}

// A host pointer the device can address directly (page-locked or mapped memory, or any host
// memory on a system with address translation from the GPU), else null.
static void* device_view(void* host) {
  void* d = nullptr;
  if (cudaHostGetDevicePointer(&d, host, 0) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return d;
}

extern "C" int mrsr_normalop_apply_host(mrsr_normalop* op, const float* x, float* y, float alpha_re, float alpha_im,
                                        float beta_re, float beta_im, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && x && y, MRSR_ERR_ARG, "NULL argument to mrsr_normalop_apply_host");
  MRSR_REQUIRE((const void*)x != (const void*)y, MRSR_ERR_ARG, "x and y must not alias");
  MRSR_REQUIRE(((uintptr_t)x & 7) == 0 && ((uintptr_t)y & 7) == 0, MRSR_ERR_ARG,
               "x and y must be aligned to their ComplexF32 elements (8 bytes)");
  const cudaStream_t st = as_stream(stream);
  OpUse use{op, st};
  const OpGeom& g = op->geo;
  const size_t bytes = sizeof(float2) * (size_t)(g.n[0] * g.n[1] * g.n[2] * g.K);
  HostIo& h = op->hio;
  if (h.x.bytes < bytes) MRSR_TRY(h.x.alloc(bytes));
  float2* xd = h.x.as<float2>();
  const void* xv = device_view(const_cast<float*>(x));
  if (xv && bytes % 16 == 0 && ((uintptr_t)xv & 15) == 0) {
    const int64_t n16 = (int64_t)(bytes / 16);
    int dev = 0, nsm = 0;
    MRSR_CHECK_CUDA(cudaGetDevice(&dev));
    MRSR_CHECK_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int64_t blocks = std::min<int64_t>(cdiv(n16, 256), (int64_t)nsm * 8);
    k_copy_in<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const float4*>(xv), reinterpret_cast<float4*>(xd), n16);
    MRSR_LAUNCH_CHECK();
  } else {
    MRSR_CHECK_CUDA(cudaMemcpyAsync(xd, x, bytes, cudaMemcpyHostToDevice, st));
  }
  const float2 alpha = make_float2(alpha_re, alpha_im), beta = make_float2(beta_re, beta_im);
  // With one coil group the inverse row pass writes every element of y once: it stores
  // straight into the host array over the CPU-GPU link, so no copy back follows the apply.
  float2* yv = cdiv(g.ncoils, op->Cg) == 1 ? static_cast<float2*>(device_view(y)) : nullptr;
  if (yv) return apply_impl(op, xd, yv, alpha, beta, st, Recorder{});
  if (h.y.bytes < bytes) MRSR_TRY(h.y.alloc(bytes));
  float2* yd = h.y.as<float2>();
  if (beta_re != 0.f || beta_im != 0.f) MRSR_CHECK_CUDA(cudaMemcpyAsync(yd, y, bytes, cudaMemcpyHostToDevice, st));
  MRSR_TRY(apply_impl(op, xd, yd, alpha, beta, st, Recorder{}));
  MRSR_CHECK_CUDA(cudaMemcpyAsync(y, yd, bytes, cudaMemcpyDeviceToHost, st));
  return MRSR_OK;
}

extern "C" int mrsr_normalop_info(const mrsr_normalop* op, int64_t* info) {
  MRSR_REQUIRE(op && info, MRSR_ERR_ARG, "NULL argument");
  const OpGeom& g = op->geo;
  int64_t v[12] = {op->kind, g.ndims, g.n[0], g.n[1], g.n[2], g.K, g.ncoils, op->nk,
                   lam_is_real(op->lam_mode) ? 0 : 1, op->precision, op->P, op->launches};
  std::memcpy(info, v, sizeof(v));
  return MRSR_OK;
}

extern "C" int mrsr_normalop_get_kmask(const mrsr_normalop* op, int64_t* out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && out, MRSR_ERR_ARG, "NULL argument");
  OpUse use{op, as_stream(stream)};
  MRSR_CHECK_CUDA(cudaMemcpyAsync(out, op->kmask.p, sizeof(int64_t) * op->nk, cudaMemcpyDeviceToDevice,
                                  as_stream(stream)));
  return MRSR_OK;
}

// packed upper triangle (P, nk) -> full (K, K, nk) complex (FFTNormalOp's Λ layout)
__global__ void k_unpack_full(const void* packed, int real, int K, int64_t nk, float2* out) {
  const int P = K * (K + 1) / 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x) {
    for (int k2 = 0; k2 < K; ++k2)
      for (int k1 = 0; k1 < K; ++k1) {
        const int a = k1 <= k2 ? k1 : k2, b = k1 <= k2 ? k2 : k1;
        const int p = a + b * (b + 1) / 2;
        float2 v = real ? make_float2(reinterpret_cast<const float*>(packed)[p + (int64_t)P * i], 0.f)
                        : reinterpret_cast<const float2*>(packed)[p + (int64_t)P * i];
        if (k1 > k2) v.y = -v.y;
        out[k1 + (int64_t)K * (k2 + (int64_t)K * i)] = v;
      }
  }
}

extern "C" int mrsr_normalop_get_lambda(const mrsr_normalop* op, void* out, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && out, MRSR_ERR_ARG, "NULL argument");
  MRSR_REQUIRE(!lam_is_diag(op->lam_mode), MRSR_ERR_UNSUPPORTED,
               "a stacked operator holds its source operator's kernel: read Λ from the source");
  cudaStream_t st = as_stream(stream);
  OpUse use{op, st};
  LamLayout l = lam_layout(op);
  const unsigned blocks = (unsigned)std::min<int64_t>(cdiv(op->nk, 256), 65535);
  if (op->kind == MRSR_KIND_FFT && op->lam_mode != LAM_FULL_CPLX) {
    const int real = op->lam_mode == LAM_PACKED_REAL;
    DevBuf packed;
    MRSR_TRY(packed.alloc((real ? 4 : 8) * (size_t)op->P * op->nk));
    if (real)
      k_lam_to_packed<float><<<blocks, 256, 0, st>>>(l, op->lam.as<float>(), op->kmask.as<int64_t>(), op->nk,
                                                     packed.as<float>());
    else
      k_lam_to_packed<float2><<<blocks, 256, 0, st>>>(l, op->lam.as<float2>(), op->kmask.as<int64_t>(), op->nk,
                                                      packed.as<float2>());
    k_unpack_full<<<blocks, 256, 0, st>>>(packed.p, real, op->geo.K, op->nk, reinterpret_cast<float2*>(out));
    MRSR_LAUNCH_CHECK();
    MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
    return MRSR_OK;
  }
  if (op->lam_mode == LAM_PACKED_REAL)
    k_lam_to_packed<float><<<blocks, 256, 0, st>>>(l, op->lam.as<float>(), op->kmask.as<int64_t>(), op->nk, (float*)out);
  else
    k_lam_to_packed<float2><<<blocks, 256, 0, st>>>(l, op->lam.as<float2>(), op->kmask.as<int64_t>(), op->nk,
                                                    (float2*)out);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

extern "C" int mrsr_normalop_profile(mrsr_normalop* op, const float* x, float* y, int iters, float* ms_per_pass,
                                     mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op && x && y && ms_per_pass && iters > 0, MRSR_ERR_ARG, "bad argument to mrsr_normalop_profile");
  cudaStream_t st = as_stream(stream);
  OpUse use{op, st};
  std::vector<double> acc(op->launches, 0.0);
  for (int it = 0; it < iters; ++it) {
    std::vector<cudaEvent_t> ev;
    Recorder rec{&ev, st};
    MRSR_TRY(rec.record());
    int s = apply_impl(op, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(y), make_float2(1.f, 0.f),
                       make_float2(0.f, 0.f), st, rec);
    if (s == MRSR_OK) s = (cudaEventSynchronize(ev.back()) == cudaSuccess) ? MRSR_OK : MRSR_ERR_CUDA;
    if (s == MRSR_OK) {
      for (int i = 0; i + 1 < (int)ev.size() && i < op->launches; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[i], ev[i + 1]);
        acc[i] += ms;
      }
    }
    for (auto e : ev) cudaEventDestroy(e);
    if (s != MRSR_OK) return s;
  }
  for (int i = 0; i < op->launches; ++i) ms_per_pass[i] = (float)(acc[i] / iters);
  return MRSR_OK;
}

extern "C" int mrsr_normalop_stack(const mrsr_normalop* src, int nrhs, mrsr_stream_t stream, mrsr_normalop** out) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(out, MRSR_ERR_ARG, "out is NULL");
  *out = nullptr;
  MRSR_REQUIRE(src, MRSR_ERR_ARG, "source operator is NULL");
  MRSR_REQUIRE(src->lam.p, MRSR_ERR_STATE, "source operator has no kernel");
  MRSR_REQUIRE(src->geo.K == 1 && src->precision == MRSR_PREC_FP32 && !lam_is_diag(src->lam_mode),
               MRSR_ERR_UNSUPPORTED, "stacking needs a float32 operator of rank K = 1 (got K = %d)", src->geo.K);
  MRSR_REQUIRE(nrhs >= 1 && nrhs <= kStackMax, MRSR_ERR_ARG, "nrhs must be in 1..%d (got %d)", kStackMax, nrhs);
  const OpGeom& g = src->geo;
  // the row and Λ passes hold every plane of a line (two copies in the generic kernels)
  const int64_t lmax = std::max(g.g[0], g.glast());
  MRSR_REQUIRE((2 * (int64_t)nrhs + 1) * lmax * 8 <= 227 * 1024, MRSR_ERR_UNSUPPORTED,
               "%d stacked right-hand sides of %lld-point lines exceed the shared memory of one block", nrhs,
               (long long)lmax);
  cudaStream_t st = as_stream(stream);
  mrsr_normalop* op = new mrsr_normalop();
  int s = op_init_geometry(op, src->kind, g.ndims, g.n, nrhs, g.ncoils, MRSR_PREC_FP32, kStackMax);
  if (s == MRSR_OK) {
    const bool real = lam_is_real(src->lam_mode);
    op->lam_mode = real ? LAM_DIAG_REAL : LAM_DIAG_CPLX;
    op->P = 1;
    op->nk = src->nk;
    choose_fc(op);
    const size_t esz = real ? sizeof(float) : sizeof(float2);
    s = op->lam.alloc(esz * (size_t)g.ngrid());
    if (s == MRSR_OK) {
      const LamLayout ls = lam_layout(src), ld = lam_layout(op);
      const unsigned blocks = (unsigned)std::min<int64_t>(cdiv(g.ngrid(), 256), 65535);
      if (real)
        k_lam_relayout<float><<<blocks, 256, 0, st>>>(ls, ld, src->lam.as<float>(), op->lam.as<float>());
      else
        k_lam_relayout<float2><<<blocks, 256, 0, st>>>(ls, ld, src->lam.as<float2>(), op->lam.as<float2>());
      if (cudaGetLastError() != cudaSuccess) {
        set_error("Λ relayout launch failed");
        s = MRSR_ERR_CUDA;
      }
    }
    if (s == MRSR_OK) s = op->kmask.alloc(sizeof(int64_t) * (size_t)src->nk);
    if (s == MRSR_OK &&
        cudaMemcpyAsync(op->kmask.p, src->kmask.p, sizeof(int64_t) * src->nk, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess) {
      set_error("kmask copy failed");
      s = MRSR_ERR_CUDA;
    }
    if (s == MRSR_OK && src->cmaps.p) s = op_set_cmaps(op, src->cmaps.as<float>(), st);
  }
  if (s == MRSR_OK) s = op_finalize(op, st);
  if (s != MRSR_OK) {
    delete op;
    return s;
  }
  mark_use(src, st);
  mark_use(op, st);
  *out = op;
  return MRSR_OK;
}

extern "C" int mrsr_normalop_check(mrsr_normalop* op, mrsr_stream_t stream) {
  MRSR_CALL_SCOPE(reinterpret_cast<cudaStream_t>(stream));
  MRSR_REQUIRE(op, MRSR_ERR_ARG, "operator is NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  int code = 0;
  MRSR_CHECK_CUDA(cudaMemcpyAsync(&code, op->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return device_error_status(op, code, st);
}

extern "C" void mrsr_normalop_destroy(mrsr_normalop* op) { delete op; }

mrsr_normalop::~mrsr_normalop() {
  if (last_use) {
    // members are freed on the library stream after the last enqueued use
    cudaStreamWaitEvent(mrsr::lib_stream(), last_use, 0);
    cudaEventDestroy(last_use);
  }
}

namespace mrsr {
int mark_use(const mrsr_normalop* cop, cudaStream_t st) {
  mrsr_normalop* op = const_cast<mrsr_normalop*>(cop);
  if (!op->last_use) MRSR_CHECK_CUDA(cudaEventCreateWithFlags(&op->last_use, cudaEventDisableTiming));
  MRSR_CHECK_CUDA(cudaEventRecord(op->last_use, st));
  return MRSR_OK;
}
}  // namespace mrsr
