// Batched in-place complex FFT along one axis of a dense column-major array,
// and the N-D transform built from it.  Used by the NUFFT (upsampled grids),
// the Toeplitz-kernel precompute and the Cartesian backprojection.
//
// Layout seen by one axis: data[outer][n][width] with the transformed index n
// of length L, `width` contiguous columns (the product of the faster axes)
// and `outer` the product of the slower axes and the batch.  A CTA takes TC
// adjacent columns of NOo consecutive outer slices (TC = 1 and width = 1 for
// the contiguous axis).
#include <algorithm>

#include "fft4.cuh"
#include "fftnd.cuh"

namespace mrsr {

struct AxisArgs {
  FftPlan pl;
  int64_t width, nouter;
  int TC, NOo, lstride;
  int64_t ntile;       // width / TC
  float sgn, scale;    // scale multiplies the output
  float2* data;
};

// generic Stockham (any 2,3,5-smooth length)
__global__ void __launch_bounds__(256) k_axis_generic(AxisArgs a) {
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* s0 = smem + a.pl.L;
  float2* s1 = s0 + a.NOo * a.lstride;
  load_twiddles(tw, a.pl);
  const int L = a.pl.L;
  const int64_t tile = blockIdx.x % a.ntile;
  const int64_t o0 = (blockIdx.x / a.ntile) * a.NOo;
  const int no = (int)min((int64_t)a.NOo, a.nouter - o0);
  float2* base = a.data + o0 * L * a.width + tile * a.TC;
  for (int e = threadIdx.x; e < a.NOo * L * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % L;
    const int o = t / L;
    s0[o * a.lstride + n * a.TC + li] = (o < no) ? base[((int64_t)o * L + n) * a.width + li] : make_float2(0.f, 0.f);
  }
  __syncthreads();
  LineLayout ly{a.NOo, a.TC, a.lstride};
  const float2* res = fft_lines(s0, s1, a.pl, ly, a.sgn, tw, false, false);
  for (int e = threadIdx.x; e < no * L * a.TC; e += blockDim.x) {
    const int li = e % a.TC;
    const int t = e / a.TC;
    const int n = t % L;
    const int o = t / L;
    base[((int64_t)o * L + n) * a.width + li] = cscale(res[o * a.lstride + n * a.TC + li], a.scale);
  }
}

// register four-step (compiled lengths)
template <class SP, int S>
__global__ void __launch_bounds__(256) k_axis_fast(AxisArgs a, Slots sl) {
  constexpr int R1 = SP::R1, R2 = SP::R2, L = SP::L;
  extern __shared__ float2 smem[];
  float2* tw = smem;
  float2* sm = smem + L;
  load_twiddles_a<SP>(tw, a.pl);
  const int64_t tile = blockIdx.x % a.ntile;
  const int64_t o0 = (blockIdx.x / a.ntile) * a.NOo;
  const int no = (int)min((int64_t)a.NOo, a.nouter - o0);
  float2* base = a.data + o0 * L * a.width + tile * a.TC;
  __syncthreads();
  step_a<SP, S, true>(sm, sl, a.NOo, tw, R1, [&](int o, int li, int n) -> float2 {
    return (o < no) ? base[((int64_t)o * L + n) * a.width + li] : make_float2(0.f, 0.f);
  });
  __syncthreads();
  step_b<SP, S>(sm, sl, a.NOo, R2, [&](int o, int li, int f1, int f2, float2 v) {
    if (o < no) base[((int64_t)o * L + f1 + R1 * f2) * a.width + li] = cscale(v, a.scale);
  });
}

template <class F>
static int with_split_axis(int L, F f) {
  switch (L) {
    case 64: return f(Split<8, 8>());
    case 128: return f(Split<8, 16>());
    case 256: return f(Split<16, 16>());
    case 384: return f(Split<12, 32>());
    case 512: return f(Split<16, 32>());
    case 768: return f(Split<24, 32>());
    case 1024: return f(Split<32, 32>());
    default: return MRSR_ERR_UNSUPPORTED;
  }
}

static int ilog2i(int x) {
  int s = 0;
  while ((1 << s) < x) ++s;
  return s;
}

int fft_axis(float2* data, const FftPlan& pl, int64_t width, int64_t nouter, int sign, float scale, cudaStream_t st) {
  const int L = pl.L;
  if (L == 1 || nouter == 0) return MRSR_OK;
  AxisArgs a;
  a.pl = pl;
  a.width = width;
  a.nouter = nouter;
  a.TC = 1;
  if (width > 1)
    while (a.TC < 8 && width % (a.TC * 2) == 0) a.TC *= 2;
  a.ntile = width / a.TC;
  a.sgn = (float)sign;
  a.scale = scale;
  a.data = data;
  const bool fast = with_split_axis(L, [](auto) { return MRSR_OK; }) == MRSR_OK;
  if (fast) {
    return with_split_axis(L, [&](auto sp) -> int {
      using SP = decltype(sp);
      Slots sl;
      sl.TC = a.TC;
      sl.tcs = ilog2i(a.TC);
      sl.W = slots_width(SP::R2, a.TC);
      int NOo = (int)std::max<int64_t>(1, 4096 / ((int64_t)a.TC * L));
      NOo = (int)std::min<int64_t>(NOo, nouter);
      a.NOo = NOo;
      a.lstride = 0;
      const size_t smem = sizeof(float2) * ((size_t)L + (size_t)NOo * SP::R1 * sl.W);
      const int64_t nblk = a.ntile * cdiv(nouter, NOo);
      auto k = sign < 0 ? k_axis_fast<SP, -1> : k_axis_fast<SP, +1>;
      if (smem > 48 * 1024) MRSR_CHECK_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      k<<<(unsigned)nblk, 256, smem, st>>>(a, sl);
      MRSR_LAUNCH_CHECK();
      return MRSR_OK;
    });
  }
  int NOo = (int)std::max<int64_t>(1, 2048 / ((int64_t)a.TC * L));
  NOo = (int)std::min<int64_t>(NOo, nouter);
  a.NOo = NOo;
  a.lstride = L * a.TC;
  const size_t smem = sizeof(float2) * ((size_t)L + 2 * (size_t)NOo * a.lstride);
  MRSR_REQUIRE(smem <= 227 * 1024, MRSR_ERR_UNSUPPORTED, "FFT length %d too long for the generic kernel", L);
  if (smem > 48 * 1024)
    MRSR_CHECK_CUDA(cudaFuncSetAttribute(k_axis_generic, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int64_t nblk = a.ntile * cdiv(nouter, NOo);
  k_axis_generic<<<(unsigned)nblk, 256, smem, st>>>(a);
  MRSR_LAUNCH_CHECK();
  return MRSR_OK;
}

int FftNd::init(int d, const int64_t* n) {
  ndims = d;
  for (int i = 0; i < 3; ++i) dims[i] = i < d ? n[i] : 1;
  for (int i = 0; i < d; ++i) MRSR_TRY(plans[i].init((int)dims[i]));
  return MRSR_OK;
}

int FftNd::run(float2* data, int64_t nbatch, int sign, float scale, cudaStream_t st) const {
  int64_t width = 1;
  int64_t total = dims[0] * dims[1] * dims[2];
  for (int ax = 0; ax < ndims; ++ax) {
    const int64_t L = dims[ax];
    const int64_t nouter = total / (width * L) * nbatch;
    const float sc = (ax == ndims - 1) ? scale : 1.0f;
    MRSR_TRY(fft_axis(data, plans[ax].plan, width, nouter, sign, sc, st));
    width *= L;
  }
  return MRSR_OK;
}

}  // namespace mrsr
