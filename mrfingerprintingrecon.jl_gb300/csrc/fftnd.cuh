// Batched N-D complex FFT on dense column-major arrays (in place).
#pragma once
#include "fft.cuh"

namespace mrsr {

// One axis: data[outer][n][width], n of length plan.L; sign -1 forward, +1 inverse
// (unnormalised); the result is multiplied by `scale`.
int fft_axis(float2* data, const FftPlan& pl, int64_t width, int64_t nouter, int sign, float scale, cudaStream_t st);

struct FftNd {
  int ndims = 0;
  int64_t dims[3] = {1, 1, 1};
  FftPlanHost plans[3];
  int init(int d, const int64_t* n);
  // transform nbatch consecutive arrays of shape dims (column-major)
  int run(float2* data, int64_t nbatch, int sign, float scale, cudaStream_t st) const;
};

}  // namespace mrsr
