// Entry points declared in mrsr.h whose kernels are not built yet: they
// report MRSR_ERR_UNSUPPORTED instead of computing anything.
#include "common.cuh"

#define MRSR_PENDING(name) \
  do { mrsr::set_error("%s is not available in this build", name); return MRSR_ERR_UNSUPPORTED; } while (0)

extern "C" {
int mrsr_grog_calib(int, int64_t, int64_t, int64_t, int, int, const float*, const float*, float*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_grog_calib");
}
int mrsr_grog_gridding(int, const int64_t*, int64_t, int64_t, int64_t, int, int, float*, const float*, const float*,
                       int32_t*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_grog_gridding");
}
}
