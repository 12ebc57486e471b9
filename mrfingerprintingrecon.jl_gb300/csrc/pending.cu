// Entry points declared in mrsr.h whose kernels are not built yet: they
// report MRSR_ERR_UNSUPPORTED instead of computing anything.
#include "common.cuh"

#define MRSR_PENDING(name) \
  do { mrsr::set_error("%s is not available in this build", name); return MRSR_ERR_UNSUPPORTED; } while (0)

extern "C" {
int mrsr_nfft_normalop_create(int, const int64_t*, int64_t, int64_t, const float*, const uint8_t*, const void*, int,
                              int, const float*, int, int, mrsr_stream_t, mrsr_normalop**) {
  MRSR_PENDING("mrsr_nfft_normalop_create");
}
int mrsr_fft_normalop_create(int, const int64_t*, int64_t, int64_t, const int32_t*, const uint8_t*, const void*, int,
                             int, int, const float*, int, int, mrsr_stream_t, mrsr_normalop**) {
  MRSR_PENDING("mrsr_fft_normalop_create");
}
int mrsr_fft_normalop_create_from_mask(int, const int64_t*, int64_t, const uint8_t*, const void*, int, int,
                                       const float*, int, int, mrsr_stream_t, mrsr_normalop**) {
  MRSR_PENDING("mrsr_fft_normalop_create_from_mask");
}
int mrsr_backprojection(int, const int64_t*, int64_t, int64_t, int, const float*, const float*, const uint8_t*,
                        const void*, int, int, const float*, int, const float*, float*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_backprojection");
}
int mrsr_backprojection_cartesian(int, const int64_t*, int64_t, int64_t, int, int, const float*, const int32_t*,
                                  const uint8_t*, const void*, int, int, const float*, float*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_backprojection_cartesian");
}
int mrsr_forward_model(int, const int64_t*, int64_t, int64_t, int, const float*, const float*, const void*, int, int,
                       const float*, float*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_forward_model");
}
int mrsr_grog_calib(int, int64_t, int64_t, int64_t, int, int, const float*, const float*, float*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_grog_calib");
}
int mrsr_grog_gridding(int, const int64_t*, int64_t, int64_t, int64_t, int, int, float*, const float*, const float*,
                       int32_t*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_grog_gridding");
}
int mrsr_cg(mrsr_normalop*, const float*, float*, int, double, double, int*, double*, mrsr_stream_t) {
  MRSR_PENDING("mrsr_cg");
}
int mrsr_cg_refined(mrsr_normalop*, mrsr_normalop*, const float*, float*, int, int, double, int*, double*,
                    mrsr_stream_t) {
  MRSR_PENDING("mrsr_cg_refined");
}
}
