// Test-only entry points declared in include/mrsr_test.h (not in the product
// ABI of mrsr.h).  They let the test suite exercise the device-error reporting
// path without making a kernel time out or fault.
#include "mrsr_test.h"
#include "normalop.cuh"

using namespace mrsr;

extern "C" int mrsr_test_set_device_error(mrsr_normalop* op, int code, mrsr_stream_t stream) {
  MRSR_REQUIRE(op, MRSR_ERR_ARG, "operator is NULL");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  MRSR_CHECK_CUDA(cudaMemcpyAsync(op->errflag.p, &code, sizeof(int), cudaMemcpyHostToDevice, st));
  MRSR_CHECK_CUDA(cudaStreamSynchronize(st));
  return MRSR_OK;
}
