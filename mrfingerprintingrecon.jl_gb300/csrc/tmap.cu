// Host-side encoding of TMA tensor maps through the driver entry point
// (the runtime resolves cuTensorMapEncodeTiled; no link against libcuda).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tmap.cuh"

namespace mrsr {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

int encode_tmap_f32_3d(CUtensorMap* map, const void* base, const uint64_t dims[3], const uint64_t strides_bytes[2],
                       const uint32_t box[3]) {
  auto fn = encode_fn();
  MRSR_REQUIRE(fn != nullptr, MRSR_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  cuuint64_t gd[3] = {dims[0], dims[1], dims[2]};
  cuuint64_t gs[2] = {strides_bytes[0], strides_bytes[1]};
  cuuint32_t bd[3] = {box[0], box[1], box[2]};
  cuuint32_t es[3] = {1, 1, 1};
  CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<void*>(base), gd, gs, bd, es,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  MRSR_REQUIRE(r == CUDA_SUCCESS, MRSR_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d) dims %llu,%llu,%llu box %u,%u,%u",
               (int)r, (unsigned long long)dims[0], (unsigned long long)dims[1], (unsigned long long)dims[2], box[0],
               box[1], box[2]);
  return MRSR_OK;
}

}  // namespace mrsr
