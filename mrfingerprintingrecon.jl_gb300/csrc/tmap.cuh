// Host helper: 3D float32 tiled tensor map (no swizzle, zero fill out of bounds).
#pragma once
#include <cuda.h>
#include <cstdint>

namespace mrsr {
int encode_tmap_f32_3d(CUtensorMap* map, const void* base, const uint64_t dims[3], const uint64_t strides_bytes[2],
                       const uint32_t box[3]);
}  // namespace mrsr
