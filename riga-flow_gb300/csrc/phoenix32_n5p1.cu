// phoenix32_n5p1.cu — the tiled FP32 kernel's instantiations for 5 assets, 1 path per thread
// (p32_tiled.cuh).
#include "p32_tiled.cuh"

namespace rg {
RG_P32_DEFINE(5, 1)
}  // namespace rg
