// phoenix32_n4p1.cu — the tiled FP32 kernel's instantiations for 4 assets, 1 path per thread
// (p32_tiled.cuh).
#include "p32_tiled.cuh"

namespace rg {
RG_P32_DEFINE(4, 1)
}  // namespace rg
