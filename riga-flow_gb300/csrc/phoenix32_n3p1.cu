// phoenix32_n3p1.cu — the tiled FP32 kernel's instantiations for 3 assets, 1 path per thread
// (p32_tiled.cuh).
#include "p32_tiled.cuh"

namespace rg {
RG_P32_DEFINE(3, 1)
}  // namespace rg
