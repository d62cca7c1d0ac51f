// phoenix32_n1p1.cu — the tiled FP32 kernel's instantiations for 1 asset, 1 path per thread
// (p32_tiled.cuh).
#include "p32_tiled.cuh"

namespace rg {
RG_P32_DEFINE(1, 1)
}  // namespace rg
