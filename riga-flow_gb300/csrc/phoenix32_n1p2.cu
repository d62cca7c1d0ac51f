// phoenix32_n1p2.cu — the tiled FP32 kernel's instantiations for 1 asset, 2 paths per thread
// (p32_tiled.cuh).
#include "p32_tiled.cuh"

namespace rg {
RG_P32_DEFINE(1, 2)
}  // namespace rg
