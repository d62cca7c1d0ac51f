// phoenix32_n2p2.cu — the tiled FP32 kernel's instantiations for 2 assets, 2 paths per thread
// (p32_tiled.cuh).
#include "p32_tiled.cuh"

namespace rg {
RG_P32_DEFINE(2, 2)
}  // namespace rg
