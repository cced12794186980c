// Explicit instantiation of the C=5 kernels (one translation unit per spinor
// size so that the build compiles them in parallel).
#include "gpe_kernels.cuh"

namespace gpe {
GPE_INSTANTIATE(float, 5)
GPE_INSTANTIATE(double, 5)
GPE_INSTANTIATE_TILE(float, 5)
GPE_INSTANTIATE_TILE(double, 5)
}  // namespace gpe
