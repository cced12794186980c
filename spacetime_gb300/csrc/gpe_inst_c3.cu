// Explicit instantiation of the C=3 kernels (one translation unit per spinor
// size so that the build compiles them in parallel).
#include "gpe_kernels.cuh"

namespace gpe {
GPE_INSTANTIATE(float, 3)
GPE_INSTANTIATE(double, 3)
GPE_INSTANTIATE_TILE(float, 3)
GPE_INSTANTIATE_TILE(double, 3)
GPE_INSTANTIATE_MARCH(float, 3)
GPE_INSTANTIATE_MARCH(double, 3)
GPE_INSTANTIATE_SLAB(float, 3)
GPE_INSTANTIATE_SLAB(double, 3)
GPE_INSTANTIATE_ROWS(float, 3)
GPE_INSTANTIATE_ROWS(double, 3)
GPE_INSTANTIATE_INIT(float, 3)
GPE_INSTANTIATE_INIT(double, 3)
GPE_INSTANTIATE_HYPER_TILE(float, 3)
GPE_INSTANTIATE_HYPER_TILE(double, 3)
GPE_INSTANTIATE_IL(3)
}  // namespace gpe
