// Explicit instantiation of the C=5 kernels (one translation unit per spinor
// size so that the build compiles them in parallel).
#include "gpe_kernels.cuh"

namespace gpe {
GPE_INSTANTIATE(float, 5)
GPE_INSTANTIATE(double, 5)
GPE_INSTANTIATE_TILE(float, 5)
GPE_INSTANTIATE_TILE(double, 5)
GPE_INSTANTIATE_MARCH(float, 5)
GPE_INSTANTIATE_MARCH(double, 5)
GPE_INSTANTIATE_SLAB(float, 5)
GPE_INSTANTIATE_SLAB(double, 5)
GPE_INSTANTIATE_ROWS(float, 5)
GPE_INSTANTIATE_ROWS(double, 5)
GPE_INSTANTIATE_INIT(float, 5)
GPE_INSTANTIATE_INIT(double, 5)
GPE_INSTANTIATE_HYPER_TILE(float, 5)
GPE_INSTANTIATE_HYPER_TILE(double, 5)
GPE_INSTANTIATE_IL(5)
}  // namespace gpe
