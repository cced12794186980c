// Explicit instantiation of the C=1 kernels (one translation unit per spinor
// size so that the build compiles them in parallel).
#include "gpe_kernels.cuh"

namespace gpe {
GPE_INSTANTIATE(float, 1)
GPE_INSTANTIATE(double, 1)
GPE_INSTANTIATE_TILE(float, 1)
GPE_INSTANTIATE_TILE(double, 1)
GPE_INSTANTIATE_MARCH(float, 1)
GPE_INSTANTIATE_MARCH(double, 1)
GPE_INSTANTIATE_SLAB(float, 1)
GPE_INSTANTIATE_SLAB(double, 1)
GPE_INSTANTIATE_ROWS(float, 1)
GPE_INSTANTIATE_ROWS(double, 1)
GPE_INSTANTIATE_INIT(float, 1)
GPE_INSTANTIATE_INIT(double, 1)
GPE_INSTANTIATE_HYPER_TILE(float, 1)
GPE_INSTANTIATE_HYPER_TILE(double, 1)
template cudaError_t launch_split<float>(const StepArgs&, int, double, cudaStream_t);
template cudaError_t launch_split<double>(const StepArgs&, int, double, cudaStream_t);

cudaError_t launch_dot(const StepArgs& a, int precision, int C, double* out, cudaStream_t s) {
    if (precision == GPE_FP64) {
        if (C == 1) return launch_dot_t<double, 1>(a, out, s);
        if (C == 3) return launch_dot_t<double, 3>(a, out, s);
        return launch_dot_t<double, 5>(a, out, s);
    }
    if (C == 1) return launch_dot_t<float, 1>(a, out, s);
    if (C == 3) return launch_dot_t<float, 3>(a, out, s);
    return launch_dot_t<float, 5>(a, out, s);
}

cudaError_t launch_pack_any(int precision, double* packed, char* dev_base, uint32_t X, uint32_t Y, uint32_t Z,
                            uint32_t vals, size_t pitch, size_t slice, bool to_device, cudaStream_t s) {
    if (precision == GPE_FP64) return launch_pack<double>(packed, dev_base, X, Y, Z, vals, pitch, slice, to_device, s);
    return launch_pack<float>(packed, dev_base, X, Y, Z, vals, pitch, slice, to_device, s);
}
GPE_INSTANTIATE_IL(1)
GPE_DEFINE_IL_CONVERT
}  // namespace gpe
