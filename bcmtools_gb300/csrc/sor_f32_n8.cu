// sor_f32_n8.cu -- float tile kernels for 8^3-cell blocks (sor_impl.cuh).
#include "sor_impl.cuh"

namespace bcmg {
template cudaError_t launch_sor_tile<float, 8>(const float*, float*, const float*, const Geom&,
                                              const SorArgs&, bool, int, cudaStream_t);
template cudaError_t launch_sor_pull<float, 8>(const float*, float*, const float*, const Geom&,
                                              const SorArgs&, int, cudaStream_t);
}  // namespace bcmg
