// sor_f64_n16.cu -- double tile kernels for 16^3-cell blocks (sor_impl.cuh).
#include "sor_impl.cuh"

namespace bcmg {
template cudaError_t launch_sor_tile<double, 16>(const double*, double*, const double*, const Geom&,
                                              const SorArgs&, bool, int, cudaStream_t);
template cudaError_t launch_sor_pull<double, 16>(const double*, double*, const double*, const Geom&,
                                              const SorArgs&, int, cudaStream_t);
}  // namespace bcmg
