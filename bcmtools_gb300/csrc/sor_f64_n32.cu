// sor_f64_n32.cu -- double tile kernels for 32^3-cell blocks (sor_impl.cuh).
#include "sor_impl.cuh"

namespace bcmg {
template cudaError_t launch_sor_tile<double, 32>(const double*, double*, const double*, const Geom&,
                                              const SorArgs&, bool, int, cudaStream_t);
}  // namespace bcmg
