// sor_f32.cu -- float instantiation of the red-black SOR kernels
// (sor_impl.cuh), compiled as its own translation unit.
#include "sor_impl.cuh"

namespace bcmg {
template cudaError_t launch_sor<float>(const float*, float*, const float*, const Geom&, const double*,
                                      double, int, int, BlockBc, PushTable, bool, int*,
                                      cudaStream_t);
}  // namespace bcmg
