// jacobi_f32.cu -- float instantiation of the fused Jacobi sweep (jacobi_impl.cuh).
#include "jacobi_impl.cuh"

namespace bcmg {
template <>
cudaError_t launch_jacobi_fused<float>(const float* x0, float* x1, const float* b, const Geom& g,
                                     const float* cf, float omega, BlockBc bc, PushTable push,
                                     int ghost_mode, int shape, double* partial, int* err,
                                     const JacPre<float>* pre,
                                     cudaStream_t st) {
  return launch_jacobi_fused_impl<float>(x0, x1, b, g, cf, omega, bc, push, ghost_mode, shape, partial,
                                       err, pre, st);
}
}  // namespace bcmg
