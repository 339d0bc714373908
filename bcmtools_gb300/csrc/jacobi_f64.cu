// jacobi_f64.cu -- double instantiation of the fused Jacobi sweep (jacobi_impl.cuh).
#include "jacobi_impl.cuh"

namespace bcmg {
template <>
cudaError_t launch_jacobi_fused<double>(const double* x0, double* x1, const double* b, const Geom& g,
                                     const double* cf, double omega, BlockBc bc, PushTable push,
                                     int ghost_mode, int shape, double* partial, int* err,
                                     const JacPre<double>* pre,
                                     cudaStream_t st) {
  return launch_jacobi_fused_impl<double>(x0, x1, b, g, cf, omega, bc, push, ghost_mode, shape, partial,
                                       err, pre, st);
}
}  // namespace bcmg
