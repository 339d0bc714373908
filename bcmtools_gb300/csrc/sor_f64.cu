// sor_f64.cu -- double entry of the red-black SOR kernels (sor_impl.cuh):
// the generic shapes here, the tile kernels in sor_f64_n*.cu.
#include "sor_impl.cuh"

namespace bcmg {
extern template cudaError_t launch_sor_tile<double, 8>(const double*, double*, const double*, const Geom&,
                                                    const SorArgs&, bool, int, cudaStream_t);
extern template cudaError_t launch_sor_tile<double, 16>(const double*, double*, const double*, const Geom&,
                                                     const SorArgs&, bool, int, cudaStream_t);
extern template cudaError_t launch_sor_tile<double, 32>(const double*, double*, const double*, const Geom&,
                                                     const SorArgs&, bool, int, cudaStream_t);

extern template cudaError_t launch_sor_pull<double, 8>(const double*, double*, const double*, const Geom&,
                                                     const SorArgs&, int, cudaStream_t);
extern template cudaError_t launch_sor_pull<double, 16>(const double*, double*, const double*, const Geom&,
                                                      const SorArgs&, int, cudaStream_t);

template <>
cudaError_t launch_sor<double>(const double* A, double* B, const double* s, const Geom& g, const double* coef,
                           double omega, int form, int n_inner, BlockBc bc, PushTable push,
                           bool fused, int* err, int variant, int pull_now, cudaStream_t st,
                           bool s_packed) {
  return launch_sor_impl<double>(A, B, s, g, coef, omega, form, n_inner, bc, push, fused, err,
                             variant, pull_now, st, s_packed);
}
template cudaError_t launch_pack_source<double>(double*, const double*, const Geom&, cudaStream_t);
}  // namespace bcmg
