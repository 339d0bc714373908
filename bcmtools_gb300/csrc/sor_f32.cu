// sor_f32.cu -- float entry of the red-black SOR kernels (sor_impl.cuh):
// the generic shapes here, the tile kernels in sor_f32_n*.cu.
#include "sor_impl.cuh"

namespace bcmg {
extern template cudaError_t launch_sor_tile<float, 8>(const float*, float*, const float*, const Geom&,
                                                    const SorArgs&, bool, int, cudaStream_t);
extern template cudaError_t launch_sor_tile<float, 16>(const float*, float*, const float*, const Geom&,
                                                     const SorArgs&, bool, int, cudaStream_t);
extern template cudaError_t launch_sor_tile<float, 32>(const float*, float*, const float*, const Geom&,
                                                     const SorArgs&, bool, int, cudaStream_t);

extern template cudaError_t launch_sor_pull<float, 8>(const float*, float*, const float*, const Geom&,
                                                     const SorArgs&, int, cudaStream_t);
extern template cudaError_t launch_sor_pull<float, 16>(const float*, float*, const float*, const Geom&,
                                                      const SorArgs&, int, cudaStream_t);

template <>
cudaError_t launch_sor<float>(const float* A, float* B, const float* s, const Geom& g, const double* coef,
                           double omega, int form, int n_inner, BlockBc bc, PushTable push,
                           bool fused, int* err, int variant, int pull_now, cudaStream_t st,
                           bool s_packed) {
  return launch_sor_impl<float>(A, B, s, g, coef, omega, form, n_inner, bc, push, fused, err,
                             variant, pull_now, st, s_packed);
}
template cudaError_t launch_pack_source<float>(float*, const float*, const Geom&, cudaStream_t);
}  // namespace bcmg
