// divcheck.cu -- self-check of the sweeps' division from a precomputed
// reciprocal (cells.cuh, div_pre) against the correctly rounded division
// instruction sequence, on seeded random operands.
#include <cstdint>

#include "bcmg.h"
#include "cells.cuh"

namespace bcmg {

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// Divisors: random sign and mantissa (every 4th with an all-ones or all-zeros
// mantissa), exponent uniform over [2^-60, 2^60]; dividends: any bit pattern
// (every 8th a power of two times a small integer, every 16th zero).
__global__ void divcheck_kernel(uint64_t seed, int64_t n, unsigned long long* bad) {
  unsigned long long nf = 0, nd = 0;
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h0 = mix64(seed ^ (uint64_t)k), h1 = mix64(h0), h2 = mix64(h1);
    // float
    {
      uint32_t mb = (uint32_t)h1 & 0x7fffffu;
      if ((k & 3) == 1) mb = 0x7fffffu;
      if ((k & 3) == 2) mb = 0;
      const int eb = (int)(h1 >> 32) % 121 - 60;  // [-60, 60]
      const uint32_t bb = ((uint32_t)(h1 >> 63) << 31) | ((uint32_t)(eb + 127) << 23) | mb;
      uint32_t ab = (uint32_t)h0;
      if ((k & 7) == 3) ab = (ab & 0x807f0000u) | 0x3f800000u;
      if ((k & 15) == 5) ab = 0;
      const float a = __uint_as_float(ab), b = __uint_as_float(bb);
      const float y = __frcp_rn(b);
      const float q = div_pre(a, b, y), ref = __fdiv_rn(a, b);
      const bool same = __float_as_uint(q) == __float_as_uint(ref) || (q != q && ref != ref);
      nf += same ? 0 : 1;
    }
    // double
    {
      uint64_t mb = h2 & 0xfffffffffffffull;
      if ((k & 3) == 1) mb = 0xfffffffffffffull;
      if ((k & 3) == 2) mb = 0;
      const int eb = (int)((h1 >> 40) % 121) - 60;
      const uint64_t bb = ((h2 >> 63) << 63) | ((uint64_t)(eb + 1023) << 52) | mb;
      uint64_t ab = mix64(h2);
      if ((k & 7) == 3) ab = (ab & 0x800ff00000000000ull) | 0x3ff0000000000000ull;
      if ((k & 15) == 5) ab = 0;
      const double a = __longlong_as_double((long long)ab), b = __longlong_as_double((long long)bb);
      const double y = __drcp_rn(b);
      const double q = div_pre(a, b, y), ref = __ddiv_rn(a, b);
      const bool same = __double_as_longlong(q) == __double_as_longlong(ref) || (q != q && ref != ref);
      nd += same ? 0 : 1;
    }
  }
  if (nf) atomicAdd(&bad[0], nf);
  if (nd) atomicAdd(&bad[1], nd);
}

}  // namespace bcmg

extern "C" BCMG_API int bcmg_check_division(uint64_t seed, int64_t n, int64_t* bad_f32,
                                            int64_t* bad_f64) {
  if (n < 0 || !bad_f32 || !bad_f64) return BCMG_USAGE;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return BCMG_CUDA_ERROR;
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMemset(d, 0, sizeof(h));
  if (e == cudaSuccess && n > 0) {
    bcmg::divcheck_kernel<<<1216, 256>>>(seed, n, d);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return BCMG_CUDA_ERROR;
  *bad_f32 = (int64_t)h[0];
  *bad_f64 = (int64_t)h[1];
  return BCMG_SUCCESS;
}
