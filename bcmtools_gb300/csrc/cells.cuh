// cells.cuh -- per-cell update rules shared by the sweep kernels: the SOR
// cell (sor1/Solver.cpp:132-153, sor2/Solver.cpp:136-160) and the squared-
// residual accumulator of the fused Jacobi sweep (calc_r2, blas.f90:650-698).
#pragma once
#include "common.cuh"

namespace bcmg {

template <typename T, int FORM>
struct SorCell;

template <int FORM>
struct SorCell<double, FORM> {
  double c0, cx, cy, cz, om, om1;
  template <class Args>
  __device__ __forceinline__ void init(const Args& a, int b) {
    const double* cf = a.coef + 4 * b;
    c0 = cf[0]; cx = cf[1]; cy = cf[2]; cz = cf[3]; om = a.omega; om1 = 1.0 - a.omega;
  }
  __device__ __forceinline__ double operator()(double fc, double sw, double ss, double sbt,
                                               double src) const {
    if (FORM == 1) {
      double a = xmul(c0, fc);
      a = xadd(a, xmul(cx, sw));
      a = xadd(a, xmul(cy, ss));
      return xadd(a, xmul(cz, sbt));
    }
    double a = xmul(cx, sw);
    a = xadd(a, xmul(cy, ss));
    a = xadd(a, xmul(cz, sbt));
    a = xsub(a, src);
    return xadd(xmul(om, xmul(c0, a)), xmul(om1, fc));
  }
};

template <int FORM>
struct SorCell<float, FORM> {
  float c0, cx, cy, cz, om, om1;
  // coefficients rounded to float once, on the host (GB300's FP64 rate makes
  // per-thread conversions visible)
  template <class Args>
  __device__ __forceinline__ void init(const Args& a, int b) {
    const float* cf = a.coef32 + 4 * b;
    c0 = cf[0]; cx = cf[1]; cy = cf[2]; cz = cf[3]; om = a.omega32; om1 = a.om1_32;
  }
  __device__ __forceinline__ float operator()(float fc, float sw, float ss, float sbt,
                                              float src) const {
    if (FORM == 1) return fmaf(cz, sbt, fmaf(cy, ss, fmaf(cx, sw, c0 * fc)));
    const float a = fmaf(cz, sbt, fmaf(cy, ss, cx * sw)) - src;
    return fmaf(om, c0 * a, om1 * fc);
  }
};

// Sum of squares in float-float for float sweeps (error-free product and
// Knuth's two-sum; one FP64 conversion per warp) and in double for double.
template <typename T>
struct SqAcc;
template <>
struct SqAcc<float> {
  float s = 0.f, c = 0.f;
  __device__ __forceinline__ void merge(float hs, float hc) {
    const float t = __fadd_rn(s, hs);
    const float bv = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(hs, bv));
    s = t;
    c = __fadd_rn(c, __fadd_rn(hc, e));
  }
  __device__ __forceinline__ void add(float r) {
    const float p = __fmul_rn(r, r);
    merge(p, __fmaf_rn(r, r, -p));
  }
  __device__ __forceinline__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) {
      const float hs = __shfl_down_sync(0xffffffffu, s, o);
      const float hc = __shfl_down_sync(0xffffffffu, c, o);
      merge(hs, hc);
    }
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};
template <>
struct SqAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double r) { s = __dadd_rn(s, __dmul_rn(r, r)); }
  __device__ __forceinline__ void warp_reduce() {
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
  }
  __device__ __forceinline__ double value() const { return s; }
};

// a / b correctly rounded, from y = RN(1/b) computed once per block on the
// host: one product and two FMA corrections.  After the first correction q
// is within one ulp of a/b; then the remainder a - b*q is exact in an FMA and
// RN(q + (a - b*q)*y) is the correctly rounded quotient (Markstein's theorem,
// P. Markstein, IBM J. Res. Dev. 34(1), 1990).  The host leaves y = 0 for
// divisors outside [2^-60, 2^60]; quotients outside that range, dividends so
// small that the remainder would be subnormal, infinities and NaN take the
// division instruction sequence.
__device__ __forceinline__ float div_pre(float a, float b, float y) {
  float q = __fmul_rn(a, y);
  const float aq = fabsf(q);
  if (y == 0.f || !(aq <= 0x1p+60f) || (aq < 0x1p-60f && aq != 0.f) ||
      (fabsf(a) < 0x1p-96f && a != 0.f))
    return __fdiv_rn(a, b);
  if (aq == 0.f) return q;  // a = 0: the sign of a/b
  float r = __fmaf_rn(-b, q, a);
  q = __fmaf_rn(r, y, q);
  r = __fmaf_rn(-b, q, a);
  return __fmaf_rn(r, y, q);
}
__device__ __forceinline__ double div_pre(double a, double b, double y) {
  double q = __dmul_rn(a, y);
  const double aq = fabs(q);
  if (y == 0.0 || !(aq <= 0x1p+60) || (aq < 0x1p-60 && aq != 0.0) ||
      (fabs(a) < 0x1p-900 && a != 0.0))
    return __ddiv_rn(a, b);
  if (aq == 0.0) return q;
  double r = __fma_rn(-b, q, a);
  q = __fma_rn(r, y, q);
  r = __fma_rn(-b, q, a);
  return __fma_rn(r, y, q);
}

// The sweeps' division by Ap: FP64 through the host reciprocal (GB300's FP64
// pipe makes the division instruction sequence costly); FP32 with the
// division instruction sequence, which measured faster than div_pre's guarded
// FMA chain in the bandwidth-bound float sweeps.
__device__ __forceinline__ float sweep_div(float a, float b, float) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double sweep_div(double a, double b, double y) {
  return div_pre(a, b, y);
}

}  // namespace bcmg
