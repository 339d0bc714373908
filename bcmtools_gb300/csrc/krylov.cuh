// krylov.cuh -- device-resident BiCGSTAB iteration (ILS3D::BiCGSTAB,
// examples/SolverTest/ILS3D.h:663-844) for block-structured fields.
//
// The iteration's scalars (rho = r.r0, alpha, omega -- gamma here as in the
// reference -- beta, the residual) live in device memory, one KSeg record per
// segment: a contiguous range of blocks solved as one system.  One segment is
// an ordinary solve; several are independent solves batched into one mesh,
// every launch advancing all of them.  Each inner product (DotAcc: exact
// products, a compensated sum along each thread's columns, FP64 across
// threads, blocks and the segment in fixed-order trees) is fused into the
// kernel that produces its operand:
//
//   kr_p       p = r + beta (p - gamma q)            (first iteration: p = r)
//   kr_ax      q = A p^   with q.r0                  (calc_ax + dot)
//              t = A s^   with t.s, t.t
//   kr_s       s = r - alpha q                       (axpyz)
//   kr_xr      x = alpha p^ + gamma s^ + x,  r = s - gamma t,
//              with r.r and r.r0                     (axpbypz, axpyz, two dots)
//   kr_scalar  per segment: the reductions of the partial sums, then the
//              scalar recurrence and the convergence test (IsConverged,
//              ILS3D.h:41-63) of that stage
//
// Vector updates keep the reference's operation order (blas.f90:242-377:
// each product and sum rounded to the field's type, scalars rounded to it).
// A segment whose solve ended (converged, broke down, hit its limit) is
// skipped by every vector kernel, so launches queued past its end change
// nothing of its x or r.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"


namespace bcmg {

struct KSeg {
  double bb;       // b.b
  double rr0;      // r.r0 of the previous iteration
  double rr1;      // r.r0 of the current iteration
  double alpha, gamma, beta;
  double res;      // |r|^2 / |b|^2 (IsConverged's residual)
  double best_rr;  // keep-best: smallest r.r so far
  double eps2;
  int count;       // iteration of the solve (ILS3D's count)
  int max_iter;
  int status;      // kRunning, else the final BCMG_* status
  int improved;    // keep-best: this iteration's x is the best so far
  int first;       // the next iteration is the first one (p = r)
  int best_saved;
  int keep_best;
  int pad;
};
constexpr int kRunning = -1;

// Stages of kr_scalar.
enum : int { KS_INIT = 0, KS_ALPHA = 1, KS_GAMMA = 2, KS_R = 3 };

// Blocks of segment s: [seg_first[s], seg_first[s+1]); seg_of[b] the segment
// of block b (null: one segment).  At the set-up stage, seg_active[s] == 0
// (null: all active) leaves segment s out of the solve, seg_eps2[s] (null:
// the launch's) is its own squared tolerance, and seg_max_iter[s]
// (null: the launch's max_iter) is its own iteration limit.
struct KSegs {
  KSeg* seg;
  const int* seg_of;
  const int* seg_first;
  int nseg;
  const unsigned char* seg_active;
  const int* seg_max_iter;
  const double* seg_eps2;
};
constexpr int kSkipped = -2;  // status of a segment left out of the solve

__device__ __forceinline__ int kseg_of(const KSegs& S, int b) { return S.seg_of ? S.seg_of[b] : 0; }

// Inner-product accumulator of one thread.  float fields: each product is
// formed exactly (x*y and its FMA remainder) and summed in float-float
// (Knuth's two-sum, about 48 significant bits, error below n 2^-48 of the sum
// of |terms| for n terms), products outside [2^-100, 2^100) -- whose
// remainder could be subnormal -- in FP64; value() hands FP64 to the block
// and segment trees.  GB300 issues FP64 at 1/64 of its FP32 rate: one FP64
// multiply-add per element for the five inner products of an iteration
// bounds the kernels that form them by the FP64 pipe, not by HBM.  double
// fields: FP64 multiply-add.
template <typename T>
struct DotAcc;
template <>
struct DotAcc<float> {
  float s = 0.f, c = 0.f;
  double wide = 0.0;
  __device__ __forceinline__ void add(float x, float y) {
    const float p = __fmul_rn(x, y);
    const float m = fabsf(p);
    if (m >= 0x1p-100f && m < 0x1p100f) {
      const float e = __fmaf_rn(x, y, -p);
      const float t = __fadd_rn(s, p);
      const float bv = __fsub_rn(t, s);
      const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bv)), __fsub_rn(p, bv));
      s = t;
      c = __fadd_rn(c, __fadd_rn(err, e));
    } else if (x != 0.f && y != 0.f) {
      wide = __fma_rn((double)x, (double)y, wide);
    }
  }
  __device__ __forceinline__ double value() const {
    return __dadd_rn(__dadd_rn((double)s, (double)c), wide);
  }
};
template <>
struct DotAcc<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double x, double y) { s = __fma_rn(x, y, s); }
  __device__ __forceinline__ double value() const { return s; }
};

// Sum of one double per thread over the CTA in a fixed tree order; the
// result is valid in thread 0.  `red` holds one double per warp.
__device__ __forceinline__ double kr_block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  }
  __syncthreads();
  return v;
}

// Threads of one CTA: one per column up to 16^3 blocks (64, 256), 512 for
// 32^3 blocks (two columns each), 256 for other shapes.  CTAs per SM they are
// compiled for: 2048 threads per SM (32 registers a thread) for the streaming
// updates and for the float 32^3 stencil kernels, 1024 (64 registers) where
// the stencil or the double accumulators would spill at 32.  Measured on the
// 2920-block 32^3 mesh: the p update at 512 threads x 4 CTAs ran 0.30 ms
// (75 % of HBM), 0.33 at 256 x 8, 0.38-0.47 with four or two columns side
// by side per thread; A.p with its inner product 0.33 ms at 512 x 4, 0.37 at
// 256 x 8 and 256 x 4.
template <int N>
__host__ __device__ constexpr int kr_nt() { return N == 8 ? 64 : N == 32 ? 512 : 256; }
template <typename T, int N, bool HEAVY>
__host__ __device__ constexpr int kr_minb() {
  return (HEAVY && (sizeof(T) == 8 || N != 32) ? 1024 : 2048) / kr_nt<N>();
}

}  // namespace bcmg
