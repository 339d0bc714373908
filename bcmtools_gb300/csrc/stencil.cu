// stencil.cu -- 7-point sweeps, residuals, inner products and BLAS-1 on
// block-structured fields.
//
// Reference routines restated for the GPU (arithmetic order kept, no
// multiply-add contraction, so results match the reference bit for bit where
// the reference is sequential):
//   jacobi_smoother        SolverTest/blas.f90:452-502
//   calc_ax / calc_r / r2  blas.f90:556-698
//   dot                    blas.f90:379-412 (float: exact products, column sums in
//                          float-float, products outside [2^-100, 2^100) in FP64;
//                          block sums in FP64)
//   axpy/xpay/axpyz/axpbypz blas.f90:242-377
// Decomposition: one CTA per block; sweeps march each (i,j) column along k.
#include "cells.cuh"
#include "common.cuh"
#include "kernels.h"
#include "tile.cuh"

namespace bcmg {


// ---------------------------------------------------------------------------
// Deterministic block reduction of one double per thread (fixed tree order).
__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;  // valid in thread 0
}

// ---------------------------------------------------------------------------
// Operator coefficients of one cell.
template <typename T, bool CC>
struct Coefs {
  T v[7];
  __device__ __forceinline__ void load_block(const Op<T>& op, int b) {
    if (CC)
      for (int c = 0; c < 7; c++) v[c] = to_t<T>(op.cc[b * 7 + c]);
  }
  __device__ __forceinline__ T get(const Op<T>& op, int c, int64_t p) const {
    return CC ? v[c] : op.A[c][p];
  }
};

// jacobi_smoother: x1 = x0 - omega (x0 - r/Ap),
// r = b - Aw xW - Ae xE - As xS - An xN - Ab xB - At xT.
template <typename T, bool CC>
__global__ void __launch_bounds__(256) jacobi_kernel(T* __restrict__ x1, const T* __restrict__ x0,
                                                     const T* __restrict__ bb, Op<T> op, Geom g,
                                                     T omega) {
  const int b = blockIdx.x;
  const int64_t base = (int64_t)b * g.bstride;
  Coefs<T, CC> cf;
  cf.load_block(op, b);
  const int nx = g.nx, ny = g.ny, nz = g.nz, sy = g.sy, sz = g.sz;
  for (int ij = threadIdx.x; ij < nx * ny; ij += blockDim.x) {
    const int i = ij % nx, j = ij / nx;
    int64_t p = base + g.at(i, j, 0);
    T xm = x0[p - sz], xc = x0[p];
    for (int k = 0; k < nz; k++, p += sz) {
      const T xp = x0[p + sz];
      T r = bb[p];
      r = xsub(r, xmul(cf.get(op, 1, p), x0[p - 1]));
      r = xsub(r, xmul(cf.get(op, 2, p), x0[p + 1]));
      r = xsub(r, xmul(cf.get(op, 3, p), x0[p - sy]));
      r = xsub(r, xmul(cf.get(op, 4, p), x0[p + sy]));
      r = xsub(r, xmul(cf.get(op, 5, p), xm));
      r = xsub(r, xmul(cf.get(op, 6, p), xp));
      const T xt = xdiv(r, cf.get(op, 0, p));
      x1[p] = xsub(xc, xmul(omega, xsub(xc, xt)));
      xm = xc;
      xc = xp;
    }
  }
}

template <typename T>
static bool cubic_fast(const Op<T>& op, const Geom& g) {
  return op.cc && op.cf8 && g.nx == g.ny && g.ny == g.nz && (g.vc == 1 || g.vc == 2) &&
         (g.nx == 8 || g.nx == 16 || g.nx == 32);
}

// jacobi_smoother on cubic blocks with a per-block constant operator: the
// same arithmetic (coefficients rounded to T, the division of the fused
// sweeps), block edge and ghost width fixed at compile time, and each thread
// walking CPT columns side by side so that their loads overlap.
template <typename T, int N, int VC, int CPT>
__global__ void __launch_bounds__(N * N / CPT, CPT > 1 ? (sizeof(T) == 4 ? 4 : 2) : 1) jacobi_cubic_kernel(
    T* __restrict__ x1, const T* __restrict__ x0, const T* __restrict__ bb,
    const T* __restrict__ cf8, Geom g, T omega) {
  using BL = BrickTile<T, N, VC>;
  constexpr int NT = N * N / CPT, LX = BL::LX, LXY = BL::LXY;
  const int b = blockIdx.x;
  const T* cf = cf8 + (int64_t)b * 8;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const T rc0 = cf[7];
  const int64_t base = (int64_t)b * g.bstride;
  int off[CPT];
  T xm[CPT], xc[CPT];
#pragma unroll
  for (int c = 0; c < CPT; c++) {
    const int ij = threadIdx.x + c * NT;
    off[c] = BL::at(ij % N, ij / N, 0);
    xm[c] = x0[base + off[c] - LXY];
    xc[c] = x0[base + off[c]];
  }
#pragma unroll 2
  for (int k = 0; k < N; k++) {
    T w[CPT], e[CPT], s_[CPT], n_[CPT], up[CPT], bv[CPT];
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      const T* q = x0 + base + off[c] + k * LXY;
      w[c] = q[-1];
      e[c] = q[1];
      s_[c] = q[-LX];
      n_[c] = q[LX];
      up[c] = q[LXY];
      bv[c] = bb[base + off[c] + k * LXY];
    }
#pragma unroll
    for (int c = 0; c < CPT; c++) {
      T r = bv[c];
      r = xsub(r, xmul(c1, w[c]));
      r = xsub(r, xmul(c2, e[c]));
      r = xsub(r, xmul(c3, s_[c]));
      r = xsub(r, xmul(c4, n_[c]));
      r = xsub(r, xmul(c5, xm[c]));
      r = xsub(r, xmul(c6, up[c]));
      const T xt = sweep_div(r, c0, rc0);
      x1[base + off[c] + k * LXY] = xsub(xc[c], xmul(omega, xsub(xc[c], xt)));
      xm[c] = xc[c];
      xc[c] = up[c];
    }
  }
}

template <typename T>
cudaError_t launch_jacobi(T* x1, const T* x0, const T* b, Op<T> op, const Geom& g, T omega,
                          cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  if (cubic_fast(op, g)) {
    switch (g.nx * 4 + g.vc) {
      case 8 * 4 + 1: jacobi_cubic_kernel<T, 8, 1, 1><<<g.nb, 64, 0, st>>>(x1, x0, b, op.cf8, g, omega); break;
      case 8 * 4 + 2: jacobi_cubic_kernel<T, 8, 2, 1><<<g.nb, 64, 0, st>>>(x1, x0, b, op.cf8, g, omega); break;
      case 16 * 4 + 1: jacobi_cubic_kernel<T, 16, 1, 1><<<g.nb, 256, 0, st>>>(x1, x0, b, op.cf8, g, omega); break;
      case 16 * 4 + 2: jacobi_cubic_kernel<T, 16, 2, 1><<<g.nb, 256, 0, st>>>(x1, x0, b, op.cf8, g, omega); break;
      case 32 * 4 + 1: jacobi_cubic_kernel<T, 32, 1, 4><<<g.nb, 256, 0, st>>>(x1, x0, b, op.cf8, g, omega); break;
      default: jacobi_cubic_kernel<T, 32, 2, 4><<<g.nb, 256, 0, st>>>(x1, x0, b, op.cf8, g, omega); break;
    }
    return cudaGetLastError();
  }
  const int threads = min(256, g.nx * g.ny);
  if (op.cc)
    jacobi_kernel<T, true><<<g.nb, threads, 0, st>>>(x1, x0, b, op, g, omega);
  else
    jacobi_kernel<T, false><<<g.nb, threads, 0, st>>>(x1, x0, b, op, g, omega);
  return cudaGetLastError();
}

// calc_ax (mode 0), calc_r (mode 1), calc_r2 (mode 2, FP64 per-block partials).
template <typename T, bool CC, int MODE>
__global__ void __launch_bounds__(256) residual_kernel(T* __restrict__ out, const T* __restrict__ x,
                                                       const T* __restrict__ bb, Op<T> op, Geom g,
                                                       double* __restrict__ partial) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  const int64_t base = (int64_t)b * g.bstride;
  Coefs<T, CC> cf;
  cf.load_block(op, b);
  const int nx = g.nx, ny = g.ny, nz = g.nz, sy = g.sy, sz = g.sz;
  double acc = 0.0;
  for (int ij = threadIdx.x; ij < nx * ny; ij += blockDim.x) {
    const int i = ij % nx, j = ij / nx;
    int64_t p = base + g.at(i, j, 0);
    T xm = x[p - sz], xc = x[p];
    for (int k = 0; k < nz; k++, p += sz) {
      const T xp = x[p + sz];
      if (MODE == 0) {
        T a = xmul(cf.get(op, 1, p), x[p - 1]);
        a = xadd(a, xmul(cf.get(op, 2, p), x[p + 1]));
        a = xadd(a, xmul(cf.get(op, 3, p), x[p - sy]));
        a = xadd(a, xmul(cf.get(op, 4, p), x[p + sy]));
        a = xadd(a, xmul(cf.get(op, 5, p), xm));
        a = xadd(a, xmul(cf.get(op, 6, p), xp));
        a = xadd(a, xmul(cf.get(op, 0, p), xc));
        out[p] = a;
      } else {
        T r = bb[p];
        r = xsub(r, xmul(cf.get(op, 1, p), x[p - 1]));
        r = xsub(r, xmul(cf.get(op, 2, p), x[p + 1]));
        r = xsub(r, xmul(cf.get(op, 3, p), x[p - sy]));
        r = xsub(r, xmul(cf.get(op, 4, p), x[p + sy]));
        r = xsub(r, xmul(cf.get(op, 5, p), xm));
        r = xsub(r, xmul(cf.get(op, 6, p), xp));
        r = xsub(r, xmul(cf.get(op, 0, p), xc));
        if (MODE == 1) out[p] = r;
        else acc += (double)r * (double)r;
      }
      xm = xc;
      xc = xp;
    }
  }
  if (MODE == 2) {
    acc = block_sum(acc, red);
    if (threadIdx.x == 0) partial[b] = acc;
  }
}

template <typename T, int MODE>
static void residual_dispatch(T* out, const T* x, const T* b, Op<T> op, const Geom& g,
                              double* partial, cudaStream_t st) {
  const int threads = min(256, g.nx * g.ny);
  if (op.cc)
    residual_kernel<T, true, MODE><<<g.nb, threads, 0, st>>>(out, x, b, op, g, partial);
  else
    residual_kernel<T, false, MODE><<<g.nb, threads, 0, st>>>(out, x, b, op, g, partial);
}

// calc_ax / calc_r / calc_r2 on cubic blocks with a constant operator: one
// thread per column, unrolled k walk, coefficients rounded to T on the host;
// calc_r2's block sum in float-float (SqAcc) for float fields.
template <typename T, int N, int VC, int MODE>
__global__ void __launch_bounds__(N * N) residual_cubic_kernel(T* __restrict__ out,
                                                               const T* __restrict__ x,
                                                               const T* __restrict__ bb,
                                                               const T* __restrict__ cf8, Geom g,
                                                               double* __restrict__ partial) {
  using BL = BrickTile<T, N, VC>;
  constexpr int NW = N * N / 32;
  __shared__ double red[NW > 0 ? NW : 1];
  const int b = blockIdx.x, i = threadIdx.x % N, j = threadIdx.x / N;
  const T* cf = cf8 + (int64_t)b * 8;
  const T c0 = cf[0], c1 = cf[1], c2 = cf[2], c3 = cf[3], c4 = cf[4], c5 = cf[5], c6 = cf[6];
  const int64_t p0 = (int64_t)b * g.bstride + BL::at(i, j, 0);
  const T* q = x + p0;
  SqAcc<T> acc;
  T xm = q[-BL::LXY], xc = q[0];
#pragma unroll
  for (int k = 0; k < N; k++) {
    const T* qk = q + k * BL::LXY;
    const T xp = qk[BL::LXY];
    if (MODE == 0) {
      T a = xmul(c1, qk[-1]);
      a = xadd(a, xmul(c2, qk[1]));
      a = xadd(a, xmul(c3, qk[-BL::LX]));
      a = xadd(a, xmul(c4, qk[BL::LX]));
      a = xadd(a, xmul(c5, xm));
      a = xadd(a, xmul(c6, xp));
      a = xadd(a, xmul(c0, xc));
      out[p0 + k * BL::LXY] = a;
    } else {
      T r = bb[p0 + k * BL::LXY];
      r = xsub(r, xmul(c1, qk[-1]));
      r = xsub(r, xmul(c2, qk[1]));
      r = xsub(r, xmul(c3, qk[-BL::LX]));
      r = xsub(r, xmul(c4, qk[BL::LX]));
      r = xsub(r, xmul(c5, xm));
      r = xsub(r, xmul(c6, xp));
      r = xsub(r, xmul(c0, xc));
      if (MODE == 1) out[p0 + k * BL::LXY] = r;
      else acc.add(r);
    }
    xm = xc;
    xc = xp;
  }
  if (MODE == 2) {
    acc.warp_reduce();
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red[w] = acc.value();
    __syncthreads();
    if (threadIdx.x == 0) {
      double v = 0.0;
      for (int q2 = 0; q2 < NW; q2++) v += red[q2];
      partial[b] = v;
    }
  }
}

template <typename T, int MODE>
static void residual_cubic(T* out, const T* x, const T* b, const Op<T>& op, const Geom& g,
                           double* partial, cudaStream_t st) {
  const int key = g.nx * 4 + g.vc;
  switch (key) {
    case 8 * 4 + 1: residual_cubic_kernel<T, 8, 1, MODE><<<g.nb, 64, 0, st>>>(out, x, b, op.cf8, g, partial); break;
    case 8 * 4 + 2: residual_cubic_kernel<T, 8, 2, MODE><<<g.nb, 64, 0, st>>>(out, x, b, op.cf8, g, partial); break;
    case 16 * 4 + 1: residual_cubic_kernel<T, 16, 1, MODE><<<g.nb, 256, 0, st>>>(out, x, b, op.cf8, g, partial); break;
    case 16 * 4 + 2: residual_cubic_kernel<T, 16, 2, MODE><<<g.nb, 256, 0, st>>>(out, x, b, op.cf8, g, partial); break;
    case 32 * 4 + 1: residual_cubic_kernel<T, 32, 1, MODE><<<g.nb, 1024, 0, st>>>(out, x, b, op.cf8, g, partial); break;
    default: residual_cubic_kernel<T, 32, 2, MODE><<<g.nb, 1024, 0, st>>>(out, x, b, op.cf8, g, partial); break;
  }
}

template <typename T>
cudaError_t launch_residual(T* out, const T* x, const T* b, Op<T> op, const Geom& g, int mode,
                            double* partial, cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  if (cubic_fast(op, g)) {
    if (mode == 0) residual_cubic<T, 0>(out, x, b, op, g, partial, st);
    else if (mode == 1) residual_cubic<T, 1>(out, x, b, op, g, partial, st);
    else residual_cubic<T, 2>(out, x, b, op, g, partial, st);
    return cudaGetLastError();
  }
  if (mode == 0) residual_dispatch<T, 0>(out, x, b, op, g, partial, st);
  else if (mode == 1) residual_dispatch<T, 1>(out, x, b, op, g, partial, st);
  else residual_dispatch<T, 2>(out, x, b, op, g, partial, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) dot_partial_kernel(const T* __restrict__ x,
                                                          const T* __restrict__ y, Geom g,
                                                          double* __restrict__ partial) {
  __shared__ double red[32];
  const int b = blockIdx.x;
  const int64_t base = (int64_t)b * g.bstride;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  double acc = 0.0;
  for (int ij = threadIdx.x; ij < nx * ny; ij += blockDim.x) {
    const int i = ij % nx, j = ij / nx;
    int64_t p = base + g.at(i, j, 0);
    if constexpr (sizeof(T) == 4) {
      // float: the column's products summed in float-float where they are
      // exact there (2^-100 <= |x y| < 2^100: the product's error term is a
      // normal float), in double otherwise; GB300's FP64 rate would bound a
      // per-element FP64 accumulation.
      float s = 0.f, c = 0.f;
      double wide = 0.0;
      for (int k = 0; k < nz; k++, p += g.sz) {
        const float xv = x[p], yv = y[p];
        const ff q = two_prod(xv, yv);
        const float m = fabsf(q.hi);
        if (m >= 0x1p-100f && m < 0x1p100f) {
          const ff t = two_sum(s, q.hi);
          s = t.hi;
          c = __fadd_rn(c, __fadd_rn(t.lo, q.lo));
        } else if (xv != 0.f && yv != 0.f) {
          wide += (double)xv * (double)yv;
        }
      }
      acc += (double)s + (double)c + wide;
    } else {
      for (int k = 0; k < nz; k++, p += g.sz) acc += (double)x[p] * (double)y[p];
    }
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) partial[b] = acc;
}

template <typename T>
cudaError_t launch_dot_partial(const T* x, const T* y, const Geom& g, double* partial,
                               cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  dot_partial_kernel<T><<<g.nb, min(256, g.nx * g.ny), 0, st>>>(x, y, g, partial);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(1024) reduce_final_kernel(const double* __restrict__ partial,
                                                            int n, double* __restrict__ out) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += partial[i];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) out[0] = acc;
}

cudaError_t launch_reduce_final(const double* partial, int n, double* out, cudaStream_t st) {
  reduce_final_kernel<<<1, 1024, 0, st>>>(partial, n, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
template <typename T, int KIND>
__global__ void __launch_bounds__(256) blas1_kernel(T* __restrict__ z, const T* __restrict__ x,
                                                    const T* __restrict__ y, T a, T bc, Geom g) {
  const int b = blockIdx.x;
  const int64_t base = (int64_t)b * g.bstride;
  const int nx = g.nx, ny = g.ny, nz = g.nz;
  for (int ij = threadIdx.x; ij < nx * ny; ij += blockDim.x) {
    const int i = ij % nx, j = ij / nx;
    int64_t p = base + g.at(i, j, 0);
    for (int k = 0; k < nz; k++, p += g.sz) {
      if (KIND == 0) z[p] = xadd(z[p], xmul(a, x[p]));                       // axpy
      else if (KIND == 1) z[p] = xadd(x[p], xmul(a, z[p]));                  // xpay
      else if (KIND == 2) z[p] = xadd(xmul(a, x[p]), y[p]);                  // axpyz
      else if (KIND == 3) z[p] = xadd(xadd(xmul(a, x[p]), xmul(bc, y[p])), z[p]);  // axpbypz
      else z[p] = xmul(a, z[p]);                                            // scal
    }
  }
}

template <typename T>
cudaError_t launch_blas1(int kind, T* z, const T* x, const T* y, T a, T b, const Geom& g,
                         cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  const int th = min(256, g.nx * g.ny);
  switch (kind) {
    case 0: blas1_kernel<T, 0><<<g.nb, th, 0, st>>>(z, x, y, a, b, g); break;
    case 1: blas1_kernel<T, 1><<<g.nb, th, 0, st>>>(z, x, y, a, b, g); break;
    case 2: blas1_kernel<T, 2><<<g.nb, th, 0, st>>>(z, x, y, a, b, g); break;
    case 3: blas1_kernel<T, 3><<<g.nb, th, 0, st>>>(z, x, y, a, b, g); break;
    default: blas1_kernel<T, 4><<<g.nb, th, 0, st>>>(z, x, y, a, b, g); break;
  }
  return cudaGetLastError();
}

template <typename T>
__global__ void fill_kernel(T* __restrict__ x, int64_t n, T v) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    x[e] = v;
}

template <typename T>
cudaError_t launch_fill(T* x, int64_t n, T v, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  fill_kernel<T><<<(int)blocks, 256, 0, st>>>(x, n, v);
  return cudaGetLastError();
}

// Seeded uniform values in [lo, hi) on the interior of blocks [b0, b0+nb)
// (ghosts untouched): value of interior cell c of local block l is a
// splitmix64 hash of (seed, l, c) scaled to the interval, so a block set
// gets the same values wherever it sits in a larger mesh.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

template <typename T>
__global__ void __launch_bounds__(256) fill_random_kernel(T* __restrict__ x, Geom g, int b0,
                                                          int nb, uint64_t seed, double lo,
                                                          double hi) {
  const int64_t cells = (int64_t)g.nx * g.ny * g.nz;
  const int64_t total = cells * nb;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = e / cells, c = e - l * cells;
    const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / ((int64_t)g.nx * g.ny));
    const uint64_t h = splitmix64(seed * 0x100000001b3ull ^ splitmix64((uint64_t)l * (uint64_t)cells + (uint64_t)c));
    const double u = (double)(h >> 11) * 0x1p-53;  // [0, 1)
    x[(int64_t)(b0 + l) * g.bstride + g.at(i, j, k)] = (T)(lo + (hi - lo) * u);
  }
}

template <typename T>
cudaError_t launch_fill_random(T* x, const Geom& g, int b0, int nb, uint64_t seed, double lo,
                               double hi, cudaStream_t st) {
  const int64_t total = (int64_t)g.nx * g.ny * g.nz * nb;
  if (total == 0) return cudaSuccess;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  fill_random_kernel<T><<<(int)blocks, 256, 0, st>>>(x, g, b0, nb, seed, lo, hi);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Boundary folding (SolverTest bca.f90:12-394, applied per block by
// BlockScalar3D::ImposeBoundaryCondition, BlockScalar3D.h:208-215).  For an
// outer face with neighbour coefficient A_nb and value xc:
//   Dirichlet  Ap -= A_nb;  b = (T)((double)b - (double)(A_nb*xc) * 2);  A_nb = 0
//   Neumann    Ap += A_nb;  b += A_nb*xc (minus faces) or -= (plus faces);  A_nb = 0
// with A_nb*xc rounded to T first (Fortran `real` operands, then the
// double-precision 2.0d0 factor).  One launch per axis; each thread takes one
// cell of the face plane and folds its minus face before its plus face.
template <typename T>
__device__ __forceinline__ void fold_cell(T* __restrict__ Ap, T* __restrict__ An,
                                          T* __restrict__ b, int q, int code, T xc, bool minus) {
  const T a = An[q];
  const T p = xmul(a, xc);
  if (code == 1) {
    Ap[q] = xsub(Ap[q], a);
    b[q] = to_t<T>(xsub((double)b[q], xmul((double)p, 2.0)));
  } else {
    Ap[q] = xadd(Ap[q], a);
    b[q] = minus ? xadd(b[q], p) : xsub(b[q], p);
  }
  An[q] = (T)0;
}

template <typename T>
__global__ void __launch_bounds__(256) fold_axis_kernel(FoldPtrs<T> p, Geom g, int ax,
                                                         const int* __restrict__ code,
                                                         const double* __restrict__ xcv) {
  const int blk = blockIdx.x;
  const int fm = 2 * ax, fp = 2 * ax + 1;
  const int cm = code[blk * 6 + fm], cp = code[blk * 6 + fp];
  if (cm == 0 && cp == 0) return;
  const T xm = (T)xcv[blk * 6 + fm], xp = (T)xcv[blk * 6 + fp];
  const int n[3] = {g.nx, g.ny, g.nz};
  const int u = ax == 0 ? 1 : 0, v = ax == 2 ? 1 : 2;  // the plane's axes
  const int64_t base = (int64_t)blk * g.bstride;
  T* Ap = p.A[0] + base;
  T* Am = p.A[1 + 2 * ax] + base;
  T* Aq = p.A[2 + 2 * ax] + base;
  T* b = p.b + base;
  for (int e = threadIdx.x; e < n[u] * n[v]; e += blockDim.x) {
    int c[3];
    c[u] = e % n[u];
    c[v] = e / n[u];
    if (cm) {
      c[ax] = 0;
      fold_cell(Ap, Am, b, g.at(c[0], c[1], c[2]), cm, xm, true);
    }
    if (cp) {
      c[ax] = n[ax] - 1;
      fold_cell(Ap, Aq, b, g.at(c[0], c[1], c[2]), cp, xp, false);
    }
  }
}

template <typename T>
cudaError_t launch_fold_boundary(FoldPtrs<T> p, const Geom& g, const int* code, const double* xc,
                                 cudaStream_t st) {
  if (g.nb == 0) return cudaSuccess;
  for (int ax = 0; ax < 3; ax++) {
    fold_axis_kernel<T><<<g.nb, 256, 0, st>>>(p, g, ax, code, xc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// Mixed precision helpers: interior FP64 -> FP32 (residual hand-off) and
// x64 += (double) d32 (correction accumulation).  Both fields share vc.
__global__ void __launch_bounds__(256) convert_kernel(float* __restrict__ dst,
                                                      const double* __restrict__ src, Geom g64,
                                                      Geom g32) {
  const int b = blockIdx.x;
  const int nx = g64.nx, ny = g64.ny, nz = g64.nz;
  for (int ij = threadIdx.x; ij < nx * ny; ij += blockDim.x) {
    const int i = ij % nx, j = ij / nx;
    for (int k = 0; k < nz; k++) {
      const int q = g64.at(i, j, k);
      dst[(int64_t)b * g32.bstride + q] = __double2float_rn(src[(int64_t)b * g64.bstride + q]);
    }
  }
}

__global__ void __launch_bounds__(256) accumulate_kernel(double* __restrict__ x,
                                                         const float* __restrict__ d, Geom g64,
                                                         Geom g32) {
  const int b = blockIdx.x;
  const int nx = g64.nx, ny = g64.ny, nz = g64.nz;
  for (int ij = threadIdx.x; ij < nx * ny; ij += blockDim.x) {
    const int i = ij % nx, j = ij / nx;
    for (int k = 0; k < nz; k++) {
      const int q = g64.at(i, j, k);
      const int64_t p = (int64_t)b * g64.bstride + q;
      x[p] = x[p] + (double)d[(int64_t)b * g32.bstride + q];
    }
  }
}

cudaError_t launch_convert_f64_to_f32(float* dst, const double* src, const Geom& g64,
                                      const Geom& g32, cudaStream_t st) {
  if (g64.nb == 0) return cudaSuccess;
  convert_kernel<<<g64.nb, min(256, g64.nx * g64.ny), 0, st>>>(dst, src, g64, g32);
  return cudaGetLastError();
}

cudaError_t launch_accumulate_f32_into_f64(double* x, const float* d, const Geom& g64,
                                           const Geom& g32, cudaStream_t st) {
  if (g64.nb == 0) return cudaSuccess;
  accumulate_kernel<<<g64.nb, min(256, g64.nx * g64.ny), 0, st>>>(x, d, g64, g32);
  return cudaGetLastError();
}

#define INST(T)                                                                              \
  template cudaError_t launch_jacobi<T>(T*, const T*, const T*, Op<T>, const Geom&, T,      \
                                        cudaStream_t);                                      \
  template cudaError_t launch_residual<T>(T*, const T*, const T*, Op<T>, const Geom&, int,  \
                                          double*, cudaStream_t);                           \
  template cudaError_t launch_dot_partial<T>(const T*, const T*, const Geom&, double*,      \
                                             cudaStream_t);                                 \
  template cudaError_t launch_blas1<T>(int, T*, const T*, const T*, T, T, const Geom&,      \
                                       cudaStream_t);                                       \
  template cudaError_t launch_fill<T>(T*, int64_t, T, cudaStream_t);                       \
  template cudaError_t launch_fill_random<T>(T*, const Geom&, int, int, uint64_t, double,  \
                                             double, cudaStream_t);                         \
  template cudaError_t launch_fold_boundary<T>(FoldPtrs<T>, const Geom&, const int*,        \
                                               const double*, cudaStream_t);
INST(float)
INST(double)
#undef INST

}  // namespace bcmg

// ---------------------------------------------------------------------------
// Inner product without any allocation, for callers that cannot call
// cudaMalloc: host code embedded in a larger application or framework that
// owns every device allocation (its own pool or allocator, nothing else may
// allocate beside it), which would otherwise have to hand this library a
// scratch buffer it does not know how to size.  The per-block partial sums,
// which bcmg_dot keeps in a per-context buffer, live here in one file-scope
// device array of fixed capacity that every GPU loading this library holds
// until the process exits.
#include <cuda.h>

#include <mutex>

#include "bcmg.h"

namespace {

__device__ __align__(256) double g_noalloc_partials[BCMG_NOALLOC_MAX_BLOCKS];

// Device address of g_noalloc_partials, looked up with cudaGetSymbolAddress
// once per device and CUDA context (with that device current).  In host code
// the array's name is only a host-side stand-in, never a device address.
// The context id (cuCtxGetId, unique for the life of the process) keys the
// cache, so that after a cudaDeviceReset or a re-created primary context the
// address is looked up again instead of reusing one that is no longer mapped.
constexpr int kMaxDevices = 64;
struct PartialsAddr {
  unsigned long long ctx_id;
  double* ptr;
};
PartialsAddr g_partials_addr[kMaxDevices] = {};
std::mutex g_partials_mu;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Driver entry points through the runtime (the library links only cudart).
bool current_context_id(unsigned long long* id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) !=
            cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) !=
            cudaSuccess || q2 != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return false;
    }
    get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
    get_id = reinterpret_cast<CtxGetIdFn>(f2);
  }
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return get_id(ctx, id) == CUDA_SUCCESS;
}

}  // namespace

extern "C" BCMG_API int bcmg_dot_noalloc(int dtype, const void* x, const void* y, int nb, int nx,
                                         int ny, int nz, int vc, int64_t block_stride,
                                         double* result, void* stream) {
  using namespace bcmg;
  if ((dtype != BCMG_F32 && dtype != BCMG_F64) || !x || !y || !result) return BCMG_USAGE;
  if (nb < 0 || nx < 1 || ny < 1 || nz < 1 || vc < 1) return BCMG_USAGE;
  // every brick index the kernels form is an int: the padded plane and the
  // padded brick must fit in int32
  const int64_t sy = (int64_t)nx + 2 * (int64_t)vc;
  const int64_t plane = sy * ((int64_t)ny + 2 * (int64_t)vc);
  const int64_t brick = plane * ((int64_t)nz + 2 * (int64_t)vc);
  if (sy > INT32_MAX || plane > INT32_MAX || brick > INT32_MAX) return BCMG_USAGE;
  if (block_stride < brick) return BCMG_USAGE;
  if (nb > BCMG_NOALLOC_MAX_BLOCKS) return BCMG_SCRATCH_LIMIT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return BCMG_NO_DEVICE;
  }
  if (dev < 0 || dev >= kMaxDevices) return BCMG_USAGE;
  double* part;
  {
    std::lock_guard<std::mutex> lock(g_partials_mu);
    unsigned long long ctx_id = 0;
    const bool have_ctx = current_context_id(&ctx_id);
    if (!have_ctx || !g_partials_addr[dev].ptr || g_partials_addr[dev].ctx_id != ctx_id) {
      // set-up for this device and context (the lookup also makes the
      // device's primary context current on a thread that has none yet)
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_partials) != cudaSuccess || !p) {
        cudaGetLastError();
        return BCMG_CUDA_ERROR;
      }
      if (!current_context_id(&ctx_id)) return BCMG_CUDA_ERROR;
      g_partials_addr[dev].ptr = static_cast<double*>(p);
      g_partials_addr[dev].ctx_id = ctx_id;
    }
    part = g_partials_addr[dev].ptr;
  }
  if (nb == 0) {
    // an empty mesh: the reduction of zero partials writes 0
    return launch_reduce_final(part, 0, result, (cudaStream_t)stream) == cudaSuccess
               ? BCMG_SUCCESS : BCMG_CUDA_ERROR;
  }
  Geom g;
  g.nx = nx; g.ny = ny; g.nz = nz; g.vc = vc;
  g.sy = (int)sy;
  g.sz = (int)plane;
  g.off0 = (int)((1 + sy + plane) * vc);
  g.bstride = block_stride;
  g.nb = nb;
  cudaError_t e = dtype == BCMG_F64
      ? launch_dot_partial<double>((const double*)x, (const double*)y, g, part, (cudaStream_t)stream)
      : launch_dot_partial<float>((const float*)x, (const float*)y, g, part, (cudaStream_t)stream);
  if (e == cudaSuccess) e = launch_reduce_final(part, nb, result, (cudaStream_t)stream);
  return e == cudaSuccess ? BCMG_SUCCESS : BCMG_CUDA_ERROR;
}
